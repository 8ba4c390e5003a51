// Absolute orientation constraints of a shot: up vector, pan, tilt and roll
// (bundle/error/absolute_motion_errors.h: UpVectorError, PanAngleError,
// TiltAngleError, RollAngleError), each under CauchyLoss(1) as
// BundleAdjuster::Run adds them (bundle_adjuster.cc:1013-1082).  They depend
// on the shot rotation, the rig instance rotation composed with the rig
// camera rotation (position_functors.h:40-63).  A handful of residuals per
// shot: evaluated on the host in FP64, with the Jacobian w.r.t. the two
// rotations from forward-mode dual numbers.
#pragma once

#include <cmath>
#include <limits>

namespace gbba {

struct OrientationTerm {
  enum Kind { kUpVector = 0, kPan = 1, kTilt = 2, kRoll = 3 };
  int kind = kUpVector;
  int instance = 0;
  int rig_camera = -1;         // the shot's rig camera (-1: none)
  double target[3] = {0, 0, 0};  // up vector: the direction (normalized here); angles: target[0]
  double scale = 1.0;          // 1 / std deviation
};

namespace orient {

// Value and derivatives w.r.t. the instance rotation (0..2) and the rig
// camera rotation (3..5).
constexpr int kN = 6;
struct D {
  double v = 0.0;
  double d[kN] = {0, 0, 0, 0, 0, 0};
  D() = default;
  D(double x) : v(x) {}  // NOLINT: constants promote implicitly
};
inline D var(double x, int k) {
  D r(x);
  r.d[k] = 1.0;
  return r;
}
inline D operator+(const D& a, const D& b) {
  D r(a.v + b.v);
  for (int k = 0; k < kN; ++k) r.d[k] = a.d[k] + b.d[k];
  return r;
}
inline D operator-(const D& a, const D& b) {
  D r(a.v - b.v);
  for (int k = 0; k < kN; ++k) r.d[k] = a.d[k] - b.d[k];
  return r;
}
inline D operator-(const D& a) {
  D r(-a.v);
  for (int k = 0; k < kN; ++k) r.d[k] = -a.d[k];
  return r;
}
inline D operator*(const D& a, const D& b) {
  D r(a.v * b.v);
  for (int k = 0; k < kN; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
  return r;
}
inline D operator/(const D& a, const D& b) {
  D r(a.v / b.v);
  for (int k = 0; k < kN; ++k) r.d[k] = (a.d[k] * b.v - a.v * b.d[k]) / (b.v * b.v);
  return r;
}
// f(a) with f'(a) = df
inline D chain(const D& a, double f, double df) {
  D r(f);
  for (int k = 0; k < kN; ++k) r.d[k] = df * a.d[k];
  return r;
}
inline D sqrt(const D& a) {
  const double s = std::sqrt(a.v);
  return chain(a, s, s > 0.0 ? 0.5 / s : 0.0);
}
inline D sin(const D& a) { return chain(a, std::sin(a.v), std::cos(a.v)); }
inline D cos(const D& a) { return chain(a, std::cos(a.v), -std::sin(a.v)); }
inline D asin(const D& a) { return chain(a, std::asin(a.v), 1.0 / std::sqrt(1.0 - a.v * a.v)); }
inline D atan2(const D& y, const D& x) {
  // d atan2(y, x) = (x dy - y dx) / (x^2 + y^2)
  const double den = x.v * x.v + y.v * y.v;
  D r(std::atan2(y.v, x.v));
  for (int k = 0; k < kN; ++k) r.d[k] = den > 0.0 ? (x.v * y.d[k] - y.v * x.d[k]) / den : 0.0;
  return r;
}

// Rotations as angle-axis vectors; quaternions scalar first.
inline void aa_to_quat(const D* a, D* q) {
  const D t2 = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
  if (t2.v > 0.0) {
    const D t = sqrt(t2);
    const D h = t * D(0.5);
    const D k = sin(h) / t;
    q[0] = cos(h);
    for (int i = 0; i < 3; ++i) q[1 + i] = a[i] * k;
  } else {
    q[0] = D(1.0);
    for (int i = 0; i < 3; ++i) q[1 + i] = a[i] * D(0.5);
  }
}
inline void quat_mul(const D* a, const D* b, D* r) {
  r[0] = a[0] * b[0] - a[1] * b[1] - a[2] * b[2] - a[3] * b[3];
  r[1] = a[0] * b[1] + a[1] * b[0] + a[2] * b[3] - a[3] * b[2];
  r[2] = a[0] * b[2] - a[1] * b[3] + a[2] * b[0] + a[3] * b[1];
  r[3] = a[0] * b[3] + a[1] * b[2] - a[2] * b[1] + a[3] * b[0];
}
inline void quat_to_aa(const D* q, D* a) {
  const D s2 = q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
  D k(2.0);
  if (s2.v > 0.0) {
    const D s = sqrt(s2);
    // the angle of the shorter rotation
    const D two_theta = q[0].v < 0.0 ? D(2.0) * atan2(-s, -q[0]) : D(2.0) * atan2(s, q[0]);
    k = two_theta / s;
  }
  for (int i = 0; i < 3; ++i) a[i] = q[1 + i] * k;
}
// R(a) p by the Rodrigues formula (first order for tiny angles)
inline void rotate(const D* a, const D* p, D* out) {
  const D t2 = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
  if (t2.v > std::numeric_limits<double>::epsilon()) {
    const D t = sqrt(t2);
    const D c = cos(t), s = sin(t);
    const D w[3] = {a[0] / t, a[1] / t, a[2] / t};
    const D wxp[3] = {w[1] * p[2] - w[2] * p[1], w[2] * p[0] - w[0] * p[2], w[0] * p[1] - w[1] * p[0]};
    const D wp = w[0] * p[0] + w[1] * p[1] + w[2] * p[2];
    const D f = wp * (D(1.0) - c);
    for (int i = 0; i < 3; ++i) out[i] = p[i] * c + wxp[i] * s + w[i] * f;
  } else {
    const D axp[3] = {a[1] * p[2] - a[2] * p[1], a[2] * p[0] - a[0] * p[2], a[0] * p[1] - a[1] * p[0]};
    for (int i = 0; i < 3; ++i) out[i] = p[i] + axp[i];
  }
}
inline D angle_diff(const D& a, double b) {
  const D d = a - D(b);
  if (d.v > M_PI) return d - D(2 * M_PI);
  if (d.v < -M_PI) return d + D(2 * M_PI);
  return d;
}

// Residuals of a term (1 or 3) at instance rotation ri and rig camera
// rotation rc; returns the count.
inline int residuals(const OrientationTerm& t, const double* ri, const double* rc, D* r) {
  D a[3], b[3], qa[4], qb[4], q[4], R[3];
  for (int k = 0; k < 3; ++k) {
    a[k] = var(ri[k], k);
    b[k] = var(rc ? rc[k] : 0.0, 3 + k);
  }
  aa_to_quat(a, qa);
  aa_to_quat(b, qb);
  quat_mul(qa, qb, q);
  quat_to_aa(q, R);
  const D ex[3] = {D(1.0), D(0.0), D(0.0)};
  const D ez[3] = {D(0.0), D(0.0), D(1.0)};
  switch (t.kind) {
    case OrientationTerm::kUpVector: {
      const D up[3] = {D(t.target[0]), D(t.target[1]), D(t.target[2])};
      D zw[3];
      rotate(R, up, zw);
      for (int k = 0; k < 3; ++k) r[k] = D(t.scale) * (zw[k] - ez[k]);
      return 3;
    }
    case OrientationTerm::kPan: {
      D zw[3];
      rotate(R, ez, zw);
      if (std::fabs(zw[0].v) < 1e-8 && std::fabs(zw[1].v) < 1e-8) r[0] = D(0.0);
      else r[0] = D(t.scale) * angle_diff(atan2(zw[0], zw[1]), t.target[0]);
      return 1;
    }
    case OrientationTerm::kTilt: {
      D z[3];
      rotate(R, ez, z);
      const D l = sqrt(z[0] * z[0] + z[1] * z[1]);
      r[0] = D(t.scale) * angle_diff(-atan2(z[2], l), t.target[0]);
      return 1;
    }
    default: {  // roll
      D x[3], z[3];
      rotate(R, ex, x);
      rotate(R, ez, z);
      D h[3] = {z[1], -z[0], D(0.0)};
      const D lh = sqrt(h[0] * h[0] + h[1] * h[1]);
      const double eps = 1e-5;
      if (lh.v < eps) {
        r[0] = D(0.0);
        return 1;
      }
      h[0] = h[0] / lh;
      h[1] = h[1] / lh;
      const D c[3] = {x[1] * h[2] - x[2] * h[1], x[2] * h[0] - x[0] * h[2], x[0] * h[1] - x[1] * h[0]};
      const D sin_roll = z[0] * c[0] + z[1] * c[1] + z[2] * c[2];
      if (sin_roll.v <= -(1.0 - eps)) {
        r[0] = D(0.0);
        return 1;
      }
      r[0] = D(t.scale) * angle_diff(asin(sin_roll), t.target[0]);
      return 1;
    }
  }
}

// Cauchy loss (a = 1) times the IRLS weight w, with the Gauss-Newton
// correction Ceres applies when rho'' < 0: residual and Jacobian scaled by
// sqrt(w rho'(s)).  Returns w rho(s).
inline double cauchy_correct(int m, D* r, double w = 1.0) {
  double s = 0.0;
  for (int q = 0; q < m; ++q) s += r[q].v * r[q].v;
  const double rho = std::log1p(s);
  const double sq = std::sqrt(w / (1.0 + s));
  for (int q = 0; q < m; ++q) r[q] = r[q] * D(sq);
  return w * rho;
}

}  // namespace orient
}  // namespace gbba
