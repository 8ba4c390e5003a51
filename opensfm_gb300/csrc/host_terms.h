// Host constraint terms on shot poses, evaluated in FP64 with forward-mode
// dual numbers: a handful of residuals per constrained shot (or pair or
// triple of shots), far too few to be worth a kernel.  The solver adds
// their Gauss-Newton blocks to the camera-side system on the device.
//
//   absolute orientation  UpVectorError, PanAngleError, TiltAngleError,
//                         RollAngleError (bundle/error/absolute_motion_errors.h:
//                         10-126) under CauchyLoss(1) (bundle_adjuster.cc:
//                         1011-1082); derivatives w.r.t. the rig instance and
//                         rig camera rotations.
//   relative rotation     RelativeRotationError (relative_motion_errors.h:
//                         66-94) under the relative-motion loss
//                         (bundle_adjuster.cc:912-956).
//   common position       CommonPositionError (relative_motion_errors.h:
//                         96-126) under TukeyLoss(1) (bundle_adjuster.cc:
//                         958-999).
//   linear motion         LinearMotionError (motion_prior_errors.h:12-74)
//                         under CauchyLoss(1) (bundle_adjuster.cc:1080-1138).
//   gauge scale           TranslationPriorError (absolute_motion_errors.h:
//                         175-190) between the two gauge shots' rig
//                         instances, no loss (bundle_adjuster.cc:1140-1157).
//   position heatmap      HeatmapdCostFunctor (absolute_motion_errors.h:
//                         128-173): a bicubic lookup of a cost grid at the
//                         shot's horizontal position, no loss
//                         (bundle_adjuster.cc:1000-1009).
//   relative motion       RelativeMotionError (relative_motion_errors.h:
//                         13-64) between two rig instances and their
//                         reconstruction scales, under the relative-motion
//                         loss scaled by the term's robust multiplier
//                         (bundle_adjuster.cc:872-910).
//   adjusted GPS          with SetAdjustAbsolutePositionStd: the position
//                         prior divided by its scale group's std multiplier
//                         (DataPriorError with adjust_scales, prior_error.h:
//                         54-93), and StdDeviationConstraint
//                         (parameters_errors.h:7-16) on each multiplier, no
//                         loss (bundle_adjuster.cc:772-838).
//
// Shot rotation and position compose the rig instance with the rig camera
// as ShotRotationFunctor / ShotPositionFunctor do (position_functors.h:
// 12-63).
#pragma once

#include <algorithm>
#include <cmath>
#include <limits>

namespace gbba {

struct OrientationTerm {
  enum Kind { kUpVector = 0, kPan = 1, kTilt = 2, kRoll = 3 };
  int kind = kUpVector;
  int instance = 0;
  int rig_camera = -1;           // the shot's rig camera (-1: none)
  double target[3] = {0, 0, 0};  // up vector: the direction (normalized here); angles: target[0]
  double scale = 1.0;            // 1 / std deviation
};

// A cost grid of AddHeatmap (bundle_adjuster.cc:331-336): row-major values,
// height = size / width rows, `resolution` metres per cell.
struct HeatmapGrid {
  const double* data = nullptr;
  int width = 0, height = 0;
  double resolution = 1.0;
};

// Constraints between two or three shots (one for a heatmap).  Each shot contributes 12
// derivative slots: instance rotation (0..2), instance position (3..5), rig
// camera rotation (6..8), rig camera position (9..11).
struct RelativeTerm {
  enum Kind {
    kRelativeRotation = 0,
    kCommonPosition = 1,
    kLinearMotion = 2,
    kGaugeScale = 3,
    kHeatmap = 4,
    kRelativeMotion = 5,
    kGpsStd = 6,
    kStdDeviation = 7
  };
  int kind = kRelativeRotation;
  int n_shots = 2;
  int instance[3] = {0, 0, 0};
  int rig_camera[3] = {-1, -1, -1};  // the rig camera used in the composition (-1: none)
  double rotation[3] = {0, 0, 0};    // relative rotation R_ij
  double scale_matrix[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  double margin = 0.0, scale = 1.0;  // common position: margin, 1 / std
  double alpha = 0.0, position_scale = 1.0, orientation_scale = 1.0;  // linear motion
  double distance = 1.0;  // gauge scale: the instances' distance at the start of the run
  HeatmapGrid grid;       // heatmap: the grid, the offsets of its centre, scale = 1 / std
  double x_offset = 0.0, y_offset = 0.0;
  // relative motion: observed rotation, translation and scale, the 7 x 7
  // scale matrix (row-major), whether the scale is observed, the loss
  // scale, and the scale blocks of the two instances (slots 24 and 25)
  double motion[7] = {0, 0, 0, 0, 0, 0, 1};
  double motion_matrix[49] = {};
  bool observed_scale = false;
  double loss_scale = 1.0;
  int scale_block[2] = {-1, -1};
  // GPS prior as a host term (the std multiplier of its scale group, or an
  // optimised camera bias): the position prior and 1 / std per axis; the
  // group's std multiplier is slot 24 (scale_block[0] < 0: none).  With a
  // fixed bias the prior is taken through it as a constant; an optimised
  // bias is read from bias_block[0] (rotation, translation: slots 6..11)
  // and bias_block[1] (scale: slot 25).
  double prior[3] = {0, 0, 0}, prior_scale[3] = {1, 1, 1};
  int bias_camera = -1;
  int bias_block[2] = {-1, -1};
};

namespace orient {

// Value and derivatives w.r.t. N parameters.
template <int N>
struct Dual {
  double v = 0.0;
  double d[N] = {};
  Dual() = default;
  Dual(double x) : v(x) {}  // NOLINT: constants promote implicitly
};
template <int N>
inline Dual<N> var(double x, int k) {
  Dual<N> r(x);
  r.d[k] = 1.0;
  return r;
}
template <int N>
inline Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r(a.v + b.v);
  for (int k = 0; k < N; ++k) r.d[k] = a.d[k] + b.d[k];
  return r;
}
template <int N>
inline Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r(a.v - b.v);
  for (int k = 0; k < N; ++k) r.d[k] = a.d[k] - b.d[k];
  return r;
}
template <int N>
inline Dual<N> operator-(const Dual<N>& a) {
  Dual<N> r(-a.v);
  for (int k = 0; k < N; ++k) r.d[k] = -a.d[k];
  return r;
}
template <int N>
inline Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r(a.v * b.v);
  for (int k = 0; k < N; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
  return r;
}
template <int N>
inline Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r(a.v / b.v);
  for (int k = 0; k < N; ++k) r.d[k] = (a.d[k] * b.v - a.v * b.d[k]) / (b.v * b.v);
  return r;
}
// f(a) with f'(a) = df
template <int N>
inline Dual<N> chain(const Dual<N>& a, double f, double df) {
  Dual<N> r(f);
  for (int k = 0; k < N; ++k) r.d[k] = df * a.d[k];
  return r;
}
template <int N>
inline Dual<N> sqrt(const Dual<N>& a) {
  const double s = std::sqrt(a.v);
  return chain(a, s, s > 0.0 ? 0.5 / s : 0.0);
}
template <int N>
inline Dual<N> sin(const Dual<N>& a) { return chain(a, std::sin(a.v), std::cos(a.v)); }
template <int N>
inline Dual<N> cos(const Dual<N>& a) { return chain(a, std::cos(a.v), -std::sin(a.v)); }
template <int N>
inline Dual<N> asin(const Dual<N>& a) { return chain(a, std::asin(a.v), 1.0 / std::sqrt(1.0 - a.v * a.v)); }
template <int N>
inline Dual<N> abs(const Dual<N>& a) { return a.v < 0.0 ? -a : a; }
template <int N>
inline Dual<N> atan2(const Dual<N>& y, const Dual<N>& x) {
  // d atan2(y, x) = (x dy - y dx) / (x^2 + y^2)
  const double den = x.v * x.v + y.v * y.v;
  Dual<N> r(std::atan2(y.v, x.v));
  for (int k = 0; k < N; ++k) r.d[k] = den > 0.0 ? (x.v * y.d[k] - y.v * x.d[k]) / den : 0.0;
  return r;
}

// Rotations as angle-axis vectors; quaternions scalar first.
template <int N>
inline void aa_to_quat(const Dual<N>* a, Dual<N>* q) {
  const Dual<N> t2 = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
  if (t2.v > 0.0) {
    const Dual<N> t = sqrt(t2);
    const Dual<N> h = t * Dual<N>(0.5);
    const Dual<N> k = sin(h) / t;
    q[0] = cos(h);
    for (int i = 0; i < 3; ++i) q[1 + i] = a[i] * k;
  } else {
    q[0] = Dual<N>(1.0);
    for (int i = 0; i < 3; ++i) q[1 + i] = a[i] * Dual<N>(0.5);
  }
}
template <int N>
inline void quat_mul(const Dual<N>* a, const Dual<N>* b, Dual<N>* r) {
  r[0] = a[0] * b[0] - a[1] * b[1] - a[2] * b[2] - a[3] * b[3];
  r[1] = a[0] * b[1] + a[1] * b[0] + a[2] * b[3] - a[3] * b[2];
  r[2] = a[0] * b[2] - a[1] * b[3] + a[2] * b[0] + a[3] * b[1];
  r[3] = a[0] * b[3] + a[1] * b[2] - a[2] * b[1] + a[3] * b[0];
}
template <int N>
inline void quat_to_aa(const Dual<N>* q, Dual<N>* a) {
  const Dual<N> s2 = q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
  Dual<N> k(2.0);
  if (s2.v > 0.0) {
    const Dual<N> s = sqrt(s2);
    // the angle of the shorter rotation
    const Dual<N> two_theta = q[0].v < 0.0 ? Dual<N>(2.0) * atan2(-s, -q[0]) : Dual<N>(2.0) * atan2(s, q[0]);
    k = two_theta / s;
  }
  for (int i = 0; i < 3; ++i) a[i] = q[1 + i] * k;
}
// the angle-axis of R(a) R(b) (MultRotations, error_utils.h:14-24)
template <int N>
inline void compose(const Dual<N>* a, const Dual<N>* b, Dual<N>* out) {
  Dual<N> qa[4], qb[4], q[4];
  aa_to_quat(a, qa);
  aa_to_quat(b, qb);
  quat_mul(qa, qb, q);
  quat_to_aa(q, out);
}
// R(a) p by the Rodrigues formula (first order for tiny angles)
template <int N>
inline void rotate(const Dual<N>* a, const Dual<N>* p, Dual<N>* out) {
  const Dual<N> t2 = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
  if (t2.v > std::numeric_limits<double>::epsilon()) {
    const Dual<N> t = sqrt(t2);
    const Dual<N> c = cos(t), s = sin(t);
    const Dual<N> w[3] = {a[0] / t, a[1] / t, a[2] / t};
    const Dual<N> wxp[3] = {w[1] * p[2] - w[2] * p[1], w[2] * p[0] - w[0] * p[2], w[0] * p[1] - w[1] * p[0]};
    const Dual<N> wp = w[0] * p[0] + w[1] * p[1] + w[2] * p[2];
    const Dual<N> f = wp * (Dual<N>(1.0) - c);
    for (int i = 0; i < 3; ++i) out[i] = p[i] * c + wxp[i] * s + w[i] * f;
  } else {
    const Dual<N> axp[3] = {a[1] * p[2] - a[2] * p[1], a[2] * p[0] - a[0] * p[2], a[0] * p[1] - a[1] * p[0]};
    for (int i = 0; i < 3; ++i) out[i] = p[i] + axp[i];
  }
}
template <int N>
inline Dual<N> angle_diff(const Dual<N>& a, double b) {
  const Dual<N> d = a - Dual<N>(b);
  if (d.v > M_PI) return d - Dual<N>(2 * M_PI);
  if (d.v < -M_PI) return d + Dual<N>(2 * M_PI);
  return d;
}

// ---- absolute orientation: 6 slots (instance rotation, rig camera rotation)
using D = Dual<6>;

// Residuals of a term (1 or 3) at instance rotation ri and rig camera
// rotation rc; returns the count.
inline int residuals(const OrientationTerm& t, const double* ri, const double* rc, D* r) {
  D a[3], b[3], R[3];
  for (int k = 0; k < 3; ++k) {
    a[k] = var<6>(ri[k], k);
    b[k] = var<6>(rc ? rc[k] : 0.0, 3 + k);
  }
  compose(a, b, R);
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

// ---- relative terms: 12 slots per shot
template <int N>
struct ShotPose {
  Dual<N> rotation[3];  // the shot rotation (instance composed with rig camera)
  Dual<N> position[3];  // the shot position
};

// pose of shot k from instance pose pi[6] and rig camera pose pc[6] (null:
// no rig camera), with slots 12k .. 12k + 11
template <int N>
inline ShotPose<N> shot_pose(int k, const double* pi, const double* pc) {
  ShotPose<N> s;
  Dual<N> ri[3], ti[3];
  for (int i = 0; i < 3; ++i) {
    ri[i] = var<N>(pi[i], 12 * k + i);
    ti[i] = var<N>(pi[3 + i], 12 * k + 3 + i);
  }
  if (!pc) {
    for (int i = 0; i < 3; ++i) {
      s.rotation[i] = ri[i];
      s.position[i] = ti[i];
    }
    return s;
  }
  Dual<N> rc[3], tc[3], off[3];
  for (int i = 0; i < 3; ++i) {
    rc[i] = var<N>(pc[i], 12 * k + 6 + i);
    tc[i] = var<N>(pc[3 + i], 12 * k + 9 + i);
  }
  compose(ri, rc, s.rotation);
  rotate(ri, tc, off);
  for (int i = 0; i < 3; ++i) s.position[i] = ti[i] + off[i];
  return s;
}

// Cubic Hermite (Catmull-Rom) interpolation between p1 and p2 at x in
// [0, 1] with tangents from the neighbours -- the spline of Ceres'
// CubicInterpolator -- and its derivative.
inline double catmull_rom(double p0, double p1, double p2, double p3, double x, double* df) {
  const double a = 0.5 * (-p0 + 3.0 * p1 - 3.0 * p2 + p3);
  const double b = 0.5 * (2.0 * p0 - 5.0 * p1 + 4.0 * p2 - p3);
  const double c = 0.5 * (-p0 + p2);
  if (df) *df = c + x * (2.0 * b + 3.0 * a * x);
  return p1 + x * (c + x * (b + x * a));
}

// Bicubic value of the grid at fractional (row, col), indices clamped to
// the grid (Grid2D's border rule), with d/d row and d/d col.
inline double bicubic(const HeatmapGrid& g, double r, double c, double* dfdr, double* dfdc) {
  auto at = [&](int i, int j) {
    i = std::min(std::max(i, 0), g.height - 1);
    j = std::min(std::max(j, 0), g.width - 1);
    return g.data[size_t(i) * g.width + j];
  };
  const int row = int(std::floor(r)), col = int(std::floor(c));
  double f[4], df[4];
  for (int k = 0; k < 4; ++k) {
    const int i = row - 1 + k;
    f[k] = catmull_rom(at(i, col - 1), at(i, col), at(i, col + 1), at(i, col + 2), c - col, &df[k]);
  }
  const double v = catmull_rom(f[0], f[1], f[2], f[3], r - row, dfdr);
  *dfdc = catmull_rom(df[0], df[1], df[2], df[3], r - row, nullptr);
  return v;
}

// Scaled residuals (at most 7) of a relative term from the shots' instance
// and rig camera poses (pc[k] null: no rig camera) and, for a relative
// motion, the two reconstruction scales (slots 24 and 25); returns the
// count.
template <int N>
inline int relative_residuals(const RelativeTerm& t, const double* const* pi, const double* const* pc, Dual<N>* r,
                              const double* scales = nullptr, const double* bias = nullptr) {
  ShotPose<N> s[3];
  for (int k = 0; k < t.n_shots; ++k) s[k] = shot_pose<N>(k, pi[k], t.kind == RelativeTerm::kRelativeMotion ? nullptr : pc[k]);
  switch (t.kind) {
    case RelativeTerm::kGpsStd: {
      // (t_k - prior_k) / (std_k m) on the instance position; with an
      // optimised bias (angle-axis w, translation b, scale c) the prior is
      // c R(w) p + b (SimilarityPriorTransform, bias.h:34-54)
      const Dual<N> m = var<N>(scales[0], 24);
      Dual<N> prior[3];
      if (bias) {
        Dual<N> w[3], p[3], rp[3];
        for (int k = 0; k < 3; ++k) {
          w[k] = var<N>(bias[k], 6 + k);
          p[k] = Dual<N>(t.prior[k]);
        }
        rotate(w, p, rp);
        const Dual<N> c = var<N>(bias[6], 25);
        for (int k = 0; k < 3; ++k) prior[k] = c * rp[k] + var<N>(bias[3 + k], 9 + k);
      } else {
        for (int k = 0; k < 3; ++k) prior[k] = Dual<N>(t.prior[k]);
      }
      for (int k = 0; k < 3; ++k) r[k] = Dual<N>(t.prior_scale[k]) * (s[0].position[k] - prior[k]) / m;
      return 3;
    }
    case RelativeTerm::kStdDeviation: {
      // log(1 / sqrt(2 pi m^2))
      const double m = scales[0];
      r[0] = Dual<N>(std::log(1.0 / std::sqrt(2.0 * M_PI * m * m)));
      r[0].d[24] = -1.0 / m;
      return 1;
    }
    case RelativeTerm::kRelativeMotion: {
      // rotation log(R_ij R_i^T R_j); translation t_ij - s_j R_j^T (t_i -
      // t_j); scale S_ij - s_j / s_i when observed; times the scale matrix.
      // A zero scale makes the residual undefined (the functor fails).
      const Dual<N> si = var<N>(scales[0], 24), sj = var<N>(scales[1], 25);
      Dual<N> e[7], rij[3], neg_i[3], neg_j[3], tmp[3], d[3], rd[3];
      for (int i = 0; i < 3; ++i) {
        rij[i] = Dual<N>(t.motion[i]);
        neg_i[i] = -s[0].rotation[i];
        neg_j[i] = -s[1].rotation[i];
        d[i] = s[0].position[i] - s[1].position[i];
      }
      compose(rij, neg_i, tmp);
      compose(tmp, s[1].rotation, e);
      rotate(neg_j, d, rd);
      for (int i = 0; i < 3; ++i) e[3 + i] = Dual<N>(t.motion[3 + i]) - sj * rd[i];
      e[6] = t.observed_scale ? Dual<N>(t.motion[6]) - sj / si : Dual<N>(0.0);
      const bool undefined = scales[0] == 0.0 || scales[1] == 0.0;
      for (int i = 0; i < 7; ++i) {
        Dual<N> acc(0.0);
        for (int j = 0; j < 7; ++j) acc = acc + Dual<N>(t.motion_matrix[7 * i + j]) * e[j];
        r[i] = undefined ? Dual<N>(std::numeric_limits<double>::quiet_NaN()) : acc;
      }
      return 7;
    }
    case RelativeTerm::kRelativeRotation: {
      // log(R_ij R_i^T R_j), then the scale matrix
      Dual<N> rij[3], neg[3], tmp[3], e[3];
      for (int i = 0; i < 3; ++i) {
        rij[i] = Dual<N>(t.rotation[i]);
        neg[i] = -s[0].rotation[i];
      }
      compose(rij, neg, tmp);
      compose(tmp, s[1].rotation, e);
      for (int i = 0; i < 3; ++i)
        r[i] = Dual<N>(t.scale_matrix[3 * i]) * e[0] + Dual<N>(t.scale_matrix[3 * i + 1]) * e[1] +
               Dual<N>(t.scale_matrix[3 * i + 2]) * e[2];
      return 3;
    }
    case RelativeTerm::kCommonPosition: {
      for (int i = 0; i < 3; ++i) {
        Dual<N> e = s[0].position[i] - s[1].position[i];
        if (i < 2) {
          e = abs(e) - Dual<N>(t.margin);
          if (e.v < 0.0) e = Dual<N>(0.0);
        }
        r[i] = Dual<N>(t.scale) * e;
      }
      return 3;
    }
    case RelativeTerm::kHeatmap: {
      // grid row = height / 2 - (y - y_offset) / resolution, column = width
      // / 2 + (x - x_offset) / resolution
      const HeatmapGrid& g = t.grid;
      const Dual<N> row = Dual<N>(0.5 * g.height) - (s[0].position[1] - Dual<N>(t.y_offset)) / Dual<N>(g.resolution);
      const Dual<N> col = Dual<N>(0.5 * g.width) + (s[0].position[0] - Dual<N>(t.x_offset)) / Dual<N>(g.resolution);
      double dfdr, dfdc;
      const double v = bicubic(g, row.v, col.v, &dfdr, &dfdc);
      Dual<N> f(v);
      for (int k = 0; k < N; ++k) f.d[k] = dfdr * row.d[k] + dfdc * col.d[k];
      r[0] = Dual<N>(t.scale) * f;
      return 1;
    }
    case RelativeTerm::kGaugeScale: {
      // log(|t_0 - t_1| / distance) on the rig instance positions alone
      Dual<N> d[3];
      for (int i = 0; i < 3; ++i) d[i] = var<N>(pi[0][3 + i], 3 + i) - var<N>(pi[1][3 + i], 15 + i);
      const Dual<N> n = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      r[0] = chain(n, std::log(n.v / t.distance), 1.0 / n.v);
      return 1;
    }
    default: {  // linear motion: shot 1 between shots 0 and 2 at fraction alpha
      Dual<N> d20[3], d10[3];
      for (int i = 0; i < 3; ++i) {
        d20[i] = s[2].position[i] - s[0].position[i];
        d10[i] = s[1].position[i] - s[0].position[i];
      }
      const Dual<N> n20 = sqrt(d20[0] * d20[0] + d20[1] * d20[1] + d20[2] * d20[2]);
      const Dual<N> n10 = sqrt(d10[0] * d10[0] + d10[1] * d10[1] + d10[2] * d10[2]);
      for (int i = 0; i < 3; ++i) {
        if (n20.v > 1e-15) r[i] = Dual<N>(t.position_scale) * (Dual<N>(t.alpha) - n10 / n20);
        else r[i] = Dual<N>(t.position_scale) * (Dual<N>(t.alpha) * d20[i] - d10[i]);
      }
      Dual<N> neg0[3], neg1[3], a[3], b[3], e[3];
      for (int i = 0; i < 3; ++i) {
        neg0[i] = -s[0].rotation[i];
        neg1[i] = -s[1].rotation[i];
      }
      compose(s[2].rotation, neg0, a);
      for (int i = 0; i < 3; ++i) a[i] = Dual<N>(t.alpha) * a[i];
      compose(s[0].rotation, neg1, b);
      compose(a, b, e);
      for (int i = 0; i < 3; ++i) r[3 + i] = Dual<N>(t.orientation_scale) * e[i];
      return 6;
    }
  }
}

// ---- losses
// rho(s) and its derivatives for the loss kinds of the projection loss
// (0 trivial, 1 Huber, 2 soft-L1, 3 Cauchy, 4 arctan) and 5 Tukey, scale a
// (Ceres' documented definitions).
inline void loss_rho(int kind, double a, double s, double* rho) {
  const double b = a * a;
  switch (kind) {
    case 1:
      if (s > b) {
        const double r = std::sqrt(s);
        rho[0] = 2.0 * a * r - b;
        rho[1] = std::max(std::numeric_limits<double>::min(), a / r);
        rho[2] = -rho[1] / (2.0 * s);
      } else {
        rho[0] = s, rho[1] = 1.0, rho[2] = 0.0;
      }
      return;
    case 2: {
      const double sum = 1.0 + s / b, tmp = std::sqrt(sum);
      rho[0] = 2.0 * b * (tmp - 1.0);
      rho[1] = std::max(std::numeric_limits<double>::min(), 1.0 / tmp);
      rho[2] = -(0.5 / b) * rho[1] / sum;
      return;
    }
    case 3: {
      const double sum = 1.0 + s / b, inv = 1.0 / sum;
      rho[0] = b * std::log1p(s / b);
      rho[1] = std::max(std::numeric_limits<double>::min(), inv);
      rho[2] = -inv * inv / b;
      return;
    }
    case 4: {
      const double inv = 1.0 / (b + s * s);
      rho[0] = a * std::atan2(s, a);
      rho[1] = std::max(std::numeric_limits<double>::min(), b * inv);
      rho[2] = -2.0 * s * b * inv * inv;
      return;
    }
    case 5:
      if (s <= b) {
        const double v = 1.0 - s / b;
        rho[0] = b / 3.0 * (1.0 - v * v * v);
        rho[1] = v * v;
        rho[2] = -2.0 * v / b;
      } else {
        rho[0] = b / 3.0, rho[1] = 0.0, rho[2] = 0.0;
      }
      return;
    default:
      rho[0] = s, rho[1] = 1.0, rho[2] = 0.0;
  }
}

// Loss times the IRLS weight w with the residual/Jacobian correction Ceres
// applies (Triggs et al.): r <- sqrt(rho') r / (1 - alpha), J <- sqrt(rho')
// (J - alpha r r^T J / |r|^2), alpha from rho''; alpha = 0 when rho'' <= 0.
// Returns w rho(|r|^2).
template <int N>
inline double loss_correct(int kind, double a, int m, Dual<N>* r, double w = 1.0) {
  double s = 0.0;
  for (int q = 0; q < m; ++q) s += r[q].v * r[q].v;
  double rho[3];
  loss_rho(kind, a, s, rho);
  for (double& v : rho) v *= w;
  const double sq1 = std::sqrt(rho[1]);
  double rscale = sq1, alpha_s = 0.0;
  if (s > 0.0 && rho[2] > 0.0) {
    const double alpha = 1.0 - std::sqrt(1.0 + 2.0 * s * rho[2] / rho[1]);
    rscale = sq1 / (1.0 - alpha);
    alpha_s = alpha / s;
  }
  for (int k = 0; k < N; ++k) {
    double rj = 0.0;
    for (int q = 0; q < m; ++q) rj += r[q].v * r[q].d[k];
    for (int q = 0; q < m; ++q) r[q].d[k] = sq1 * (r[q].d[k] - alpha_s * r[q].v * rj);
  }
  for (int q = 0; q < m; ++q) r[q].v *= rscale;
  return rho[0];
}

// Cauchy loss (a = 1) times the IRLS weight w, the loss of the orientation
// constraints.  Returns w rho(s).
inline double cauchy_correct(int m, D* r, double w = 1.0) { return loss_correct<6>(3, 1.0, m, r, w); }

}  // namespace orient
}  // namespace gbba
