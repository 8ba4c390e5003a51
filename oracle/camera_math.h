// Oracle (test infrastructure only) -- FP64 CPU restatement of the camera
// models and pose transform on the bundle-adjustment path of OpenSfM.
//
// This header is the checker for the CUDA kernels: only tests, the smoke
// entry point and the bench's CPU-baseline leg may link it.  Nothing in the
// product path includes it.
//
// Every model is written as PROJ -> DISTO -> AFFINE with the parameter
// vector ordered [PROJ params | DISTO params | AFFINE params], as the
// reference composes them:
//   opensfm/src/lib/geometry/camera_instances.h:138-199 (ProjectGeneric,
//     model aliases), :8-20 (ProjectionType order)
//   opensfm/src/lib/geometry/functions.h:28-97 (chain rule, parameter order)
//   opensfm/src/lib/geometry/src/camera.cc:11-172 (parameter order per model)
// Forward maps follow
//   camera_projections_functions.h:8-230, camera_distortions_functions.h:12-837,
//   transformations_functions.h:13-107.
// The analytic derivatives restate the closed forms of those files; tests
// check them against the dual-number forward-mode AD below and against FP64
// central differences.
#pragma once

#include <cmath>
#include <cstring>

namespace oracle {

enum Model {
  PERSPECTIVE = 0,
  BROWN = 1,
  FISHEYE = 2,
  FISHEYE_OPENCV = 3,
  FISHEYE62 = 4,
  FISHEYE624 = 5,
  SPHERICAL = 6,
  DUAL = 7,
  RADIAL = 8,
  SIMPLE_RADIAL = 9,
  NUM_MODELS = 10
};

enum ProjKind { P_PERSPECTIVE, P_FISHEYE, P_DUAL, P_SPHERICAL };
enum DistoKind { D_NONE, D_K1, D_K1K2, D_K1K4, D_BROWN, D_62, D_624 };
enum AffKind { A_NONE, A_SCALE, A_AFFINE };

struct ModelDesc {
  ProjKind proj;
  DistoKind disto;
  AffKind aff;
  int n_proj, n_disto, n_aff;  // parameter counts
  int n_params;                // max(1, sum) -- spherical keeps 1 dummy
};

inline int disto_size(DistoKind d) {
  switch (d) {
    case D_NONE: return 0;
    case D_K1: return 1;
    case D_K1K2: return 2;
    case D_K1K4: return 4;
    case D_BROWN: return 5;
    case D_62: return 8;
    case D_624: return 12;
  }
  return 0;
}
inline int aff_size(AffKind a) { return a == A_NONE ? 0 : (a == A_SCALE ? 1 : 4); }

inline ModelDesc model_desc(int m) {
  ModelDesc d{};
  switch (m) {
    case PERSPECTIVE: d = {P_PERSPECTIVE, D_K1K2, A_SCALE}; break;
    case BROWN: d = {P_PERSPECTIVE, D_BROWN, A_AFFINE}; break;
    case FISHEYE: d = {P_FISHEYE, D_K1K2, A_SCALE}; break;
    case FISHEYE_OPENCV: d = {P_FISHEYE, D_K1K4, A_AFFINE}; break;
    case FISHEYE62: d = {P_FISHEYE, D_62, A_AFFINE}; break;
    case FISHEYE624: d = {P_FISHEYE, D_624, A_AFFINE}; break;
    case SPHERICAL: d = {P_SPHERICAL, D_NONE, A_NONE}; break;
    case DUAL: d = {P_DUAL, D_K1K2, A_SCALE}; break;
    case RADIAL: d = {P_PERSPECTIVE, D_K1K2, A_AFFINE}; break;
    case SIMPLE_RADIAL: d = {P_PERSPECTIVE, D_K1, A_AFFINE}; break;
  }
  d.n_proj = (d.proj == P_DUAL) ? 1 : 0;
  d.n_disto = disto_size(d.disto);
  d.n_aff = aff_size(d.aff);
  int s = d.n_proj + d.n_disto + d.n_aff;
  d.n_params = s < 1 ? 1 : s;
  return d;
}

// ---------------------------------------------------------------------------
// Forward-mode dual numbers (used as the autodiff check of the analytic
// Jacobians, the role Eigen::AutoDiffScalar plays in the reference tests
// bundle/test/reprojection_errors_test.cc:23-190).
template <int N>
struct Dual {
  double v;
  double d[N];
  Dual() : v(0) { std::memset(d, 0, sizeof(d)); }
  Dual(double x) : v(x) { std::memset(d, 0, sizeof(d)); }  // NOLINT
  static Dual var(double x, int i) {
    Dual r(x);
    r.d[i] = 1.0;
    return r;
  }
};
template <int N> inline Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r(a.v + b.v);
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <int N> inline Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r(a.v - b.v);
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <int N> inline Dual<N> operator-(const Dual<N>& a) {
  Dual<N> r(-a.v);
  for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
  return r;
}
template <int N> inline Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r(a.v * b.v);
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
template <int N> inline Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r(a.v / b.v);
  const double ib = 1.0 / b.v;
  for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
  return r;
}
template <int N> inline Dual<N> operator+(const Dual<N>& a, double b) { return a + Dual<N>(b); }
template <int N> inline Dual<N> operator+(double a, const Dual<N>& b) { return Dual<N>(a) + b; }
template <int N> inline Dual<N> operator-(const Dual<N>& a, double b) { return a - Dual<N>(b); }
template <int N> inline Dual<N> operator-(double a, const Dual<N>& b) { return Dual<N>(a) - b; }
template <int N> inline Dual<N> operator*(const Dual<N>& a, double b) { return a * Dual<N>(b); }
template <int N> inline Dual<N> operator*(double a, const Dual<N>& b) { return Dual<N>(a) * b; }
template <int N> inline Dual<N> operator/(const Dual<N>& a, double b) { return a / Dual<N>(b); }
template <int N> inline Dual<N> operator/(double a, const Dual<N>& b) { return Dual<N>(a) / b; }
template <int N> inline bool operator>(const Dual<N>& a, double b) { return a.v > b; }
template <int N> inline bool operator<(const Dual<N>& a, double b) { return a.v < b; }
template <int N> inline Dual<N> sqrt(const Dual<N>& a) {
  Dual<N> r(std::sqrt(a.v));
  const double k = 0.5 / r.v;
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * k;
  return r;
}
template <int N> inline Dual<N> sin(const Dual<N>& a) {
  Dual<N> r(std::sin(a.v));
  const double c = std::cos(a.v);
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * c;
  return r;
}
template <int N> inline Dual<N> cos(const Dual<N>& a) {
  Dual<N> r(std::cos(a.v));
  const double s = -std::sin(a.v);
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * s;
  return r;
}
template <int N> inline Dual<N> log(const Dual<N>& a) {
  Dual<N> r(std::log(a.v));
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] / a.v;
  return r;
}
template <int N> inline Dual<N> atan2(const Dual<N>& y, const Dual<N>& x) {
  Dual<N> r(std::atan2(y.v, x.v));
  const double den = 1.0 / (x.v * x.v + y.v * y.v);
  for (int i = 0; i < N; ++i) r.d[i] = (x.v * y.d[i] - y.v * x.d[i]) * den;
  return r;
}
inline double value_of(double x) { return x; }
template <int N> inline double value_of(const Dual<N>& x) { return x.v; }

// ---------------------------------------------------------------------------
// Forward maps (generic scalar T, so the same code runs on Dual for AD).

// camera_projections_functions.h:67-72 (perspective), :8-15 (fisheye),
// :99-112 (dual), :193-202 (spherical).  The fisheye radius uses only x,y
// (functions.h:6-9 SquaredNorm sums the first two components).
template <class T>
inline void proj_forward(ProjKind k, const T* p, const T* prm, T* out) {
  using std::atan2;
  using std::sqrt;
  switch (k) {
    case P_PERSPECTIVE:
      out[0] = p[0] / p[2];
      out[1] = p[1] / p[2];
      break;
    case P_FISHEYE: {
      const T r = sqrt(p[0] * p[0] + p[1] * p[1]);
      const T th = atan2(r, p[2]);
      out[0] = th / r * p[0];
      out[1] = th / r * p[1];
      break;
    }
    case P_DUAL: {
      const T px = p[0] / p[2], py = p[1] / p[2];
      const T r = sqrt(p[0] * p[0] + p[1] * p[1]);
      const T th = atan2(r, p[2]);
      const T fx = th / r * p[0], fy = th / r * p[1];
      out[0] = prm[0] * px + (1.0 - prm[0]) * fx;
      out[1] = prm[0] * py + (1.0 - prm[0]) * fy;
      break;
    }
    case P_SPHERICAL: {
      const T lon = atan2(p[0], p[2]);
      const T lat = atan2(-p[1], sqrt(p[0] * p[0] + p[2] * p[2]));
      out[0] = lon * (1.0 / (2.0 * M_PI));
      out[1] = -lat * (1.0 / (2.0 * M_PI));
      break;
    }
  }
}

// camera_distortions_functions.h: Disto2 :16-21, Disto24 :106-112,
// Disto2468 :207-214, Disto62 :331-345, Disto624 :509-532, DistoBrown :706-716.
template <class T>
inline void disto_forward(DistoKind k, const T* q, const T* c, T* out) {
  const T x = q[0], y = q[1];
  const T r2 = x * x + y * y;
  T radial = T(1.0), tx = T(0.0), ty = T(0.0);
  switch (k) {
    case D_NONE:
      out[0] = x;
      out[1] = y;
      return;
    case D_K1: radial = 1.0 + r2 * c[0]; break;
    case D_K1K2: radial = 1.0 + r2 * (c[0] + c[1] * r2); break;
    case D_K1K4: radial = 1.0 + r2 * (c[0] + r2 * (c[1] + r2 * (c[2] + r2 * c[3]))); break;
    case D_BROWN:
      radial = 1.0 + r2 * (c[0] + r2 * (c[1] + r2 * c[2]));
      tx = 2.0 * c[3] * x * y + c[4] * (r2 + 2.0 * x * x);
      ty = 2.0 * c[4] * x * y + c[3] * (r2 + 2.0 * y * y);
      break;
    case D_62:
    case D_624:
      radial = 1.0 + r2 * (c[0] + r2 * (c[1] + r2 * (c[2] + r2 * (c[3] + r2 * (c[4] + r2 * c[5])))));
      tx = 2.0 * c[6] * x * y + c[7] * (r2 + 2.0 * x * x);
      ty = 2.0 * c[7] * x * y + c[6] * (r2 + 2.0 * y * y);
      if (k == D_624) {
        tx = tx + c[8] * r2 + c[9] * r2 * r2;
        ty = ty + c[10] * r2 + c[11] * r2 * r2;
      }
      break;
  }
  out[0] = x * radial + tx;
  out[1] = y * radial + ty;
}

// transformations_functions.h: Affine :13-33 [focal, aspect, cx, cy],
// UniformScale :53-62 [focal], Identity :84-91.
template <class T>
inline void aff_forward(AffKind k, const T* q, const T* a, T* out) {
  switch (k) {
    case A_NONE:
      out[0] = q[0];
      out[1] = q[1];
      break;
    case A_SCALE:
      out[0] = a[0] * q[0];
      out[1] = a[0] * q[1];
      break;
    case A_AFFINE:
      out[0] = a[0] * q[0] + a[2];
      out[1] = a[0] * a[1] * q[1] + a[3];
      break;
  }
}

template <class T>
inline void project(int model, const T* p, const T* params, T* uv) {
  const ModelDesc d = model_desc(model);
  T a[2], b[2];
  proj_forward<T>(d.proj, p, params, a);
  disto_forward<T>(d.disto, a, params + d.n_proj, b);
  aff_forward<T>(d.aff, b, params + d.n_proj + d.n_disto, uv);
}

// ---------------------------------------------------------------------------
// Analytic derivatives (double).  Layout: J_in is 2x3 (projection) or 2x2
// row-major; J_prm is 2xP row-major.

// camera_projections_functions.h:74-87 (perspective), :17-47 (fisheye),
// :114-150 (dual), :204-220 (spherical).
inline void proj_jac(ProjKind k, const double* p, const double* prm, double* out,
                     double* Jin /*2x3*/, double* Jprm /*2x1*/) {
  const double x = p[0], y = p[1], z = p[2];
  auto fisheye_jac = [&](double* J) {
    const double r2 = x * x + y * y, r = std::sqrt(r2), R2 = r2 + z * z;
    const double th = std::atan2(r, z);
    const double x2 = x * x, y2 = y * y, z2 = z * z;
    const double inv = 1.0 / (r2 * R2 * r);
    J[0] = (x2 * y2 * th + y2 * y2 * th + y2 * z2 * th + x2 * z * r) * inv;
    J[1] = x * (y * z * r - y * th * R2) * inv;
    J[2] = -x / R2;
    J[3] = y * (x * z * r - x * th * R2) * inv;
    J[4] = (x2 * y2 * th + x2 * x2 * th + x2 * z2 * th + y2 * z * r) * inv;
    J[5] = -y / R2;
  };
  auto persp_jac = [&](double* J) {
    J[0] = 1.0 / z;
    J[1] = 0.0;
    J[2] = -x / (z * z);
    J[3] = 0.0;
    J[4] = 1.0 / z;
    J[5] = -y / (z * z);
  };
  proj_forward<double>(k, p, prm, out);
  switch (k) {
    case P_PERSPECTIVE: persp_jac(Jin); break;
    case P_FISHEYE: fisheye_jac(Jin); break;
    case P_DUAL: {
      double Jp[6], Jf[6], pp[2], pf[2];
      persp_jac(Jp);
      fisheye_jac(Jf);
      proj_forward<double>(P_PERSPECTIVE, p, prm, pp);
      proj_forward<double>(P_FISHEYE, p, prm, pf);
      for (int i = 0; i < 6; ++i) Jin[i] = prm[0] * Jp[i] + (1.0 - prm[0]) * Jf[i];
      Jprm[0] = pp[0] - pf[0];
      Jprm[1] = pp[1] - pf[1];
      break;
    }
    case P_SPHERICAL: {
      const double rt2 = x * x + z * z, rt = std::sqrt(rt2);
      const double R2 = x * x + y * y + z * z;
      const double tp = 2.0 * M_PI;
      Jin[0] = z / (tp * rt2);
      Jin[1] = 0.0;
      Jin[2] = -x / (tp * rt2);
      Jin[3] = -(x * y) / (tp * R2 * rt);
      Jin[4] = rt / (tp * R2);
      Jin[5] = -(y * z) / (tp * R2 * rt);
      break;
    }
  }
}

// Distortion derivatives: camera_distortions_functions.h:23-44 (Disto2),
// :114-142 (Disto24), :216-258 (Disto2468), :347-411 (Disto62),
// :534-617 (Disto624), :718-764 (DistoBrown).
inline void disto_jac(DistoKind k, const double* q, const double* c, double* out,
                      double* Jin /*2x2*/, double* Jprm /*2xP*/) {
  const double x = q[0], y = q[1];
  const double x2 = x * x, y2 = y * y, r2 = x2 + y2;
  const int P = disto_size(k);
  disto_forward<double>(k, q, c, out);
  switch (k) {
    case D_NONE:
      Jin[0] = 1; Jin[1] = 0; Jin[2] = 0; Jin[3] = 1;
      return;
    case D_K1: {
      const double k1 = c[0];
      Jin[0] = 3.0 * k1 * x2 + k1 * y2 + 1.0;
      Jin[1] = x * 2.0 * k1 * y;
      Jin[2] = y * 2.0 * k1 * x;
      Jin[3] = k1 * (3.0 * y2 + x2) + 1.0;
      Jprm[0] = x * r2;
      Jprm[P] = y * r2;
      return;
    }
    case D_K1K2: {
      const double k1 = c[0], k2 = c[1];
      const double x4 = x2 * x2, y4 = y2 * y2;
      Jin[0] = 5.0 * k2 * x4 + 3.0 * k1 * x2 + 6.0 * k2 * x2 * y2 + k2 * y4 + k1 * y2 + 1.0;
      Jin[1] = x * (2.0 * k1 * y + 4.0 * k2 * y * r2);
      Jin[2] = y * (2.0 * k1 * x + 4.0 * k2 * x * r2);
      Jin[3] = 5.0 * k2 * y4 + 3.0 * k1 * y2 + 6.0 * k2 * y2 * x2 + k2 * x4 + k1 * x2 + 1.0;
      Jprm[0] = x * r2;
      Jprm[1] = x * r2 * r2;
      Jprm[P + 0] = y * r2;
      Jprm[P + 1] = y * r2 * r2;
      return;
    }
    case D_K1K4: {
      const double k1 = c[0], k2 = c[1], k3 = c[2], k4 = c[3];
      const double dr = 2.0 * k1 + 4.0 * k2 * r2 + 6.0 * k3 * r2 * r2 + 8.0 * k4 * r2 * r2 * r2;
      const double rad = k1 * r2 + k2 * r2 * r2 + k3 * r2 * r2 * r2 + k4 * r2 * r2 * r2 * r2 + 1.0;
      Jin[0] = x * (dr * x) + rad;
      Jin[1] = x * (dr * y);
      Jin[2] = y * (dr * x);
      Jin[3] = y * (dr * y) + rad;
      double rp = r2;
      for (int i = 0; i < 4; ++i) {
        Jprm[i] = x * rp;
        Jprm[P + i] = y * rp;
        rp *= r2;
      }
      return;
    }
    case D_BROWN: {
      const double k1 = c[0], k2 = c[1], k3 = c[2], p1 = c[3], p2 = c[4];
      const double x4 = x2 * x2, y4 = y2 * y2, r4 = r2 * r2, r6 = r4 * r2;
      Jin[0] = 5.0 * k2 * x4 + 3.0 * k1 * x2 + 6.0 * k3 * x2 * r4 + 6.0 * k2 * x2 * y2 + k3 * r6 +
               k2 * y4 + k1 * y2 + 1.0 + 2.0 * p1 * y + 6.0 * p2 * x;
      Jin[1] = x * (2.0 * k1 * y + 4.0 * k2 * y * r2 + 6.0 * k3 * y * r4) + 2.0 * p1 * x + 2.0 * p2 * y;
      Jin[3] = 5.0 * k2 * y4 + 3.0 * k1 * y2 + 6.0 * k3 * y2 * r4 + 6.0 * k2 * x2 * y2 + k3 * r6 +
               k2 * x4 + k1 * x2 + 1.0 + 2.0 * p2 * x + 6.0 * p1 * y;
      Jin[2] = y * (2.0 * k1 * x + 4.0 * k2 * x * r2 + 6.0 * k3 * x * r4) + 2.0 * p2 * y + 2.0 * p1 * x;
      Jprm[0] = x * r2;
      Jprm[1] = x * r2 * r2;
      Jprm[2] = x * r2 * r2 * r2;
      Jprm[3] = 2.0 * x * y;
      Jprm[4] = 3.0 * x2 + y2;
      Jprm[P + 0] = y * r2;
      Jprm[P + 1] = y * r2 * r2;
      Jprm[P + 2] = y * r2 * r2 * r2;
      Jprm[P + 3] = 3.0 * y2 + x2;
      Jprm[P + 4] = 2.0 * x * y;
      return;
    }
    case D_62:
    case D_624: {
      const double k1 = c[0], k2 = c[1], k3 = c[2], k4 = c[3], k5 = c[4], k6 = c[5];
      const double p1 = c[6], p2 = c[7];
      const double r2_2 = r2 * r2, r2_3 = r2_2 * r2, r2_4 = r2_3 * r2, r2_5 = r2_4 * r2;
      const double dx_dxt = 2.0 * y * p1 + 6.0 * p2 * x;
      const double dx_dyt = 2.0 * x * p1 + 2.0 * p2 * y;
      const double dy_dxt = dx_dyt;
      const double dy_dyt = 2.0 * x * p2 + 6.0 * p1 * y;
      const double p = 1.0 + r2 * (k1 + r2 * (k2 + r2 * (k3 + r2 * (k4 + r2 * (k5 + r2 * k6)))));
      const double dp_dr = k1 + 2.0 * k2 * r2 + 3.0 * k3 * r2_2 + 4.0 * k4 * r2_3 +
                           5.0 * k5 * r2_4 + 6.0 * k6 * r2_5;
      double a00 = p + x * dp_dr * 2.0 * x + dx_dxt;
      double a01 = x * dp_dr * 2.0 * y + dx_dyt;
      double a10 = y * dp_dr * 2.0 * x + dy_dxt;
      double a11 = p + y * dp_dr * 2.0 * y + dy_dyt;
      if (k == D_624) {
        const double s0 = c[8], s1 = c[9], s2 = c[10], s3 = c[11];
        a00 += s0 * 2.0 * x + s1 * 4.0 * x * r2;
        a01 += s0 * 2.0 * y + s1 * 4.0 * y * r2;
        a10 += s2 * 2.0 * x + s3 * 4.0 * x * r2;
        a11 += s2 * 2.0 * y + s3 * 4.0 * y * r2;
      }
      Jin[0] = a00; Jin[1] = a01; Jin[2] = a10; Jin[3] = a11;
      double rp = r2;
      for (int i = 0; i < 6; ++i) {
        Jprm[i] = x * rp;
        Jprm[P + i] = y * rp;
        rp *= r2;
      }
      Jprm[6] = 2.0 * x * y;
      Jprm[7] = 3.0 * x2 + y2;
      Jprm[P + 6] = 3.0 * y2 + x2;
      Jprm[P + 7] = 2.0 * x * y;
      if (k == D_624) {
        Jprm[8] = r2; Jprm[9] = r2_2; Jprm[10] = 0.0; Jprm[11] = 0.0;
        Jprm[P + 8] = 0.0; Jprm[P + 9] = 0.0; Jprm[P + 10] = r2; Jprm[P + 11] = r2_2;
      }
      return;
    }
  }
}

// transformations_functions.h:135-154 (Affine), :174-186 (UniformScale),
// :203-212 (Identity).
inline void aff_jac(AffKind k, const double* q, const double* a, double* out,
                    double* Jin /*2x2*/, double* Jprm /*2xP*/) {
  aff_forward<double>(k, q, a, out);
  switch (k) {
    case A_NONE:
      Jin[0] = 1; Jin[1] = 0; Jin[2] = 0; Jin[3] = 1;
      break;
    case A_SCALE:
      Jin[0] = a[0]; Jin[1] = 0; Jin[2] = 0; Jin[3] = a[0];
      Jprm[0] = q[0];
      Jprm[1] = q[1];
      break;
    case A_AFFINE:
      Jin[0] = a[0]; Jin[1] = 0; Jin[2] = 0; Jin[3] = a[0] * a[1];
      // columns: focal, aspect, cx, cy
      Jprm[0] = q[0]; Jprm[1] = 0.0; Jprm[2] = 1.0; Jprm[3] = 0.0;
      Jprm[4] = q[1] * a[1]; Jprm[5] = q[1] * a[0]; Jprm[6] = 0.0; Jprm[7] = 1.0;
      break;
  }
}

// Full model: uv and d(uv)/d(point_cam) (2x3) and d(uv)/d(params) (2xC),
// composed by the chain rule exactly as ComposeForwardDerivatives does
// (functions.h:77-97): J = [J_aff_in * J_dis_in * J_proj_in | ... ].
inline void project_jac(int model, const double* p, const double* params, double* uv,
                        double* Jp /*2x3*/, double* Jc /*2xC*/) {
  const ModelDesc d = model_desc(model);
  const int C = d.n_params;
  double a[2], b[2];
  double Jpp[6] = {0}, Jpt[2] = {0};
  double Jdi[4] = {0}, Jdt[2 * 12] = {0};
  double Jai[4] = {0}, Jat[2 * 4] = {0};
  proj_jac(d.proj, p, params, a, Jpp, Jpt);
  disto_jac(d.disto, a, params + d.n_proj, b, Jdi, Jdt);
  aff_jac(d.aff, b, params + d.n_proj + d.n_disto, uv, Jai, Jat);
  // M = Jai * Jdi  (2x2)
  double M[4];
  M[0] = Jai[0] * Jdi[0] + Jai[1] * Jdi[2];
  M[1] = Jai[0] * Jdi[1] + Jai[1] * Jdi[3];
  M[2] = Jai[2] * Jdi[0] + Jai[3] * Jdi[2];
  M[3] = Jai[2] * Jdi[1] + Jai[3] * Jdi[3];
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 3; ++j) Jp[i * 3 + j] = M[i * 2 + 0] * Jpp[j] + M[i * 2 + 1] * Jpp[3 + j];
  for (int i = 0; i < 2 * C; ++i) Jc[i] = 0.0;
  int col = 0;
  if (d.n_proj) {
    for (int i = 0; i < 2; ++i) Jc[i * C + col] = M[i * 2 + 0] * Jpt[0] + M[i * 2 + 1] * Jpt[1];
    col += 1;
  }
  for (int t = 0; t < d.n_disto; ++t) {
    for (int i = 0; i < 2; ++i)
      Jc[i * C + col + t] = Jai[i * 2 + 0] * Jdt[t] + Jai[i * 2 + 1] * Jdt[d.n_disto + t];
  }
  col += d.n_disto;
  for (int t = 0; t < d.n_aff; ++t) {
    for (int i = 0; i < 2; ++i) Jc[i * C + col + t] = Jat[i * d.n_aff + t];
  }
}

// ---------------------------------------------------------------------------
// Pose transform x_cam = R(-r) * (X - t) with the angle-axis Rodrigues formula
// and its small-angle branch (transformations_functions.h:221-258).
template <class T>
inline void pose_forward_t(const T* X, const T* rt, T* out) {
  using std::cos;
  using std::sin;
  using std::sqrt;
  const T x = X[0] - rt[3], y = X[1] - rt[4], z = X[2] - rt[5];
  const T a = -rt[0], b = -rt[1], c = -rt[2];
  const T cpx = b * z - c * y, cpy = c * x - a * z, cpz = a * y - b * x;
  const T th2 = a * a + b * b + c * c;
  if (value_of(th2) > 2.220446049250313e-16) {
    const T th = sqrt(th2);
    const T ct = cos(th);
    const T st = sin(th) / th;
    const T dd = (a * x + b * y + c * z) * (1.0 - ct) / th2;
    out[0] = x * ct + st * cpx + a * dd;
    out[1] = y * ct + st * cpy + b * dd;
    out[2] = z * ct + st * cpz + c * dd;
  } else {
    out[0] = x + cpx;
    out[1] = y + cpy;
    out[2] = z + cpz;
  }
}

// Rotation matrix (row-major) of angle-axis aa with the small-angle branch
// R = I + [aa]x (transformations_functions.h:330-376).
template <class T>
inline void angle_axis_to_rotation(const T* aa, T* R) {
  using std::cos;
  using std::sin;
  using std::sqrt;
  const T th2 = aa[0] * aa[0] + aa[1] * aa[1] + aa[2] * aa[2];
  if (value_of(th2) < 2.220446049250313e-16) {
    R[0] = T(1.0); R[1] = -aa[2]; R[2] = aa[1];
    R[3] = aa[2]; R[4] = T(1.0); R[5] = -aa[0];
    R[6] = -aa[1]; R[7] = aa[0]; R[8] = T(1.0);
    return;
  }
  const T th = sqrt(th2);
  const T c = cos(th), s = sin(th), t = 1.0 - c;
  const T it2 = 1.0 / th2, it = 1.0 / th;
  const T xx = aa[0] * aa[0] * it2, xy = aa[0] * aa[1] * it2, xz = aa[0] * aa[2] * it2;
  const T yy = aa[1] * aa[1] * it2, yz = aa[1] * aa[2] * it2, zz = aa[2] * aa[2] * it2;
  const T xs = aa[0] * it * s, ys = aa[1] * it * s, zs = aa[2] * it * s;
  R[0] = t * xx + c; R[1] = t * xy - zs; R[2] = t * xz + ys;
  R[3] = t * xy + zs; R[4] = t * yy + c; R[5] = t * yz - xs;
  R[6] = t * xz - ys; R[7] = t * yz + xs; R[8] = t * zz + c;
}

// Pose Jacobian as PoseFunctor::ForwardDerivatives produces it
// (transformations_functions.h:260-327): 3x9 row-major, columns
// [d/dX (3) | d/d(rx,ry,rz) (3) | d/d(tx,ty,tz) (3)].  dR/d(rt) comes from
// forward-mode duals seeded with -e_k on R(-rt), as the reference does.
inline void pose_jac(const double* X, const double* rt, double* out, double* J /*3x9*/) {
  Dual<3> aa[3];
  for (int k = 0; k < 3; ++k) {
    aa[k] = Dual<3>(-rt[k]);
    aa[k].d[k] = -1.0;
  }
  Dual<3> R[9];
  angle_axis_to_rotation<Dual<3>>(aa, R);
  const double v[3] = {X[0] - rt[3], X[1] - rt[4], X[2] - rt[5]};
  for (int i = 0; i < 3; ++i) {
    for (int k = 0; k < 3; ++k) {
      double s = 0;
      for (int j = 0; j < 3; ++j) s += v[j] * R[i * 3 + j].d[k];
      J[i * 9 + 3 + k] = s;
    }
    for (int j = 0; j < 3; ++j) {
      J[i * 9 + j] = R[i * 3 + j].v;
      J[i * 9 + 6 + j] = -R[i * 3 + j].v;
    }
  }
  pose_forward_t<double>(X, rt, out);
}

}  // namespace oracle
