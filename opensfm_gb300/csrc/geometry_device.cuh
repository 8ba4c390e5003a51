// Per-shot pose precompute and per-observation residual/Jacobian evaluation.
//
// The pose of a shot is the composition of its rig instance and rig camera
// poses, both stored camera-to-world as [angle-axis | camera centre]
// (opensfm/src/lib/bundle/data/pose.h:17,34-43).  A world point X is mapped
// to the camera frame as R(-r_rc) (R(-r_inst) (X - c_inst) - c_rc)
// (bundle/error/error_utils.h:449-461, geometry/transformations_functions.h:
// 221-258).
//
// Rotation derivative.  The reference differentiates R(-r) with dual
// numbers for every observation (transformations_functions.h:260-327).
// Here each shot stores R and the SO(3) right Jacobian J_r of phi = -r, and
// an observation uses
//     d(R v)/d r = R [v]x J_r(phi),
// so a residual row with point-Jacobian row j = a R becomes (j x v)^T J_r:
// 18 values per shot instead of a 27-entry derivative tensor, and 15 FMAs per
// row.  (J_r(phi) = I - (1 - cos t)/t^2 [phi]x + (t - sin t)/t^3 [phi]x^2,
// t = |phi|.)
//
// Camera-centred coordinates.  In FP64 mode points and centres are FP64.
// In mixed mode they are stored as double-float pairs (hi = float(x),
// lo = float(x - hi)); v = (X_hi - c_hi) + (X_lo - c_lo) is then accurate
// to FP32 relative precision of v itself even at UTM offsets (x ~ 5e5,
// y ~ 4e6 m), with no FP64 instruction per observation (FP64 runs at a small
// fraction of the FP32 rate on this GPU).
#pragma once

#include <cstdint>

#include "camera_models.cuh"

namespace gbba {

// FP64 3-vector padded to 32 bytes.
struct alignas(32) Point4 {
  double x, y, z, w;
};
// Double-float 3-vector: hi = float(x), lo = float(x - hi).
struct alignas(32) PointF2 {
  float hx, hy, hz, pad0, lx, ly, lz, pad1;
};

template <typename R> struct PointStore;
template <> struct PointStore<double> { using type = Point4; };
template <> struct PointStore<float> { using type = PointF2; };

GB_HD Point4 make_point_store(double x, double y, double z, double*) { return {x, y, z, 0.0}; }
GB_HD PointF2 make_point_store(double x, double y, double z, float*) {
  const float hx = float(x), hy = float(y), hz = float(z);
  return {hx, hy, hz, 0.0f, float(x - double(hx)), float(y - double(hy)), float(z - double(hz)), 0.0f};
}

// ---------------------------------------------------------------------------
// Per-shot geometry in the working precision R (128 B in FP32):
//   rot[9]  world -> camera rotation R_rc * R_inst (row-major)
//   jr[9]   right Jacobian J_r(-r_inst) (row-major)
//   tc[3]   camera-frame offset -R_rc * c_rc (zero without rig camera)
//   cam     camera index of the shot (exact small integer)
//   chi[3], clo[3]  rig instance centre (double-float in FP32; lo = 0 in FP64)
//   inst, rig  rig instance and rig camera indices (rig = -1: none)
template <typename R>
struct alignas(16) ShotGeom {
  R rot[9];
  R jr[9];
  R tc[3];
  R cam;
  R chi[3];
  R clo[3];
  R inst;
  R rig;
  R pad[sizeof(R) == 4 ? 2 : 0 + 2];
};

#ifdef __CUDACC__
// v = X - c_inst in the working precision.
__device__ __forceinline__ void centred(const Point4* X, const ShotGeom<double>& g, double* v) {
  const double2* a = reinterpret_cast<const double2*>(X);
  const double2 a0 = __ldg(a), a1 = __ldg(a + 1);
  v[0] = a0.x - g.chi[0];
  v[1] = a0.y - g.chi[1];
  v[2] = a1.x - g.chi[2];
}
__device__ __forceinline__ void centred(const PointF2* X, const ShotGeom<float>& g, float* v) {
  const float4* a = reinterpret_cast<const float4*>(X);
  const float4 ah = __ldg(a), al = __ldg(a + 1);
  v[0] = (ah.x - g.chi[0]) + (al.x - g.clo[0]);
  v[1] = (ah.y - g.chi[1]) + (al.y - g.clo[1]);
  v[2] = (ah.z - g.chi[2]) + (al.z - g.clo[2]);
}
#endif

// Extra per-shot data used only when rig cameras are optimised:
//   rinst[9] R_inst; rrc[9] R_rc; jrc[9] J_r(-r_rc); crc[3] rig camera centre.
template <typename R>
struct alignas(16) RigGeom {
  R rinst[9];
  R rrc[9];
  R jrc[9];
  R crc[3];
  R pad[2];
};

#ifdef __CUDACC__
template <typename T>
__device__ __forceinline__ void ldg_copy(const T* src, T& dst) {
  static_assert(sizeof(T) % 16 == 0, "vector copy needs 16-byte multiples");
  const float4* s = reinterpret_cast<const float4*>(src);
  float4* d = reinterpret_cast<float4*>(&dst);
#pragma unroll
  for (int i = 0; i < int(sizeof(T) / 16); ++i) d[i] = __ldg(s + i);
}
#endif

// Rodrigues rotation of angle-axis w (row-major) with the first-order branch
// I + [w]x below machine epsilon (transformations_functions.h:330-376).
GB_HD void rodrigues(const double* w, double* Rm) {
  const double th2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
  if (th2 < 2.220446049250313e-16) {
    Rm[0] = 1.0; Rm[1] = -w[2]; Rm[2] = w[1];
    Rm[3] = w[2]; Rm[4] = 1.0; Rm[5] = -w[0];
    Rm[6] = -w[1]; Rm[7] = w[0]; Rm[8] = 1.0;
    return;
  }
  const double th = sqrt(th2);
  const double c = cos(th), s = sin(th), t = 1.0 - c;
  const double it2 = 1.0 / th2, it = 1.0 / th;
  const double xx = w[0] * w[0] * it2, xy = w[0] * w[1] * it2, xz = w[0] * w[2] * it2;
  const double yy = w[1] * w[1] * it2, yz = w[1] * w[2] * it2, zz = w[2] * w[2] * it2;
  const double xs = w[0] * it * s, ys = w[1] * it * s, zs = w[2] * it * s;
  Rm[0] = t * xx + c; Rm[1] = t * xy - zs; Rm[2] = t * xz + ys;
  Rm[3] = t * xy + zs; Rm[4] = t * yy + c; Rm[5] = t * yz - xs;
  Rm[6] = t * xz - ys; Rm[7] = t * yz + xs; Rm[8] = t * zz + c;
}

// Right Jacobian of SO(3) at phi (row-major), with its Taylor expansion
// near zero.
GB_HD void right_jacobian(const double* phi, double* J) {
  const double th2 = phi[0] * phi[0] + phi[1] * phi[1] + phi[2] * phi[2];
  double a, b;
  if (th2 < 1e-8) {
    a = 0.5 - th2 / 24.0;
    b = 1.0 / 6.0 - th2 / 120.0;
  } else {
    const double th = sqrt(th2);
    a = (1.0 - cos(th)) / th2;
    b = (th - sin(th)) / (th2 * th);
  }
  const double K[9] = {0.0, -phi[2], phi[1], phi[2], 0.0, -phi[0], -phi[1], phi[0], 0.0};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double k2 = 0.0;
      for (int m = 0; m < 3; ++m) k2 += K[i * 3 + m] * K[m * 3 + j];
      J[i * 3 + j] = (i == j ? 1.0 : 0.0) - a * K[i * 3 + j] + b * k2;
    }
}

// R(-r) and J_r(-r) for a camera-to-world angle-axis r.
GB_HD void pose_rotation(const double* r, double* Rm, double* Jr) {
  const double phi[3] = {-r[0], -r[1], -r[2]};
  rodrigues(phi, Rm);
  right_jacobian(phi, Jr);
}

// ---------------------------------------------------------------------------
// Record layout (row-major blocks, NR residual rows):
//   [ r (NR) | J_point (NR x 3) | J_instance (NR x 6: rx ry rz tx ty tz)
//     | J_camera (NR x CMAX) | J_rig (NR x 6, only when RIG) ]
// The columns of J_instance and J_rig follow the parameter order of
// bundle::Pose (RX, RY, RZ, TX, TY, TZ; data/pose.h:17).
template <int NR, int CMAX, bool RIG>
struct RecordLayout {
  static constexpr int kR = 0;
  static constexpr int kPt = NR;
  static constexpr int kInst = kPt + 3 * NR;
  static constexpr int kCam = kInst + 6 * NR;
  static constexpr int kRig = kCam + CMAX * NR;
  static constexpr int kWidth = kRig + (RIG ? 6 * NR : 0);
};

// Projection of a camera-frame point for a runtime model id (mixed-model
// kernels) or a compile-time model M >= 0.
template <int M, int CMAX, typename R>
__device__ __forceinline__ void project_dispatch(int model, const R* p, const R* prm, R* uv,
                                                 R* Jp, R* Jc) {
  if constexpr (M >= 0) {
    static_assert(ModelTraits<M>::kSize <= CMAX, "record too narrow for model");
    R Jtmp[2 * ModelTraits<M>::kSize];
    project_model<M, R>(p, prm, uv, Jp, Jtmp);
    constexpr int C = ModelTraits<M>::kSize;
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < CMAX; ++j) Jc[i * CMAX + j] = j < C ? Jtmp[i * C + j] : R(0);
  } else {
#define GB_CASE(MM)                                                                 \
  case MM: {                                                                        \
    if constexpr (ModelTraits<MM>::kSize <= CMAX) {                                 \
      constexpr int C = ModelTraits<MM>::kSize;                                     \
      R Jtmp[2 * C];                                                                \
      project_model<MM, R>(p, prm, uv, Jp, Jtmp);                                   \
      _Pragma("unroll") for (int i = 0; i < 2; ++i)                                 \
      _Pragma("unroll") for (int j = 0; j < CMAX; ++j) Jc[i * CMAX + j] =           \
          j < C ? Jtmp[i * C + j] : R(0);                                           \
    }                                                                               \
    break;                                                                          \
  }
    switch (model) {
      GB_CASE(kPerspective)
      GB_CASE(kBrown)
      GB_CASE(kFisheye)
      GB_CASE(kFisheyeOpencv)
      GB_CASE(kFisheye62)
      GB_CASE(kFisheye624)
      GB_CASE(kDual)
      GB_CASE(kRadial)
      GB_CASE(kSimpleRadial)
      default:
        break;
    }
#undef GB_CASE
  }
}

// Inputs of one observation evaluation (all in registers).
template <typename R>
struct ObsInputs {
  R ox, oy;     // observed normalized coordinates (or bearing angles / 2pi)
  R w;          // 1 / std_deviation
  R v[3];       // camera-centred world point X - c_inst
  ShotGeom<R> g;
  const RigGeom<R>* rg;  // only read when RIG
  const R* cam;          // camera parameters
  int model;
};

// Evaluates the scaled residual and (if JAC) its Jacobian into rec[] using
// RecordLayout<NR, CMAX, RIG>.  Follows ReprojectionError2DAnalytic<C>::
// Evaluate (projection_errors.h:67-207) and ReprojectionError3DAnalytic
// (:255-374) for spherical cameras.  A depth prior (negative weight, see
// ObsPack) follows RelativeDepthError (bundle/error/relative_depth_error.h):
// one residual (depth(p) - value) / std, depth(p) = |p| when radial, else
// p.z, on the same camera-frame point p (so the same pose chain rule), with
// no camera columns.  Only the solver's slots hold depth priors: kernels of
// other callers instantiate DEPTH = false and carry no depth branch.
template <typename R, int M, int NR, int CMAX, bool RIG, bool JAC, bool DEPTH = false>
__device__ __forceinline__ void eval_observation(const ObsInputs<R>& in, R* rec) {
  using L = RecordLayout<NR, CMAX, RIG>;
  const R v0 = in.v[0], v1 = in.v[1], v2 = in.v[2];
  const ShotGeom<R>& g = in.g;
  R p[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) p[i] = g.rot[i * 3 + 0] * v0 + g.rot[i * 3 + 1] * v1 + g.rot[i * 3 + 2] * v2 + g.tc[i];

  const bool depth = DEPTH && in.w < R(0);
  const R w = depth ? -in.w : in.w;
  R Jq[NR * 3];  // d(residual)/d(p) before scaling
  if (depth) {
    R d;
    if (in.oy > R(0.5)) {
      d = sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
      const R id = R(1) / d;
      Jq[0] = p[0] * id;
      Jq[1] = p[1] * id;
      Jq[2] = p[2] * id;
    } else {
      d = p[2];
      Jq[0] = Jq[1] = R(0);
      Jq[2] = R(1);
    }
    rec[L::kR + 0] = w * (d - in.ox);
#pragma unroll
    for (int i = 1; i < NR; ++i) rec[L::kR + i] = R(0);
    if (JAC) {
#pragma unroll
      for (int i = 3; i < NR * 3; ++i) Jq[i] = R(0);
#pragma unroll
      for (int i = 0; i < NR * CMAX; ++i) rec[L::kCam + i] = R(0);
    }
  } else if (NR == 3 && in.model == kSpherical) {
    // bearing residual: normalize(p) - b(obs), obs = (lon, lat) / 2pi
    R o[3];
    normalize_stage<R>(p, o, Jq);
    const R lon = in.ox * R(2.0 * M_PI), lat = -in.oy * R(2.0 * M_PI);
    const R cl = cos(lat);
    const R b[3] = {cl * sin(lon), -sin(lat), cl * cos(lon)};
#pragma unroll
    for (int i = 0; i < NR; ++i) rec[L::kR + i] = w * (o[i] - b[i]);
    if (JAC) {
#pragma unroll
      for (int i = 0; i < NR * CMAX; ++i) rec[L::kCam + i] = R(0);
    }
  } else {
    R uv[2], Jc[2 * CMAX], Jp2[6];
    project_dispatch<M, CMAX, R>(in.model, p, in.cam, uv, Jp2, Jc);
    rec[L::kR + 0] = w * (uv[0] - in.ox);
    rec[L::kR + 1] = w * (uv[1] - in.oy);
    if (NR == 3) rec[L::kR + 2] = R(0);
    if (JAC) {
#pragma unroll
      for (int i = 0; i < 6; ++i) Jq[i] = Jp2[i];
      if (NR == 3) {
        Jq[6] = Jq[7] = Jq[8] = R(0);
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < CMAX; ++j) rec[L::kCam + i * CMAX + j] = w * Jc[i * CMAX + j];
      if (NR == 3) {
#pragma unroll
        for (int j = 0; j < CMAX; ++j) rec[L::kCam + 2 * CMAX + j] = R(0);
      }
    }
  }
  if constexpr (JAC) {
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    const R a0 = w * Jq[i * 3 + 0], a1 = w * Jq[i * 3 + 1], a2 = w * Jq[i * 3 + 2];
    R jp[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      jp[j] = a0 * g.rot[0 * 3 + j] + a1 * g.rot[1 * 3 + j] + a2 * g.rot[2 * 3 + j];
      rec[L::kPt + i * 3 + j] = jp[j];
      rec[L::kInst + i * 6 + 3 + j] = -jp[j];  // d/d(centre) = -d/dX
    }
    // rotation: (jp x v)^T J_r
    const R c0 = jp[1] * v2 - jp[2] * v1;
    const R c1 = jp[2] * v0 - jp[0] * v2;
    const R c2 = jp[0] * v1 - jp[1] * v0;
#pragma unroll
    for (int k = 0; k < 3; ++k) rec[L::kInst + i * 6 + k] = c0 * g.jr[0 * 3 + k] + c1 * g.jr[1 * 3 + k] + c2 * g.jr[2 * 3 + k];
    if constexpr (RIG) {
      // shots without an applied rig camera have a zero rig-camera block
      // (projection_errors.h:184-188)
      if (g.rig < R(0)) {
#pragma unroll
        for (int k = 0; k < 6; ++k) rec[L::kRig + i * 6 + k] = R(0);
        continue;
      }
      // p = R_rc (y - c_rc), y = R_inst v:  d p / d r_rc = R_rc [y - c_rc]x J_rc,
      // d p / d c_rc = -R_rc
      const RigGeom<R>& rg = *in.rg;
      R e[3], q[3];
#pragma unroll
      for (int k = 0; k < 3; ++k)
        e[k] = rg.rinst[k * 3 + 0] * v0 + rg.rinst[k * 3 + 1] * v1 + rg.rinst[k * 3 + 2] * v2 - rg.crc[k];
#pragma unroll
      for (int k = 0; k < 3; ++k) q[k] = a0 * rg.rrc[0 * 3 + k] + a1 * rg.rrc[1 * 3 + k] + a2 * rg.rrc[2 * 3 + k];
      const R d0 = q[1] * e[2] - q[2] * e[1];
      const R d1 = q[2] * e[0] - q[0] * e[2];
      const R d2 = q[0] * e[1] - q[1] * e[0];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        rec[L::kRig + i * 6 + k] = d0 * rg.jrc[0 * 3 + k] + d1 * rg.jrc[1 * 3 + k] + d2 * rg.jrc[2 * 3 + k];
        rec[L::kRig + i * 6 + 3 + k] = -q[k];
      }
    }
  }
  }  // JAC
}

}  // namespace gbba
