// Per-shot pose precompute and per-observation residual/Jacobian evaluation.
//
// The pose of a shot is the composition of its rig instance and rig camera
// poses, both stored camera-to-world as [angle-axis | camera centre]
// (opensfm/src/lib/bundle/data/pose.h:17,34-43).  A world point X is mapped
// to the camera frame as R(-r_rc) (R(-r_inst) (X - c_inst) - c_rc)
// (bundle/error/error_utils.h:449-461, geometry/transformations_functions.h:
// 221-258).  The rotation and its derivative with respect to the angle-axis
// parameters are computed once per shot in FP64 (the reference recomputes
// them for every observation, transformations_functions.h:260-327); the
// observation kernels only contract them with X - c_inst.
//
// Mixed precision: X - c_inst is formed in FP64 (georeferenced coordinates,
// e.g. UTM with x ~ 5e5 m) and only the camera-centred difference is cast to
// the working type R, so FP32 never sees the large offsets.
#pragma once

#include <cstdint>

#include "camera_models.cuh"

namespace gbba {

// FP64 3-vector padded to 32 bytes (world points, shot centres).
struct alignas(32) Point4 {
  double x, y, z, w;
};
#ifdef __CUDACC__
__device__ __forceinline__ Point4 ldg_point4(const Point4* p) {
  const double2* q = reinterpret_cast<const double2*>(p);
  const double2 a = __ldg(q), b = __ldg(q + 1);
  return {a.x, a.y, b.x, b.y};
}
#endif

// ---------------------------------------------------------------------------
// Per-shot geometry in the working precision R.
//   rot[9]    world -> camera rotation R_rc * R_inst (row-major)
//   drot[27]  d(rot)/d(r_inst) as drot[(m*3 + j)*3 + k] = d rot[m][j] / d r_inst[k]
//   tc[3]     camera-frame offset -R_rc * c_rc (zero without rig camera)
template <typename R>
struct alignas(16) ShotGeom {
  R rot[9];
  R drot[27];
  R tc[3];
  R pad;
};

// Extra per-shot data used only when rig cameras are optimised.
//   rinst[9]  R_inst;  rrc[9] R_rc;  drrc[27] d(R_rc)/d(r_rc);  crc[3]
template <typename R>
struct alignas(16) RigGeom {
  R rinst[9];
  R rrc[9];
  R drrc[27];
  R crc[3];
};

// Forward-mode dual number with three derivative slots (FP64), used for the
// derivative of the Rodrigues rotation with respect to its angle-axis.
struct D3 {
  double v, d0, d1, d2;
};
GB_HD D3 d3(double v) { return {v, 0.0, 0.0, 0.0}; }
GB_HD D3 operator+(D3 a, D3 b) { return {a.v + b.v, a.d0 + b.d0, a.d1 + b.d1, a.d2 + b.d2}; }
GB_HD D3 operator-(D3 a, D3 b) { return {a.v - b.v, a.d0 - b.d0, a.d1 - b.d1, a.d2 - b.d2}; }
GB_HD D3 operator*(D3 a, D3 b) {
  return {a.v * b.v, a.d0 * b.v + a.v * b.d0, a.d1 * b.v + a.v * b.d1, a.d2 * b.v + a.v * b.d2};
}
GB_HD D3 operator*(double s, D3 a) { return {s * a.v, s * a.d0, s * a.d1, s * a.d2}; }
GB_HD D3 d3_inv(D3 a) {
  const double iv = 1.0 / a.v, k = -iv * iv;
  return {iv, k * a.d0, k * a.d1, k * a.d2};
}
GB_HD D3 d3_sqrt(D3 a) {
  const double s = sqrt(a.v), k = 0.5 / s;
  return {s, k * a.d0, k * a.d1, k * a.d2};
}
GB_HD D3 d3_sin(D3 a) {
  const double c = cos(a.v);
  return {sin(a.v), c * a.d0, c * a.d1, c * a.d2};
}
GB_HD D3 d3_cos(D3 a) {
  const double s = -sin(a.v);
  return {cos(a.v), s * a.d0, s * a.d1, s * a.d2};
}

// Rodrigues rotation of angle-axis w (row-major) with the first-order branch
// I + [w]x below machine epsilon (transformations_functions.h:330-376).
GB_HD void rodrigues_d3(const D3* w, D3* Rm) {
  const D3 th2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
  if (th2.v < 2.220446049250313e-16) {
    const D3 one = d3(1.0), mz = d3(0.0) - w[2], my = d3(0.0) - w[1], mx = d3(0.0) - w[0];
    Rm[0] = one; Rm[1] = mz; Rm[2] = w[1];
    Rm[3] = w[2]; Rm[4] = one; Rm[5] = mx;
    Rm[6] = my; Rm[7] = w[0]; Rm[8] = one;
    return;
  }
  const D3 th = d3_sqrt(th2);
  const D3 c = d3_cos(th), s = d3_sin(th), t = d3(1.0) - c;
  const D3 it2 = d3_inv(th2), it = d3_inv(th);
  const D3 xx = w[0] * w[0] * it2, xy = w[0] * w[1] * it2, xz = w[0] * w[2] * it2;
  const D3 yy = w[1] * w[1] * it2, yz = w[1] * w[2] * it2, zz = w[2] * w[2] * it2;
  const D3 xs = w[0] * it * s, ys = w[1] * it * s, zs = w[2] * it * s;
  Rm[0] = t * xx + c; Rm[1] = t * xy - zs; Rm[2] = t * xz + ys;
  Rm[3] = t * xy + zs; Rm[4] = t * yy + c; Rm[5] = t * yz - xs;
  Rm[6] = t * xz - ys; Rm[7] = t * yz + xs; Rm[8] = t * zz + c;
}

// R(-r) and d R(-r) / d r for a camera-to-world angle-axis r: the dual
// seeds are -e_k, as PoseFunctor::ForwardDerivatives seeds them.
GB_HD void pose_rotation(const double* r, double* Rm, double* dR /*27*/) {
  D3 w[3];
  w[0] = {-r[0], -1.0, 0.0, 0.0};
  w[1] = {-r[1], 0.0, -1.0, 0.0};
  w[2] = {-r[2], 0.0, 0.0, -1.0};
  D3 M[9];
  rodrigues_d3(w, M);
  for (int i = 0; i < 9; ++i) {
    Rm[i] = M[i].v;
    dR[i * 3 + 0] = M[i].d0;
    dR[i * 3 + 1] = M[i].d1;
    dR[i * 3 + 2] = M[i].d2;
  }
}

// ---------------------------------------------------------------------------
// Per-observation residual and Jacobian in registers.
//
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
  static constexpr int kPlanes4 = (kWidth + 3) / 4;  // float4 planes
  static constexpr int kPlanes2 = (kWidth + 1) / 2;  // double2 planes
};

// Projection of a camera-frame point for a runtime model id (used by the
// mixed-model kernels) or a compile-time model M >= 0.
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

// Inputs of one observation evaluation.
template <typename R>
struct ObsInputs {
  R ox, oy;      // observed normalized coordinates (or bearing angles)
  R w;           // 1 / std_deviation
  double X[3];   // world point (FP64)
  double c[3];   // rig instance centre (FP64)
  const ShotGeom<R>* g;
  const RigGeom<R>* rg;  // only read when RIG
  const R* cam;          // camera parameters
  int model;
};

// Evaluates the scaled residual and (if JAC) its Jacobian into rec[] using
// RecordLayout<NR, CMAX, RIG>.  Follows ReprojectionError2DAnalytic<C>::
// Evaluate (projection_errors.h:67-207) and ReprojectionError3DAnalytic
// (:255-374) for spherical cameras.
template <typename R, int M, int NR, int CMAX, bool RIG, bool JAC>
__device__ __forceinline__ void eval_observation(const ObsInputs<R>& in, R* rec) {
  using L = RecordLayout<NR, CMAX, RIG>;
  // camera-centred point: FP64 subtraction, then cast
  const R v0 = R(in.X[0] - in.c[0]);
  const R v1 = R(in.X[1] - in.c[1]);
  const R v2 = R(in.X[2] - in.c[2]);
  const ShotGeom<R>& g = *in.g;
  R p[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) p[i] = g.rot[i * 3 + 0] * v0 + g.rot[i * 3 + 1] * v1 + g.rot[i * 3 + 2] * v2 + g.tc[i];

  R Jq[NR * 3];  // d(residual)/d(p) before scaling
  if (NR == 3 && in.model == kSpherical) {
    // bearing residual: normalize(p) - b(obs), obs = (lon, lat) / 2pi
    R o[3];
    normalize_stage<R>(p, o, Jq);
    const R lon = in.ox * R(2.0 * M_PI), lat = -in.oy * R(2.0 * M_PI);
    const R cl = cos(lat);
    const R b[3] = {cl * sin(lon), -sin(lat), cl * cos(lon)};
#pragma unroll
    for (int i = 0; i < NR; ++i) rec[L::kR + i] = in.w * (o[i] - b[i]);
    if (JAC) {
#pragma unroll
      for (int i = 0; i < NR * CMAX; ++i) rec[L::kCam + i] = R(0);
    }
  } else {
    R uv[2], Jc[2 * CMAX], Jp2[6];
    project_dispatch<M, CMAX, R>(in.model, p, in.cam, uv, Jp2, Jc);
    rec[L::kR + 0] = in.w * (uv[0] - in.ox);
    rec[L::kR + 1] = in.w * (uv[1] - in.oy);
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
        for (int j = 0; j < CMAX; ++j) rec[L::kCam + i * CMAX + j] = in.w * Jc[i * CMAX + j];
      if (NR == 3) {
#pragma unroll
        for (int j = 0; j < CMAX; ++j) rec[L::kCam + 2 * CMAX + j] = R(0);
      }
    }
  }
  if (!JAC) return;

  // E[m][k] = sum_j drot[m][j][k] v_j  (3x3): derivative of p wrt r_inst
  R E[9];
#pragma unroll
  for (int m = 0; m < 3; ++m)
#pragma unroll
    for (int k = 0; k < 3; ++k)
      E[m * 3 + k] = g.drot[(m * 3 + 0) * 3 + k] * v0 + g.drot[(m * 3 + 1) * 3 + k] * v1 +
                     g.drot[(m * 3 + 2) * 3 + k] * v2;
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    const R a0 = in.w * Jq[i * 3 + 0], a1 = in.w * Jq[i * 3 + 1], a2 = in.w * Jq[i * 3 + 2];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const R jp = a0 * g.rot[0 * 3 + j] + a1 * g.rot[1 * 3 + j] + a2 * g.rot[2 * 3 + j];
      rec[L::kPt + i * 3 + j] = jp;
      rec[L::kInst + i * 6 + 3 + j] = -jp;  // d/d(centre) = -d/dX
      rec[L::kInst + i * 6 + j] = a0 * E[0 * 3 + j] + a1 * E[1 * 3 + j] + a2 * E[2 * 3 + j];
    }
    if constexpr (RIG) {
      // d p / d r_rc = dR_rc (R_inst v - c_rc); d p / d c_rc = -R_rc
      const RigGeom<R>& rg = *in.rg;
      R y[3];
#pragma unroll
      for (int k = 0; k < 3; ++k)
        y[k] = rg.rinst[k * 3 + 0] * v0 + rg.rinst[k * 3 + 1] * v1 + rg.rinst[k * 3 + 2] * v2 - rg.crc[k];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        R s = R(0);
#pragma unroll
        for (int m = 0; m < 3; ++m) {
          const R e = rg.drrc[(m * 3 + 0) * 3 + k] * y[0] + rg.drrc[(m * 3 + 1) * 3 + k] * y[1] +
                      rg.drrc[(m * 3 + 2) * 3 + k] * y[2];
          s += (m == 0 ? a0 : (m == 1 ? a1 : a2)) * e;
        }
        rec[L::kRig + i * 6 + k] = s;
        rec[L::kRig + i * 6 + 3 + k] = -(a0 * rg.rrc[0 * 3 + k] + a1 * rg.rrc[1 * 3 + k] + a2 * rg.rrc[2 * 3 + k]);
      }
    }
  }
}

}  // namespace gbba
