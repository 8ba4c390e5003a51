// Camera models of the bundle-adjustment path as device/host code.
//
// Each model is PROJECTION -> DISTORTION -> AFFINE; the parameter vector is
// ordered [projection | distortion | affine] and the model ids follow
// geometry::ProjectionType (opensfm/src/lib/geometry/camera_instances.h:8-20,
// :418-430 for the compositions, geometry/src/camera.cc:11-172 for the
// parameter order).  The math restates
//   camera_projections_functions.h:8-230 (projections),
//   camera_distortions_functions.h:12-837 (distortions),
//   transformations_functions.h:13-107 (affine / uniform scale / identity),
// evaluated in a single fused pass that returns the projected point and its
// derivatives with respect to the camera-frame point and to the intrinsics
// (the composition ComposeForwardDerivatives of functions.h:77-97 performs).
//
// The affine stage has a diagonal input Jacobian, so d(uv)/d(point) is
// formed as diag(ax, ay) * D * P without generic 2x2 products.
#pragma once

#include <cmath>

#ifdef __CUDACC__
#define GB_HD __host__ __device__ __forceinline__
#else
#define GB_HD inline
#endif

namespace gbba {

enum Projection : int {
  kPerspective = 0,
  kBrown = 1,
  kFisheye = 2,
  kFisheyeOpencv = 3,
  kFisheye62 = 4,
  kFisheye624 = 5,
  kSpherical = 6,
  kDual = 7,
  kRadial = 8,
  kSimpleRadial = 9,
  kNumProjections = 10
};

constexpr int kMaxCameraParams = 16;

// Parameter counts per model: {projection, distortion, affine}.
template <int M> struct ModelTraits;
#define GB_MODEL(M, NP, ND, NA, PK, DK, AK)                 \
  template <> struct ModelTraits<M> {                       \
    static constexpr int kProj = NP, kDisto = ND, kAff = NA; \
    static constexpr int kSize = (NP + ND + NA) < 1 ? 1 : (NP + ND + NA); \
    static constexpr int kProjKind = PK, kDistoKind = DK, kAffKind = AK;  \
  };
// projection kinds: 0 perspective, 1 fisheye, 2 dual, 3 spherical
// distortion kinds: 0 none, 1 k1, 2 k1k2, 3 k1..k4, 4 brown, 5 62, 6 624
// affine kinds: 0 identity, 1 uniform scale, 2 affine
GB_MODEL(kPerspective, 0, 2, 1, 0, 2, 1)
GB_MODEL(kBrown, 0, 5, 4, 0, 4, 2)
GB_MODEL(kFisheye, 0, 2, 1, 1, 2, 1)
GB_MODEL(kFisheyeOpencv, 0, 4, 4, 1, 3, 2)
GB_MODEL(kFisheye62, 0, 8, 4, 1, 5, 2)
GB_MODEL(kFisheye624, 0, 12, 4, 1, 6, 2)
GB_MODEL(kSpherical, 0, 0, 0, 3, 0, 0)
GB_MODEL(kDual, 1, 2, 1, 2, 2, 1)
GB_MODEL(kRadial, 0, 2, 4, 0, 2, 2)
GB_MODEL(kSimpleRadial, 0, 1, 4, 0, 1, 2)
#undef GB_MODEL

GB_HD int model_num_params(int m) {
  switch (m) {
    case kPerspective: return 3;
    case kBrown: return 9;
    case kFisheye: return 3;
    case kFisheyeOpencv: return 8;
    case kFisheye62: return 12;
    case kFisheye624: return 16;
    case kSpherical: return 1;
    case kDual: return 4;
    case kRadial: return 6;
    case kSimpleRadial: return 5;
  }
  return 0;
}

template <typename R> GB_HD R gb_sqrt(R x) { return sqrt(x); }
template <typename R> GB_HD R gb_atan2(R y, R x) { return atan2(y, x); }
#ifdef __CUDACC__
template <> GB_HD float gb_sqrt<float>(float x) { return sqrtf(x); }
template <> GB_HD float gb_atan2<float>(float y, float x) { return atan2f(y, x); }
#endif

// Projection stage: a = P(p), Pa = dP/dp (2x3 row-major), Pt = dP/dtransition.
template <int PK, typename R>
GB_HD void projection_stage(const R* p, const R* prm, R* a, R* Pa, R* Pt) {
  const R x = p[0], y = p[1], z = p[2];
  if (PK == 0) {  // perspective: (x/z, y/z)
    const R iz = R(1) / z;
    a[0] = x * iz;
    a[1] = y * iz;
    Pa[0] = iz; Pa[1] = R(0); Pa[2] = -x * iz * iz;
    Pa[3] = R(0); Pa[4] = iz; Pa[5] = -y * iz * iz;
  } else if (PK == 1 || PK == 2) {
    // fisheye: theta/r * (x, y) with r = |(x, y)|, theta = atan2(r, z)
    const R x2 = x * x, y2 = y * y, z2 = z * z;
    const R r2 = x2 + y2;
    const R r = gb_sqrt(r2);
    const R R2 = r2 + z2;
    const R th = gb_atan2(r, z);
    const R s = th / r;
    R fa0 = s * x, fa1 = s * y;
    const R inv = R(1) / (r2 * R2 * r);
    const R iR2 = R(1) / R2;
    R F[6];
    F[0] = (y2 * th * R2 + x2 * z * r) * inv;  // (x2 y2 + y4 + y2 z2) th = y2 th R2
    F[1] = x * (y * z * r - y * th * R2) * inv;
    F[2] = -x * iR2;
    F[3] = y * (x * z * r - x * th * R2) * inv;
    F[4] = (x2 * th * R2 + y2 * z * r) * inv;
    F[5] = -y * iR2;
    if (PK == 1) {
      a[0] = fa0; a[1] = fa1;
#pragma unroll
      for (int i = 0; i < 6; ++i) Pa[i] = F[i];
    } else {
      // dual: t * perspective + (1 - t) * fisheye
      const R t = prm[0], u = R(1) - t;
      const R iz = R(1) / z;
      const R px = x * iz, py = y * iz;
      a[0] = t * px + u * fa0;
      a[1] = t * py + u * fa1;
      Pa[0] = t * iz + u * F[0]; Pa[1] = u * F[1]; Pa[2] = t * (-x * iz * iz) + u * F[2];
      Pa[3] = u * F[3]; Pa[4] = t * iz + u * F[4]; Pa[5] = t * (-y * iz * iz) + u * F[5];
      Pt[0] = px - fa0;
      Pt[1] = py - fa1;
    }
  }
}

// Distortion stage: b = D(a), Db = dD/da (2x2), Dk = dD/dk (2xND row-major).
template <int DK, int ND, typename R>
GB_HD void distortion_stage(const R* a, const R* k, R* b, R* Db, R* Dk) {
  const R x = a[0], y = a[1];
  const R x2 = x * x, y2 = y * y, r2 = x2 + y2;
  if (DK == 0) {
    b[0] = x; b[1] = y;
    Db[0] = R(1); Db[1] = R(0); Db[2] = R(0); Db[3] = R(1);
    return;
  }
  // Radial polynomial d(r2) = 1 + k1 r2 + k2 r2^2 + ... and its derivative
  // with respect to r2; tangential (p1, p2) and thin-prism (s0..s3) terms.
  R rad, drad;  // radial factor and d(rad)/d(r2)
  constexpr int NK = DK == 1 ? 1 : DK == 2 ? 2 : DK == 3 ? 4 : DK == 4 ? 3 : 6;
  {
    R acc = k[NK - 1], dacc = R(NK) * k[NK - 1];
#pragma unroll
    for (int i = NK - 2; i >= 0; --i) {
      acc = k[i] + r2 * acc;
      dacc = R(i + 1) * k[i] + r2 * dacc;
    }
    rad = R(1) + r2 * acc;
    drad = dacc;
  }
  R tx = R(0), ty = R(0);
  R t00 = R(0), t01 = R(0), t10 = R(0), t11 = R(0);
  if (DK >= 4) {
    const R p1 = k[NK], p2 = k[NK + 1];
    const R xy = x * y;
    tx = R(2) * p1 * xy + p2 * (r2 + R(2) * x2);
    ty = R(2) * p2 * xy + p1 * (r2 + R(2) * y2);
    t00 = R(2) * p1 * y + R(6) * p2 * x;
    t01 = R(2) * p1 * x + R(2) * p2 * y;
    t10 = t01;
    t11 = R(2) * p2 * x + R(6) * p1 * y;
    if (DK == 6) {
      const R s0 = k[8], s1 = k[9], s2 = k[10], s3 = k[11];
      tx += s0 * r2 + s1 * r2 * r2;
      ty += s2 * r2 + s3 * r2 * r2;
      t00 += R(2) * x * (s0 + R(2) * s1 * r2);
      t01 += R(2) * y * (s0 + R(2) * s1 * r2);
      t10 += R(2) * x * (s2 + R(2) * s3 * r2);
      t11 += R(2) * y * (s2 + R(2) * s3 * r2);
    }
  }
  b[0] = x * rad + tx;
  b[1] = y * rad + ty;
  const R g = R(2) * drad;  // d(rad)/dx = g x, d(rad)/dy = g y
  Db[0] = rad + g * x2 + t00;
  Db[1] = g * x * y + t01;
  Db[2] = g * x * y + t10;
  Db[3] = rad + g * y2 + t11;
  // parameter derivatives
  R rp = r2;
#pragma unroll
  for (int i = 0; i < NK; ++i) {
    Dk[i] = x * rp;
    Dk[ND + i] = y * rp;
    rp *= r2;
  }
  if (DK >= 4) {
    Dk[NK] = R(2) * x * y;
    Dk[NK + 1] = R(3) * x2 + y2;
    Dk[ND + NK] = R(3) * y2 + x2;
    Dk[ND + NK + 1] = R(2) * x * y;
    if (DK == 6) {
      Dk[8] = r2; Dk[9] = r2 * r2; Dk[10] = R(0); Dk[11] = R(0);
      Dk[ND + 8] = R(0); Dk[ND + 9] = R(0); Dk[ND + 10] = r2; Dk[ND + 11] = r2 * r2;
    }
  }
}

// Full model.  uv: projected point; Jp: d(uv)/d(p) 2x3; Jc: d(uv)/d(params)
// 2xC row-major.  Spherical cameras never come here (bearing residuals).
template <int M, typename R>
GB_HD void project_model(const R* p, const R* prm, R* uv, R* Jp, R* Jc) {
  using T = ModelTraits<M>;
  constexpr int C = T::kSize;
  constexpr int ND = T::kDisto;
  R a[2], Pa[6], Pt[2] = {R(0), R(0)};
  projection_stage<T::kProjKind, R>(p, prm, a, Pa, Pt);
  R b[2], Db[4], Dk[2 * (ND > 0 ? ND : 1)];
  distortion_stage<T::kDistoKind, ND, R>(a, prm + T::kProj, b, Db, Dk);
  const R* af = prm + T::kProj + T::kDisto;
  R ax = R(1), ay = R(1);
  if (T::kAffKind == 1) {
    ax = ay = af[0];
    uv[0] = ax * b[0];
    uv[1] = ay * b[1];
  } else if (T::kAffKind == 2) {
    ax = af[0];
    ay = af[0] * af[1];
    uv[0] = ax * b[0] + af[2];
    uv[1] = ay * b[1] + af[3];
  } else {
    uv[0] = b[0];
    uv[1] = b[1];
  }
  // M = diag(ax, ay) * Db
  const R m00 = ax * Db[0], m01 = ax * Db[1], m10 = ay * Db[2], m11 = ay * Db[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    Jp[j] = m00 * Pa[j] + m01 * Pa[3 + j];
    Jp[3 + j] = m10 * Pa[j] + m11 * Pa[3 + j];
  }
  int col = 0;
  if (T::kProj) {
    Jc[0] = m00 * Pt[0] + m01 * Pt[1];
    Jc[C] = m10 * Pt[0] + m11 * Pt[1];
    col = 1;
  }
#pragma unroll
  for (int t = 0; t < ND; ++t) {
    Jc[col + t] = ax * Dk[t];
    Jc[C + col + t] = ay * Dk[ND + t];
  }
  col += ND;
  if (T::kAffKind == 1) {
    Jc[col] = b[0];
    Jc[C + col] = b[1];
  } else if (T::kAffKind == 2) {
    Jc[col + 0] = b[0];       Jc[C + col + 0] = af[1] * b[1];
    Jc[col + 1] = R(0);       Jc[C + col + 1] = af[0] * b[1];
    Jc[col + 2] = R(1);       Jc[C + col + 2] = R(0);
    Jc[col + 3] = R(0);       Jc[C + col + 3] = R(1);
  }
}

// Spherical bearing residual stage (projection_errors.h:210-375):
// out = p / |p| and d(out)/dp (3x3).
template <typename R>
GB_HD void normalize_stage(const R* p, R* out, R* J) {
  const R x = p[0], y = p[1], z = p[2];
  const R x2 = x * x, y2 = y * y, z2 = z * z, n2 = x2 + y2 + z2;
  const R n = gb_sqrt(n2);
  const R in = R(1) / n;
  const R i3 = in / n2;
  out[0] = x * in; out[1] = y * in; out[2] = z * in;
  J[0] = (y2 + z2) * i3; J[1] = -x * y * i3; J[2] = -x * z * i3;
  J[3] = -x * y * i3; J[4] = (x2 + z2) * i3; J[5] = -y * z * i3;
  J[6] = -x * z * i3; J[7] = -y * z * i3; J[8] = (x2 + y2) * i3;
}

}  // namespace gbba
