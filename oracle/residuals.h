// Oracle (test infrastructure only) -- reprojection residuals with Jacobian
// blocks, restating
//   opensfm/src/lib/bundle/error/projection_errors.h:15-57 (ReprojectionError2D),
//   :59-208 (ReprojectionError2DAnalytic<C>: blocks camera | rig instance |
//   rig camera | point, scaled by 1/std), :210-375 (ReprojectionError3D for
//   spherical cameras: residual = (normalize(x_cam) - bearing(obs)) / std).
//   opensfm/src/lib/bundle/error/error_utils.h:449-461 (rig composition: the
//   instance pose first, then the rig-camera pose).
#pragma once

#include "camera_math.h"

namespace oracle {

// Number of residual rows for a model (spherical cameras use bearings).
inline int residual_size(int model) { return model == SPHERICAL ? 3 : 2; }

// Observed bearing of a spherical observation (projection_errors.h:214-223).
inline void spherical_bearing(const double* obs, double* b) {
  const double lon = obs[0] * 2 * M_PI;
  const double lat = -obs[1] * 2 * M_PI;
  b[0] = std::cos(lat) * std::sin(lon);
  b[1] = -std::sin(lat);
  b[2] = std::cos(lat) * std::cos(lon);
}

// Generic-scalar residual (no Jacobians), used for AD checks and for
// residual-only cost evaluation.  rig may be null (rig camera not used).
template <class T>
inline void residual_generic(int model, const T* cam, const T* inst, const T* rig, const T* X,
                             const double* obs, double std_dev, T* r) {
  T p1[3], p2[3];
  pose_forward_t<T>(X, inst, p1);
  const T* pc = p1;
  if (rig) {
    pose_forward_t<T>(p1, rig, p2);
    pc = p2;
  }
  const double scale = 1.0 / std_dev;
  if (model == SPHERICAL) {
    using std::sqrt;
    const T n = sqrt(pc[0] * pc[0] + pc[1] * pc[1] + pc[2] * pc[2]);
    double b[3];
    spherical_bearing(obs, b);
    for (int i = 0; i < 3; ++i) r[i] = scale * (pc[i] / n - b[i]);
    return;
  }
  T uv[2];
  project<T>(model, pc, cam, uv);
  r[0] = scale * (uv[0] - obs[0]);
  r[1] = scale * (uv[1] - obs[1]);
}

// Analytic residual + Jacobian blocks (row-major, NR rows):
//   Jcam NRxC, Jinst NRx6, Jrig NRx6 (zeros when rig == null), Jpt NRx3.
// Mirrors the chain rule ComposeForwardDerivatives<TYPE, Pose, Pose> of
// camera_instances.h:275-318.
inline void residual_jac(int model, const double* cam, const double* inst, const double* rig,
                         const double* X, const double* obs, double std_dev, double* r,
                         double* Jcam, double* Jinst, double* Jrig, double* Jpt) {
  const ModelDesc d = model_desc(model);
  const int C = d.n_params;
  const int NR = residual_size(model);
  const double scale = 1.0 / std_dev;
  double p1[3], P1[27];
  pose_jac(X, inst, p1, P1);
  double pc[3];
  // dpc/dX (3x3), dpc/dinst (3x6), dpc/drig (3x6)
  double dX[9], dI[18], dR[18] = {0};
  if (rig) {
    double P2[27];
    pose_jac(p1, rig, pc, P2);
    // dpc/dp1 = P2[:, 0:3]
    for (int i = 0; i < 3; ++i) {
      for (int j = 0; j < 3; ++j) {
        double s = 0;
        for (int k = 0; k < 3; ++k) s += P2[i * 9 + k] * P1[k * 9 + j];
        dX[i * 3 + j] = s;
      }
      for (int j = 0; j < 6; ++j) {
        double s = 0;
        for (int k = 0; k < 3; ++k) s += P2[i * 9 + k] * P1[k * 9 + 3 + j];
        dI[i * 6 + j] = s;
        dR[i * 6 + j] = P2[i * 9 + 3 + j];
      }
    }
  } else {
    for (int i = 0; i < 3; ++i) {
      pc[i] = p1[i];
      for (int j = 0; j < 3; ++j) dX[i * 3 + j] = P1[i * 9 + j];
      for (int j = 0; j < 6; ++j) dI[i * 6 + j] = P1[i * 9 + 3 + j];
    }
  }
  double Jin[9];  // NR x 3: d(out)/d(pc)
  double out[3];
  if (model == SPHERICAL) {
    const double x = pc[0], y = pc[1], z = pc[2];
    const double x2 = x * x, y2 = y * y, z2 = z * z, n2 = x2 + y2 + z2;
    const double n = std::sqrt(n2), i3 = 1.0 / (n * n2);
    // transformations_functions.h:388-418 (Normalize)
    Jin[0] = (y2 + z2) * i3; Jin[1] = -x * y * i3; Jin[2] = -x * z * i3;
    Jin[3] = -y * x * i3; Jin[4] = (x2 + z2) * i3; Jin[5] = -y * z * i3;
    Jin[6] = -z * x * i3; Jin[7] = -z * y * i3; Jin[8] = (x2 + y2) * i3;
    const double inv = 1.0 / std::sqrt(x2 + y2 + z2);
    double b[3];
    spherical_bearing(obs, b);
    for (int i = 0; i < 3; ++i) {
      out[i] = pc[i] * inv;
      r[i] = scale * (out[i] - b[i]);
    }
    for (int i = 0; i < NR * C; ++i) Jcam[i] = 0.0;
  } else {
    double Jc[2 * 16];
    project_jac(model, pc, cam, out, Jin, Jc);
    for (int i = 0; i < 2 * C; ++i) Jcam[i] = scale * Jc[i];
    r[0] = scale * (out[0] - obs[0]);
    r[1] = scale * (out[1] - obs[1]);
  }
  for (int i = 0; i < NR; ++i) {
    for (int j = 0; j < 3; ++j) {
      double s = 0;
      for (int k = 0; k < 3; ++k) s += Jin[i * 3 + k] * dX[k * 3 + j];
      Jpt[i * 3 + j] = scale * s;
    }
    for (int j = 0; j < 6; ++j) {
      double s = 0, t = 0;
      for (int k = 0; k < 3; ++k) {
        s += Jin[i * 3 + k] * dI[k * 6 + j];
        t += Jin[i * 3 + k] * dR[k * 6 + j];
      }
      Jinst[i * 6 + j] = scale * s;
      Jrig[i * 6 + j] = rig ? scale * t : 0.0;
    }
  }
}

// ---------------------------------------------------------------------------
// Depth prior of an observation, restating RelativeDepthError
// (opensfm/src/lib/bundle/error/relative_depth_error.h): the world point in
// the camera frame (WorldToCameraCoordinatesRig with unit scale: the
// instance pose, then the rig-camera pose when it is used), its depth z, or
// its distance to the camera when radial, and the residual
// (depth - value) / std.  value and std are floats in the reference
// (map::Depth, map/observation.h:10-18); callers pass them rounded.
template <class T>
inline T depth_residual_generic(const T* inst, const T* rig, const T* X, double value, double std_dev,
                                bool radial) {
  using std::sqrt;
  T p1[3], p2[3];
  pose_forward_t<T>(X, inst, p1);
  const T* pc = p1;
  if (rig) {
    pose_forward_t<T>(p1, rig, p2);
    pc = p2;
  }
  const T d = radial ? sqrt(pc[0] * pc[0] + pc[1] * pc[1] + pc[2] * pc[2]) : pc[2];
  return (1.0 / std_dev) * (d - value);
}

// The same with its Jacobian rows: Jinst [6], Jrig [6] (zeros when
// rig == null), Jpt [3]; chain rule through pose_jac as residual_jac.
inline double depth_residual_jac(const double* inst, const double* rig, const double* X, double value,
                                 double std_dev, bool radial, double* Jinst, double* Jrig, double* Jpt) {
  const double scale = 1.0 / std_dev;
  double p1[3], P1[27];
  pose_jac(X, inst, p1, P1);
  double pc[3], dX[9], dI[18], dR[18] = {0};
  if (rig) {
    double P2[27];
    pose_jac(p1, rig, pc, P2);
    for (int i = 0; i < 3; ++i) {
      for (int j = 0; j < 3; ++j) {
        double s = 0;
        for (int k = 0; k < 3; ++k) s += P2[i * 9 + k] * P1[k * 9 + j];
        dX[i * 3 + j] = s;
      }
      for (int j = 0; j < 6; ++j) {
        double s = 0;
        for (int k = 0; k < 3; ++k) s += P2[i * 9 + k] * P1[k * 9 + 3 + j];
        dI[i * 6 + j] = s;
        dR[i * 6 + j] = P2[i * 9 + 3 + j];
      }
    }
  } else {
    for (int i = 0; i < 3; ++i) {
      pc[i] = p1[i];
      for (int j = 0; j < 3; ++j) dX[i * 3 + j] = P1[i * 9 + j];
      for (int j = 0; j < 6; ++j) dI[i * 6 + j] = P1[i * 9 + 3 + j];
    }
  }
  double d, g[3];  // depth and d(depth)/d(pc)
  if (radial) {
    d = std::sqrt(pc[0] * pc[0] + pc[1] * pc[1] + pc[2] * pc[2]);
    for (int k = 0; k < 3; ++k) g[k] = pc[k] / d;
  } else {
    d = pc[2];
    g[0] = g[1] = 0.0;
    g[2] = 1.0;
  }
  for (int j = 0; j < 3; ++j) Jpt[j] = scale * (g[0] * dX[j] + g[1] * dX[3 + j] + g[2] * dX[6 + j]);
  for (int j = 0; j < 6; ++j) {
    Jinst[j] = scale * (g[0] * dI[j] + g[1] * dI[6 + j] + g[2] * dI[12 + j]);
    Jrig[j] = rig ? scale * (g[0] * dR[j] + g[1] * dR[6 + j] + g[2] * dR[12 + j]) : 0.0;
  }
  return scale * (d - value);
}

// ---------------------------------------------------------------------------
// Robust losses rho(s), rho'(s), rho''(s) with s = |r|^2, following the
// definitions in Ceres Solver's public documentation (LossFunction section):
//   Trivial s; Huber(a): s <= a^2 ? s : 2a sqrt(s) - a^2;
//   SoftLOne(a): 2b (sqrt(1 + s/b) - 1); Cauchy(a): b log(1 + s/b);
//   Arctan(a): a atan2(s, a); with b = a^2.
enum Loss { LOSS_TRIVIAL = 0, LOSS_HUBER = 1, LOSS_SOFTL1 = 2, LOSS_CAUCHY = 3, LOSS_ARCTAN = 4 };

inline void loss_eval(int loss, double a, double s, double* rho) {
  const double b = a * a;
  switch (loss) {
    case LOSS_HUBER:
      if (s > b) {
        const double r = std::sqrt(s);
        rho[0] = 2.0 * a * r - b;
        rho[1] = a / r;
        rho[2] = -rho[1] / (2.0 * s);
      } else {
        rho[0] = s; rho[1] = 1.0; rho[2] = 0.0;
      }
      return;
    case LOSS_SOFTL1: {
      const double sum = 1.0 + s / b;
      const double tmp = std::sqrt(sum);
      rho[0] = 2.0 * b * (tmp - 1.0);
      rho[1] = 1.0 / tmp;
      rho[2] = -(0.5 / b) * rho[1] / sum;
      return;
    }
    case LOSS_CAUCHY: {
      const double sum = 1.0 + s / b;
      const double inv = 1.0 / sum;
      rho[0] = b * std::log(sum);
      rho[1] = inv;
      rho[2] = -inv * inv / b;
      return;
    }
    case LOSS_ARCTAN: {
      const double inv = 1.0 / (a * a + s * s);
      rho[0] = a * std::atan2(s, a);
      rho[1] = a * a * inv;
      rho[2] = -2.0 * s * b * inv * inv;
      return;
    }
    default:
      rho[0] = s; rho[1] = 1.0; rho[2] = 0.0;
  }
}

}  // namespace oracle
