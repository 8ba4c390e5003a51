// Oracle (test infrastructure only) -- FP64 CPU bundle-adjustment solver.
//
// Restates the optimisation the reference runs through Ceres
// (bundle_adjuster.cc:670-1203, irls_solver.cc:93-474, mixture_reweighting.cc)
// with an exact linear solve: points are eliminated by the Schur complement
// and the dense reduced camera system is factorised by Cholesky (the
// reference's DENSE_SCHUR).  The trust-region and robust-loss rules follow
// Ceres' public documentation:
//   * Levenberg-Marquardt, initial radius 1e4, max radius 1e8, min relative
//     decrease 1e-3, radius /= max(1/3, 1 - (2 rho - 1)^3) on success,
//     radius /= factor and factor *= 2 on failure; non-monotonic steps;
//   * Jacobi scaling 1/(1 + |J_j|) from the first iteration, LM diagonal
//     clamped to [1e-6, 1e32];
//   * robust loss through the residual/Jacobian correction of Triggs et al.;
//   * IRLS mixture reweighting every max_iterations/10 successful iterations
//     or on inner convergence, terminating on a relative log-likelihood
//     change below 1e-3.
// Cost, gradient and every linear-algebra step are FP64.  Only the tests and
// the bench's CPU-baseline leg call it.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

#include "residuals.h"

using namespace oracle;

namespace {

constexpr double kEps = 2.220446049250313e-16;

}  // namespace

extern "C" {

struct OracleProblem {
  int32_t n_cameras;
  const int32_t* camera_model;
  const double* camera_values;  // [n][16]
  const double* camera_prior;   // [n][16]
  const double* camera_sigma;   // [n][16]
  const uint8_t* camera_free;   // [n][16]
  const uint8_t* camera_log;    // [n][16]
  int32_t n_instances;
  const double* instance_poses;  // [n][6]
  const uint8_t* instance_free;  // [n][6]
  const uint8_t* instance_has_gps;
  const double* gps_position;  // [n][3]
  const double* gps_std;       // [n][3]
  int32_t n_rig_cameras;
  const double* rig_poses;  // [n][6]
  const uint8_t* rig_free;  // [n][6]
  const uint8_t* rig_used;
  const uint8_t* rig_has_prior;
  const double* rig_prior;  // [n][6]
  const double* rig_sigma;  // [n][6]
  int32_t n_shots;
  const int32_t* shot_instance;
  const int32_t* shot_rig;
  const int32_t* shot_camera;
  int64_t n_points;
  const double* points;  // [n][3]
  const uint8_t* point_free;
  const uint8_t* point_has_prior;
  const double* point_prior;  // [n][3]
  const double* point_sigma;  // [n][3]
  const uint8_t* point_has_altitude;
  int64_t n_obs;
  const int32_t* obs_shot;
  const int32_t* obs_point;
  const double* obs_xy;
  const double* obs_std;
  const uint8_t* obs_gcp;
  // absolute orientation constraints of shots
  int32_t n_orient;
  const int32_t* orient_kind;   // 0 up vector, 1 pan, 2 tilt, 3 roll
  const int32_t* orient_shot;
  const double* orient_target;  // [n][3]: the up vector, or the angle in [0]
  const double* orient_std;
  // constraints between shots
  int32_t n_rel;
  const int32_t* rel_kind;     // 0 relative rotation, 1 common position, 2 linear motion, 3 gauge, 4 heatmap,
                               // 5 relative motion
  const int32_t* rel_shots;    // [n][3]
  // [n][64]: rotation[3] + scale matrix[9]; margin, std; alpha, position
  // std, orientation std; distance; x offset, y offset, std; motion[7],
  // observed flag, scale matrix[49], robust multiplier, scale indices i, j
  const double* rel_params;
  int32_t rel_loss;            // loss of the relative rotations (projection loss kinds)
  double rel_loss_threshold;
  // the heatmap of the kind-4 constraints (params: x offset, y offset, std)
  const double* heat_grid;
  int64_t heat_n;
  int32_t heat_width;
  double heat_resolution;
  // reconstruction scales (the unknowns of the relative motions)
  int32_t n_scales;
  const double* scales;
  const uint8_t* scale_free;
  // depth priors of observations (RelativeDepthError, IRLS group DEPTH,
  // under the projection loss): terms n_obs .. n_obs + n_depth - 1
  int64_t n_depth;
  const int64_t* depth_obs;     // [n] the observation it belongs to
  const double* depth_value;    // [n]
  const double* depth_std;      // [n]
  const uint8_t* depth_radial;  // [n]
};

struct OracleOptions {
  int32_t max_iterations;
  int32_t loss;
  double loss_threshold;
  int32_t irls;  // 0 none, 1 mixture
  double density_ratio;
  int32_t skip_initial_reweighting;
  int32_t threads;
};

struct OracleResult {
  double* camera_values;   // [n][16]
  double* instance_poses;  // [n][6]
  double* rig_poses;       // [n][6]
  double* points;          // [n][3]
  double* scales;          // [n_scales]
  double* obs_weights;     // [n_obs]
  double* obs_errors;      // [n_obs][3] unscaled residuals
  double* trace_cost;      // [capacity]
  int32_t trace_capacity;
  int32_t trace_n;
  double initial_cost;
  double final_cost;
  int32_t iterations;
  int32_t successful;
  int32_t termination;  // 0 no convergence, 1 convergence, 2 IRLS success, 3 failure
};

}  // extern "C"

namespace {

struct State {
  std::vector<double> cam, inst, rig, pts;  // cam [n][16], inst/rig [n][6], pts [n][3]
  std::vector<double> scl;                  // reconstruction scales
};

// Compact indices of the optimised camera-side coordinates.
struct Index {
  std::vector<int> inst, rig, cam, scl;  // -1 for fixed coordinates
  int n = 0;
};

constexpr int kRelParams = 64;

struct Mixture {
  double ll = 0.0;
};

// ---- absolute orientation constraints
// UpVectorError, PanAngleError, TiltAngleError and RollAngleError
// (bundle/error/absolute_motion_errors.h:10-126) on the shot rotation, the
// rig instance rotation composed with the rig camera rotation
// (bundle/error/position_functors.h:40-63).  Restated with rotation
// matrices: R = R(instance) R(rig camera), and R e_x, R e_z are its first
// and third columns.  Derivatives w.r.t. the two rotations (slots 0..2 and
// 3..5) by forward-mode duals.
using D6 = Dual<6>;

D6 asin6(const D6& a) {
  D6 r(std::asin(a.v));
  const double k = 1.0 / std::sqrt(1.0 - a.v * a.v);
  for (int i = 0; i < 6; ++i) r.d[i] = a.d[i] * k;
  return r;
}

// Rodrigues: R = cos t I + sin t [k]x + (1 - cos t) k k^T, k = a / t
template <class T>
void rotation_matrix(const T* a, T* M) {
  const T t2 = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
  if (t2.v > kEps) {
    const T t = sqrt(t2);
    const T k[3] = {a[0] / t, a[1] / t, a[2] / t};
    const T c = cos(t), sn = sin(t), v = 1.0 - c;
    M[0] = c + v * k[0] * k[0];
    M[1] = v * k[0] * k[1] - sn * k[2];
    M[2] = v * k[0] * k[2] + sn * k[1];
    M[3] = v * k[1] * k[0] + sn * k[2];
    M[4] = c + v * k[1] * k[1];
    M[5] = v * k[1] * k[2] - sn * k[0];
    M[6] = v * k[2] * k[0] - sn * k[1];
    M[7] = v * k[2] * k[1] + sn * k[0];
    M[8] = c + v * k[2] * k[2];
  } else {
    M[0] = T(1.0), M[1] = -a[2], M[2] = a[1];
    M[3] = a[2], M[4] = T(1.0), M[5] = -a[0];
    M[6] = -a[1], M[7] = a[0], M[8] = T(1.0);
  }
}

template <class T>
T wrap_angle(const T& d) {
  if (d.v > M_PI) return d - 2 * M_PI;
  if (d.v < -M_PI) return d + 2 * M_PI;
  return d;
}

// Scaled residuals (1 or 3) of one constraint; returns the count.
int orientation_residual(int kind, const double* target, double std_dev, const double* ri, const double* rc,
                         D6* r) {
  D6 a[3], b[3], A[9], B[9], R[9];
  for (int k = 0; k < 3; ++k) {
    a[k] = D6::var(ri[k], k);
    b[k] = D6::var(rc[k], 3 + k);
  }
  rotation_matrix(a, A);
  rotation_matrix(b, B);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) R[3 * i + j] = A[3 * i] * B[j] + A[3 * i + 1] * B[3 + j] + A[3 * i + 2] * B[6 + j];
  const double scale = 1.0 / std_dev;
  const D6 z[3] = {R[2], R[5], R[8]}, x[3] = {R[0], R[3], R[6]};
  if (kind == 0) {
    const double n = std::sqrt(target[0] * target[0] + target[1] * target[1] + target[2] * target[2]);
    const double u[3] = {target[0] / n, target[1] / n, target[2] / n};
    for (int i = 0; i < 3; ++i) {
      const D6 v = R[3 * i] * u[0] + R[3 * i + 1] * u[1] + R[3 * i + 2] * u[2];
      r[i] = scale * (v - (i == 2 ? 1.0 : 0.0));
    }
    return 3;
  }
  if (kind == 1) {
    if (std::fabs(z[0].v) < 1e-8 && std::fabs(z[1].v) < 1e-8) r[0] = D6(0.0);
    else r[0] = scale * wrap_angle(atan2(z[0], z[1]) - target[0]);
    return 1;
  }
  if (kind == 2) {
    const D6 l = sqrt(z[0] * z[0] + z[1] * z[1]);
    r[0] = scale * wrap_angle(-atan2(z[2], l) - target[0]);
    return 1;
  }
  // roll: the angle of the camera x axis out of the horizontal plane
  const double eps = 1e-5;
  D6 h[2] = {z[1], -z[0]};
  const D6 lh = sqrt(h[0] * h[0] + h[1] * h[1]);
  if (lh.v < eps) {
    r[0] = D6(0.0);
    return 1;
  }
  h[0] = h[0] / lh;
  h[1] = h[1] / lh;
  // c = x cross (h0, h1, 0)
  const D6 c[3] = {-x[2] * h[1], x[2] * h[0], x[0] * h[1] - x[1] * h[0]};
  const D6 sin_roll = z[0] * c[0] + z[1] * c[1] + z[2] * c[2];
  if (sin_roll.v <= -(1.0 - eps)) {
    r[0] = D6(0.0);
    return 1;
  }
  r[0] = scale * wrap_angle(asin6(sin_roll) - target[0]);
  return 1;
}

// ---- constraints between shots
// RelativeRotationError, CommonPositionError (relative_motion_errors.h:
// 66-126) and LinearMotionError (motion_prior_errors.h:12-74) on the shot
// poses (position_functors.h:12-63).  Restated with rotation matrices: the
// shot rotation is R(instance) R(rig camera), its position the instance
// position plus R(instance) times the rig camera position, and a composed
// rotation's angle-axis is the matrix logarithm (atan2 of the skew part's
// norm and the trace).  12 derivative slots per shot: instance rotation,
// instance position, rig camera rotation, rig camera position.
using D36 = Dual<36>;

template <class T>
void matmul3(const T* A, const T* B, T* C, bool transpose_b = false) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      T acc(0.0);
      for (int k = 0; k < 3; ++k) acc = acc + A[3 * i + k] * (transpose_b ? B[3 * j + k] : B[3 * k + j]);
      C[3 * i + j] = acc;
    }
}

template <class T>
void log_rotation(const T* M, T* a) {
  const T v[3] = {(M[7] - M[5]) * 0.5, (M[2] - M[6]) * 0.5, (M[3] - M[1]) * 0.5};
  const T c = (M[0] + M[4] + M[8] - 1.0) * 0.5;
  const T s2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
  T k(1.0);
  if (s2.v > 1e-24) {
    const T sn = sqrt(s2);
    k = atan2(sn, c) / sn;
  }
  for (int i = 0; i < 3; ++i) a[i] = v[i] * k;
}

struct ShotFrame {
  D36 R[9];
  D36 p[3];
};

ShotFrame shot_frame(int k, const double* pi, const double* pc) {
  ShotFrame f;
  D36 ri[3], rc[3], tc[3], Ri[9], Rc[9];
  for (int i = 0; i < 3; ++i) {
    ri[i] = D36::var(pi[i], 12 * k + i);
    f.p[i] = D36::var(pi[3 + i], 12 * k + 3 + i);
    rc[i] = D36::var(pc ? pc[i] : 0.0, 12 * k + 6 + i);
    tc[i] = D36::var(pc ? pc[3 + i] : 0.0, 12 * k + 9 + i);
  }
  rotation_matrix(ri, Ri);
  if (!pc) {
    for (int i = 0; i < 9; ++i) f.R[i] = Ri[i];
    return f;
  }
  rotation_matrix(rc, Rc);
  matmul3(Ri, Rc, f.R);
  for (int i = 0; i < 3; ++i) f.p[i] = f.p[i] + Ri[3 * i] * tc[0] + Ri[3 * i + 1] * tc[1] + Ri[3 * i + 2] * tc[2];
  return f;
}

// ---- position heatmap (HeatmapdCostFunctor, absolute_motion_errors.h:
// 128-173): bicubic convolution of the grid with the Catmull-Rom kernel
// (Keys, a = -1/2) as four weights per axis, indices clamped to the grid.
struct HeatGrid {
  const double* data;
  int64_t n;
  int width;
  double resolution;
};

void keys_weights(double t, double* w, double* dw) {
  const double t2 = t * t, t3 = t2 * t;
  w[0] = 0.5 * (-t3 + 2.0 * t2 - t);
  w[1] = 0.5 * (3.0 * t3 - 5.0 * t2 + 2.0);
  w[2] = 0.5 * (-3.0 * t3 + 4.0 * t2 + t);
  w[3] = 0.5 * (t3 - t2);
  dw[0] = 0.5 * (-3.0 * t2 + 4.0 * t - 1.0);
  dw[1] = 0.5 * (9.0 * t2 - 10.0 * t);
  dw[2] = 0.5 * (-9.0 * t2 + 8.0 * t + 1.0);
  dw[3] = 0.5 * (3.0 * t2 - 2.0 * t);
}

double heat_value(const HeatGrid& g, double r, double c, double* fr, double* fc) {
  const int height = int(g.n / g.width);
  const double r0 = std::floor(r), c0 = std::floor(c);
  double wr[4], dwr[4], wc[4], dwc[4];
  keys_weights(r - r0, wr, dwr);
  keys_weights(c - c0, wc, dwc);
  double f = 0.0;
  *fr = *fc = 0.0;
  for (int i = 0; i < 4; ++i) {
    const int ri = std::min(std::max(int(r0) - 1 + i, 0), height - 1);
    for (int j = 0; j < 4; ++j) {
      const int cj = std::min(std::max(int(c0) - 1 + j, 0), g.width - 1);
      const double v = g.data[int64_t(ri) * g.width + cj];
      f += wr[i] * wc[j] * v;
      *fr += dwr[i] * wc[j] * v;
      *fc += wr[i] * dwc[j] * v;
    }
  }
  return f;
}

int relative_residual(int kind, const double* const* pi, const double* const* pc, const double* prm, D36* r,
                      const HeatGrid* grid = nullptr, const double* scales = nullptr) {
  if (kind == 8) {
    // DataPriorError with SimilarityPriorTransform (prior_error.h:19-114,
    // bias.h:34-54): (t - (c R(w) p + b)) / (std m) on the instance
    // position t, the camera bias (w, b, c) in slots 12..18 (scales[1..7]),
    // the std multiplier m in slot 24 (scales[0])
    const D36 m = D36::var(scales[0], 24);
    D36 w[3], Rw[9];
    for (int k = 0; k < 3; ++k) w[k] = D36::var(scales[1 + k], 12 + k);
    rotation_matrix(w, Rw);
    const D36 c = D36::var(scales[7], 18);
    for (int k = 0; k < 3; ++k) {
      const D36 rp = Rw[3 * k] * prm[0] + Rw[3 * k + 1] * prm[1] + Rw[3 * k + 2] * prm[2];
      const D36 prior = c * rp + D36::var(scales[4 + k], 15 + k);
      r[k] = (D36::var(pi[0][3 + k], 3 + k) - prior) / (m * prm[3 + k]);
    }
    return 3;
  }
  if (kind == 6) {
    // DataPriorError with adjust_scales (prior_error.h:54-93): (t - prior) /
    // (std m) on the instance position, m in slot 24
    const D36 m = D36::var(scales[0], 24);
    for (int k = 0; k < 3; ++k) r[k] = (D36::var(pi[0][3 + k], 3 + k) - prm[k]) / (m * prm[3 + k]);
    return 3;
  }
  if (kind == 7) {
    // StdDeviationConstraint (parameters_errors.h:7-16)
    const D36 m = D36::var(scales[0], 24);
    r[0] = log(1.0 / sqrt(m * m * (2.0 * M_PI)));
    return 1;
  }
  if (kind == 5) {
    // RelativeMotionError (relative_motion_errors.h:13-64) on the instance
    // poses alone: rotation log(R_ij R_i^T R_j), translation t_ij - s_j
    // R_j^T (t_i - t_j), scale S_ij - s_j / s_i when observed; then the 7 x
    // 7 matrix.  Scales in slots 24, 25.
    const ShotFrame fi = shot_frame(0, pi[0], nullptr), fj = shot_frame(1, pi[1], nullptr);
    const D36 si = D36::var(scales[0], 24), sj = D36::var(scales[1], 25);
    D36 rij[3], Rij[9], T1[9], T2[9], e[7];
    for (int i = 0; i < 3; ++i) rij[i] = D36(prm[i]);
    rotation_matrix(rij, Rij);
    matmul3(Rij, fi.R, T1, true);
    matmul3(T1, fj.R, T2);
    log_rotation(T2, e);
    for (int i = 0; i < 3; ++i) {
      D36 v(0.0);
      for (int k = 0; k < 3; ++k) v = v + fj.R[3 * k + i] * (fi.p[k] - fj.p[k]);  // (R_j^T d)_i
      e[3 + i] = prm[3 + i] - sj * v;
    }
    e[6] = prm[7] != 0.0 ? prm[6] - sj / si : D36(0.0);
    const bool undefined = scales[0] == 0.0 || scales[1] == 0.0;
    for (int i = 0; i < 7; ++i) {
      D36 acc(0.0);
      for (int k = 0; k < 7; ++k) acc = acc + e[k] * prm[8 + 7 * i + k];
      r[i] = undefined ? D36(std::numeric_limits<double>::quiet_NaN()) : acc;
    }
    return 7;
  }
  if (kind == 4) {
    const ShotFrame f = shot_frame(0, pi[0], pc[0]);
    const int height = int(grid->n / grid->width);
    const D36 row = (f.p[1] - prm[1]) * (-1.0 / grid->resolution) + 0.5 * height;
    const D36 col = (f.p[0] - prm[0]) * (1.0 / grid->resolution) + 0.5 * grid->width;
    double fr, fc;
    D36 v(heat_value(*grid, row.v, col.v, &fr, &fc));
    for (int k = 0; k < 36; ++k) v.d[k] = fr * row.d[k] + fc * col.d[k];
    r[0] = v * (1.0 / prm[2]);
    return 1;
  }
  if (kind == 3) {
    // TranslationPriorError (absolute_motion_errors.h:175-190) on the
    // instance positions: log of the distance ratio
    D36 d[3];
    for (int i = 0; i < 3; ++i) d[i] = D36::var(pi[0][3 + i], 3 + i) - D36::var(pi[1][3 + i], 15 + i);
    r[0] = log(sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) / prm[0]);
    return 1;
  }
  const int n = kind == 2 ? 3 : 2;
  ShotFrame f[3];
  for (int k = 0; k < n; ++k) f[k] = shot_frame(k, pi[k], pc[k]);
  if (kind == 0) {
    D36 rij[3], Rij[9], T1[9], T2[9], e[3];
    for (int i = 0; i < 3; ++i) rij[i] = D36(prm[i]);
    rotation_matrix(rij, Rij);
    matmul3(Rij, f[0].R, T1, true);  // R_ij R_i^T
    matmul3(T1, f[1].R, T2);
    log_rotation(T2, e);
    for (int i = 0; i < 3; ++i) r[i] = e[0] * prm[3 + 3 * i] + e[1] * prm[4 + 3 * i] + e[2] * prm[5 + 3 * i];
    return 3;
  }
  if (kind == 1) {
    const double scale = 1.0 / prm[1];
    for (int i = 0; i < 3; ++i) {
      D36 e = f[0].p[i] - f[1].p[i];
      if (i < 2) {
        if (e.v < 0.0) e = -e;
        e = e - prm[0];
        if (e.v < 0.0) e = D36(0.0);
      }
      r[i] = e * scale;
    }
    return 3;
  }
  const double alpha = prm[0], ps = 1.0 / prm[1], os = 1.0 / prm[2];
  D36 d20[3], d10[3];
  for (int i = 0; i < 3; ++i) {
    d20[i] = f[2].p[i] - f[0].p[i];
    d10[i] = f[1].p[i] - f[0].p[i];
  }
  const D36 n20 = sqrt(d20[0] * d20[0] + d20[1] * d20[1] + d20[2] * d20[2]);
  const D36 n10 = sqrt(d10[0] * d10[0] + d10[1] * d10[1] + d10[2] * d10[2]);
  for (int i = 0; i < 3; ++i) r[i] = n20.v > 1e-15 ? (alpha - n10 / n20) * ps : (d20[i] * alpha - d10[i]) * ps;
  D36 M20[9], M01[9], a[3], b[3], Ra[9], Rb[9], Rab[9], e[3];
  matmul3(f[2].R, f[0].R, M20, true);  // R2 R0^T
  matmul3(f[0].R, f[1].R, M01, true);  // R0 R1^T
  log_rotation(M20, a);
  log_rotation(M01, b);
  for (int i = 0; i < 3; ++i) a[i] = a[i] * alpha;
  rotation_matrix(a, Ra);
  rotation_matrix(b, Rb);
  matmul3(Ra, Rb, Rab);
  log_rotation(Rab, e);
  for (int i = 0; i < 3; ++i) r[3 + i] = e[i] * os;
  return 6;
}

// rho of the losses, Tukey (kind 5) included (Ceres' documented forms)
void loss_rho5(int kind, double a, double s, double* rho) {
  if (kind != 5) {
    loss_eval(kind, a, s, rho);
    return;
  }
  const double b = a * a;
  if (s <= b) {
    const double v = 1.0 - s / b;
    rho[0] = b / 3.0 * (1.0 - v * v * v);
    rho[1] = v * v;
    rho[2] = -2.0 * v / b;
  } else {
    rho[0] = b / 3.0, rho[1] = 0.0, rho[2] = 0.0;
  }
}

struct Solver {
  const OracleProblem& P;
  const OracleOptions& O;
  Index idx;
  std::vector<double> w_obs, w_cam, w_rig, w_gps, w_pp, w_orient, w_rel;
  std::vector<int> gps_list, pp_list;
  int threads;

  Solver(const OracleProblem& p, const OracleOptions& o) : P(p), O(o) {
    threads = std::max(1, o.threads);
    idx.inst.assign(6 * P.n_instances, -1);
    idx.rig.assign(6 * std::max(0, P.n_rig_cameras), -1);
    idx.cam.assign(16 * P.n_cameras, -1);
    for (int i = 0; i < P.n_instances; ++i)
      for (int k = 0; k < 6; ++k)
        if (P.instance_free[6 * i + k]) idx.inst[6 * i + k] = idx.n++;
    for (int r = 0; r < P.n_rig_cameras; ++r)
      for (int k = 0; k < 6; ++k)
        if (P.rig_used[r] && P.rig_free[6 * r + k]) idx.rig[6 * r + k] = idx.n++;
    for (int c = 0; c < P.n_cameras; ++c) {
      const int C = model_desc(P.camera_model[c]).n_params;
      for (int k = 0; k < C; ++k)
        if (P.camera_free[16 * c + k]) idx.cam[16 * c + k] = idx.n++;
    }
    idx.scl.assign(std::max(0, P.n_scales), -1);
    for (int k = 0; k < P.n_scales; ++k)
      if (P.scale_free[k]) idx.scl[k] = idx.n++;
    w_obs.assign(n_terms(), 1.0);
    w_cam.assign(P.n_cameras, 1.0);
    w_rig.assign(P.n_rig_cameras, 1.0);
    for (int i = 0; i < P.n_instances; ++i)
      if (P.instance_has_gps[i]) gps_list.push_back(i);
    w_gps.assign(gps_list.size(), 1.0);
    for (int64_t p = 0; p < P.n_points; ++p)
      if (P.point_has_prior[p]) pp_list.push_back(int(p));
    w_pp.assign(pp_list.size(), 1.0);
    w_orient.assign(std::max(0, P.n_orient), 1.0);
    w_rel.assign(std::max(0, P.n_rel), 1.0);
  }

  // Constraint q between shots at state s: residuals and Jacobian after the
  // loss correction (Triggs; alpha = 0 when rho'' <= 0) times the IRLS
  // weight, the compact columns of the 36 slots, w rho through *rho and the
  // raw residuals through raw.
  int relative_term(const State& s, int q, D36* r, int* col, double* rho, double* raw = nullptr) const {
    const int kind = P.rel_kind[q], n = kind == 2 ? 3 : (kind == 4 || kind == 6 || kind == 8) ? 1 : kind == 7 ? 0 : 2;
    const double* prm = P.rel_params + kRelParams * q;
    const double* pi[3] = {nullptr, nullptr, nullptr};
    const double* pc[3] = {nullptr, nullptr, nullptr};
    for (int a = 0; a < 36; ++a) col[a] = -1;
    for (int k = 0; k < n; ++k) {
      const int sh = P.rel_shots[3 * q + k];
      const int inst = P.shot_instance[sh], rc = P.shot_rig[sh];
      pi[k] = &s.inst[6 * inst];
      for (int a = 0; a < 6; ++a) col[12 * k + a] = idx.inst[6 * inst + a];
      // the heatmap functor always composes the rig camera; the relative
      // motion and the GPS prior none
      if (rc >= 0 && (P.rig_used[rc] || kind == 4) && kind != 5 && kind != 6 && kind != 8) {
        pc[k] = &s.rig[6 * rc];
        for (int a = 0; a < 6; ++a) col[12 * k + 6 + a] = idx.rig[6 * rc + a];
      }
    }
    const HeatGrid grid{P.heat_grid, P.heat_n, P.heat_width, P.heat_resolution};
    double scales[2] = {1.0, 1.0};
    if (kind == 5)
      for (int k = 0; k < 2; ++k) {
        const int si = int(prm[58 + k]);
        scales[k] = s.scl[si];
        col[24 + k] = idx.scl[si];
      }
    if (kind == 6 || kind == 7) {
      // the std multiplier: params[6] (GPS prior) or params[0] (regulariser)
      const int si = int(prm[kind == 6 ? 6 : 0]);
      scales[0] = s.scl[si];
      col[24] = idx.scl[si];
    }
    double biased[8] = {1, 0, 0, 0, 0, 0, 0, 1};
    if (kind == 8) {
      // the std multiplier (params[6], -1: none) and the seven bias
      // unknowns (params[7..13])
      if (prm[6] >= 0) {
        biased[0] = s.scl[int(prm[6])];
        col[24] = idx.scl[int(prm[6])];
      }
      for (int j = 0; j < 7; ++j) {
        const int si = int(prm[7 + j]);
        biased[1 + j] = s.scl[si];
        col[12 + j] = idx.scl[si];
      }
    }
    const int m = relative_residual(kind, pi, pc, prm, r, &grid, kind == 8 ? biased : scales);
    double sq = 0.0;
    for (int a = 0; a < m; ++a) {
      sq += r[a].v * r[a].v;
      if (raw) raw[a] = r[a].v;
    }
    // relative rotation and motion: the relative-motion loss (a motion's at
    // threshold x robust multiplier); Tukey(1); Cauchy(1); none; none
    static const int kLoss[9] = {-1, 5, LOSS_CAUCHY, LOSS_TRIVIAL, LOSS_TRIVIAL, -1, LOSS_TRIVIAL, LOSS_TRIVIAL,
                                 LOSS_TRIVIAL};
    const int loss = (kind == 0 || kind == 5) ? P.rel_loss : kLoss[kind];
    const double la = kind == 0 ? P.rel_loss_threshold : kind == 5 ? P.rel_loss_threshold * prm[57] : 1.0;
    double rh[3];
    loss_rho5(loss, la, sq, rh);
    for (double& v : rh) v *= w_rel[q];
    *rho = rh[0];
    const double sq1 = std::sqrt(rh[1]);
    double rs = sq1, as = 0.0;
    if (sq > 0.0 && rh[2] > 0.0) {
      const double alpha = 1.0 - std::sqrt(1.0 + 2.0 * sq * rh[2] / rh[1]);
      rs = sq1 / (1.0 - alpha);
      as = alpha / sq;
    }
    for (int k = 0; k < 36; ++k) {
      double rj = 0.0;
      for (int a = 0; a < m; ++a) rj += r[a].v * r[a].d[k];
      for (int a = 0; a < m; ++a) r[a].d[k] = sq1 * (r[a].d[k] - as * r[a].v * rj);
    }
    for (int a = 0; a < m; ++a) r[a].v *= rs;
    return m;
  }

  // Orientation constraint q at state s under CauchyLoss(1) and its IRLS
  // weight: the residuals and Jacobian corrected by sqrt(w rho'(|r|^2))
  // (rho'' < 0, so no second-order term), the compact columns of the two
  // rotations (-1: fixed), and w rho(|r|^2) through *rho.
  int orientation_term(const State& s, int q, D6* r, int* col, double* rho, double* raw = nullptr) const {
    const int sh = P.orient_shot[q];
    const int inst = P.shot_instance[sh], rc = P.shot_rig[sh];
    const bool use_rig = rc >= 0 && P.rig_used[rc];
    static const double zero[3] = {0, 0, 0};
    const int m = orientation_residual(P.orient_kind[q], P.orient_target + 3 * q, P.orient_std[q], &s.inst[6 * inst],
                                       use_rig ? &s.rig[6 * rc] : zero, r);
    for (int k = 0; k < 3; ++k) {
      col[k] = idx.inst[6 * inst + k];
      col[3 + k] = use_rig ? idx.rig[6 * rc + k] : -1;
    }
    double sq = 0.0;
    for (int a = 0; a < m; ++a) {
      sq += r[a].v * r[a].v;
      if (raw) raw[a] = r[a].v;
    }
    *rho = w_orient[q] * std::log1p(sq);
    const double f = std::sqrt(w_orient[q] / (1.0 + sq));
    for (int a = 0; a < m; ++a) r[a] = r[a] * f;
    return m;
  }

  template <typename F>
  void par(int64_t n, F&& f) const {
    if (threads <= 1 || n < 2048) {
      for (int64_t i = 0; i < n; ++i) f(i, 0);
      return;
    }
    std::vector<std::thread> pool;
    const int64_t chunk = (n + threads - 1) / threads;
    for (int t = 0; t < threads; ++t) {
      const int64_t b = t * chunk, e = std::min(n, b + chunk);
      if (b >= e) break;
      pool.emplace_back([b, e, t, &f] {
        for (int64_t i = b; i < e; ++i) f(i, t);
      });
    }
    for (auto& th : pool) th.join();
  }

  // Residual terms: the observations, then the depth priors.
  int64_t n_terms() const { return P.n_obs + std::max<int64_t>(0, P.n_depth); }
  int64_t term_obs(int64_t i) const { return i < P.n_obs ? i : P.depth_obs[i - P.n_obs]; }
  int term_point(int64_t i) const { return P.obs_point[term_obs(i)]; }

  // depth prior k: the scaled residual and (when Ji) its Jacobian rows
  double depth_term(const State& s, int64_t k, double* Ji = nullptr, double* Jr = nullptr, double* Jp = nullptr,
                    bool* use_rig_out = nullptr) const {
    const int64_t o = P.depth_obs[k];
    const int sh = P.obs_shot[o];
    const int rc = P.shot_rig[sh];
    const bool use_rig = rc >= 0 && P.rig_used[rc];
    if (use_rig_out) *use_rig_out = use_rig;
    const double* inst = &s.inst[6 * P.shot_instance[sh]];
    const double* rig = use_rig ? &s.rig[6 * rc] : nullptr;
    const double* X = &s.pts[3 * P.obs_point[o]];
    if (Ji) return depth_residual_jac(inst, rig, X, P.depth_value[k], P.depth_std[k], P.depth_radial[k] != 0, Ji, Jr, Jp);
    return depth_residual_generic<double>(inst, rig, X, P.depth_value[k], P.depth_std[k], P.depth_radial[k] != 0);
  }

  // scaled residual of term i at state s
  int obs_residual(const State& s, int64_t i, double* r) const {
    if (i >= P.n_obs) {
      r[0] = depth_term(s, i - P.n_obs);
      r[1] = r[2] = 0.0;
      return 1;
    }
    const int sh = P.obs_shot[i];
    const int cam = P.shot_camera[sh];
    const int model = P.camera_model[cam];
    const int rc = P.shot_rig[sh];
    const double* rig = (rc >= 0 && P.rig_used[rc]) ? &s.rig[6 * rc] : nullptr;
    residual_generic<double>(model, &s.cam[16 * cam], &s.inst[6 * P.shot_instance[sh]], rig,
                             &s.pts[3 * P.obs_point[i]], P.obs_xy + 2 * i, P.obs_std[i], r);
    return residual_size(model);
  }

  // prior residuals
  int cam_prior(const State& s, int c, double* r, double* J) const {
    const int C = model_desc(P.camera_model[c]).n_params;
    for (int k = 0; k < C; ++k) {
      const double scale = 1.0 / std::max(P.camera_sigma[16 * c + k], kEps);
      const double v = s.cam[16 * c + k], pr = P.camera_prior[16 * c + k];
      if (P.camera_log[16 * c + k]) {
        r[k] = scale * std::log(v / pr);
        J[k] = scale / v;
      } else {
        r[k] = scale * (v - pr);
        J[k] = scale;
      }
    }
    return C;
  }

  // resid: [terms][3] when given (sized for every term or for the
  // observations only)
  double cost(const State& s, std::vector<double>* resid) const {
    std::vector<double> part(threads, 0.0);
    par(n_terms(), [&](int64_t i, int t) {
      double r[3] = {0, 0, 0};
      const int nr = obs_residual(s, i, r);
      double sq = 0.0;
      for (int k = 0; k < nr; ++k) sq += r[k] * r[k];
      double rho[3];
      loss_eval(O.loss, O.loss_threshold, sq, rho);
      part[t] += 0.5 * w_obs[i] * rho[0];
      if (resid && resid->size() >= size_t(3 * (i + 1)))
        for (int k = 0; k < 3; ++k) (*resid)[3 * i + k] = r[k];
    });
    double c = 0.0;
    for (double v : part) c += v;
    c += prior_cost(s);
    return c;
  }

  double prior_cost(const State& s) const {
    double c = 0.0;
    for (int q = 0; q < P.n_rel; ++q) {
      D36 r[7];
      int col[36];
      double rho;
      relative_term(s, q, r, col, &rho);
      c += 0.5 * rho;
    }
    for (int q = 0; q < P.n_orient; ++q) {
      D6 r[3];
      int col[6];
      double rho;
      orientation_term(s, q, r, col, &rho);
      c += 0.5 * rho;
    }
    double r[16], J[16];
    for (int k = 0; k < P.n_cameras; ++k) {
      const int n = cam_prior(s, k, r, J);
      for (int j = 0; j < n; ++j) c += 0.5 * w_cam[k] * r[j] * r[j];
    }
    for (int rc = 0; rc < P.n_rig_cameras; ++rc) {
      if (!P.rig_has_prior[rc]) continue;
      for (int j = 0; j < 6; ++j) {
        const double v = (s.rig[6 * rc + j] - P.rig_prior[6 * rc + j]) / std::max(P.rig_sigma[6 * rc + j], kEps);
        c += 0.5 * w_rig[rc] * v * v;
      }
    }
    for (size_t g = 0; g < gps_list.size(); ++g) {
      const int i = gps_list[g];
      for (int j = 0; j < 3; ++j) {
        const double v = (s.inst[6 * i + 3 + j] - P.gps_position[3 * i + j]) / std::max(P.gps_std[3 * i + j], kEps);
        c += 0.5 * w_gps[g] * v * v;
      }
    }
    for (size_t g = 0; g < pp_list.size(); ++g) {
      const int p = pp_list[g];
      const int n = P.point_has_altitude[p] ? 3 : 2;
      for (int j = 0; j < n; ++j) {
        const double v = (s.pts[3 * p + j] - P.point_prior[3 * p + j]) / std::max(P.point_sigma[3 * p + j], kEps);
        c += 0.5 * w_pp[g] * v * v;
      }
    }
    return c;
  }

  // ---- linearization storage
  struct ObsLin {
    int nr = 0;
    double r[3];
    double Jp[9];
    int m = 0;        // camera-side columns
    int col[28];      // compact indices
    double Jc[3 * 28];
  };
  std::vector<ObsLin> lin;
  std::vector<double> U, g;            // camera side (dense)
  std::vector<double> V, gp;           // points [n][9], [n][3]
  std::vector<double> colnorm_c, colnorm_p;

  void linearize(const State& s) {
    const int n = idx.n;
    lin.assign(n_terms(), ObsLin());
    par(n_terms(), [&](int64_t i, int) {
      ObsLin& L = lin[i];
      const int64_t o = term_obs(i);
      const bool depth = i >= P.n_obs;
      const int sh = P.obs_shot[o];
      const int cam = P.shot_camera[sh];
      const int model = P.camera_model[cam];
      const int C = model_desc(model).n_params;
      const int inst = P.shot_instance[sh];
      const int rc = P.shot_rig[sh];
      const bool use_rig = rc >= 0 && P.rig_used[rc];
      double r[3] = {0, 0, 0}, Jc[48] = {0}, Ji[18] = {0}, Jr[18] = {0}, Jp[9] = {0};
      int nr;
      if (depth) {
        r[0] = depth_term(s, i - P.n_obs, Ji, Jr, Jp);
        nr = 1;
      } else {
        residual_jac(model, &s.cam[16 * cam], &s.inst[6 * inst], use_rig ? &s.rig[6 * rc] : nullptr,
                     &s.pts[3 * P.obs_point[o]], P.obs_xy + 2 * o, P.obs_std[o], r, Jc, Ji, Jr, Jp);
        nr = residual_size(model);
      }
      L.nr = nr;
      // gather camera-side columns
      int m = 0;
      double cols[3][28];
      auto add_col = [&](int ci, const double* J, int stride, int k) {
        if (ci < 0) return;
        L.col[m] = ci;
        for (int a = 0; a < nr; ++a) cols[a][m] = J[a * stride + k];
        ++m;
      };
      for (int k = 0; k < 6; ++k) add_col(idx.inst[6 * inst + k], Ji, 6, k);
      if (use_rig)
        for (int k = 0; k < 6; ++k) add_col(idx.rig[6 * rc + k], Jr, 6, k);
      if (model != SPHERICAL && !depth)
        for (int k = 0; k < C; ++k) add_col(idx.cam[16 * cam + k], Jc, C, k);
      L.m = m;
      // robust correction
      double sq = 0.0;
      for (int a = 0; a < nr; ++a) sq += r[a] * r[a];
      double rho[3];
      loss_eval(O.loss, O.loss_threshold, sq, rho);
      for (double& v : rho) v *= w_obs[i];
      const double sq1 = std::sqrt(rho[1]);
      double rs = sq1, as = 0.0;
      if (sq > 0.0 && rho[2] > 0.0) {
        const double D = 1.0 + 2.0 * sq * rho[2] / rho[1];
        const double alpha = 1.0 - std::sqrt(D);
        rs = sq1 / (1.0 - alpha);
        as = alpha / sq;
      }
      auto corr = [&](double* colv /*nr values with stride*/, int stride) {
        double rj = 0.0;
        for (int a = 0; a < nr; ++a) rj += r[a] * colv[a * stride];
        for (int a = 0; a < nr; ++a) colv[a * stride] = sq1 * (colv[a * stride] - as * r[a] * rj);
      };
      for (int k = 0; k < 3; ++k) corr(Jp + k, 3);
      for (int k = 0; k < m; ++k) corr(&cols[0][k], 28);
      for (int a = 0; a < nr; ++a) {
        L.r[a] = rs * r[a];
        for (int k = 0; k < 3; ++k) L.Jp[a * 3 + k] = P.point_free[P.obs_point[o]] ? Jp[a * 3 + k] : 0.0;
        for (int k = 0; k < m; ++k) L.Jc[a * 28 + k] = cols[a][k];
      }
    });
    U.assign(size_t(n) * n, 0.0);
    g.assign(n, 0.0);
    V.assign(9 * P.n_points, 0.0);
    gp.assign(3 * P.n_points, 0.0);
    for (int64_t i = 0; i < n_terms(); ++i) {
      const ObsLin& L = lin[i];
      const int p = term_point(i);
      for (int a = 0; a < L.nr; ++a) {
        for (int k = 0; k < L.m; ++k) {
          g[L.col[k]] += L.Jc[a * 28 + k] * L.r[a];
          for (int l = 0; l < L.m; ++l) U[size_t(L.col[k]) * n + L.col[l]] += L.Jc[a * 28 + k] * L.Jc[a * 28 + l];
        }
        for (int k = 0; k < 3; ++k) {
          gp[3 * p + k] += L.Jp[a * 3 + k] * L.r[a];
          for (int l = 0; l < 3; ++l) V[9 * p + 3 * k + l] += L.Jp[a * 3 + k] * L.Jp[a * 3 + l];
        }
      }
    }
    // priors (diagonal Jacobians)
    double r[16], J[16];
    for (int c = 0; c < P.n_cameras; ++c) {
      const int C = cam_prior(s, c, r, J);
      for (int k = 0; k < C; ++k) {
        const int ci = idx.cam[16 * c + k];
        if (ci < 0) continue;
        g[ci] += w_cam[c] * J[k] * r[k];
        U[size_t(ci) * n + ci] += w_cam[c] * J[k] * J[k];
      }
    }
    for (int rc = 0; rc < P.n_rig_cameras; ++rc) {
      if (!P.rig_has_prior[rc]) continue;
      for (int k = 0; k < 6; ++k) {
        const int ci = idx.rig[6 * rc + k];
        if (ci < 0) continue;
        const double sc = 1.0 / std::max(P.rig_sigma[6 * rc + k], kEps);
        g[ci] += w_rig[rc] * sc * sc * (s.rig[6 * rc + k] - P.rig_prior[6 * rc + k]);
        U[size_t(ci) * n + ci] += w_rig[rc] * sc * sc;
      }
    }
    for (size_t q = 0; q < gps_list.size(); ++q) {
      const int i = gps_list[q];
      for (int k = 0; k < 3; ++k) {
        const int ci = idx.inst[6 * i + 3 + k];
        if (ci < 0) continue;
        const double sc = 1.0 / std::max(P.gps_std[3 * i + k], kEps);
        g[ci] += w_gps[q] * sc * sc * (s.inst[6 * i + 3 + k] - P.gps_position[3 * i + k]);
        U[size_t(ci) * n + ci] += w_gps[q] * sc * sc;
      }
    }
    for (size_t q = 0; q < pp_list.size(); ++q) {
      const int p = pp_list[q];
      if (!P.point_free[p]) continue;
      const int nn = P.point_has_altitude[p] ? 3 : 2;
      for (int k = 0; k < nn; ++k) {
        const double sc = 1.0 / std::max(P.point_sigma[3 * p + k], kEps);
        gp[3 * p + k] += w_pp[q] * sc * sc * (s.pts[3 * p + k] - P.point_prior[3 * p + k]);
        V[9 * p + 4 * k] += w_pp[q] * sc * sc;
      }
    }
    for (int q = 0; q < P.n_orient; ++q) {
      D6 rr[3];
      int col[6];
      double rho;
      const int m = orientation_term(s, q, rr, col, &rho);
      for (int a = 0; a < 6; ++a) {
        if (col[a] < 0) continue;
        for (int t = 0; t < m; ++t) g[col[a]] += rr[t].d[a] * rr[t].v;
        for (int b = 0; b < 6; ++b) {
          if (col[b] < 0) continue;
          for (int t = 0; t < m; ++t) U[size_t(col[a]) * n + col[b]] += rr[t].d[a] * rr[t].d[b];
        }
      }
    }
    for (int q = 0; q < P.n_rel; ++q) {
      D36 rr[7];
      int col[36];
      double rho;
      const int m = relative_term(s, q, rr, col, &rho);
      for (int a = 0; a < 36; ++a) {
        if (col[a] < 0) continue;
        for (int t = 0; t < m; ++t) g[col[a]] += rr[t].d[a] * rr[t].v;
        for (int b = 0; b < 36; ++b) {
          if (col[b] < 0) continue;
          for (int t = 0; t < m; ++t) U[size_t(col[a]) * n + col[b]] += rr[t].d[a] * rr[t].d[b];
        }
      }
    }
  }

  // ---- linear step
  std::vector<double> scale_c, scale_p;
  bool solve(double mu, bool first, std::vector<double>& dc, std::vector<double>& dp, double& model_change) {
    const int n = idx.n;
    if (first) {
      scale_c.assign(n, 1.0);
      for (int j = 0; j < n; ++j) scale_c[j] = 1.0 / (1.0 + std::sqrt(U[size_t(j) * n + j]));
      scale_p.assign(3 * P.n_points, 1.0);
      for (int64_t p = 0; p < P.n_points; ++p)
        for (int k = 0; k < 3; ++k) scale_p[3 * p + k] = 1.0 / (1.0 + std::sqrt(V[9 * p + 4 * k]));
    }
    auto damp = [&](double d, double s) {
      double c = s * s * d;
      c = std::min(std::max(c, 1e-6), 1e32);
      return c / (s * s) * mu;
    };
    std::vector<double> S(U), b(n);
    for (int j = 0; j < n; ++j) {
      S[size_t(j) * n + j] += damp(U[size_t(j) * n + j], scale_c[j]);
      b[j] = -g[j];
    }
    // point inverses
    std::vector<double> Vi(9 * P.n_points, 0.0);
    for (int64_t p = 0; p < P.n_points; ++p) {
      if (!P.point_free[p]) continue;
      double A[9];
      for (int k = 0; k < 9; ++k) A[k] = V[9 * p + k];
      for (int k = 0; k < 3; ++k) A[4 * k] += damp(V[9 * p + 4 * k], scale_p[3 * p + k]);
      const double det = A[0] * (A[4] * A[8] - A[5] * A[7]) - A[1] * (A[3] * A[8] - A[5] * A[6]) +
                         A[2] * (A[3] * A[7] - A[4] * A[6]);
      if (!(std::fabs(det) > 0.0)) continue;
      double* I = &Vi[9 * p];
      I[0] = (A[4] * A[8] - A[5] * A[7]) / det;
      I[1] = (A[2] * A[7] - A[1] * A[8]) / det;
      I[2] = (A[1] * A[5] - A[2] * A[4]) / det;
      I[3] = (A[5] * A[6] - A[3] * A[8]) / det;
      I[4] = (A[0] * A[8] - A[2] * A[6]) / det;
      I[5] = (A[2] * A[3] - A[0] * A[5]) / det;
      I[6] = (A[3] * A[7] - A[4] * A[6]) / det;
      I[7] = (A[1] * A[6] - A[0] * A[7]) / det;
      I[8] = (A[0] * A[4] - A[1] * A[3]) / det;
    }
    // Schur complement, grouped by point
    const int64_t nt = n_terms();
    std::vector<int64_t> order(nt);
    for (int64_t i = 0; i < nt; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t c) { return term_point(a) < term_point(c); });
    std::vector<int> wcol;
    std::vector<double> wval;  // [3] per entry: W = J_c^T J_p (entry per column)
    for (int64_t a = 0; a < nt;) {
      const int p = term_point(order[a]);
      int64_t e = a;
      while (e < nt && term_point(order[e]) == p) ++e;
      if (P.point_free[p]) {
        wcol.clear();
        wval.clear();
        for (int64_t q = a; q < e; ++q) {
          const ObsLin& L = lin[order[q]];
          for (int k = 0; k < L.m; ++k) {
            double w3[3] = {0, 0, 0};
            for (int r = 0; r < L.nr; ++r)
              for (int l = 0; l < 3; ++l) w3[l] += L.Jc[r * 28 + k] * L.Jp[r * 3 + l];
            // merge equal columns
            int pos = -1;
            for (size_t t = 0; t < wcol.size(); ++t)
              if (wcol[t] == L.col[k]) pos = int(t);
            if (pos < 0) {
              wcol.push_back(L.col[k]);
              wval.insert(wval.end(), w3, w3 + 3);
            } else {
              for (int l = 0; l < 3; ++l) wval[3 * pos + l] += w3[l];
            }
          }
        }
        const double* I = &Vi[9 * p];
        const size_t m = wcol.size();
        std::vector<double> T(3 * m);  // W V^-1
        for (size_t t = 0; t < m; ++t)
          for (int l = 0; l < 3; ++l)
            T[3 * t + l] = wval[3 * t] * I[l] + wval[3 * t + 1] * I[3 + l] + wval[3 * t + 2] * I[6 + l];
        for (size_t t = 0; t < m; ++t) {
          for (size_t u = 0; u < m; ++u) {
            const double v = T[3 * t] * wval[3 * u] + T[3 * t + 1] * wval[3 * u + 1] + T[3 * t + 2] * wval[3 * u + 2];
            S[size_t(wcol[t]) * n + wcol[u]] -= v;
          }
          b[wcol[t]] += T[3 * t] * gp[3 * p] + T[3 * t + 1] * gp[3 * p + 1] + T[3 * t + 2] * gp[3 * p + 2];
        }
      }
      a = e;
    }
    // Cholesky solve
    std::vector<double> Lm(S);
    for (int j = 0; j < n; ++j) {
      double d = Lm[size_t(j) * n + j];
      for (int k = 0; k < j; ++k) d -= Lm[size_t(j) * n + k] * Lm[size_t(j) * n + k];
      if (!(d > 0.0)) return false;
      d = std::sqrt(d);
      Lm[size_t(j) * n + j] = d;
      for (int i = j + 1; i < n; ++i) {
        double s = Lm[size_t(i) * n + j];
        for (int k = 0; k < j; ++k) s -= Lm[size_t(i) * n + k] * Lm[size_t(j) * n + k];
        Lm[size_t(i) * n + j] = s / d;
      }
    }
    dc.assign(n, 0.0);
    std::vector<double> y(n);
    for (int i = 0; i < n; ++i) {
      double s = b[i];
      for (int k = 0; k < i; ++k) s -= Lm[size_t(i) * n + k] * y[k];
      y[i] = s / Lm[size_t(i) * n + i];
    }
    for (int i = n - 1; i >= 0; --i) {
      double s = y[i];
      for (int k = i + 1; k < n; ++k) s -= Lm[size_t(k) * n + i] * dc[k];
      dc[i] = s / Lm[size_t(i) * n + i];
    }
    // back-substitution
    std::vector<double> wd(3 * P.n_points, 0.0);
    for (int64_t i = 0; i < nt; ++i) {
      const ObsLin& L = lin[i];
      const int p = term_point(i);
      for (int r = 0; r < L.nr; ++r) {
        double t = 0.0;
        for (int k = 0; k < L.m; ++k) t += L.Jc[r * 28 + k] * dc[L.col[k]];
        for (int l = 0; l < 3; ++l) wd[3 * p + l] += L.Jp[r * 3 + l] * t;
      }
    }
    dp.assign(3 * P.n_points, 0.0);
    for (int64_t p = 0; p < P.n_points; ++p) {
      if (!P.point_free[p]) continue;
      const double* I = &Vi[9 * p];
      double q[3];
      for (int l = 0; l < 3; ++l) q[l] = -gp[3 * p + l] - wd[3 * p + l];
      for (int l = 0; l < 3; ++l) dp[3 * p + l] = I[3 * l] * q[0] + I[3 * l + 1] * q[1] + I[3 * l + 2] * q[2];
    }
    // linear model decrease
    double mc = 0.0;
    for (int64_t i = 0; i < nt; ++i) {
      const ObsLin& L = lin[i];
      const int p = term_point(i);
      for (int r = 0; r < L.nr; ++r) {
        double t = 0.0;
        for (int k = 0; k < L.m; ++k) t += L.Jc[r * 28 + k] * dc[L.col[k]];
        for (int l = 0; l < 3; ++l) t += L.Jp[r * 3 + l] * dp[3 * p + l];
        mc += -0.5 * t * (2.0 * L.r[r] + t);
      }
    }
    // priors: J diagonal -> model change from g restricted to priors is
    // already inside U, g; compute it directly
    mc += prior_model_change(dc, dp);
    model_change = mc;
    return true;
  }

  const State* cur = nullptr;
  double prior_model_change(const std::vector<double>& dc, const std::vector<double>& dp) const {
    const State& s = *cur;
    double mc = 0.0;
    auto term = [](double w, double r, double J, double d) { return -0.5 * w * (J * d) * (2.0 * r + J * d); };
    double r[16], J[16];
    for (int c = 0; c < P.n_cameras; ++c) {
      const int C = cam_prior(s, c, r, J);
      for (int k = 0; k < C; ++k) {
        const int ci = idx.cam[16 * c + k];
        if (ci >= 0) mc += term(w_cam[c], r[k], J[k], dc[ci]);
      }
    }
    for (int rc = 0; rc < P.n_rig_cameras; ++rc) {
      if (!P.rig_has_prior[rc]) continue;
      for (int k = 0; k < 6; ++k) {
        const int ci = idx.rig[6 * rc + k];
        if (ci < 0) continue;
        const double sc = 1.0 / std::max(P.rig_sigma[6 * rc + k], kEps);
        mc += term(w_rig[rc], sc * (s.rig[6 * rc + k] - P.rig_prior[6 * rc + k]), sc, dc[ci]);
      }
    }
    for (size_t q = 0; q < gps_list.size(); ++q) {
      const int i = gps_list[q];
      for (int k = 0; k < 3; ++k) {
        const int ci = idx.inst[6 * i + 3 + k];
        if (ci < 0) continue;
        const double sc = 1.0 / std::max(P.gps_std[3 * i + k], kEps);
        mc += term(w_gps[q], sc * (s.inst[6 * i + 3 + k] - P.gps_position[3 * i + k]), sc, dc[ci]);
      }
    }
    for (size_t q = 0; q < pp_list.size(); ++q) {
      const int p = pp_list[q];
      if (!P.point_free[p]) continue;
      const int nn = P.point_has_altitude[p] ? 3 : 2;
      for (int k = 0; k < nn; ++k) {
        const double sc = 1.0 / std::max(P.point_sigma[3 * p + k], kEps);
        mc += term(w_pp[q], sc * (s.pts[3 * p + k] - P.point_prior[3 * p + k]), sc, dp[3 * p + k]);
      }
    }
    for (int q = 0; q < P.n_orient; ++q) {
      D6 rr[3];
      int col[6];
      double rho;
      const int m = orientation_term(s, q, rr, col, &rho);
      for (int t = 0; t < m; ++t) {
        double jd = 0.0;
        for (int a = 0; a < 6; ++a)
          if (col[a] >= 0) jd += rr[t].d[a] * dc[col[a]];
        mc += -0.5 * jd * (2.0 * rr[t].v + jd);
      }
    }
    for (int q = 0; q < P.n_rel; ++q) {
      D36 rr[7];
      int col[36];
      double rho;
      const int m = relative_term(s, q, rr, col, &rho);
      for (int t = 0; t < m; ++t) {
        double jd = 0.0;
        for (int a = 0; a < 36; ++a)
          if (col[a] >= 0) jd += rr[t].d[a] * dc[col[a]];
        mc += -0.5 * jd * (2.0 * rr[t].v + jd);
      }
    }
    return mc;
  }

  State apply(const State& s, const std::vector<double>& dc, const std::vector<double>& dp) const {
    State t = s;
    for (int i = 0; i < P.n_instances; ++i)
      for (int k = 0; k < 6; ++k)
        if (idx.inst[6 * i + k] >= 0) t.inst[6 * i + k] += dc[idx.inst[6 * i + k]];
    for (int r = 0; r < P.n_rig_cameras; ++r)
      for (int k = 0; k < 6; ++k)
        if (idx.rig[6 * r + k] >= 0) t.rig[6 * r + k] += dc[idx.rig[6 * r + k]];
    for (int c = 0; c < P.n_cameras; ++c)
      for (int k = 0; k < 16; ++k)
        if (idx.cam[16 * c + k] >= 0) t.cam[16 * c + k] += dc[idx.cam[16 * c + k]];
    for (int64_t p = 0; p < P.n_points; ++p)
      if (P.point_free[p])
        for (int k = 0; k < 3; ++k) t.pts[3 * p + k] += dp[3 * p + k];
    for (int k = 0; k < P.n_scales; ++k)
      if (idx.scl[k] >= 0) t.scl[k] += dc[idx.scl[k]];
    return t;
  }

  // ---- IRLS mixture (mixture_reweighting.cc:10-109)
  static double mixture(const std::vector<std::vector<double>>& res, std::vector<double*>& w, double ratio) {
    if (res.size() < 10) return 0.0;
    const int k = int(res[0].size());
    double prev = std::numeric_limits<double>::max(), ll = 0.0;
    for (int it = 0; it < 5; ++it) {
      std::vector<double> S(k * k, 0.0);
      double W = 0.0;
      for (size_t i = 0; i < res.size(); ++i) {
        if (int(res[i].size()) != k) continue;
        for (int a = 0; a < k; ++a)
          for (int b = 0; b < k; ++b) S[a * k + b] += *w[i] * res[i][a] * res[i][b];
        W += *w[i];
      }
      if (W < 1e-9) return 0.0;
      for (auto& v : S) v /= W;
      for (int a = 0; a < k; ++a) S[a * k + a] += 0.025;
      // determinant and inverse by Gauss-Jordan with partial pivoting
      std::vector<double> M(S), I(k * k, 0.0);
      for (int a = 0; a < k; ++a) I[a * k + a] = 1.0;
      double det = 1.0;
      for (int c = 0; c < k; ++c) {
        int piv = c;
        for (int r = c + 1; r < k; ++r)
          if (std::fabs(M[r * k + c]) > std::fabs(M[piv * k + c])) piv = r;
        if (M[piv * k + c] == 0.0) {
          det = 0.0;
          break;
        }
        if (piv != c) {
          for (int j = 0; j < k; ++j) {
            std::swap(M[piv * k + j], M[c * k + j]);
            std::swap(I[piv * k + j], I[c * k + j]);
          }
          det = -det;
        }
        const double d = M[c * k + c];
        det *= d;
        for (int j = 0; j < k; ++j) {
          M[c * k + j] /= d;
          I[c * k + j] /= d;
        }
        for (int r = 0; r < k; ++r) {
          if (r == c) continue;
          const double f = M[r * k + c];
          for (int j = 0; j < k; ++j) {
            M[r * k + j] -= f * M[c * k + j];
            I[r * k + j] -= f * I[c * k + j];
          }
        }
      }
      if (det < 1e-3) {
        det = 0.025 * 0.025;
        std::fill(I.begin(), I.end(), 0.0);
        for (int a = 0; a < k; ++a) I[a * k + a] = 1.0 / 0.025;
      }
      const double sqn = std::sqrt(std::pow(2 * M_PI, k) * det);
      const double K = ratio / sqn;
      ll = 0.0;
      for (size_t i = 0; i < res.size(); ++i) {
        if (int(res[i].size()) != k) continue;
        double m = 0.0;
        for (int a = 0; a < k; ++a)
          for (int b = 0; b < k; ++b) m += res[i][a] * I[a * k + b] * res[i][b];
        const double pin = std::exp(-0.5 * m) / sqn;
        ll += std::log(pin + K);
        *w[i] = std::max(1e-10, std::min(pin / (pin + K), 1.0));
      }
      const double change = std::fabs(ll - prev) / std::fabs(prev);
      if (change < 1e-3) break;
      prev = ll;
    }
    return ll;
  }

  double reweight(const State& s) {
    std::vector<double> resid(3 * n_terms());
    cost(s, &resid);
    double total = 0.0;
    // projection groups: one per shot, plus GCP2D; then DEPTH
    // (bundle_adjuster.cc:559-562,599-602)
    std::vector<std::vector<int64_t>> groups(P.n_shots + 2);
    for (int64_t i = 0; i < P.n_obs; ++i) groups[P.obs_gcp[i] ? P.n_shots : P.obs_shot[i]].push_back(i);
    for (int64_t i = P.n_obs; i < n_terms(); ++i) groups[P.n_shots + 1].push_back(i);
    for (auto& grp : groups) {
      std::vector<std::vector<double>> res;
      std::vector<double*> w;
      for (int64_t i : grp) {
        const int model = P.camera_model[P.shot_camera[P.obs_shot[term_obs(i)]]];
        const int nr = i >= P.n_obs ? 1 : residual_size(model);
        res.emplace_back(&resid[3 * i], &resid[3 * i] + nr);
        w.push_back(&w_obs[i]);
      }
      total += mixture(res, w, O.density_ratio);
    }
    {
      std::vector<std::vector<double>> res;
      std::vector<double*> w;
      double r[16], J[16];
      for (int c = 0; c < P.n_cameras; ++c) {
        const int C = cam_prior(s, c, r, J);
        res.emplace_back(r, r + C);
        w.push_back(&w_cam[c]);
      }
      total += mixture(res, w, O.density_ratio);
    }
    {
      std::vector<std::vector<double>> res;
      std::vector<double*> w;
      for (int rc = 0; rc < P.n_rig_cameras; ++rc) {
        if (!P.rig_has_prior[rc]) continue;
        std::vector<double> r(6);
        for (int k = 0; k < 6; ++k)
          r[k] = (s.rig[6 * rc + k] - P.rig_prior[6 * rc + k]) / std::max(P.rig_sigma[6 * rc + k], kEps);
        res.push_back(r);
        w.push_back(&w_rig[rc]);
      }
      total += mixture(res, w, O.density_ratio);
    }
    {
      std::vector<std::vector<double>> res;
      std::vector<double*> w;
      for (size_t q = 0; q < gps_list.size(); ++q) {
        const int i = gps_list[q];
        std::vector<double> r(3);
        for (int k = 0; k < 3; ++k)
          r[k] = (s.inst[6 * i + 3 + k] - P.gps_position[3 * i + k]) / std::max(P.gps_std[3 * i + k], kEps);
        res.push_back(r);
        w.push_back(&w_gps[q]);
      }
      total += mixture(res, w, O.density_ratio);
    }
    {
      std::vector<std::vector<double>> res;
      std::vector<double*> w;
      for (size_t q = 0; q < pp_list.size(); ++q) {
        const int p = pp_list[q];
        const int nn = P.point_has_altitude[p] ? 3 : 2;
        std::vector<double> r(nn);
        for (int k = 0; k < nn; ++k)
          r[k] = (s.pts[3 * p + k] - P.point_prior[3 * p + k]) / std::max(P.point_sigma[3 * p + k], kEps);
        res.push_back(r);
        w.push_back(&w_pp[q]);
      }
      total += mixture(res, w, O.density_ratio);
    }
    for (int kind = 0; kind < 4; ++kind) {  // groups UP, PAN, TILT, ROLL
      std::vector<std::vector<double>> res;
      std::vector<double*> w;
      for (int q = 0; q < P.n_orient; ++q) {
        if (P.orient_kind[q] != kind) continue;
        D6 rr[3];
        int col[6];
        double rho, raw[3];
        const int m = orientation_term(s, q, rr, col, &rho, raw);
        res.emplace_back(raw, raw + m);
        w.push_back(&w_orient[q]);
      }
      total += mixture(res, w, O.density_ratio);
    }
    for (int kind = 0; kind < 8; ++kind) {  // groups ROT, POS, MOTION, GAUGE, HEATMAP, REL, GPS, STDDEV
      std::vector<std::vector<double>> res;
      std::vector<double*> w;
      for (int q = 0; q < P.n_rel; ++q) {
        // a GPS prior through an optimised bias (kind 8) is in group GPS
        if (P.rel_kind[q] != kind && !(kind == 6 && P.rel_kind[q] == 8)) continue;
        D36 rr[7];
        int col[36];
        double rho, raw[7];
        const int m = relative_term(s, q, rr, col, &rho, raw);
        res.emplace_back(raw, raw + m);
        w.push_back(&w_rel[q]);
      }
      total += mixture(res, w, O.density_ratio);
    }
    return total;
  }
};

}  // namespace

// One group of MixtureReweighting::ComputeGroupWeights
// (mixture_reweighting.cc:10-109): n residual vectors of dimension k
// (row-major), weights updated in place; returns the log-likelihood.
extern "C" double oracle_mixture_group(int k, int64_t n, const double* residuals, double* weights,
                                       double density_ratio) {
  std::vector<std::vector<double>> res(n, std::vector<double>(k));
  std::vector<double*> w(n);
  for (int64_t i = 0; i < n; ++i) {
    for (int a = 0; a < k; ++a) res[i][a] = residuals[i * k + a];
    w[i] = weights + i;
  }
  return Solver::mixture(res, w, density_ratio);
}

// One depth prior's scaled residual and its Jacobian rows: d/d instance
// pose [6], d/d rig camera pose [6] (rig_camera_pose null: not composed,
// zeros), d/d point [3].
extern "C" double oracle_depth_residual(const double* instance_pose, const double* rig_camera_pose,
                                        const double* point, double value, double std_dev, int radial,
                                        double* jac_instance, double* jac_rig, double* jac_point) {
  return depth_residual_jac(instance_pose, rig_camera_pose, point, value, std_dev, radial != 0, jac_instance, jac_rig,
                            jac_point);
}

// One orientation constraint's scaled residuals and Jacobian [m][6]
// (d/d instance rotation, d/d rig camera rotation); returns m.
extern "C" int oracle_orientation_residual(int kind, const double* target, double std_dev, const double* ri,
                                           const double* rc, double* r, double* J) {
  static const double zero[3] = {0, 0, 0};
  D6 d[3];
  const int m = orientation_residual(kind, target, std_dev, ri, rc ? rc : zero, d);
  for (int q = 0; q < m; ++q) {
    r[q] = d[q].v;
    for (int k = 0; k < 6; ++k) J[6 * q + k] = d[q].d[k];
  }
  return m;
}

// One constraint between shots: scaled residuals and Jacobian [m][36]
// (kind and params as OracleProblem holds them; rig camera poses may be
// null); returns m.
extern "C" int oracle_relative_residual(int kind, const double* instance_poses, const double* rig_camera_poses,
                                        const double* params, const double* scales, double* r, double* J) {
  const int n = kind == 2 ? 3 : (kind == 6 || kind == 8) ? 1 : kind == 7 ? 0 : 2;
  const double* pi[3] = {nullptr, nullptr, nullptr};
  const double* pc[3] = {nullptr, nullptr, nullptr};
  for (int k = 0; k < n; ++k) {
    pi[k] = instance_poses + 6 * k;
    pc[k] = rig_camera_poses ? rig_camera_poses + 6 * k : nullptr;
  }
  D36 d[7];
  const int m = relative_residual(kind, pi, pc, params, d, nullptr, scales);
  for (int q = 0; q < m; ++q) {
    r[q] = d[q].v;
    for (int k = 0; k < 36; ++k) J[36 * q + k] = d[q].d[k];
  }
  return m;
}

// The heatmap residual and its Jacobian [12] at one instance pose and rig
// camera pose (null: none).
extern "C" double oracle_heatmap_residual(const double* grid, int64_t n, int width, double resolution,
                                          const double* params, const double* instance_pose,
                                          const double* rig_camera_pose, double* J) {
  const HeatGrid g{grid, n, width, resolution};
  const double* pi[3] = {instance_pose, nullptr, nullptr};
  const double* pc[3] = {rig_camera_pose, nullptr, nullptr};
  D36 r[7];
  relative_residual(4, pi, pc, params, r, &g);
  for (int k = 0; k < 12; ++k) J[k] = r[0].d[k];
  return r[0].v;
}

extern "C" int oracle_solve(const OracleProblem* Pp, const OracleOptions* Op, OracleResult* out) {
  const OracleProblem& P = *Pp;
  const OracleOptions& O = *Op;
  // Index checks: a problem whose counts disagree with its index arrays is
  // refused (-1) before anything is read out of range.
  for (int s = 0; s < P.n_shots; ++s)
    if (P.shot_instance[s] < 0 || P.shot_instance[s] >= P.n_instances || P.shot_camera[s] < 0 ||
        P.shot_camera[s] >= P.n_cameras || P.shot_rig[s] < -1 || P.shot_rig[s] >= std::max(1, P.n_rig_cameras))
      return -1;
  for (int64_t i = 0; i < P.n_obs; ++i)
    if (P.obs_shot[i] < 0 || P.obs_shot[i] >= P.n_shots || P.obs_point[i] < 0 || P.obs_point[i] >= P.n_points)
      return -1;
  for (int64_t k = 0; k < P.n_depth; ++k)
    if (P.depth_obs[k] < 0 || P.depth_obs[k] >= P.n_obs || !(P.depth_std[k] > 0.0)) return -1;
  Solver S(P, O);
  State x;
  x.cam.assign(P.camera_values, P.camera_values + 16 * P.n_cameras);
  x.inst.assign(P.instance_poses, P.instance_poses + 6 * P.n_instances);
  x.rig.assign(P.rig_poses, P.rig_poses + 6 * std::max(0, P.n_rig_cameras));
  x.pts.assign(P.points, P.points + 3 * P.n_points);
  x.scl.assign(P.scales, P.scales + std::max(0, P.n_scales));
  S.cur = &x;
  double ll = -std::numeric_limits<double>::infinity();
  const bool irls = O.irls == 1;
  if (irls && !O.skip_initial_reweighting) ll = S.reweight(x);
  double cost = S.cost(x, nullptr);
  out->initial_cost = cost;
  out->trace_n = 0;
  auto trace = [&](double c) {
    if (out->trace_cost && out->trace_n < out->trace_capacity) out->trace_cost[out->trace_n++] = c;
  };
  trace(cost);
  double radius = 1e4, decrease = 2.0;
  double reference_cost = cost, candidate_cost = cost, minimum_cost = cost, acc_ref = 0.0, acc_cand = 0.0;
  int n_nonmono = 0, invalid = 0;
  const int interval = std::max(1, O.max_iterations / 10);
  bool first = true;
  S.linearize(x);
  out->termination = 0;
  out->successful = 0;
  int iter;
  for (iter = 1; iter <= O.max_iterations; ++iter) {
    std::vector<double> dc, dp;
    double mc = 0.0;
    S.cur = &x;
    const bool ok = S.solve(1.0 / radius, first, dc, dp, mc);
    first = false;
    bool success = false;
    double new_cost = cost;
    State cand;
    double step2 = 0.0;
    if (ok && mc > 0.0 && std::isfinite(mc)) {
      for (double v : dc) step2 += v * v;
      for (double v : dp) step2 += v * v;
      cand = S.apply(x, dc, dp);
      new_cost = S.cost(cand, nullptr);
      if (std::isfinite(new_cost)) {
        invalid = 0;
        double rho = (cost - new_cost) / mc;
        rho = std::max(rho, (reference_cost - new_cost) / (acc_ref + mc));
        success = rho > 1e-3;
        if (success) {
          acc_cand += mc;
          acc_ref += mc;
          if (new_cost < minimum_cost) {
            minimum_cost = new_cost;
            candidate_cost = new_cost;
            acc_cand = 0.0;
            n_nonmono = 0;
          } else {
            ++n_nonmono;
            if (new_cost > candidate_cost) {
              candidate_cost = new_cost;
              acc_cand = 0.0;
            }
          }
          if (n_nonmono == 5) {
            reference_cost = candidate_cost;
            acc_ref = acc_cand;
          }
          radius = std::min(1e8, radius / std::max(1.0 / 3.0, 1.0 - std::pow(2.0 * rho - 1.0, 3)));
          decrease = 2.0;
        }
      } else {
        ++invalid;
      }
    } else {
      ++invalid;
    }
    double cost_change = 0.0, grad_max = 0.0;
    if (success) {
      cost_change = cost - new_cost;
      x = cand;
      cost = new_cost;
      S.cur = &x;
      S.linearize(x);
      for (double v : S.g) grad_max = std::max(grad_max, std::fabs(v));
      for (double v : S.gp) grad_max = std::max(grad_max, std::fabs(v));
      out->successful++;
    } else {
      radius /= decrease;
      decrease *= 2.0;
    }
    trace(cost);
    bool inner = false;
    if (success) {
      if (std::fabs(cost_change) <= 1e-7 * cost) inner = true;
      else if (grad_max <= 1e-10) inner = true;
      else {
        double xn = 0.0;
        for (double v : x.cam) xn += v * v;
        for (double v : x.inst) xn += v * v;
        for (double v : x.rig) xn += v * v;
        for (double v : x.pts) xn += v * v;
        for (double v : x.scl) xn += v * v;
        if (std::sqrt(step2) <= 1e-8 * (std::sqrt(xn) + 1e-8)) inner = true;
      }
    }
    if (irls) {
      if ((success && iter % interval == 0) || inner) {
        const double prev = ll;
        ll = S.reweight(x);
        cost = S.cost(x, nullptr);
        reference_cost = candidate_cost = minimum_cost = cost;
        acc_ref = acc_cand = 0.0;
        n_nonmono = 0;
        S.linearize(x);
        if (prev > -std::numeric_limits<double>::infinity() &&
            std::fabs(ll - prev) / (std::fabs(prev) + 1e-20) < 1e-3) {
          out->termination = 2;
          break;
        }
      }
    } else if (inner) {
      out->termination = 1;
      break;
    }
    if (radius < 1e-32) {
      out->termination = 1;
      break;
    }
    if (invalid >= 5) {
      out->termination = 3;
      break;
    }
  }
  out->iterations = std::min(iter, O.max_iterations);
  out->final_cost = cost;
  std::memcpy(out->camera_values, x.cam.data(), sizeof(double) * x.cam.size());
  std::memcpy(out->instance_poses, x.inst.data(), sizeof(double) * x.inst.size());
  if (P.n_rig_cameras) std::memcpy(out->rig_poses, x.rig.data(), sizeof(double) * x.rig.size());
  std::memcpy(out->points, x.pts.data(), sizeof(double) * x.pts.size());
  if (out->scales && P.n_scales > 0) std::memcpy(out->scales, x.scl.data(), sizeof(double) * x.scl.size());
  std::vector<double> resid(3 * P.n_obs);
  S.cost(x, &resid);
  for (int64_t i = 0; i < P.n_obs; ++i) {
    if (out->obs_weights) out->obs_weights[i] = S.w_obs[i];
    if (out->obs_errors)
      for (int k = 0; k < 3; ++k) out->obs_errors[3 * i + k] = resid[3 * i + k] * P.obs_std[i];
  }
  return 0;
}
