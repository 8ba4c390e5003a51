// GPU Levenberg-Marquardt bundle-adjustment solver (see solver.h): the
// implementation, compiled once per working precision by solver_fp64.cu and
// solver_mixed.cu.
#pragma once
#include <algorithm>
#include <array>
#include <map>
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>
#include <numeric>
#include <sstream>
#include <vector>

#include "coarse_kernels.cuh"
#include "coarse_space.h"
#include "dense_cholesky.h"
#include "dense_schur.cuh"
#include "host_blocks.cuh"
#include "device_buffer.h"
#include "solver.h"
#include "solver_kernels.cuh"
#include "solver_shot_major.cuh"
#include "kernel_config.cuh"
#include "record_passes.cuh"

namespace gbba {

namespace {

constexpr double kEps = 2.220446049250313e-16;
// Iterative refinement of the mixed-precision linear solve: used when the
// requested PCG tolerance is tighter than kRefineThreshold; every FP32 PCG
// round reduces the residual by kRefineInnerTolerance; at most
// kMaxRefinements FP64 residual evaluations per step.
constexpr double kRefineThreshold = 1e-4;
constexpr double kRefineInnerTolerance = 1e-3;
constexpr int kMaxRefinements = 4;
// PCG tolerance of the step that confirms convergence of an inexact solve.
constexpr double kConfirmTolerance = 1e-6;
// Dense mode: relative residual of the solution, and the most FP64
// conjugate-gradient iterations (preconditioned by the factor) per step.
constexpr double kDenseTolerance = 1e-12;
constexpr int kDenseMaxRefinements = 50;

template <int C>
constexpr int tri_pad() {
  return TriSize<C>::kPad;
}

int slot_grid(int64_t n) {
  const int64_t want = (n + 255) / 256;
  return int(std::max<int64_t>(1, std::min<int64_t>(want, 152 * 8)));
}
int elem_grid(int64_t n, int block = 256) { return int(std::max<int64_t>(1, (n + block - 1) / block)); }

// One of the record-reading passes (RecordPassArgs::Which) of the solver,
// launched with stored records by dispatch_config(kc, f), or matrix-free by
// launch_evaluated(kc, f) (DeviceSolver::record_pass picks).
template <typename R>
struct RecordPassLaunch : RecordPassArgs<R> {
  using Args = RecordPassArgs<R>;
  RecordPassLaunch(typename Args::Which w, const SolveView<R>& view, const ShotMajorView<R>& shot_major = {}) {
    this->which = w;
    this->v = view;
    this->sm = shot_major;
    this->grid = slot_grid(view.scene.n_slots);
  }
  template <int M, int NR, int CMAX, bool RIG>
  void run() {
    using L = RecordLayout<NR, CMAX, RIG>;
    this->template launch<M, NR, CMAX, RIG>(
        StoredRecords<R, planes_of<R>(L::kWidth)>{this->v.rec, this->sm.rec, this->v.stride});
  }
};

// ---------------------------------------------------------------------------
// Slot construction from the uploaded observations (point-major order given
// by `order`): observation packs, point index, GCP flag and unit IRLS
// weights; padding slots get point -1.
template <typename R>
__global__ void build_slots_kernel(int64_t n_terms, int64_t n_proj, int64_t n_slots,
                                   const Observation* __restrict__ raw, const int32_t* __restrict__ order,
                                   ObsPack<R>* __restrict__ ob, ObsPack<double>* __restrict__ ob64,
                                   int* __restrict__ opt, uint8_t* __restrict__ gcp, R* __restrict__ weight) {
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  for (int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; s < n_slots; s += stride) {
    ObsPack<R> o{};
    ObsPack<double> o64{};
    int pt = -1;
    uint8_t g = 0;
    if (s < n_terms) {
      const int32_t t = order[s];
      const Observation q = raw[t];
      if (t < n_proj) {
        const double w = 1.0 / q.std_dev;
        o.x = R(q.x);
        o.y = R(q.y);
        o.w = R(w);
        o64.x = q.x;
        o64.y = q.y;
        o64.w = w;
        g = q.is_gcp ? kSlotGcp : kSlotProjection;
      } else {
        // a depth prior (ObsPack doc: negative weight, value, radial flag)
        const double w = 1.0 / double(q.depth_std);
        o.x = R(q.depth);
        o.y = R(q.depth_radial ? 1 : 0);
        o.w = R(-w);
        o64.x = double(q.depth);
        o64.y = q.depth_radial ? 1.0 : 0.0;
        o64.w = -w;
        g = kSlotDepth;
      }
      o.shot = q.shot;
      o64.shot = q.shot;
      pt = q.point;
    }
    ob[s] = o;
    if (ob64) ob64[s] = o64;
    opt[s] = pt;
    gcp[s] = g;
    weight[s] = R(1);
  }
}

// Point and shot of every shot-major slot.
template <typename R>
__global__ void build_shot_major_kernel(int64_t n_slots, const int32_t* __restrict__ src, const int* __restrict__ opt,
                                        const ObsPack<R>* __restrict__ ob, int* __restrict__ pt,
                                        int* __restrict__ sh) {
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  for (int64_t j = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < n_slots; j += stride) {
    const int s = src[j];
    pt[j] = s >= 0 ? opt[s] : -1;
    sh[j] = s >= 0 ? ob[s].shot : 0;
  }
}

// ---------------------------------------------------------------------------
// Small camera-side kernels.

template <typename R>
__global__ void cam_damp_kernel(int n, const R* __restrict__ dc, const double* __restrict__ pdiag,
                                const uint8_t* __restrict__ mask, R* __restrict__ cscale, R* __restrict__ damp,
                                double mu, int first) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  if (!mask[j]) {
    damp[j] = R(0);
    if (first) cscale[j] = R(1);
    return;
  }
  const double d = double(dc[j]) + pdiag[j];
  if (first) cscale[j] = R(1.0 / (1.0 + sqrt(d)));
  const double s = double(cscale[j]);
  double c = s * s * d;
  c = c < 1e-6 ? 1e-6 : (c > 1e32 ? 1e32 : c);
  damp[j] = R(c / (s * s) * mu);
}

template <typename R>
__global__ void rhs_finish_kernel(int n, const double* __restrict__ gc, const double* __restrict__ pgrad,
                                  const uint8_t* __restrict__ mask, double* __restrict__ rhs64, R* __restrict__ rhs,
                                  double* __restrict__ bb) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  double v = 0.0;
  if (j < n) {
    const double b = mask[j] ? rhs64[j] - gc[j] - pgrad[j] : 0.0;
    rhs64[j] = b;
    rhs[j] = R(b);
    v = b * b;
  }
  block_sum_add<256>(v, bb);
}

// Inverts a symmetric positive definite n x n matrix (row-major, double) in
// place by Cholesky; returns false if not positive definite.
__device__ inline bool spd_inverse(double* A, int n, int ld) {
  // Cholesky A = L L^T (lower stored in A)
  for (int j = 0; j < n; ++j) {
    double d = A[j * ld + j];
    for (int k = 0; k < j; ++k) d -= A[j * ld + k] * A[j * ld + k];
    if (!(d > 0.0)) return false;
    d = sqrt(d);
    A[j * ld + j] = d;
    for (int i = j + 1; i < n; ++i) {
      double s = A[i * ld + j];
      for (int k = 0; k < j; ++k) s -= A[i * ld + k] * A[j * ld + k];
      A[i * ld + j] = s / d;
    }
  }
  // inverse of L in place (lower)
  for (int j = 0; j < n; ++j) {
    A[j * ld + j] = 1.0 / A[j * ld + j];
    for (int i = j + 1; i < n; ++i) {
      double s = 0.0;
      for (int k = j; k < i; ++k) s -= A[i * ld + k] * A[k * ld + j];
      A[i * ld + j] = s / A[i * ld + i];
    }
  }
  // A^-1 = L^-T L^-1, write full symmetric
  for (int i = 0; i < n; ++i)
    for (int j = 0; j <= i; ++j) {
      double s = 0.0;
      for (int k = i; k < n; ++k) s += A[k * ld + i] * A[k * ld + j];
      A[j * ld + i] = s;  // upper
    }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < i; ++j) A[i * ld + j] = A[j * ld + i];
  return true;
}

// Assembles and inverts the block-Jacobi preconditioner blocks.
//   block = schur_tri + diag(pdiag + damp) on optimised coordinates,
//   identity-free rows/columns for fixed coordinates (their inverse rows are 0).
template <typename R>
__global__ void precond_invert_kernel(CamLayout cl, int cam_tri_stride, int cmax, const R* __restrict__ tri_inst,
                                      const R* __restrict__ tri_rig, const R* __restrict__ tri_cam,
                                      const double* __restrict__ pdiag, const R* __restrict__ damp,
                                      const uint8_t* __restrict__ mask, R* __restrict__ minv_inst,
                                      R* __restrict__ minv_rig, R* __restrict__ minv_cam, int* __restrict__ n_bad) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  const int nb = cl.n_inst + cl.n_rig + cl.n_cam;
  if (b >= nb) return;
  int size, start;
  const R* tri;
  R* out;
  int w;  // logical block width
  if (b < cl.n_inst) {
    size = 8; w = 6; start = 8 * b; tri = tri_inst + 24 * int64_t(b); out = minv_inst + 64 * int64_t(b);
  } else if (b < cl.n_inst + cl.n_rig) {
    const int r = b - cl.n_inst;
    size = 8; w = 6; start = cl.rig_base + 8 * r; tri = tri_rig + 24 * int64_t(r); out = minv_rig + 64 * int64_t(r);
  } else {
    const int k = b - cl.n_inst - cl.n_rig;
    size = 16; w = cmax; start = cl.cam_base + 16 * k; tri = tri_cam + int64_t(cam_tri_stride) * k;
    out = minv_cam + 256 * int64_t(k);
  }
  double A[16 * 16];
  int idx[16];
  int m = 0;
  for (int a = 0; a < w; ++a)
    if (mask[start + a]) idx[m++] = a;
  // unpack the upper triangle (row-major over a <= c)
  auto tri_at = [&](int a, int c) {
    if (a > c) { const int t = a; a = c; c = t; }
    const int off = a * w - a * (a - 1) / 2 + (c - a);
    return double(tri[off]);
  };
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < m; ++j) {
      double v = tri_at(idx[i], idx[j]);
      if (i == j) v += pdiag[start + idx[i]] + double(damp[start + idx[i]]);
      A[i * 16 + j] = v;
    }
  for (int i = 0; i < size * size; ++i) out[i] = R(0);
  if (m == 0) return;
  if (!spd_inverse(A, m, 16)) {
    atomicAdd(n_bad, 1);
    // fall back to the inverse diagonal
    for (int i = 0; i < m; ++i) {
      const double d = tri_at(idx[i], idx[i]) + pdiag[start + idx[i]] + double(damp[start + idx[i]]);
      out[idx[i] * size + idx[i]] = R(d > 0.0 ? 1.0 / d : 0.0);
    }
    return;
  }
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < m; ++j) out[idx[i] * size + idx[j]] = R(A[i * 16 + j]);
}

// z = M^-1 r (block diagonal), rz += r . z
template <typename R>
__global__ void precond_apply_kernel(CamLayout cl, const R* __restrict__ minv_inst, const R* __restrict__ minv_rig,
                                     const R* __restrict__ minv_cam, const R* __restrict__ r, R* __restrict__ z,
                                     double* __restrict__ rz) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  double acc = 0.0;
  if (j < cl.n) {
    const R* M;
    int start, size, row;
    if (j < cl.rig_base) {
      const int b = j >> 3;
      start = 8 * b; size = 8; row = j & 7; M = minv_inst + 64 * int64_t(b);
    } else if (j < cl.cam_base) {
      const int b = (j - cl.rig_base) >> 3;
      start = cl.rig_base + 8 * b; size = 8; row = (j - cl.rig_base) & 7; M = minv_rig + 64 * int64_t(b);
    } else {
      const int b = (j - cl.cam_base) >> 4;
      start = cl.cam_base + 16 * b; size = 16; row = (j - cl.cam_base) & 15; M = minv_cam + 256 * int64_t(b);
    }
    R s = R(0);
    for (int k = 0; k < size; ++k) s += M[row * size + k] * r[start + k];
    z[j] = s;
    acc = double(r[j]) * double(s);
  }
  block_sum_add<256>(acc, rz);
}

// y = mask (y + diag p), pq += p . y
template <typename R>
__global__ void spmv_finish_kernel(int n, const R* __restrict__ p, const double* __restrict__ pdiag,
                                   const R* __restrict__ damp, const uint8_t* __restrict__ mask, R* __restrict__ y,
                                   double* __restrict__ pq) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  double acc = 0.0;
  if (j < n) {
    R v = R(0);
    if (mask[j]) v = y[j] + R(pdiag[j] + double(damp[j])) * p[j];
    y[j] = v;
    acc = double(p[j]) * double(v);
  }
  block_sum_add<256>(acc, pq);
}

// x += alpha p, r -= alpha y, rr += r . r with alpha = s[RZ] / s[PQ]
enum { kRZ = 0, kPQ = 1, kRR = 2, kRZN = 3, kBB = 4 };
template <typename R>
__global__ void pcg_step_kernel(int n, const double* __restrict__ s, R* __restrict__ x, R* __restrict__ r,
                                const R* __restrict__ p, const R* __restrict__ y, double* __restrict__ rr) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  double acc = 0.0;
  const double pq = s[kPQ];
  const double alpha = pq > 0.0 ? s[kRZ] / pq : 0.0;
  if (j < n) {
    x[j] += R(alpha) * p[j];
    const R rv = r[j] - R(alpha) * y[j];
    r[j] = rv;
    acc = double(rv) * double(rv);
  }
  block_sum_add<256>(acc, rr);
}

// p = z + beta p, beta = s[RZN] / s[RZ]
template <typename R>
__global__ void pcg_dir_kernel(int n, const double* __restrict__ s, R* __restrict__ p, const R* __restrict__ z) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const double beta = s[kRZ] != 0.0 ? s[kRZN] / s[kRZ] : 0.0;
  p[j] = z[j] + R(beta) * p[j];
}

template <typename From, typename To>
__global__ void convert_kernel(int n, const From* __restrict__ a, To* __restrict__ b) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) b[j] = To(a[j]);
}

// Residual of iterative refinement: r = b - (y + (pdiag + damp) x) on the
// free coordinates, in FP64 (y = the FP64 implicit Schur product W/V part);
// writes r in the working precision for the next PCG round and |r|^2.
template <typename R>
__global__ void refine_residual_kernel(int n, const double* __restrict__ x, const double* __restrict__ pdiag,
                                       const R* __restrict__ damp, const uint8_t* __restrict__ mask,
                                       const double* __restrict__ b, const double* __restrict__ y,
                                       R* __restrict__ r, double* __restrict__ rr) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  double acc = 0.0;
  if (j < n) {
    double v = 0.0;
    if (mask[j]) v = b[j] - (y[j] + (pdiag[j] + double(damp[j])) * x[j]);
    r[j] = R(v);
    acc = v * v;
  }
  block_sum_add<256>(acc, rr);
}

// x64 += e (the correction from a PCG round).
template <typename R>
__global__ void add_correction_kernel(int n, const R* __restrict__ e, double* __restrict__ x) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) x[j] += double(e[j]);
}

static __global__ void pcg_rotate_kernel(double* s) {
  s[kRZ] = s[kRZN];
  s[kPQ] = 0.0;
  s[kRR] = 0.0;
  s[kRZN] = 0.0;
}

// The stopping test of one PCG iteration in the device-side loop (the host
// loop's test after pcg_step_kernel): counts the iteration in ctl[0] and
// ends the loop on a non-positive curvature p.Sp, a residual within
// tolerance (*tol2 = tol^2 |b|^2), a non-finite residual, or ctl[1]
// iterations -- the last bound ends the loop whatever the scalars are.
static __global__ void pcg_control_kernel(const double* __restrict__ s, int* __restrict__ ctl,
                                          const double* __restrict__ tol2, cudaGraphConditionalHandle cond) {
  const int it = ctl[0] + 1;
  ctl[0] = it;
  const double pq = s[kPQ], rr = s[kRR];
  const bool stop = !(pq > 0.0) || rr <= *tol2 || !isfinite(rr) || it >= ctl[1];
  cudaGraphSetConditional(cond, stop ? 0u : 1u);
}

template <typename R>
__global__ void copy_kernel(int n, const R* __restrict__ a, R* __restrict__ b) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) b[j] = a[j];
}

// Point priors (GCP3D, prior_error.h:19-114 with indexes PX, PY[, PZ]):
// r_j = (X_j - prior_j) / sigma_j, weighted by the group's IRLS weight.
struct PointPriorDev {
  int point;
  int n;  // 2 or 3 constrained coordinates
  double prior[3];
  double scale[3];
};

template <typename R>
__global__ void point_prior_linearize_kernel(int n, const PointPriorDev* __restrict__ pp, const double* __restrict__ w,
                                             const Point4* __restrict__ X, const uint8_t* __restrict__ point_free,
                                             R* __restrict__ Vp, R* __restrict__ gp) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const PointPriorDev P = pp[k];
  if (!point_free[P.point]) return;
  const Point4 x = X[P.point];
  const double v[3] = {x.x, x.y, x.z};
  const int dg[3] = {0, 3, 5};
  for (int j = 0; j < P.n; ++j) {
    const double r = P.scale[j] * (v[j] - P.prior[j]);
    atomicAdd(Vp + 8 * int64_t(P.point) + dg[j], R(w[k] * P.scale[j] * P.scale[j]));
    atomicAdd(gp + 4 * int64_t(P.point) + j, R(w[k] * P.scale[j] * r));
  }
}

static __global__ void point_prior_cost_kernel(int n, const PointPriorDev* __restrict__ pp, const double* __restrict__ w,
                                               const Point4* __restrict__ X, double* __restrict__ resid,
                                               double* __restrict__ out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  double acc = 0.0;
  if (k < n) {
    const PointPriorDev P = pp[k];
    const Point4 x = X[P.point];
    const double v[3] = {x.x, x.y, x.z};
    for (int j = 0; j < 3; ++j) {
      const double r = j < P.n ? P.scale[j] * (v[j] - P.prior[j]) : 0.0;
      resid[3 * k + j] = r;
      acc += 0.5 * w[k] * r * r;
    }
  }
  block_sum_add<256>(acc, out);
}

template <typename R>
__global__ void point_prior_model_kernel(int n, const PointPriorDev* __restrict__ pp, const double* __restrict__ w,
                                         const Point4* __restrict__ X, const R* __restrict__ dp,
                                         const uint8_t* __restrict__ point_free, double* __restrict__ out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  double acc = 0.0;
  if (k < n) {
    const PointPriorDev P = pp[k];
    if (point_free[P.point]) {
      const Point4 x = X[P.point];
      const double v[3] = {x.x, x.y, x.z};
      for (int j = 0; j < P.n; ++j) {
        const double r = P.scale[j] * (v[j] - P.prior[j]);
        const double jd = P.scale[j] * double(dp[4 * int64_t(P.point) + j]);
        acc += -0.5 * w[k] * jd * (2.0 * r + jd);
      }
    }
  }
  block_sum_add<256>(acc, out);
}

// ---------------------------------------------------------------------------
// Host helpers: mixture reweighting of one group of residual vectors
// (mixture_reweighting.cc:10-109 with ComputeWhitening, irls_helpers.cc:
// 220-277).  res holds `count` residual vectors of dimension k; blocks with
// another dimension are skipped (dims[i] != k).
struct MixtureResult {
  double log_likelihood = 0.0;
  int outliers = 0;
  int total = 0;
};

bool small_cholesky(std::vector<double>& A, int k, double& det) {
  det = 1.0;
  for (int j = 0; j < k; ++j) {
    double d = A[j * k + j];
    for (int m = 0; m < j; ++m) d -= A[j * k + m] * A[j * k + m];
    if (!(d > 0.0)) return false;
    det *= d;
    d = std::sqrt(d);
    A[j * k + j] = d;
    for (int i = j + 1; i < k; ++i) {
      double s = A[i * k + j];
      for (int m = 0; m < j; ++m) s -= A[i * k + m] * A[j * k + m];
      A[i * k + j] = s / d;
    }
  }
  return true;
}

// Determinant and inverse of a small symmetric matrix (LU with pivoting, so
// that indefinite matrices behave like Eigen's determinant()/inverse()).
bool small_det_inverse(const std::vector<double>& A, int k, double& det, std::vector<double>& inv) {
  std::vector<double> M = A;
  std::vector<int> perm(k);
  std::iota(perm.begin(), perm.end(), 0);
  det = 1.0;
  for (int c = 0; c < k; ++c) {
    int p = c;
    for (int r = c + 1; r < k; ++r)
      if (std::fabs(M[r * k + c]) > std::fabs(M[p * k + c])) p = r;
    if (M[p * k + c] == 0.0) {
      det = 0.0;
      return false;
    }
    if (p != c) {
      for (int j = 0; j < k; ++j) std::swap(M[p * k + j], M[c * k + j]);
      std::swap(perm[p], perm[c]);
      det = -det;
    }
    det *= M[c * k + c];
    for (int r = c + 1; r < k; ++r) {
      const double f = M[r * k + c] / M[c * k + c];
      M[r * k + c] = f;
      for (int j = c + 1; j < k; ++j) M[r * k + j] -= f * M[c * k + j];
    }
  }
  inv.assign(k * k, 0.0);
  for (int col = 0; col < k; ++col) {
    std::vector<double> b(k, 0.0);
    for (int i = 0; i < k; ++i) b[i] = perm[i] == col ? 1.0 : 0.0;
    for (int i = 0; i < k; ++i)
      for (int j = 0; j < i; ++j) b[i] -= M[i * k + j] * b[j];
    for (int i = k - 1; i >= 0; --i) {
      for (int j = i + 1; j < k; ++j) b[i] -= M[i * k + j] * b[j];
      b[i] /= M[i * k + i];
    }
    for (int i = 0; i < k; ++i) inv[i * k + col] = b[i];
  }
  return true;
}

constexpr double kMinDeterminant = 1e-3;
constexpr double kMinVariance = 0.025;
constexpr double kMinWeight = 1e-10;
constexpr int kMinSampleSize = 10;
constexpr int kMaxInnerIterations = 5;
constexpr double kConvergenceThreshold = 1e-3;

// Group covariance -> (inverse, 1/sqrt((2pi)^k det), K), mixture_reweighting.cc:34-58.
void mixture_params(const std::vector<double>& cov_in, int k, double density_ratio, std::vector<double>& inv,
                    double& norm, double& K) {
  std::vector<double> cov = cov_in;
  for (int i = 0; i < k; ++i) cov[i * k + i] += kMinVariance;
  double det;
  small_det_inverse(cov, k, det, inv);
  if (det < kMinDeterminant) {
    det = kMinVariance * kMinVariance;
    inv.assign(k * k, 0.0);
    for (int i = 0; i < k; ++i) inv[i * k + i] = 1.0 / kMinVariance;
  }
  const double normalizer = std::pow(2 * M_PI, k) * det;
  const double sq = std::sqrt(normalizer);
  norm = 1.0 / sq;
  K = density_ratio / sq;
}

// One host constraint term linearized at a camera-side state: the residuals
// and Jacobian after the loss correction (m rows, ns derivative slots), the
// loss-free residuals the IRLS mixture reads, the free camera-side
// coordinate of every slot (-1: fixed), and w rho(|r|^2).
struct HostTermLin {
  static constexpr int kMaxRows = 7, kMaxSlots = 36;
  int m = 0, ns = 0;
  double r[kMaxRows] = {}, raw[kMaxRows] = {};
  double J[kMaxRows][kMaxSlots] = {};
  int coord[kMaxSlots] = {};
  double rho = 0.0;
};

// IRLS groups of the host constraint terms: UP, PAN, TILT, ROLL (by
// orientation kind), ROT, POS, MOTION, GAUGE, HEATMAP, REL, GPS, STDDEV (by
// relative kind)
constexpr int kHostGroups = 12;
const char* const kHostGroupNames[kHostGroups] = {"UP",     "PAN",    "TILT",    "ROLL", "ROT", "POS",
                                                  "MOTION", "GAUGE", "HEATMAP", "REL",  "GPS", "STDDEV"};

MixtureResult mixture_group(const std::vector<std::vector<double>>& res, std::vector<double>& weights,
                            double density_ratio) {
  MixtureResult out;
  out.total = int(res.size());
  if (res.empty() || int(res.size()) < kMinSampleSize) return out;
  const int k = int(res[0].size());
  double prev = std::numeric_limits<double>::max();
  double ll = 0.0;
  int outl = 0;
  for (int it = 0; it < kMaxInnerIterations; ++it) {
    std::vector<double> S(k * k, 0.0);
    double W = 0.0;
    for (size_t i = 0; i < res.size(); ++i) {
      if (int(res[i].size()) != k) continue;
      for (int a = 0; a < k; ++a)
        for (int b = 0; b < k; ++b) S[a * k + b] += weights[i] * res[i][a] * res[i][b];
      W += weights[i];
    }
    if (W < 1e-9) return out;
    for (auto& s : S) s /= W;
    std::vector<double> inv;
    double norm, K;
    mixture_params(S, k, density_ratio, inv, norm, K);
    ll = 0.0;
    outl = 0;
    for (size_t i = 0; i < res.size(); ++i) {
      if (int(res[i].size()) != k) continue;
      double m = 0.0;
      for (int a = 0; a < k; ++a)
        for (int b = 0; b < k; ++b) m += res[i][a] * inv[a * k + b] * res[i][b];
      const double p_in = std::exp(-0.5 * m) * norm;
      ll += std::log(p_in + K);
      double w = p_in / (p_in + K);
      w = std::max(kMinWeight, std::min(w, 1.0));
      weights[i] = w;
      if (w < 0.5) ++outl;
    }
    const double change = std::fabs(ll - prev) / std::fabs(prev);
    if (change < kConvergenceThreshold) break;
    prev = ll;
  }
  out.log_likelihood = ll;
  out.outliers = outl;
  return out;
}

// Angle-axis rotation of a vector (for the GPS-prior bias transform).
void rotate_aa(const double* r, const double* p, double* out) {
  const double th2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
  if (th2 < kEps) {
    out[0] = p[0] + r[1] * p[2] - r[2] * p[1];
    out[1] = p[1] + r[2] * p[0] - r[0] * p[2];
    out[2] = p[2] + r[0] * p[1] - r[1] * p[0];
    return;
  }
  const double th = std::sqrt(th2), c = std::cos(th), s = std::sin(th);
  const double k[3] = {r[0] / th, r[1] / th, r[2] / th};
  const double kxp[3] = {k[1] * p[2] - k[2] * p[1], k[2] * p[0] - k[0] * p[2], k[0] * p[1] - k[1] * p[0]};
  const double kp = k[0] * p[0] + k[1] * p[1] + k[2] * p[2];
  for (int i = 0; i < 3; ++i) out[i] = p[i] * c + kxp[i] * s + k[i] * kp * (1 - c);
}

double now_seconds() {
  using clk = std::chrono::steady_clock;
  return std::chrono::duration<double>(clk::now().time_since_epoch()).count();
}

}  // namespace
}  // namespace gbba

namespace gbba {
namespace {

template <typename R>
class DeviceSolver : public SolverBase {
 protected:
  using V16 = typename Vec16<R>::type;
  using PS = typename PointStore<R>::type;
  static constexpr bool kMixed = sizeof(R) == 4;

 public:
  SolveSummary solve(Problem& P, const SolverOptions& opts) override;
  void reprojection(std::vector<double>& errors, std::vector<double>& weights) override {
    errors = last_errors_;
    weights = last_weights_;
  }
  bool covariances(std::vector<double>& cov) override {
    cov = cov_;
    return cov_valid_;
  }
  ~DeviceSolver() override { release_pcg_graph(); }

 protected:
  // ---- setup
  void setup(const Problem& P, const SolverOptions& opts);
  void upload_camera_side(const std::vector<double>& x, bool working, bool fp64);
  // ---- device passes
  SolveView<R> view();
  ShotMajorView<R> sm_view();
  SceneView<double> view64(bool candidate);
  double cost_pass(bool candidate, bool store_residuals);
  void linearize();
  void point_priors_linearize(bool candidate);
  // ---- host priors and orientation constraints
  double prior_terms(const std::vector<double>& x, bool want_derivs);
  // y += H x for the host-computed Gauss-Newton blocks
  template <typename A>
  void host_blocks_apply(const A* x, A* y, cudaStream_t st = 0) {
    if (n_hblocks_ == 0) return;
    host_block_spmv_kernel<A><<<(8 * n_hblocks_ + 255) / 256, 256, 0, st>>>(n_hblocks_, d_hbase_.get(),
                                                                           d_hval_.get(), x, y);
    ++launches_;
  }
  double prior_model_change(const std::vector<double>& x, const std::vector<double>& dx);
  // host constraint terms: the orientation terms, then the relative terms
  int n_host_terms() const { return int(prob_->orientation_terms.size() + prob_->relative_terms.size()); }
  int host_term_group(int q) const;
  void host_term(int q, const std::vector<double>& x, HostTermLin& L) const;
  // ---- linear solve
  int solve_step(double mu, bool first, double& model_change, std::vector<double>& dxc);
  int run_pcg(const R* rhs, double bb, double tol, int max_it);
  // the PCG iterations as one CUDA graph launch: a while node whose body is
  // one iteration and pcg_control_kernel (built on first use, again when
  // the host-term blocks move); single-rank solves only
  int run_pcg_device_loop(int max_it, double tol2);
  void build_pcg_graph();
  void release_pcg_graph();
  cudaStream_t pcg_st_ = nullptr;
  cudaGraph_t pcg_graph_ = nullptr;
  cudaGraphExec_t pcg_exec_ = nullptr;
  const void* pcg_graph_key_ = nullptr;  // the host-term block values the graph reads
  int pcg_graph_blocks_ = -1;
  // the views the recorded passes read (matrix-free passes evaluate the
  // current state, whose buffers trade places with the candidate's on an
  // accepted step): the graph is rebuilt when they change
  SolveView<R> pcg_view_{};
  ShotMajorView<R> pcg_sm_view_{};
  // The view as far as the recorded passes read it: passes over stored
  // records read neither the points nor the FP64 residuals (whose buffers
  // trade places with the candidate's on every accepted step), so those
  // do not force a rebuild there.
  SolveView<R> pcg_graph_view() {
    SolveView<R> v = view();
    if (!matrix_free_) {
      v.scene.points = nullptr;
      v.resid64 = nullptr;
    }
    return v;
  }
  bool pcg_graph_coarse_ = false;  // the graph applies the coarse correction
  int64_t pcg_body_nodes_ = 0;
  DeviceArray<int> d_pcg_ctl_;      // [iterations done, iteration limit]
  DeviceArray<double> d_pcg_tol2_;  // tol^2 |b|^2
  int solve_dense(double mu);
  void assemble_dense(double mu);
  bool compute_covariances();
  // launches a record pass with stored or evaluated records
  void record_pass(RecordPassLaunch<R>& f) {
    if (matrix_free_) launch_evaluated<R>(kc_, f);
    else dispatch_config(kc_, f);
  }
  // ---- IRLS
  double compute_weights(std::vector<std::string>& groups_report, int& proj_out, int& proj_total,
                         std::vector<std::pair<std::string, std::pair<int, int>>>& other);
  // ---- results
  void finish(Problem& P);
  // ---- sharded solve (opts_.shard): collectives over the ranks, no-ops on
  // a single rank.  Observation sums are reduced right after the record
  // pass that forms them, before any prior or host term (replicated on
  // every rank) is added.  Decisions taken on values that every rank
  // computes for itself (PCG scalars, the camera step) use rank 0's values,
  // so that all ranks take the same branches and issue the same collectives.
  bool sharded() const { return opts_.shard.active(); }
  void shard_reduce(double* h, int64_t n, int op);
  void shard_bcast(double* h, int64_t n);
  template <typename T>
  void shard_reduce_device(T* d, int64_t n);

  Problem* prob_ = nullptr;
  SolverOptions opts_;
  KernelConfig kc_{};
  CamLayout cl_{};
  int n_inst_ = 0, n_rig_ = 0, n_cam_ = 0, n_shots_ = 0;
  int64_t n_pt_ = 0, n_obs_ = 0, n_terms_ = 0, n_slots_ = 0;
  std::vector<int64_t> depth_obs_;  // the observations with a depth prior, in observation order
  int n_planes_ = 0;
  uint64_t plane_mask_ = 0;
  int cam_tri_stride_ = 0;
  std::vector<int64_t> slot_obs_;
  std::vector<double> xc_, xc_cand_;
  std::vector<uint8_t> cmask_;
  std::vector<double> pgrad_, pdiag_;
  // orientation constraints: Gauss-Newton blocks (8 x 8, keyed by coordinate
  // group bases) and their diagonal (for the LM damping)
  std::map<std::pair<int, int>, std::array<double, 64>> hblocks_;
  std::vector<double> hdiag_;
  int n_hblocks_ = 0;
  std::vector<double> host_weight_;  // IRLS weight of every host constraint term
  // the host terms linearized at the current state (the linear-model
  // decrease of a step reads them instead of evaluating the terms again)
  std::vector<HostTermLin> host_lin_;
  std::vector<int> group_count_, group_dim_;
  std::vector<double> group_ratio_;
  std::vector<double> prior_weight_cam_, prior_weight_rig_, prior_weight_gps_;
  std::vector<int> gps_inst_;
  std::vector<PointPriorDev> point_priors_;
  int64_t pp_offset_ = 0, n_pp_total_ = 0;  // this rank's first point prior in the GCP3D group, the group size
  std::vector<double> point_prior_w_;
  double ratio_cam_ = 1e-3, ratio_rig_ = 1e-3, ratio_gps_ = 1e-3, ratio_gcp3d_ = 1e-3;
  int64_t launches_ = 0;
  int64_t refinements_ = 0;  // FP64 residual evaluations of iterative refinement
  int64_t confirmations_ = 0;  // convergence confirmations with a refined step (mixed)
  double pcg_tolerance_override_ = 0.0;  // > 0: PCG tolerance of the next steps
  // dense mode: explicit reduced camera system over the n_dense_ optimised
  // camera-side coordinates, factored by DenseSpdSolver
  // matrix-free: no stored records; every record pass evaluates them again
  bool matrix_free_ = false;
  bool dense_ = false;
  bool dense_ready_ = false;  // the dense structures exist (dense steps or covariances)
  int n_dense_ = 0;
  std::vector<int> dmap_host_;
  std::vector<double> cov_;  // [n_inst][6][6] pose covariances of the final state
  bool cov_valid_ = false;
  int64_t n_pairs_ = 0;
  int64_t dense_failures_ = 0;  // factorizations that found the system not positive definite
  DenseSpdSolver dense_solver_;
  // two-level preconditioner (coarse_space.h): built at the first PCG
  // step; the Galerkin matrix is probed once per linearization and
  // factored with the damping of every step
  void coarse_prepare();
  void coarse_apply(const R* r, R* z, double* rz, cudaStream_t st);
  bool coarse_built_ = false, coarse_stale_ = true, coarse_active_ = false, coarse_have_e_ = false;
  CoarseSpace cs_;
  int64_t coarse_probes_ = 0;
  int last_pcg_iterations_ = 0, prev_pcg_iterations_ = 0;  // of the last two linear solves
  DeviceArray<double> d_cbasis_, d_cE_, d_cW_, d_cw_, d_cu_, d_cscal_;
  DeviceArray<int> d_ccluster_, d_ccolour_, d_cpartner_, d_cmstart_, d_cmembers_;
  DeviceArray<R> d_czero_, d_cprobe_;
  DeviceArray<float> d_cinv_;  // E^-1 through the FP32 factor, [m][ld]
  int coarse_ld_ = 0;
  DenseSpdSolver coarse_solver_;
  std::vector<double> last_errors_, last_weights_;

  // device state
  DeviceArray<ObsPack<R>> d_obs_;
  DeviceArray<ObsPack<double>> d_obs64_;
  DeviceArray<int> d_obs_point_;
  DeviceArray<uint8_t> d_gcp_;
  DeviceArray<R> d_weight_;
  // FP64 residuals of the current state, and (mixed mode) of the last
  // candidate: swapped in when the candidate is accepted
  DeviceArray<double> d_resid_, d_resid_cand_;
  DeviceArray<V16> d_rec_;
  // shot-major order: point-major slot, point and shot of every shot-major
  // slot, and the shot-major copy of the records
  DeviceArray<int> d_sm_src_, d_sm_point_, d_sm_shot_;
  DeviceArray<V16> d_rec_sm_;
  // geometry: working precision of the current state (d_geom_, d_cam_), FP64
  // of the current state (mixed mode only; in FP64 mode d_geom_ is it), FP64
  // of the candidate state (d_geomc_, d_camc_)
  DeviceArray<ShotGeom<R>> d_geom_;
  DeviceArray<ShotGeom<double>> d_geom64_, d_geomc_;
  DeviceArray<RigGeom<R>> d_rig_;
  DeviceArray<R> d_cam_;
  DeviceArray<double> d_cam64_, d_camc_;
  DeviceArray<int> d_cam_model_, d_shot_inst_, d_shot_rig_, d_shot_cam_;
  DeviceArray<double> d_inst_pose_, d_rig_pose_;
  DeviceArray<uint8_t> d_rig_used_;
  DeviceArray<Point4> d_X_, d_Xc_;
  DeviceArray<PS> d_Xw_;
  DeviceArray<uint8_t> d_inst_free_, d_cam_free_, d_rig_free_, d_point_free_, d_cmask_;
  DeviceArray<R> d_Vp_, d_gp_, d_Vinv_, d_pscale_, d_zbuf_, d_dp_;
  DeviceArray<double> d_gc_, d_rhs64_;  // FP64 sums: gradient, reduced right-hand side
  // iterative refinement (mixed mode): FP64 step, FP64 Schur product, the
  // FP32 residual handed to PCG and its squared norm
  DeviceArray<double> d_x64_, d_zbuf64_, d_y64_, d_rr64_;
  DeviceArray<R> d_rref_;
  DeviceArray<R> d_dc_, d_rhs_, d_cscale_, d_damp_;
  DeviceArray<double> d_pdiag_, d_pgrad_;
  DeviceArray<double> d_pdamp_;  // pdiag + orientation-term diagonal: the LM diagonal of the host terms
  DeviceArray<int2> d_hbase_;
  DeviceArray<double> d_hval_;
  DeviceArray<R> d_x_, d_r_, d_z_, d_p_, d_y_;
  DeviceArray<R> d_tri_inst_, d_tri_rig_, d_tri_cam_, d_minv_inst_, d_minv_rig_, d_minv_cam_;
  DeviceArray<double> d_scal_;
  DeviceArray<int> d_bad_;
  DeviceArray<double> d_irls_stats_, d_irls_ll_;
  DeviceArray<IrlsGroupParams> d_irls_params_;
  DeviceArray<int> d_group_dim_;
  DeviceArray<PointPriorDev> d_pp_;
  DeviceArray<double> d_pp_w_, d_pp_res_;
  DeviceArray<int> d_dmap_, d_didx_;
  DeviceArray<int2> d_pairs_;
  DeviceArray<int> d_pair_key_;
  DeviceArray<double> d_S_, d_WT_, d_bd_, d_xd_;
  DeviceArray<double> d_V64_, d_Vinv64_, d_gp64_;  // FP64 point blocks of the dense path
};

// ---------------------------------------------------------------------------
template <typename R>
void DeviceSolver<R>::setup(const Problem& P, const SolverOptions& opts) {
  opts_ = opts;
  n_inst_ = int(P.instances.size());
  n_rig_ = int(P.rig_cameras.size());
  n_cam_ = int(P.cameras.size());
  n_shots_ = int(P.shots.size());
  n_pt_ = int64_t(P.points.size());
  n_obs_ = int64_t(P.observations.size());
  // residual terms on slots: every observation, then its depth prior if it
  // has one (RelativeDepthError, added beside the projection error at
  // bundle_adjuster.cc:861-869)
  depth_obs_.clear();
  for (int64_t o = 0; o < n_obs_; ++o)
    if (P.observations[size_t(o)].has_depth) depth_obs_.push_back(o);
  n_terms_ = n_obs_ + int64_t(depth_obs_.size());

  // kernel configuration
  bool any_sph = false, single = true, any_rig_free = false, any_rig_used = false;
  int first = -1;
  for (const Shot& s : P.shots) {
    const int m = P.cameras[s.camera].model;
    if (m == kSpherical) any_sph = true;
    if (first < 0) first = m;
    else if (m != first) single = false;
    if (s.rig_camera >= 0 && P.rig_cameras[s.rig_camera].used) {
      any_rig_used = true;
      const PoseBlock& rc = P.rig_cameras[s.rig_camera];
      for (int k = 0; k < 6; ++k) any_rig_free |= rc.free_mask[k] != 0;
    }
  }
  kc_.nr = any_sph ? 3 : 2;
  kc_.rig = any_rig_free;
  if (single && !any_sph && !any_rig_used && first >= 0) {
    kc_.model = first;
    kc_.cmax = model_num_params(first);
  } else {
    kc_.model = kDyn;
    kc_.cmax = 16;
  }
  const int width = kc_.nr + 3 * kc_.nr + 6 * kc_.nr + kc_.cmax * kc_.nr + (kc_.rig ? 6 * kc_.nr : 0);
  n_planes_ = planes_of<R>(width);
  bool any_cam_free = false;
  for (const CameraBlock& c : P.cameras)
    for (int k = 0; k < c.n; ++k) any_cam_free |= c.free_mask[k] != 0;
  // planes holding only intrinsics columns are not written when every
  // camera is fixed
  plane_mask_ = 0;
  {
    const int cam_begin = 10 * kc_.nr;                      // RecordLayout::kCam
    const int cam_end = cam_begin + kc_.cmax * kc_.nr;      // RecordLayout::kRig
    const int VN = Vec16<R>::kN;
    for (int p = 0; p < n_planes_; ++p) {
      const bool cam_only = p * VN >= cam_begin && (p + 1) * VN <= cam_end;
      if (!any_cam_free && cam_only) continue;
      plane_mask_ |= uint64_t(1) << p;
    }
  }

  // camera-side layout
  cl_.n_inst = n_inst_;
  cl_.n_rig = n_rig_;
  cl_.n_cam = n_cam_;
  cl_.rig_base = 8 * n_inst_;
  cl_.cam_base = cl_.rig_base + 8 * n_rig_;
  cl_.n = cl_.cam_base + 16 * n_cam_;
  xc_.assign(cl_.n, 0.0);
  cmask_.assign(cl_.n, 0);
  for (int i = 0; i < n_inst_; ++i)
    for (int k = 0; k < 6; ++k) {
      xc_[8 * i + k] = P.instances[i].value[k];
      cmask_[8 * i + k] = P.instances[i].free_mask[k];
    }
  for (int r = 0; r < n_rig_; ++r)
    for (int k = 0; k < 6; ++k) {
      xc_[cl_.rig_base + 8 * r + k] = P.rig_cameras[r].value[k];
      cmask_[cl_.rig_base + 8 * r + k] =
          (P.rig_cameras[r].used && (kc_.rig || P.rig_cameras[r].scale_block)) ? P.rig_cameras[r].free_mask[k] : 0;
    }
  for (int c = 0; c < n_cam_; ++c)
    for (int k = 0; k < P.cameras[c].n; ++k) {
      xc_[cl_.cam_base + 16 * c + k] = P.cameras[c].value[k];
      cmask_[cl_.cam_base + 16 * c + k] = P.cameras[c].free_mask[k];
    }

  // Slots.  Point-major order: observations sorted by point (stable
  // counting sort), padded to a warp multiple.  Shot-major order of the same
  // slots: by rig instance, then shot, then point (a stable counting sort of
  // the point-major slots by shot rank); padding slots go last.  The host
  // makes three sequential passes over the observations (counts, point
  // scatter, shot scatter); the per-slot arrays are built on the device from
  // the uploaded observations.
  if (n_terms_ > int64_t(std::numeric_limits<int32_t>::max()) - 32)
    throw std::invalid_argument("more observations than a 32-bit slot index can address");
  n_slots_ = std::max<int64_t>(32, (n_terms_ + 31) / 32 * 32);
  // observation of term t (a depth prior's is the observation it belongs to)
  auto term = [&](int64_t t) -> const Observation& {
    return P.observations[size_t(t < n_obs_ ? t : depth_obs_[size_t(t - n_obs_)])];
  };
  std::vector<int> rank(n_shots_);
  {
    std::vector<int> shots(n_shots_);
    std::iota(shots.begin(), shots.end(), 0);
    std::stable_sort(shots.begin(), shots.end(),
                     [&](int a, int b) { return P.shots[a].instance < P.shots[b].instance; });
    for (int r = 0; r < n_shots_; ++r) rank[shots[r]] = r;
  }
  std::vector<int64_t> pstart(n_pt_ + 1, 0), sstart(n_shots_ + 1, 0);
  // IRLS groups of the slots: one per shot, GCP2D, DEPTH
  group_count_.assign(n_shots_ + 2, 0);
  int gcp_shot = -1;
  for (int64_t t = 0; t < n_terms_; ++t) {
    const Observation& q = term(t);
    ++pstart[q.point + 1];
    ++sstart[rank[q.shot] + 1];
    ++group_count_[t >= n_obs_ ? n_shots_ + 1 : q.is_gcp ? n_shots_ : q.shot];
    if (t < n_obs_ && q.is_gcp && gcp_shot < 0) gcp_shot = q.shot;
  }
  for (int64_t p = 0; p < n_pt_; ++p) pstart[p + 1] += pstart[p];
  for (int r = 0; r < n_shots_; ++r) sstart[r + 1] += sstart[r];
  std::vector<int32_t> order(n_terms_);
  for (int64_t o = 0; o < n_terms_; ++o) order[pstart[term(o).point]++] = int32_t(o);
  std::vector<int32_t> src(n_slots_, -1);
  for (int64_t s = 0; s < n_terms_; ++s) src[sstart[rank[term(order[s]).shot]]++] = int32_t(s);
  slot_obs_.assign(n_slots_, -1);  // the observation of a projection slot; -1: depth prior or padding
  for (int64_t s = 0; s < n_terms_; ++s) slot_obs_[s] = order[s] < n_obs_ ? order[s] : -1;
  {
    DeviceArray<Observation> raw(size_t(std::max<int64_t>(1, n_terms_)));
    DeviceArray<int32_t> d_order;
    if (n_obs_)
      GB_CUDA(cudaMemcpyAsync(raw.get(), P.observations.data(), size_t(n_obs_) * sizeof(Observation),
                              cudaMemcpyHostToDevice));
    if (!depth_obs_.empty()) {
      std::vector<Observation> dt(depth_obs_.size());
      for (size_t k = 0; k < dt.size(); ++k) dt[k] = P.observations[size_t(depth_obs_[k])];
      GB_CUDA(cudaMemcpy(raw.get() + n_obs_, dt.data(), dt.size() * sizeof(Observation), cudaMemcpyHostToDevice));
    }
    d_order.upload(order);
    d_sm_src_.upload(src);
    d_obs_.resize(n_slots_);
    if (kMixed) d_obs64_.resize(n_slots_);
    d_obs_point_.resize(n_slots_);
    d_gcp_.resize(n_slots_);
    d_weight_.resize(n_slots_);
    d_sm_point_.resize(n_slots_);
    d_sm_shot_.resize(n_slots_);
    build_slots_kernel<R><<<elem_grid(n_slots_), 256>>>(n_terms_, n_obs_, n_slots_, raw.get(), d_order.get(),
                                                         d_obs_.get(),
                                                         kMixed ? d_obs64_.get() : nullptr, d_obs_point_.get(),
                                                         d_gcp_.get(), d_weight_.get());
    build_shot_major_kernel<R><<<elem_grid(n_slots_), 256>>>(n_slots_, d_sm_src_.get(), d_obs_point_.get(),
                                                              d_obs_.get(), d_sm_point_.get(), d_sm_shot_.get());
    launches_ += 2;
    GB_CUDA(cudaGetLastError());
    GB_CUDA(cudaDeviceSynchronize());  // raw and d_order are released here
  }
  d_resid_.resize(4 * n_slots_);
  d_resid_.zero();
  if (kMixed) {
    d_resid_cand_.resize(4 * n_slots_);
    d_resid_cand_.zero();
  }

  // Dense mode: the reduced camera system is formed explicitly and factored
  // when the linear solver type asks for an exact solve (Ceres' DENSE_*,
  // SPARSE_SCHUR and SPARSE_NORMAL_CHOLESKY) and the optimised camera-side
  // coordinates number at most opts.dense_max_unknowns; ITERATIVE_SCHUR,
  // CGNR and larger systems use PCG on the implicit Schur product.
  {
    const std::string& ls = opts.linear_solver;
    const bool exact = ls == "DENSE_SCHUR" || ls == "DENSE_QR" || ls == "DENSE_NORMAL_CHOLESKY" ||
                       ls == "SPARSE_SCHUR" || ls == "SPARSE_NORMAL_CHOLESKY";
    std::vector<int> dmap(cl_.n, -1);
    n_dense_ = 0;
    for (int j = 0; j < cl_.n; ++j)
      if (cmask_[j]) dmap[j] = n_dense_++;
    // a sharded solve takes its steps from PCG on the implicit Schur product
    // (one camera-side all-reduce per iteration); the explicit system and
    // the covariances are single-rank features
    dense_ = !sharded() && exact && n_dense_ > 0 && n_dense_ <= opts.dense_max_unknowns;
    if (dense_ != exact_dense_steps(P, opts) || (exact && n_dense_ != camera_side_unknowns(P)))
      throw std::logic_error("dense mode: camera-side unknown count disagrees with camera_side_unknowns()");
    dense_ready_ = !sharded() && (dense_ || opts.compute_covariances) && n_dense_ > 0 &&
                   n_dense_ <= opts.dense_max_unknowns;
    dmap_host_ = dmap;
    if (dense_ready_) {
      // pairs (o1 >= o2) of the observations of every point, as point-major
      // slot indices, sorted (stable counting sort) by the block of S they
      // add to: key = (shot(o1) * n_shots + shot(o2)) * 2 + (o1 == o2)
      const int64_t n_keys = int64_t(n_shots_) * n_shots_ * 2;
      if (n_keys > int64_t(std::numeric_limits<int>::max()))
        throw std::invalid_argument("dense mode: too many shots");
      std::vector<int2> raw_pairs;
      std::vector<int> raw_keys;
      {
        int64_t s0 = 0;
        while (s0 < n_terms_) {
          const int p = term(order[s0]).point;
          int64_t s1 = s0 + 1;
          while (s1 < n_terms_ && term(order[s1]).point == p) ++s1;
          for (int64_t a = s0; a < s1; ++a) {
            const int64_t sa = term(order[a]).shot;
            for (int64_t b = s0; b <= a; ++b) {
              const int64_t sb = term(order[b]).shot;
              raw_pairs.push_back(make_int2(int(a), int(b)));
              raw_keys.push_back(int((sa * n_shots_ + sb) * 2 + (a == b ? 1 : 0)));
            }
          }
          s0 = s1;
        }
      }
      n_pairs_ = int64_t(raw_pairs.size());
      std::vector<int64_t> kstart(static_cast<size_t>(n_keys) + 1, 0);
      for (int k : raw_keys) ++kstart[size_t(k) + 1];
      for (int64_t k = 0; k < n_keys; ++k) kstart[k + 1] += kstart[k];
      std::vector<int2> sorted_pairs(static_cast<size_t>(n_pairs_));
      std::vector<int> pair_key(static_cast<size_t>(n_pairs_));
      for (size_t q = 0; q < raw_keys.size(); ++q) {
        const int k = raw_keys[q];
        const size_t dst = size_t(kstart[size_t(k)]++);
        sorted_pairs.data()[dst] = raw_pairs.data()[q];
        pair_key.data()[dst] = k;
      }
      d_pair_key_.upload(pair_key);
      const int W = 6 + kc_.cmax + (kc_.rig ? 6 : 0);
      d_dmap_.upload(dmap);
      d_pairs_.upload(sorted_pairs);
      d_didx_.resize(size_t(n_slots_) * W);
      d_WT_.resize(size_t(n_slots_) * 9 * W);  // dense_record<W>()
      d_S_.resize(size_t(n_dense_) * n_dense_);
      d_bd_.resize(n_dense_);
      d_xd_.resize(n_dense_);
      d_x64_.resize(cl_.n);
      const size_t np1 = size_t(std::max<int64_t>(1, n_pt_));
      d_V64_.resize(8 * np1);
      d_Vinv64_.resize(8 * np1);
      d_gp64_.resize(4 * np1);
    }
  }

  // Records: stored (two copies, point-major and shot-major) unless they
  // would take more than 60% of the free device memory, or the caller asks
  // for matrix-free passes.  The dense path reads stored records (its
  // systems are small) and keeps them.
  {
    const size_t record_bytes = 2 * size_t(n_planes_) * size_t(n_slots_) * sizeof(V16);
    size_t free_bytes = 0, total_bytes = 0;
    GB_CUDA(cudaMemGetInfo(&free_bytes, &total_bytes));
    if (opts.matrix_free > 0) matrix_free_ = true;
    else if (opts.matrix_free < 0) matrix_free_ = false;
    else matrix_free_ = double(record_bytes) > 0.6 * double(free_bytes);
    if (dense_ready_) matrix_free_ = false;
    if (!matrix_free_) {
      d_rec_.resize(size_t(n_planes_) * n_slots_);
      d_rec_.zero();  // planes skipped by plane_mask_ must read as zero
      d_rec_sm_.resize(size_t(n_planes_) * n_slots_);
      d_rec_sm_.zero();
      // the staged Schur-product passes' shared-memory limit, set before
      // any pass is recorded into a graph
      StagedPrepare<R> prep;
      dispatch_config(kc_, prep);
    } else {
      d_rec_.release();
      d_rec_sm_.release();
    }
  }

  // shots / cameras / rigs
  std::vector<int> si(n_shots_), sr(n_shots_), sc(n_shots_);
  for (int s = 0; s < n_shots_; ++s) {
    si[s] = P.shots[s].instance;
    sr[s] = P.shots[s].rig_camera;
    sc[s] = P.shots[s].camera;
  }
  d_shot_inst_.upload(si);
  d_shot_rig_.upload(sr);
  d_shot_cam_.upload(sc);
  std::vector<int> cm(n_cam_);
  for (int c = 0; c < n_cam_; ++c) cm[c] = P.cameras[c].model;
  d_cam_model_.upload(cm);
  std::vector<uint8_t> ru(std::max(1, n_rig_), 0);
  for (int r = 0; r < n_rig_; ++r) ru[r] = P.rig_cameras[r].used ? 1 : 0;
  d_rig_used_.upload(ru);
  d_geom_.resize(std::max(1, n_shots_));
  if (kMixed) d_geom64_.resize(std::max(1, n_shots_));
  d_geomc_.resize(std::max(1, n_shots_));
  if (kc_.rig) d_rig_.resize(std::max(1, n_shots_));
  d_inst_pose_.resize(std::max(1, n_inst_) * 6);
  d_rig_pose_.resize(std::max(1, n_rig_) * 6);
  d_cam_.resize(std::max(1, n_cam_) * 16);
  if (kMixed) d_cam64_.resize(std::max(1, n_cam_) * 16);
  d_camc_.resize(std::max(1, n_cam_) * 16);

  // free flags
  std::vector<uint8_t> fi(std::max(1, n_inst_), 0), fc(std::max(1, n_cam_), 0), fr(std::max(1, n_rig_), 0);
  for (int i = 0; i < n_inst_; ++i)
    for (int k = 0; k < 6; ++k) fi[i] |= cmask_[8 * i + k];
  for (int r = 0; r < n_rig_; ++r)
    for (int k = 0; k < 6; ++k) fr[r] |= cmask_[cl_.rig_base + 8 * r + k];
  for (int c = 0; c < n_cam_; ++c)
    for (int k = 0; k < 16; ++k) fc[c] |= cmask_[cl_.cam_base + 16 * c + k];
  d_inst_free_.upload(fi);
  d_cam_free_.upload(fc);
  d_rig_free_.upload(fr);
  d_cmask_.upload(cmask_);

  // points
  std::vector<Point4> X(std::max<int64_t>(1, n_pt_));
  std::vector<uint8_t> pf(std::max<int64_t>(1, n_pt_), 0);
  for (int64_t p = 0; p < n_pt_; ++p) {
    X[p] = Point4{P.points[p].value[0], P.points[p].value[1], P.points[p].value[2], 0.0};
    pf[p] = P.points[p].free ? 1 : 0;
  }
  d_X_.upload(X);
  d_Xc_.resize(X.size());
  if (kMixed) d_Xw_.resize(X.size());
  d_point_free_.upload(pf);
  const size_t np = X.size();
  d_Vp_.resize(8 * np);
  d_gp_.resize(4 * np);
  d_Vinv_.resize(8 * np);
  d_pscale_.resize(3 * np);
  d_zbuf_.resize(4 * np);
  d_dp_.resize(4 * np);
  d_dp_.zero();
  if (kMixed) {
    d_zbuf64_.resize(4 * np);
    d_x64_.resize(cl_.n);
    d_y64_.resize(cl_.n);
    d_rref_.resize(cl_.n);
    d_rr64_.resize(1);
  }

  // camera-side vectors
  for (auto* a : {&d_dc_, &d_rhs_, &d_cscale_, &d_damp_, &d_x_, &d_r_, &d_z_, &d_p_, &d_y_}) a->resize(cl_.n);
  d_gc_.resize(cl_.n);
  d_rhs64_.resize(cl_.n);
  d_pdiag_.resize(cl_.n);
  d_pgrad_.resize(cl_.n);
  d_pdamp_.resize(cl_.n);
  hdiag_.assign(cl_.n, 0.0);
  d_tri_inst_.resize(24 * std::max(1, n_inst_));
  d_tri_rig_.resize(24 * std::max(1, n_rig_));
  cam_tri_stride_ = (kc_.cmax * (kc_.cmax + 1) / 2 + 3) / 4 * 4;
  d_tri_cam_.resize(size_t(cam_tri_stride_) * std::max(1, n_cam_));
  d_minv_inst_.resize(64 * std::max(1, n_inst_));
  d_minv_rig_.resize(64 * std::max(1, n_rig_));
  d_minv_cam_.resize(256 * std::max(1, n_cam_));
  d_scal_.resize(8);
  d_bad_.resize(2);

  // IRLS slot groups: one per shot, GCP2D, and DEPTH (one residual each),
  // counted with the slots
  group_dim_.assign(n_shots_ + 2, 2);
  for (int s = 0; s < n_shots_; ++s) group_dim_[s] = P.cameras[P.shots[s].camera].model == kSpherical ? 3 : 2;
  if (gcp_shot >= 0) group_dim_[n_shots_] = group_dim_[gcp_shot];
  group_dim_[n_shots_ + 1] = 1;
  if (sharded()) {
    // group sizes over every rank's observations (the small-group rule reads
    // them); the GCP2D group takes the larger residual size found on any rank
    std::vector<double> cnt(group_count_.begin(), group_count_.end());
    shard_reduce(cnt.data(), int64_t(cnt.size()), 0);
    for (size_t g = 0; g < cnt.size(); ++g) group_count_[g] = int(cnt[g] + 0.5);
    double gd = gcp_shot >= 0 ? double(group_dim_[n_shots_]) : 0.0;
    shard_reduce(&gd, 1, 1);
    if (gd > 0.0) group_dim_[n_shots_] = int(gd);
  }
  group_ratio_ = P.group_density_ratio;
  if (group_ratio_.size() != size_t(n_shots_ + 1)) group_ratio_.assign(n_shots_ + 1, opts.default_density_ratio);
  group_ratio_.push_back(P.ratio_depth);
  d_group_dim_.upload(group_dim_);
  d_irls_stats_.resize(8 * (n_shots_ + 2));
  d_irls_ll_.resize(2 * (n_shots_ + 2));
  d_irls_params_.resize(n_shots_ + 2);

  // priors
  prior_weight_cam_.assign(n_cam_, 1.0);
  prior_weight_rig_.assign(n_rig_, 1.0);
  gps_inst_.clear();
  for (int i = 0; i < n_inst_; ++i)
    if (P.instances[i].has_position_prior) gps_inst_.push_back(i);
  prior_weight_gps_.assign(gps_inst_.size(), 1.0);
  host_weight_.assign(P.orientation_terms.size() + P.relative_terms.size(), 1.0);
  point_priors_.clear();
  for (int64_t p = 0; p < n_pt_; ++p) {
    const PointBlock& b = P.points[p];
    if (!b.has_prior) continue;
    PointPriorDev d{};
    d.point = int(p);
    d.n = b.has_altitude ? 3 : 2;
    for (int j = 0; j < 3; ++j) {
      d.prior[j] = b.prior[j];
      d.scale[j] = 1.0 / std::max(b.sigma[j], kEps);
    }
    point_priors_.push_back(d);
  }
  point_prior_w_.assign(point_priors_.size(), 1.0);
  // the GCP3D reweighting group spans the point priors of every rank, in
  // rank order
  pp_offset_ = 0;
  n_pp_total_ = int64_t(point_priors_.size());
  if (sharded()) {
    std::vector<double> cnt(size_t(opts.shard.world), 0.0);
    cnt[size_t(opts.shard.rank)] = double(point_priors_.size());
    shard_reduce(cnt.data(), int64_t(cnt.size()), 0);
    n_pp_total_ = 0;
    for (int r = 0; r < opts.shard.world; ++r) {
      if (r == opts.shard.rank) pp_offset_ = n_pp_total_;
      n_pp_total_ += int64_t(cnt[size_t(r)] + 0.5);
    }
  }
  if (!point_priors_.empty()) {
    d_pp_.upload(point_priors_);
    d_pp_w_.upload(point_prior_w_);
    d_pp_res_.resize(3 * point_priors_.size());
  }
  pgrad_.assign(cl_.n, 0.0);
  pdiag_.assign(cl_.n, 0.0);
  GB_CUDA(cudaDeviceSynchronize());
}

// Uploads camera-side FP64 parameters and rebuilds per-shot geometry.
//   working = true:  geometry of the current state in the working precision
//                    (linearization) and, with fp64 in mixed mode, its FP64
//                    copy (cost passes of the current state);
//   working = false: FP64 geometry of a candidate state (d_geomc_, d_camc_).
template <typename R>
void DeviceSolver<R>::upload_camera_side(const std::vector<double>& x, bool working, bool fp64) {
  std::vector<double> ip(std::max(1, n_inst_) * 6, 0.0), rp(std::max(1, n_rig_) * 6, 0.0);
  for (int i = 0; i < n_inst_; ++i)
    for (int k = 0; k < 6; ++k) ip[6 * i + k] = x[8 * i + k];
  for (int r = 0; r < n_rig_; ++r)
    for (int k = 0; k < 6; ++k) rp[6 * r + k] = x[cl_.rig_base + 8 * r + k];
  d_inst_pose_.upload(ip);
  d_rig_pose_.upload(rp);
  std::vector<double> cam(std::max(1, n_cam_) * 16, 0.0);
  for (int c = 0; c < n_cam_; ++c)
    for (int k = 0; k < 16; ++k) cam[16 * c + k] = x[cl_.cam_base + 16 * c + k];
  const int blocks = (n_shots_ + 127) / 128;
  if (working) {
    std::vector<R> cw(cam.size());
    for (size_t i = 0; i < cam.size(); ++i) cw[i] = R(cam[i]);
    d_cam_.upload(cw);
    if (n_shots_ > 0) {
      shot_prep_kernel<R><<<blocks, 128>>>(n_shots_, d_shot_inst_.get(), d_shot_rig_.get(), d_shot_cam_.get(),
                                           d_inst_pose_.get(), d_rig_pose_.get(), d_rig_used_.get(), d_geom_.get(),
                                           kc_.rig ? d_rig_.get() : nullptr);
      ++launches_;
    }
  }
  if (fp64 && (kMixed || !working)) {
    DeviceArray<ShotGeom<double>>& geom = working ? d_geom64_ : d_geomc_;
    DeviceArray<double>& cams = working ? d_cam64_ : d_camc_;
    cams.upload(cam);
    if (n_shots_ > 0) {
      shot_prep_kernel<double><<<blocks, 128>>>(n_shots_, d_shot_inst_.get(), d_shot_rig_.get(),
                                                d_shot_cam_.get(), d_inst_pose_.get(), d_rig_pose_.get(),
                                                d_rig_used_.get(), geom.get(), nullptr);
      ++launches_;
    }
  }
  GB_CUDA(cudaGetLastError());
}

template <typename R>
SolveView<R> DeviceSolver<R>::view() {
  SolveView<R> v{};
  SceneView<R>& s = v.scene;
  s.n_slots = n_slots_;
  s.n_cameras = n_cam_;
  s.geom = d_geom_.get();
  s.rig = kc_.rig ? d_rig_.get() : nullptr;
  s.cam_model = d_cam_model_.get();
  s.cam_params = d_cam_.get();
  if constexpr (kMixed) s.points = d_Xw_.get();
  else s.points = reinterpret_cast<const PS*>(d_X_.get());
  s.obs = d_obs_.get();
  s.obs_point = d_obs_point_.get();
  v.rec = d_rec_.get();
  v.stride = n_slots_;
  v.weight = d_weight_.get();
  v.loss = opts_.loss;
  v.loss_a = R(opts_.loss_threshold);
  v.cl = cl_;
  v.inst_free = d_inst_free_.get();
  v.cam_free = d_cam_free_.get();
  v.rig_free = d_rig_free_.get();
  v.point_free = d_point_free_.get();
  v.Vp = d_Vp_.get();
  v.gp = d_gp_.get();
  v.Vinv = d_Vinv_.get();
  v.gc = d_gc_.get();
  v.dc = d_dc_.get();
  v.resid64 = kMixed ? d_resid_.get() : nullptr;
  return v;
}

template <typename R>
ShotMajorView<R> DeviceSolver<R>::sm_view() {
  return ShotMajorView<R>{d_sm_src_.get(), d_sm_point_.get(), d_sm_shot_.get(), d_rec_sm_.get()};
}

template <typename R>
SceneView<double> DeviceSolver<R>::view64(bool candidate) {
  SceneView<double> s{};
  s.n_slots = n_slots_;
  s.n_cameras = n_cam_;
  s.rig = nullptr;  // the cost kernels evaluate residuals only
  if (candidate) {
    s.geom = d_geomc_.get();
    s.cam_params = d_camc_.get();
  } else if constexpr (kMixed) {
    s.geom = d_geom64_.get();
    s.cam_params = d_cam64_.get();
  } else {
    s.geom = reinterpret_cast<const ShotGeom<double>*>(d_geom_.get());
    s.cam_params = reinterpret_cast<const double*>(d_cam_.get());
  }
  if constexpr (kMixed) s.obs = d_obs64_.get();
  else s.obs = reinterpret_cast<const ObsPack<double>*>(d_obs_.get());
  s.cam_model = d_cam_model_.get();
  s.points = candidate ? d_Xc_.get() : d_X_.get();
  s.obs_point = d_obs_point_.get();
  return s;
}

// ---------------------------------------------------------------------------
template <typename R>
struct CostLaunch {
  SceneView<double> s;
  const R* w;
  int loss;
  double a;
  double* resid;
  double* out;
  template <int M, int NR, int CMAX, bool RIG>
  void run() {
    const float* wf = nullptr;
    const double* wd = nullptr;
    if constexpr (sizeof(R) == 4) wf = reinterpret_cast<const float*>(w);
    else wd = reinterpret_cast<const double*>(w);
    cost_kernel<M, NR, CMAX, RIG><<<slot_grid(s.n_slots), 256>>>(s, wf, wd, loss, a, resid, out);
  }
};

template <typename R>
void DeviceSolver<R>::shard_reduce(double* h, int64_t n, int op) {
  if (!sharded() || n <= 0) return;
  if (opts_.shard.allreduce(opts_.shard.ctx, h, n, op) != 0)
    throw std::runtime_error("sharded solve: the all-reduce failed on rank " + std::to_string(opts_.shard.rank));
}

// rank 0's values on every rank (a sum to which the other ranks add zeros)
template <typename R>
void DeviceSolver<R>::shard_bcast(double* h, int64_t n) {
  if (!sharded() || n <= 0) return;
  if (opts_.shard.rank != 0) std::fill(h, h + n, 0.0);
  shard_reduce(h, n, 0);
}

// Sums a device buffer over the ranks (through host memory, in FP64).
template <typename R>
template <typename T>
void DeviceSolver<R>::shard_reduce_device(T* d, int64_t n) {
  if (!sharded() || n <= 0) return;
  std::vector<T> t(static_cast<size_t>(n));
  GB_CUDA(cudaMemcpy(t.data(), d, sizeof(T) * size_t(n), cudaMemcpyDeviceToHost));
  std::vector<double> h(t.begin(), t.end());
  shard_reduce(h.data(), n, 0);
  for (int64_t i = 0; i < n; ++i) t[size_t(i)] = T(h[size_t(i)]);
  GB_CUDA(cudaMemcpy(d, t.data(), sizeof(T) * size_t(n), cudaMemcpyHostToDevice));
}

// FP64 cost of the current (or candidate) state; projection part on the
// device, priors on the host.  In mixed mode a candidate's residuals are
// always kept (d_resid_cand_): the next linearization uses them if the
// candidate is accepted.
template <typename R>
double DeviceSolver<R>::cost_pass(bool candidate, bool store_residuals) {
  GB_CUDA(cudaMemset(d_scal_.get() + 6, 0, 2 * sizeof(double)));
  double* resid = nullptr;
  if (candidate && kMixed) resid = d_resid_cand_.get();
  else if (store_residuals) resid = d_resid_.get();
  CostLaunch<R> f{view64(candidate), d_weight_.get(), opts_.loss, opts_.loss_threshold, resid,
                  d_scal_.get() + 6};
  dispatch_config(kc_, f);
  ++launches_;
  if (!point_priors_.empty()) {
    point_prior_cost_kernel<<<elem_grid(int64_t(point_priors_.size())), 256>>>(
        int(point_priors_.size()), d_pp_.get(), d_pp_w_.get(), candidate ? d_Xc_.get() : d_X_.get(),
        d_pp_res_.get(), d_scal_.get() + 7);
    ++launches_;
  }
  GB_CUDA(cudaGetLastError());
  double c[2];
  GB_CUDA(cudaMemcpy(c, d_scal_.get() + 6, sizeof(c), cudaMemcpyDeviceToHost));
  shard_reduce(c, 2, 0);  // observations and point priors of every rank
  return c[0] + c[1] + prior_terms(candidate ? xc_cand_ : xc_, false);
}

template <typename R>
struct LinearizeLaunch {
  SolveView<R> v;
  uint64_t mask;
  template <int M, int NR, int CMAX, bool RIG>
  void run() {
    linearize_kernel<R, M, NR, CMAX, RIG><<<slot_grid(v.scene.n_slots), 256>>>(v, mask);
  }
};

template <typename R>
void DeviceSolver<R>::linearize() {
  coarse_stale_ = true;
  d_Vp_.zero();
  d_gp_.zero();
  d_gc_.zero();
  d_dc_.zero();
  LinearizeLaunch<R> f{view(), matrix_free_ ? uint64_t(0) : plane_mask_};
  dispatch_config(kc_, f);
  // the camera-side gradient and column norms, summed in shot-major order
  // (and, with stored records, the shot-major copy of the records)
  RecordPassLaunch<R> p{RecordPassLaunch<R>::kPermute, view(), sm_view()};
  p.plane_mask = matrix_free_ ? uint64_t(0) : plane_mask_;
  record_pass(p);
  launches_ += 2;
  shard_reduce_device(d_gc_.get(), int64_t(d_gc_.size()));
  shard_reduce_device(d_dc_.get(), int64_t(d_dc_.size()));
  if (!point_priors_.empty()) {
    point_prior_linearize_kernel<R><<<elem_grid(int64_t(point_priors_.size())), 256>>>(
        int(point_priors_.size()), d_pp_.get(), d_pp_w_.get(), d_X_.get(), d_point_free_.get(), d_Vp_.get(),
        d_gp_.get());
    ++launches_;
  }
  GB_CUDA(cudaGetLastError());
  prior_terms(xc_, true);
  d_pgrad_.upload(pgrad_);
  d_pdiag_.upload(pdiag_);
  std::vector<double> pdamp(cl_.n);
  for (int j = 0; j < cl_.n; ++j) pdamp[j] = pdiag_[j] + hdiag_[j];
  d_pdamp_.upload(pdamp);
  n_hblocks_ = int(hblocks_.size());
  if (n_hblocks_) {
    std::vector<int2> base;
    std::vector<double> val;
    for (const auto& kv : hblocks_) {
      base.push_back(make_int2(kv.first.first, kv.first.second));
      val.insert(val.end(), kv.second.begin(), kv.second.end());
    }
    d_hbase_.upload(base);
    d_hval_.upload(val);
  }
}

// Camera, rig-camera and GPS priors at camera-side state x (FP64, host).
// Returns their cost; with want_derivs also fills pgrad_ / pdiag_ (J^T r and
// diag(J^T J); every prior Jacobian is diagonal).
//   camera   DataPriorError<Camera>, LOG scale for focal and aspect ratio
//            (bundle_adjuster.cc:643-668, prior_error.h:54-93)
//   rig cam  DataPriorError<Pose> on all six parameters (:839-851)
//   GPS      DataPriorError<Pose, SimilarityPriorTransform> on TX TY TZ with
//            the camera bias applied to the prior (:806-838, bias.h:34-54)
template <typename R>
double DeviceSolver<R>::prior_terms(const std::vector<double>& x, bool want_derivs) {
  const Problem& P = *prob_;
  if (want_derivs) {
    std::fill(pgrad_.begin(), pgrad_.end(), 0.0);
    std::fill(pdiag_.begin(), pdiag_.end(), 0.0);
    std::fill(hdiag_.begin(), hdiag_.end(), 0.0);
    hblocks_.clear();
  }
  double cost = 0.0;
  for (int c = 0; c < n_cam_; ++c) {
    const CameraBlock& cb = P.cameras[c];
    const double w = prior_weight_cam_[c];
    for (int k = 0; k < cb.n; ++k) {
      const int j = cl_.cam_base + 16 * c + k;
      const double scale = 1.0 / std::max(cb.sigma[k], kEps);
      const double v = x[j];
      double r, J;
      if (cb.log_prior[k]) {
        r = scale * std::log(v / cb.prior[k]);
        J = scale / v;
      } else {
        r = scale * (v - cb.prior[k]);
        J = scale;
      }
      cost += 0.5 * w * r * r;
      if (want_derivs && cmask_[j]) {
        pgrad_[j] += w * J * r;
        pdiag_[j] += w * J * J;
      }
    }
  }
  for (int rc = 0; rc < n_rig_; ++rc) {
    const PoseBlock& b = P.rig_cameras[rc];
    if (!b.has_prior) continue;
    const double w = prior_weight_rig_[rc];
    for (int k = 0; k < 6; ++k) {
      const int j = cl_.rig_base + 8 * rc + k;
      const double scale = 1.0 / std::max(b.sigma[k], kEps);
      const double r = scale * (x[j] - b.prior[k]);
      cost += 0.5 * w * r * r;
      if (want_derivs && cmask_[j]) {
        pgrad_[j] += w * scale * r;
        pdiag_[j] += w * scale * scale;
      }
    }
  }
  for (size_t g = 0; g < gps_inst_.size(); ++g) {
    const int i = gps_inst_[g];
    const PoseBlock& b = P.instances[i];
    double prior[3] = {b.position_prior[0], b.position_prior[1], b.position_prior[2]};
    if (b.bias_camera >= 0) {
      const Bias& bs = P.biases[b.bias_camera];
      double rp[3];
      rotate_aa(bs.r, prior, rp);
      for (int k = 0; k < 3; ++k) prior[k] = bs.s * rp[k] + bs.t[k];
    }
    const double w = prior_weight_gps_[g];
    for (int k = 0; k < 3; ++k) {
      const int j = 8 * i + 3 + k;
      const double scale = 1.0 / std::max(b.position_sigma[k], kEps);
      const double r = scale * (x[j] - prior[k]);
      cost += 0.5 * w * r * r;
      if (want_derivs && cmask_[j]) {
        pgrad_[j] += w * scale * r;
        pdiag_[j] += w * scale * scale;
      }
    }
  }
  // host constraint terms: J^T r and J^T J over their free coordinates,
  // as 8 x 8 blocks of the coordinate groups they couple
  if (want_derivs) host_lin_.assign(size_t(n_host_terms()), HostTermLin());
  for (int q = 0; q < n_host_terms(); ++q) {
    HostTermLin tmp;
    HostTermLin& L = want_derivs ? host_lin_[size_t(q)] : tmp;
    host_term(q, x, L);
    cost += 0.5 * L.rho;
    if (!want_derivs) continue;
    for (int a = 0; a < L.ns; ++a) {
      if (L.coord[a] < 0) continue;
      double g = 0.0;
      for (int i = 0; i < L.m; ++i) g += L.J[i][a] * L.r[i];
      pgrad_[L.coord[a]] += g;
      for (int b = 0; b < L.ns; ++b) {
        if (L.coord[b] < 0) continue;
        double h = 0.0;
        for (int i = 0; i < L.m; ++i) h += L.J[i][a] * L.J[i][b];
        const int ga = L.coord[a] & ~7, gb = L.coord[b] & ~7;
        hblocks_[{ga, gb}][8 * (L.coord[a] - ga) + (L.coord[b] - gb)] += h;
        if (L.coord[a] == L.coord[b]) hdiag_[L.coord[a]] += h;
      }
    }
  }
  return cost;
}

template <typename R>
int DeviceSolver<R>::host_term_group(int q) const {
  const int no = int(prob_->orientation_terms.size());
  return q < no ? prob_->orientation_terms[q].kind : 4 + prob_->relative_terms[q - no].kind;
}

// Host term q at camera-side state x.  Orientation terms: slots 0..2 the
// instance rotation, 3..5 the rig camera rotation.  Relative terms: 12
// slots per shot (instance rotation, instance position, rig camera
// rotation, rig camera position).  Slots of coordinates shared by several
// shots map to the same coordinate and their derivatives add up.
template <typename R>
void DeviceSolver<R>::host_term(int q, const std::vector<double>& x, HostTermLin& L) const {
  const Problem& P = *prob_;
  const int no = int(P.orientation_terms.size());
  const double w = host_weight_[q];
  auto coord_of = [&](int j) { return cmask_[j] ? j : -1; };
  if (q < no) {
    const OrientationTerm& t = P.orientation_terms[q];
    const bool rig = t.rig_camera >= 0;
    const int ib = 8 * t.instance, rb = rig ? cl_.rig_base + 8 * t.rig_camera : -1;
    for (int k = 0; k < 3; ++k) {
      L.coord[k] = coord_of(ib + k);
      L.coord[3 + k] = rig ? coord_of(rb + k) : -1;
    }
    orient::D r[3];
    L.m = orient::residuals(t, &x[ib], rig ? &x[rb] : nullptr, r);
    L.ns = 6;
    for (int i = 0; i < L.m; ++i) L.raw[i] = r[i].v;
    L.rho = orient::cauchy_correct(L.m, r, w);
    for (int i = 0; i < L.m; ++i) {
      L.r[i] = r[i].v;
      for (int a = 0; a < 6; ++a) L.J[i][a] = r[i].d[a];
    }
    return;
  }
  const RelativeTerm& t = P.relative_terms[q - no];
  constexpr int N = HostTermLin::kMaxSlots;
  const double* pi[3] = {nullptr, nullptr, nullptr};
  const double* pc[3] = {nullptr, nullptr, nullptr};
  for (int k = 0; k < 3; ++k)
    for (int a = 0; a < 12; ++a) L.coord[12 * k + a] = -1;
  for (int k = 0; k < t.n_shots; ++k) {
    const int ib = 8 * t.instance[k];
    pi[k] = &x[ib];
    for (int a = 0; a < 6; ++a) L.coord[12 * k + a] = coord_of(ib + a);
    if (t.rig_camera[k] >= 0) {
      const int rb = cl_.rig_base + 8 * t.rig_camera[k];
      pc[k] = &x[rb];
      for (int a = 0; a < 6; ++a) L.coord[12 * k + 6 + a] = coord_of(rb + a);
    }
  }
  // the reconstruction scales or the GPS std multiplier: value[0] of their
  // blocks, slots 24 and 25
  double scales[2] = {1.0, 1.0};
  const int n_scales = t.kind == RelativeTerm::kRelativeMotion ? 2
                       : (t.kind == RelativeTerm::kGpsStd || t.kind == RelativeTerm::kStdDeviation) ? 1
                                                                                                     : 0;
  for (int k = 0; k < n_scales; ++k) {
    if (t.scale_block[k] < 0) continue;  // a GPS prior without a std multiplier: 1
    const int sb = cl_.rig_base + 8 * t.scale_block[k];
    scales[k] = x[sb];
    L.coord[24 + k] = coord_of(sb);
  }
  orient::Dual<N> r[7];
  if (t.kind == RelativeTerm::kGpsStd && t.bias_block[0] >= 0) {
    // optimised camera bias: rotation and translation in slots 6..11, the
    // scale in slot 25
    const int pb = cl_.rig_base + 8 * t.bias_block[0], sb = cl_.rig_base + 8 * t.bias_block[1];
    double bias[7];
    for (int k = 0; k < 6; ++k) {
      bias[k] = x[pb + k];
      L.coord[6 + k] = coord_of(pb + k);
    }
    bias[6] = x[sb];
    L.coord[25] = coord_of(sb);
    L.m = orient::relative_residuals<N>(t, pi, pc, r, scales, bias);
  } else if (t.kind == RelativeTerm::kGpsStd && t.bias_camera >= 0) {
    // the prior through the camera bias, as the diagonal GPS prior takes it
    RelativeTerm tb = t;
    const Bias& bs = P.biases[t.bias_camera];
    double rp[3];
    rotate_aa(bs.r, t.prior, rp);
    for (int k = 0; k < 3; ++k) tb.prior[k] = bs.s * rp[k] + bs.t[k];
    L.m = orient::relative_residuals<N>(tb, pi, pc, r, scales);
  } else {
    L.m = orient::relative_residuals<N>(t, pi, pc, r, scales);
  }
  L.ns = N;
  for (int i = 0; i < L.m; ++i) L.raw[i] = r[i].v;
  // relative rotation and motion: the relative-motion loss (for a motion
  // at its threshold times the term's robust multiplier); common position
  // Tukey(1); linear motion Cauchy(1); gauge, heatmap and adjusted GPS none
  static const int kLoss[8] = {-1, 5, 3, 0, 0, -1, 0, 0};
  const bool rel_loss = t.kind == RelativeTerm::kRelativeRotation || t.kind == RelativeTerm::kRelativeMotion;
  const int loss = rel_loss ? P.relative_loss : kLoss[t.kind];
  const double a = t.kind == RelativeTerm::kRelativeRotation ? P.relative_loss_threshold
                   : t.kind == RelativeTerm::kRelativeMotion ? t.loss_scale
                                                             : 1.0;
  L.rho = orient::loss_correct<N>(loss, a, L.m, r, w);
  for (int i = 0; i < L.m; ++i) {
    L.r[i] = r[i].v;
    for (int k = 0; k < N; ++k) L.J[i][k] = r[i].d[k];
  }
}

// Linear-model decrease of the priors for a camera-side step dx.
template <typename R>
double DeviceSolver<R>::prior_model_change(const std::vector<double>& x, const std::vector<double>& dx) {
  // every prior residual depends on one coordinate: r(x + d) ~ r + J d
  double total = 0.0;
  const Problem& P = *prob_;
  auto term = [&](double w, double r, double J, double d) { return -0.5 * w * (J * d) * (2.0 * r + J * d); };
  for (int c = 0; c < n_cam_; ++c) {
    const CameraBlock& cb = P.cameras[c];
    for (int k = 0; k < cb.n; ++k) {
      const int j = cl_.cam_base + 16 * c + k;
      if (!cmask_[j]) continue;
      const double scale = 1.0 / std::max(cb.sigma[k], kEps);
      const double v = x[j];
      const double r = cb.log_prior[k] ? scale * std::log(v / cb.prior[k]) : scale * (v - cb.prior[k]);
      const double J = cb.log_prior[k] ? scale / v : scale;
      total += term(prior_weight_cam_[c], r, J, dx[j]);
    }
  }
  for (int rc = 0; rc < n_rig_; ++rc) {
    const PoseBlock& b = P.rig_cameras[rc];
    if (!b.has_prior) continue;
    for (int k = 0; k < 6; ++k) {
      const int j = cl_.rig_base + 8 * rc + k;
      if (!cmask_[j]) continue;
      const double scale = 1.0 / std::max(b.sigma[k], kEps);
      total += term(prior_weight_rig_[rc], scale * (x[j] - b.prior[k]), scale, dx[j]);
    }
  }
  for (size_t g = 0; g < gps_inst_.size(); ++g) {
    const int i = gps_inst_[g];
    const PoseBlock& b = P.instances[i];
    double prior[3] = {b.position_prior[0], b.position_prior[1], b.position_prior[2]};
    if (b.bias_camera >= 0) {
      const Bias& bs = P.biases[b.bias_camera];
      double rp[3];
      rotate_aa(bs.r, prior, rp);
      for (int k = 0; k < 3; ++k) prior[k] = bs.s * rp[k] + bs.t[k];
    }
    for (int k = 0; k < 3; ++k) {
      const int j = 8 * i + 3 + k;
      if (!cmask_[j]) continue;
      const double scale = 1.0 / std::max(b.position_sigma[k], kEps);
      total += term(prior_weight_gps_[g], scale * (x[j] - prior[k]), scale, dx[j]);
    }
  }
  // x is the state the solver linearized at: the cached linearization
  const bool cached = &x == &xc_ && host_lin_.size() == size_t(n_host_terms());
  for (int q = 0; q < n_host_terms(); ++q) {
    HostTermLin tmp;
    if (!cached) host_term(q, x, tmp);
    const HostTermLin& L = cached ? host_lin_[size_t(q)] : tmp;
    for (int i = 0; i < L.m; ++i) {
      double jd = 0.0;
      for (int a = 0; a < L.ns; ++a)
        if (L.coord[a] >= 0) jd += L.J[i][a] * dx[L.coord[a]];
      total += -0.5 * jd * (2.0 * L.r[i] + jd);
    }
  }
  return total;
}

}  // namespace
}  // namespace gbba

#include "solver_loop.inc"
#include "batch_loop.inc"
