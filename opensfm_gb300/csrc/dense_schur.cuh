// Explicit reduced camera system for the dense linear solver.
//
// S = sum_o J_c^T J_c - sum_p W_p^T V_p^-1 W_p + diag(prior + damping) over
// the optimised camera-side coordinates, compressed to a dense index (dmap:
// padded camera-side index -> dense index, -1 for locked or padding
// coordinates).  This is the matrix Ceres' Schur eliminator forms for its
// DENSE_SCHUR and SPARSE_SCHUR solvers (bundle_adjuster.cc:1159-1190), and
// the operator the implicit Schur product of the PCG path applies.
//
// Only the lower triangle is accumulated (FP64 atomics): a contribution v
// to the symmetric pair (r, c), (c, r) is added once at (max, min).
//   dense_point_v_kernel        V_p = sum_o J_p^T J_p in FP64 (per observation)
//   dense_point_inverse_kernel  V_p + LM damping, inverted in FP64
//   dense_slot_kernel           per observation: U part J_c^T J_c, W_o =
//                               J_c^T J_p and T_o = W_o V_p^-1, and the
//                               right-hand side term T_o g_p
//   dense_pair_kernel           per pair (o1, o2) of observations of one
//                               point (o1 >= o2): -T_o1 W_o2^T
// The right-hand side is b = sum_o T_o g_p - g_c - g_prior (the reduced
// gradient of the Gauss-Newton system).
#pragma once

#include "solver_kernels.cuh"

namespace gbba {
namespace {

template <int CMAX, bool RIG>
constexpr int dense_width() {
  return 6 + CMAX + (RIG ? 6 : 0);
}

__device__ __forceinline__ void s_lower_add(double* S, int ld, int r, int c, double v) {
  if (r < c) {
    const int t = r;
    r = c;
    c = t;
  }
  atomicAdd(S + int64_t(r) * ld + c, v);
}

// Camera-side Jacobian entry (row q, column a) of a record: columns are the
// instance pose (6), the intrinsics (CMAX), then the rig camera pose (6).
template <typename R, int NR, int CMAX, bool RIG>
__device__ __forceinline__ double jc_at(const R* rec, int q, int a) {
  using L = RecordLayout<NR, CMAX, RIG>;
  if (a < 6) return double(rec[L::kInst + q * 6 + a]);
  if (a < 6 + CMAX) return double(rec[L::kCam + q * CMAX + a - 6]);
  return double(rec[L::kRig + q * 6 + a - 6 - CMAX]);
}

template <typename R, int NR, int CMAX, bool RIG>
__global__ void __launch_bounds__(256) dense_point_v_kernel(SolveView<R> v, double* __restrict__ V64) {
  using L = RecordLayout<NR, CMAX, RIG>;
  constexpr int NP = planes_of<R>(L::kWidth);
  constexpr int VN = Vec16<R>::kN;
  const SceneView<R>& s = v.scene;
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= s.n_slots) return;
  const int pt = s.obs_point[i];
  if (pt < 0 || !v.point_free[pt]) return;
  R rec[NP * VN];
  load_record<R, NP>(v.rec, v.stride, i, rec);
  double a[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
#pragma unroll
  for (int q = 0; q < NR; ++q) {
    const double j0 = double(rec[L::kPt + q * 3]), j1 = double(rec[L::kPt + q * 3 + 1]),
                 j2 = double(rec[L::kPt + q * 3 + 2]);
    a[0] += j0 * j0; a[1] += j0 * j1; a[2] += j0 * j2;
    a[3] += j1 * j1; a[4] += j1 * j2; a[5] += j2 * j2;
  }
#pragma unroll
  for (int k = 0; k < 6; ++k) atomicAdd(V64 + 8 * int64_t(pt) + k, a[k]);
}

// The LM damping of point_solve_kernel (same Jacobi scales), in FP64.
template <typename R>
__global__ void dense_point_inverse_kernel(int64_t n_points, const uint8_t* __restrict__ point_free,
                                           const double* __restrict__ V64, const R* __restrict__ pscale, double mu,
                                           double* __restrict__ Vinv64) {
  const int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (p >= n_points) return;
  double out[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  if (point_free[p]) {
    double a[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) a[k] = V64[8 * p + k];
    const int dg[3] = {0, 3, 5};
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const double d = a[dg[j]];
      const double sc = double(pscale[3 * p + j]);
      double c = sc * sc * d;
      c = c < 1e-6 ? 1e-6 : (c > 1e32 ? 1e32 : c);
      a[dg[j]] = d + c / (sc * sc) * mu;
    }
    if (!chol3_inverse(a, out)) {
#pragma unroll
      for (int k = 0; k < 6; ++k) out[k] = 0.0;
    }
  }
#pragma unroll
  for (int k = 0; k < 8; ++k) Vinv64[8 * p + k] = out[k];
}

// delta_p = V_p^-1 (-g_p - zbuf_p) with the FP64 inverses of the dense path.
template <typename R>
__global__ void dense_point_delta_kernel(int64_t n_points, const uint8_t* __restrict__ point_free,
                                         const double* __restrict__ Vinv64, const R* __restrict__ gp,
                                         const R* __restrict__ zbuf, R* __restrict__ dp) {
  const int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (p >= n_points) return;
  double d[3] = {0.0, 0.0, 0.0};
  if (point_free[p]) {
    double Vi[6], b[3];
#pragma unroll
    for (int k = 0; k < 6; ++k) Vi[k] = Vinv64[8 * p + k];
#pragma unroll
    for (int k = 0; k < 3; ++k) b[k] = -double(gp[4 * p + k]) - double(zbuf[4 * p + k]);
    sym3_mul(Vi, b, d);
  }
  dp[4 * p] = R(d[0]);
  dp[4 * p + 1] = R(d[1]);
  dp[4 * p + 2] = R(d[2]);
  dp[4 * p + 3] = R(0);
}

template <typename R, int NR, int CMAX, bool RIG>
__global__ void __launch_bounds__(128) dense_slot_kernel(SolveView<R> v, const int* __restrict__ dmap,
                                                         const double* __restrict__ Vinv64, double* __restrict__ S,
                                                         int lds, int* __restrict__ didx, double* __restrict__ WT,
                                                         double* __restrict__ bd) {
  using L = RecordLayout<NR, CMAX, RIG>;
  constexpr int W = dense_width<CMAX, RIG>();
  constexpr int NP = planes_of<R>(L::kWidth);
  constexpr int VN = Vec16<R>::kN;
  const SceneView<R>& s = v.scene;
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= s.n_slots) return;
  const int pt = s.obs_point[i];
  if (pt < 0) return;
  R rec[NP * VN];
  load_record<R, NP>(v.rec, v.stride, i, rec);
  int inst, cam, rig;
  shot_indices(s, shot_of(s, i), inst, cam, rig);
  int d[W];
#pragma unroll
  for (int a = 0; a < 6; ++a) d[a] = dmap[8 * inst + a];
#pragma unroll
  for (int a = 0; a < CMAX; ++a) d[6 + a] = dmap[v.cl.cam_base + 16 * cam + a];
  if constexpr (RIG) {
#pragma unroll
    for (int a = 0; a < 6; ++a) d[6 + CMAX + a] = rig >= 0 ? dmap[v.cl.rig_base + 8 * rig + a] : -1;
  }
  // U part
#pragma unroll
  for (int a = 0; a < W; ++a) {
    if (d[a] < 0) continue;
#pragma unroll
    for (int b = 0; b <= a; ++b) {
      if (d[b] < 0) continue;
      double u = 0.0;
#pragma unroll
      for (int q = 0; q < NR; ++q) u += jc_at<R, NR, CMAX, RIG>(rec, q, a) * jc_at<R, NR, CMAX, RIG>(rec, q, b);
      if (u != 0.0) s_lower_add(S, lds, d[a], d[b], u);
    }
  }
  // W_o and T_o = W_o V_p^-1 (V^-1 is zero for fixed points); b += T_o g_p
  double vi[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) vi[k] = Vinv64[8 * int64_t(pt) + k];
  const double g0 = double(v.gp[4 * int64_t(pt)]), g1 = double(v.gp[4 * int64_t(pt) + 1]),
               g2 = double(v.gp[4 * int64_t(pt) + 2]);
  double* out = WT + i * (6 * W);
  int* di = didx + i * W;
#pragma unroll
  for (int a = 0; a < W; ++a) {
    double w[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int q = 0; q < NR; ++q) {
      const double j = jc_at<R, NR, CMAX, RIG>(rec, q, a);
#pragma unroll
      for (int m = 0; m < 3; ++m) w[m] += j * double(rec[L::kPt + q * 3 + m]);
    }
    double t[3];
    sym3_mul(vi, w, t);
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      out[a * 3 + m] = w[m];
      out[3 * W + a * 3 + m] = t[m];
    }
    di[a] = d[a];
    if (d[a] >= 0) {
      const double tb = t[0] * g0 + t[1] * g1 + t[2] * g2;
      if (tb != 0.0) atomicAdd(bd + d[a], tb);
    }
  }
}

template <int W>
__global__ void __launch_bounds__(256) dense_pair_kernel(int64_t n_pairs, const int2* __restrict__ pairs,
                                                         const int* __restrict__ didx,
                                                         const double* __restrict__ WT, double* __restrict__ S,
                                                         int lds) {
  const int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (p >= n_pairs) return;
  const int2 pr = pairs[p];
  const bool same = pr.x == pr.y;
  const int* di = didx + int64_t(pr.x) * W;
  const int* dj = didx + int64_t(pr.y) * W;
  const double* Ti = WT + int64_t(pr.x) * (6 * W) + 3 * W;
  const double* Wj = WT + int64_t(pr.y) * (6 * W);
  for (int a = 0; a < W; ++a) {
    const int ra = di[a];
    if (ra < 0) continue;
    const double t0 = Ti[3 * a], t1 = Ti[3 * a + 1], t2 = Ti[3 * a + 2];
    if (t0 == 0.0 && t1 == 0.0 && t2 == 0.0) continue;
    const int bend = same ? a + 1 : W;
    for (int b = 0; b < bend; ++b) {
      const int cb = dj[b];
      if (cb < 0) continue;
      double val = -(t0 * Wj[3 * b] + t1 * Wj[3 * b + 1] + t2 * Wj[3 * b + 2]);
      // the pair adds B at (o1, o2) and B^T at (o2, o1): one lower entry,
      // twice on the diagonal (a coordinate both observations share)
      if (!same && ra == cb) val *= 2.0;
      if (val != 0.0) s_lower_add(S, lds, ra, cb, val);
    }
  }
}

// Prior curvature and LM damping on the diagonal.
template <typename R>
__global__ void dense_diag_kernel(int n, const int* __restrict__ dmap, const double* __restrict__ pdiag,
                                  const R* __restrict__ damp, double* __restrict__ S, int lds) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int d = dmap[j];
  if (d < 0) return;
  S[int64_t(d) * lds + d] += pdiag[j] + double(damp[j]);
}

// b = -g_c - g_prior on the dense coordinates (dense_slot_kernel adds the
// point terms).
__global__ void dense_rhs_init_kernel(int n, const int* __restrict__ dmap, const double* __restrict__ gc,
                                      const double* __restrict__ pgrad, double* __restrict__ bd) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int d = dmap[j];
  if (d >= 0) bd[d] = -gc[j] - pgrad[j];
}

template <typename R>
__global__ void dense_scatter_kernel(int n, const int* __restrict__ dmap, const double* __restrict__ xd,
                                     double* __restrict__ x64, R* __restrict__ x) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int d = dmap[j];
  const double v = d >= 0 && xd ? xd[d] : 0.0;
  x64[j] = v;
  x[j] = R(v);
}

}  // namespace
}  // namespace gbba
