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
//   dense_slot_kernel           per observation: W_o = J_c^T J_p, T_o =
//                               W_o V_p^-1, J_c, and the right-hand side
//                               term T_o g_p
//   dense_pair_kernel           per pair (o1, o2) of observations of one
//                               point (o1 >= o2): -T_o1 W_o2^T, plus the U
//                               part J_c^T J_c on the pairs (o, o)
// The right-hand side is b = sum_o T_o g_p - g_c - g_prior (the reduced
// gradient of the Gauss-Newton system).
#pragma once

#include "solver_kernels.cuh"
#include "solver_shot_major.cuh"

namespace gbba {
namespace {

template <int CMAX, bool RIG>
constexpr int dense_width() {
  return 6 + CMAX + (RIG ? 6 : 0);
}

// Per-observation record of the dense assembly (FP64): W_o = J_c^T J_p
// [W][3], T_o = W_o V_p^-1 [W][3], J_c^T [W][3] (up to three residual rows).
template <int W>
constexpr int dense_record() {
  return 9 * W;
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
  GB_WARP_SLOT_LOOP(s.n_slots) {
    const int64_t i = base + lane;
    const int pt = s.obs_point[i];
    const bool valid = pt >= 0 && v.point_free[pt];
    double a[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    if (valid) {
      R rec[NP * VN];
      load_record<R, NP>(v.rec, v.stride, i, rec);
#pragma unroll
      for (int q = 0; q < NR; ++q) {
        const double j0 = double(rec[L::kPt + q * 3]), j1 = double(rec[L::kPt + q * 3 + 1]),
                     j2 = double(rec[L::kPt + q * 3 + 2]);
        a[0] += j0 * j0; a[1] += j0 * j1; a[2] += j0 * j2;
        a[3] += j1 * j1; a[4] += j1 * j2; a[5] += j2 * j2;
      }
    }
    // point-major slots: one sum per run of the same point
    const bool tail = warp_segment_sum<6, double>(valid ? pt : -1, a);
    if (tail && valid) {
#pragma unroll
      for (int k = 0; k < 6; ++k) atomicAdd(V64 + 8 * int64_t(pt) + k, a[k]);
    }
  }
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

// Walks the shot-major copy of the records, so that a warp's observations
// mostly share one shot and the right-hand side sums are reduced across the
// warp before the atomic adds.
template <typename R, int NR, int CMAX, bool RIG>
__global__ void __launch_bounds__(256) dense_slot_kernel(SolveView<R> v, ShotMajorView<R> sm,
                                                         const int* __restrict__ dmap,
                                                         const double* __restrict__ Vinv64, double* __restrict__ S,
                                                         int lds, int* __restrict__ didx, double* __restrict__ WT,
                                                         double* __restrict__ bd) {
  using L = RecordLayout<NR, CMAX, RIG>;
  constexpr int W = dense_width<CMAX, RIG>();
  constexpr int NP = planes_of<R>(L::kWidth);
  constexpr int VN = Vec16<R>::kN;
  const SceneView<R>& s = v.scene;
  GB_WARP_SLOT_LOOP(s.n_slots) {
    const int64_t i = base + lane;
    const int src = sm.src[i];
    const int pt = src >= 0 ? sm.point[i] : -1;
    const bool valid = pt >= 0;
    R rec[NP * VN];
#pragma unroll
    for (int k = 0; k < NP * VN; ++k) rec[k] = R(0);
    int d[W];
#pragma unroll
    for (int a = 0; a < W; ++a) d[a] = -1;
    int key = -1;
    if (valid) {
      load_record<R, NP>(sm.rec, v.stride, i, rec);
      const int shot = sm.shot[i];
      key = shot;
      int inst, cam, rig;
      shot_indices(s, shot, inst, cam, rig);
#pragma unroll
      for (int a = 0; a < 6; ++a) d[a] = dmap[8 * inst + a];
#pragma unroll
      for (int a = 0; a < CMAX; ++a) d[6 + a] = dmap[v.cl.cam_base + 16 * cam + a];
      if constexpr (RIG) {
#pragma unroll
        for (int a = 0; a < 6; ++a) d[6 + CMAX + a] = rig >= 0 ? dmap[v.cl.rig_base + 8 * rig + a] : -1;
      }
    }
    // W_o and T_o = W_o V_p^-1 (V^-1 is zero for fixed points); b += T_o g_p
    double vi[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    double g0 = 0.0, g1 = 0.0, g2 = 0.0;
    if (valid) {
#pragma unroll
      for (int k = 0; k < 6; ++k) vi[k] = Vinv64[8 * int64_t(pt) + k];
      g0 = double(v.gp[4 * int64_t(pt)]);
      g1 = double(v.gp[4 * int64_t(pt) + 1]);
      g2 = double(v.gp[4 * int64_t(pt) + 2]);
    }
    double tb[W];
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
      if (valid) {
        double* out = WT + int64_t(src) * dense_record<W>();
#pragma unroll
        for (int m = 0; m < 3; ++m) {
          out[a * 3 + m] = w[m];
          out[3 * W + a * 3 + m] = t[m];
        }
#pragma unroll
        for (int q = 0; q < 3; ++q) out[6 * W + a * 3 + q] = q < NR ? jc_at<R, NR, CMAX, RIG>(rec, q, a) : 0.0;
        didx[int64_t(src) * W + a] = d[a];
      }
      tb[a] = t[0] * g0 + t[1] * g1 + t[2] * g2;
    }
    const bool tail = warp_segment_sum<W, double>(key, tb);
    if (tail && valid) {
#pragma unroll
      for (int a = 0; a < W; ++a)
        if (d[a] >= 0 && tb[a] != 0.0) atomicAdd(bd + d[a], tb[a]);
    }
  }
}

// Pairs come sorted by their block key (the two shots and whether the pair
// is an observation with itself), so a run of pairs adds to one block of S.
// A warp takes kPairChunks x 32 consecutive pairs; lane l walks pairs l,
// l + 32, ... of them, keeping a running sum of row a of the block and
// flushing it (FP64 atomic adds) only when its key changes; at the end the
// lanes' sums are reduced over runs of equal keys across the warp.  The FP64
// work per pair is the 3 W^2 fused multiply-adds of -T_o1 W_o2^T (and, on
// the pairs (o, o), 3 W^2 more for J_c^T J_c).
constexpr int kPairChunks = 16;

template <int W>
__device__ __forceinline__ void pair_flush_row(int a, int2 pr, const int* __restrict__ didx, const double* acc,
                                               double* __restrict__ S, int lds) {
  const int ra = didx[int64_t(pr.x) * W + a];
  if (ra < 0) return;
  const bool same = pr.x == pr.y;
  const int* dj = didx + int64_t(pr.y) * W;
#pragma unroll
  for (int b = 0; b < W; ++b) {
    if (same && b > a) continue;
    const int cb = dj[b];
    if (cb < 0 || acc[b] == 0.0) continue;
    // the pair adds B at (o1, o2) and B^T at (o2, o1): one lower entry,
    // twice on the diagonal (a coordinate both observations share)
    s_lower_add(S, lds, ra, cb, (!same && ra == cb) ? -2.0 * acc[b] : -acc[b]);
  }
}

template <int W>
__global__ void __launch_bounds__(256) dense_pair_kernel(int64_t n_pairs, const int2* __restrict__ pairs,
                                                         const int* __restrict__ pair_key,
                                                         const int* __restrict__ didx,
                                                         const double* __restrict__ WT, double* __restrict__ S,
                                                         int lds) {
  const int lane = int(threadIdx.x & 31u);
  const int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int64_t p0 = warp * 32 * kPairChunks;
  if (p0 >= n_pairs) return;  // warp-uniform
  const int64_t p1 = min(n_pairs, p0 + int64_t(32 * kPairChunks));
#pragma unroll 1
  for (int a = 0; a < W; ++a) {
    double acc[W];
#pragma unroll
    for (int b = 0; b < W; ++b) acc[b] = 0.0;
    int cur = -1;
    int2 cur_pr = make_int2(0, 0);
    for (int64_t p = p0 + lane; p < p1; p += 32) {
      const int key = pair_key[p];
      const int2 pr = pairs[p];
      if (key != cur) {
        if (cur >= 0) {
          pair_flush_row<W>(a, cur_pr, didx, acc, S, lds);
#pragma unroll
          for (int b = 0; b < W; ++b) acc[b] = 0.0;
        }
        cur = key;
        cur_pr = pr;
      }
      const double* Ri = WT + int64_t(pr.x) * dense_record<W>();
      const double t0 = Ri[3 * W + 3 * a], t1 = Ri[3 * W + 3 * a + 1], t2 = Ri[3 * W + 3 * a + 2];
      const double* Wj = WT + int64_t(pr.y) * dense_record<W>();
#pragma unroll
      for (int b = 0; b < W; ++b) acc[b] = fma(t0, Wj[3 * b], fma(t1, Wj[3 * b + 1], fma(t2, Wj[3 * b + 2], acc[b])));
      if (pr.x == pr.y) {
        // U part of observation o: acc holds the negated contribution
        const double j0 = Ri[6 * W + 3 * a], j1 = Ri[6 * W + 3 * a + 1], j2 = Ri[6 * W + 3 * a + 2];
        const double* Jo = Ri + 6 * W;
#pragma unroll
        for (int b = 0; b < W; ++b)
          acc[b] = fma(-j0, Jo[3 * b], fma(-j1, Jo[3 * b + 1], fma(-j2, Jo[3 * b + 2], acc[b])));
      }
    }
    const bool tail = warp_segment_sum<W, double>(cur, acc);
    if (tail && cur >= 0) pair_flush_row<W>(a, cur_pr, didx, acc, S, lds);
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
