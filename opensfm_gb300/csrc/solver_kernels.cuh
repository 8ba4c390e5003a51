// Device kernels of the Levenberg-Marquardt bundle-adjustment solver.
//
// Data layout.  Observations live in "slots" sorted by point (the point-major
// order), padded to a multiple of 32 with slots whose point index is -1.
// Each slot owns a residual/Jacobian record (planes of 16 bytes, see
// eval_kernels.cuh).  The unknowns are split as in Schur-complement BA
// (the elimination Ceres' SCHUR solvers perform for the reference,
// bundle_adjuster.cc:1159-1190):
//   point side   3 per point, eliminated through 3x3 blocks V_p;
//   camera side  rig instances (6), rig cameras (6) and intrinsics (C), laid
//                out as padded blocks -- instance i at [8i, 8i+6), rig camera
//                r at rig_base + 8r, camera k at cam_base + 16k -- so a block
//                update is one or two 16-byte vector reductions.
// Per-point sums (V_p = sum J_p^T J_p, g_p = sum J_p^T r, and the point
// halves of the Schur products) are warp-level segmented reductions over the
// point-major slots; each segment tail adds its sum to global memory.
// Camera-side sums run over a shot-major copy of the records
// (solver_shot_major.cuh).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "eval_kernels.cuh"

namespace gbba {

constexpr unsigned kFullMask = 0xffffffffu;

// Camera-side layout.
struct CamLayout {
  int n_inst, n_rig, n_cam;
  int rig_base, cam_base, n;  // n = total padded length
};

// Point index of a slot; padding slots hold -1.
// Segmented inclusive reduction of K values over runs of equal `key` in a
// warp; afterwards the last lane of every run holds the run's sum.
template <int K, typename T>
__device__ __forceinline__ bool warp_segment_sum(int key, T (&v)[K]) {
  const unsigned lane = threadIdx.x & 31u;
  const int prev = __shfl_up_sync(kFullMask, key, 1);
  const int next = __shfl_down_sync(kFullMask, key, 1);
  const bool head = lane == 0 || prev != key;
  const bool tail = lane == 31 || next != key;
  const unsigned heads = __ballot_sync(kFullMask, head);
  const unsigned below = heads & ((2u << lane) - 1u);
  const int start = 31 - __clz(below);
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const T up = __shfl_up_sync(kFullMask, v[k], d);
      if (int(lane) >= start + d) v[k] += up;
    }
  }
  return tail;
}

// Segmented sum followed by a broadcast of the run sum to every lane of the
// run (used when every observation of a point needs the point's total).
template <int K, typename T>
__device__ __forceinline__ void warp_segment_allreduce(int key, T (&v)[K]) {
  const unsigned lane = threadIdx.x & 31u;
  const int next = __shfl_down_sync(kFullMask, key, 1);
  const bool tail = lane == 31 || next != key;
  warp_segment_sum<K, T>(key, v);
  const unsigned tails = __ballot_sync(kFullMask, tail);
  const unsigned above = tails & ~((1u << lane) - 1u);
  const int end = __ffs(above) - 1;
#pragma unroll
  for (int k = 0; k < K; ++k) v[k] = __shfl_sync(kFullMask, v[k], end);
}

// Vector reductions into global memory.
__device__ __forceinline__ void red_add4(float* dst, float a, float b, float c, float d) {
  atomicAdd(reinterpret_cast<float4*>(dst), make_float4(a, b, c, d));
}
__device__ __forceinline__ void red_add4(double* dst, double a, double b, double c, double d) {
  atomicAdd(dst + 0, a);
  atomicAdd(dst + 1, b);
  atomicAdd(dst + 2, c);
  atomicAdd(dst + 3, d);
}
__device__ __forceinline__ void red_add(float* dst, float a) { atomicAdd(dst, a); }
__device__ __forceinline__ void red_add(double* dst, double a) { atomicAdd(dst, a); }

// Adds an 8-wide (6 used) block vector to a padded instance / rig block.
template <typename R>
__device__ __forceinline__ void red_block6(R* dst, const R* v) {
  red_add4(dst, v[0], v[1], v[2], v[3]);
  red_add4(dst + 4, v[4], v[5], R(0), R(0));
}

// Record access helpers.
template <typename R, int NP>
__device__ __forceinline__ void load_record(const typename Vec16<R>::type* planes, int64_t stride, int64_t i,
                                            R* rec) {
#pragma unroll
  for (int p = 0; p < NP; ++p) load_plane<R>(planes + p * stride + i, rec + p * Vec16<R>::kN);
}

// Robust-loss values rho(s), rho'(s), rho''(s) (Ceres LossFunction
// definitions; threshold a, b = a^2) scaled by the IRLS weight w
// (irls_solver.cc:68-91: rho = w * rho_loss, or w * s without a loss).
template <typename R>
__device__ __forceinline__ void robust_rho(int loss, R a, R w, R s, R& rho0, R& rho1, R& rho2) {
  const R b = a * a;
  switch (loss) {
    case 1:  // Huber
      if (s > b) {
        const R r = sqrt(s);
        rho0 = R(2) * a * r - b;
        rho1 = a / r;
        rho2 = -rho1 / (R(2) * s);
      } else {
        rho0 = s; rho1 = R(1); rho2 = R(0);
      }
      break;
    case 2: {  // SoftLOne
      const R sum = R(1) + s / b;
      const R tmp = sqrt(sum);
      rho0 = R(2) * b * (tmp - R(1));
      rho1 = R(1) / tmp;
      rho2 = -(R(0.5) / b) * rho1 / sum;
      break;
    }
    case 3: {  // Cauchy
      const R sum = R(1) + s / b;
      const R inv = R(1) / sum;
      rho0 = b * log(sum);
      rho1 = inv;
      rho2 = -inv * inv / b;
      break;
    }
    case 4: {  // Arctan
      const R inv = R(1) / (a * a + s * s);
      rho0 = a * atan2(s, a);
      rho1 = a * a * inv;
      rho2 = R(-2) * s * b * inv * inv;
      break;
    }
    default:
      rho0 = s; rho1 = R(1); rho2 = R(0);
  }
  rho0 *= w;
  rho1 *= w;
  rho2 *= w;
}

// Applies the robust-loss correction to a residual block (Triggs et al.,
// "Bundle Adjustment -- A Modern Synthesis", sec. 4.3; the form Ceres'
// Corrector uses): with s = |r|^2,
//   alpha = 1 - sqrt(1 + 2 s rho''/rho')  (0 when s = 0 or rho'' <= 0),
//   r <- sqrt(rho') / (1 - alpha) r,
//   J <- sqrt(rho') (I - alpha/s r r^T) J.
template <typename R, int NR, int WB>
__device__ __forceinline__ void correct_block(R* blk, const R* r, R alpha_s, R sq1) {
#pragma unroll
  for (int c = 0; c < WB; ++c) {
    R rj = R(0);
#pragma unroll
    for (int i = 0; i < NR; ++i) rj += r[i] * blk[i * WB + c];
#pragma unroll
    for (int i = 0; i < NR; ++i) blk[i * WB + c] = sq1 * (blk[i * WB + c] - alpha_s * r[i] * rj);
  }
}

// Returns rho(s) (weighted) of the uncorrected residual.
template <typename R, int NR, int CMAX, bool RIG>
__device__ __forceinline__ R robust_correct(int loss, R a, R w, R* rec) {
  using L = RecordLayout<NR, CMAX, RIG>;
  R s = R(0);
#pragma unroll
  for (int i = 0; i < NR; ++i) s += rec[L::kR + i] * rec[L::kR + i];
  R rho0, rho1, rho2;
  robust_rho<R>(loss, a, w, s, rho0, rho1, rho2);
  const R sq1 = sqrt(rho1);
  R rscale = sq1, alpha_s = R(0);
  if (s > R(0) && rho2 > R(0)) {
    const R D = R(1) + R(2) * s * rho2 / rho1;
    const R alpha = R(1) - sqrt(D);
    rscale = sq1 / (R(1) - alpha);
    alpha_s = alpha / s;
  }
  R r[NR];
#pragma unroll
  for (int i = 0; i < NR; ++i) r[i] = rec[L::kR + i];
  correct_block<R, NR, 3>(rec + L::kPt, r, alpha_s, sq1);
  correct_block<R, NR, 6>(rec + L::kInst, r, alpha_s, sq1);
  correct_block<R, NR, CMAX>(rec + L::kCam, r, alpha_s, sq1);
  if constexpr (RIG) correct_block<R, NR, 6>(rec + L::kRig, r, alpha_s, sq1);
#pragma unroll
  for (int i = 0; i < NR; ++i) rec[L::kR + i] *= rscale;
  return rho0;
}

}  // namespace gbba

namespace gbba {

// Everything the slot kernels of one LM iteration read or write.
template <typename R>
struct SolveView {
  SceneView<R> scene;
  typename Vec16<R>::type* rec;  // record planes (written by linearize)
  int64_t stride;                // plane stride (= n_slots)
  const R* weight;               // [n_slots] IRLS weights
  int loss;
  R loss_a;
  CamLayout cl;
  const uint8_t* inst_free;      // [n_inst] any parameter optimised
  const uint8_t* cam_free;       // [n_cam]
  const uint8_t* rig_free;       // [n_rig]
  const uint8_t* point_free;     // [n_points]
  R* Vp;                         // [n_points][8] xx xy xz yy yz zz
  R* gp;                         // [n_points][4]
  R* Vinv;                       // [n_points][8]
  double* gc;                    // [cl.n] camera-side gradient J^T r (FP64 sums)
  R* dc;                         // [cl.n] camera-side squared column norms
  const double* resid64;         // [n_slots][4] FP64 residuals of the current state, or null
  // batched solves: the problem of every point and whether each problem's
  // linear solve is still running (the Schur products skip the others); null
  // for a single problem
  const int* point_pid;
  const int* active;
  const int* any_active;  // number of problems still active (0: nothing to do)
};

template <typename R>
__device__ __forceinline__ bool slot_active(const SolveView<R>& v, int pt) {
  return v.active == nullptr || v.active[v.point_pid[pt]] != 0;
}

template <typename R>
__device__ __forceinline__ int shot_of(const SceneView<R>& s, int64_t i) {
  return s.obs[i].shot;
}

// Gathers of the camera-side unknowns of one observation.
template <typename R, int CMAX>
struct CamGather {
  R xi[6], xc[CMAX], xr[6];
};

template <typename R, int CMAX, bool RIG>
__device__ __forceinline__ void gather_cam(const R* x, const CamLayout& cl, int inst, int cam, int rig,
                                           CamGather<R, CMAX>& g) {
  const R* pi = x + 8 * inst;
#pragma unroll
  for (int k = 0; k < 6; ++k) g.xi[k] = pi[k];
  const R* pc = x + cl.cam_base + 16 * cam;
#pragma unroll
  for (int k = 0; k < CMAX; ++k) g.xc[k] = pc[k];
  if constexpr (RIG) {
    if (rig >= 0) {
      const R* pr = x + cl.rig_base + 8 * rig;
#pragma unroll
      for (int k = 0; k < 6; ++k) g.xr[k] = pr[k];
    } else {
#pragma unroll
      for (int k = 0; k < 6; ++k) g.xr[k] = R(0);
    }
  }
}

// t = J_c x_c for every residual row.
template <typename R, int NR, int CMAX, bool RIG>
__device__ __forceinline__ void apply_cam(const R* rec, const CamGather<R, CMAX>& g, R* t) {
  using L = RecordLayout<NR, CMAX, RIG>;
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    R s = R(0);
#pragma unroll
    for (int k = 0; k < 6; ++k) s += rec[L::kInst + i * 6 + k] * g.xi[k];
#pragma unroll
    for (int k = 0; k < CMAX; ++k) s += rec[L::kCam + i * CMAX + k] * g.xc[k];
    if constexpr (RIG) {
#pragma unroll
      for (int k = 0; k < 6; ++k) s += rec[L::kRig + i * 6 + k] * g.xr[k];
    }
    t[i] = s;
  }
}

// Shot indices of a slot (valid slots only).
template <typename R>
__device__ __forceinline__ void shot_indices(const SceneView<R>& s, int sh, int& inst, int& cam, int& rig) {
  const ShotGeom<R>* g = s.geom + sh;
  inst = int(g->inst);
  cam = int(g->cam);
  rig = int(g->rig);
}

// Iterates the slots warp by warp so that every lane of a warp is active in
// each iteration (segmented reductions need full warps).
#define GB_WARP_SLOT_LOOP(n_slots)                                                   \
  const int lane = int(threadIdx.x & 31u);                                           \
  const int64_t warp0 = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;       \
  const int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;                     \
  for (int64_t base = warp0 * 32; base < (n_slots); base += nwarps * 32)

// ---------------------------------------------------------------------------
// Linearization: records (with robust correction) and point blocks.
template <typename R, int M, int NR, int CMAX, bool RIG>
__global__ void __launch_bounds__(256) linearize_kernel(SolveView<R> v, uint64_t plane_mask) {
  using L = RecordLayout<NR, CMAX, RIG>;
  constexpr int NP = planes_of<R>(L::kWidth);
  constexpr int VN = Vec16<R>::kN;
  __shared__ R s_cam[kSharedCameras * kMaxCameraParams];
  __shared__ int s_model[kSharedCameras];
  const int* models;
  const R* cams = stage_cameras(v.scene, s_cam, s_model, models);
  const SceneView<R>& s = v.scene;
  GB_WARP_SLOT_LOOP(s.n_slots) {
    const int64_t i = base + lane;
    const int pt = s.obs_point[i];
    const bool valid = pt >= 0;
    R rec[NP * VN];
#pragma unroll
    for (int k = 0; k < NP * VN; ++k) rec[k] = R(0);
    if (valid) {
      ObsPack<R> ob;
      ldg_copy(s.obs + i, ob);
      ObsInputs<R> in;
      load_inputs<R, M>(s, ob, pt, cams, models, in);
      eval_observation<R, M, NR, CMAX, RIG, true, true>(in, rec);
      if (v.resid64) {
        // mixed precision: the residual itself comes from the FP64 cost pass
        // of the same state (the FP32 one carries ~1e-4 sigma of rounding
        // at normalized-coordinate magnitudes); the Jacobian stays FP32
#pragma unroll
        for (int q = 0; q < NR; ++q) rec[L::kR + q] = R(v.resid64[4 * i + q]);
      }
      robust_correct<R, NR, CMAX, RIG>(v.loss, v.loss_a, v.weight[i], rec);
    }
#pragma unroll
    for (int p = 0; p < NP; ++p)
      if (plane_mask & (uint64_t(1) << p)) store_plane<R>(v.rec + p * v.stride + i, rec + p * VN);

    // point block: V = J_p^T J_p (upper triangle), g = J_p^T r
    R acc[9];
    {
      const R* J = rec + L::kPt;
      const R* r = rec + L::kR;
      R a00 = R(0), a01 = R(0), a02 = R(0), a11 = R(0), a12 = R(0), a22 = R(0), b0 = R(0), b1 = R(0), b2 = R(0);
#pragma unroll
      for (int q = 0; q < NR; ++q) {
        const R j0 = J[q * 3], j1 = J[q * 3 + 1], j2 = J[q * 3 + 2];
        a00 += j0 * j0; a01 += j0 * j1; a02 += j0 * j2;
        a11 += j1 * j1; a12 += j1 * j2; a22 += j2 * j2;
        b0 += j0 * r[q]; b1 += j1 * r[q]; b2 += j2 * r[q];
      }
      acc[0] = a00; acc[1] = a01; acc[2] = a02; acc[3] = a11; acc[4] = a12; acc[5] = a22;
      acc[6] = b0; acc[7] = b1; acc[8] = b2;
    }
    const bool tail = warp_segment_sum<9, R>(valid ? pt : -1, acc);
    if (tail && valid && v.point_free[pt]) {
      red_add4(v.Vp + 8 * int64_t(pt), acc[0], acc[1], acc[2], acc[3]);
      red_add4(v.Vp + 8 * int64_t(pt) + 4, acc[4], acc[5], R(0), R(0));
      red_add4(v.gp + 4 * int64_t(pt), acc[6], acc[7], acc[8], R(0));
    }
    // the camera-side gradient and column norms are summed in shot-major
    // order by permute_records_kernel
  }
}

// ---------------------------------------------------------------------------
// Point blocks: Jacobi scaling (first iteration), LM damping and inverse.
//   D_j = clamp(s_j^2 V_jj, min_diag, max_diag) / s_j^2 * mu,  mu = 1/radius
// (Levenberg-Marquardt diagonal of the column-scaled Jacobian, documented
// Ceres defaults min_lm_diagonal 1e-6, max_lm_diagonal 1e32, scale
// s_j = 1 / (1 + |J_j|)).
template <typename R>
__device__ __forceinline__ bool chol3_inverse(const R* a /*xx xy xz yy yz zz*/, R* inv) {
  const R l00s = a[0];
  if (!(l00s > R(0))) return false;
  const R l00 = sqrt(l00s);
  const R l10 = a[1] / l00, l20 = a[2] / l00;
  const R l11s = a[3] - l10 * l10;
  if (!(l11s > R(0))) return false;
  const R l11 = sqrt(l11s);
  const R l21 = (a[4] - l20 * l10) / l11;
  const R l22s = a[5] - l20 * l20 - l21 * l21;
  if (!(l22s > R(0))) return false;
  const R l22 = sqrt(l22s);
  // inverse of L
  const R i00 = R(1) / l00, i11 = R(1) / l11, i22 = R(1) / l22;
  const R i10 = -l10 * i00 * i11;
  const R i21 = -l21 * i11 * i22;
  const R i20 = -(l20 * i00 + l21 * i10) * i22;
  // A^-1 = L^-T L^-1
  inv[0] = i00 * i00 + i10 * i10 + i20 * i20;
  inv[1] = i10 * i11 + i20 * i21;
  inv[2] = i20 * i22;
  inv[3] = i11 * i11 + i21 * i21;
  inv[4] = i21 * i22;
  inv[5] = i22 * i22;
  return true;
}

template <typename R>
__global__ void point_solve_kernel(int64_t n_points, const uint8_t* __restrict__ point_free, const R* __restrict__ Vp,
                                   R* __restrict__ pscale, R* __restrict__ Vinv, double mu, int first,
                                   int* __restrict__ n_bad) {
  const int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (p >= n_points) return;
  R out[8] = {R(0), R(0), R(0), R(0), R(0), R(0), R(0), R(0)};
  if (point_free[p]) {
    R a[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) a[k] = Vp[8 * p + k];
    const int dg[3] = {0, 3, 5};
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const R d = a[dg[j]];
      if (first) pscale[3 * p + j] = R(1) / (R(1) + sqrt(d));
      const R s = pscale[3 * p + j];
      R c = s * s * d;
      c = c < R(1e-6) ? R(1e-6) : (c > R(1e32) ? R(1e32) : c);
      a[dg[j]] = d + R(double(c / (s * s)) * mu);
    }
    if (!chol3_inverse(a, out)) {
      atomicAdd(n_bad, 1);
#pragma unroll
      for (int k = 0; k < 6; ++k) out[k] = R(0);
    }
  }
#pragma unroll
  for (int k = 0; k < 8; ++k) Vinv[8 * p + k] = out[k];
}

template <typename R>
__device__ __forceinline__ void sym3_mul(const R* m, const R* x, R* y) {
  y[0] = m[0] * x[0] + m[1] * x[1] + m[2] * x[2];
  y[1] = m[1] * x[0] + m[3] * x[1] + m[4] * x[2];
  y[2] = m[2] * x[0] + m[4] * x[1] + m[5] * x[2];
}

// ---------------------------------------------------------------------------
// Reduced-camera-system right-hand side contribution sum_o J_c^T J_p V^-1 g_p
// and Schur-Jacobi preconditioner blocks
//   B = sum_o J_c^T J_c - (J_c^T J_p) V^-1 (J_p^T J_c)
// restricted to the diagonal blocks (instance 6x6 upper triangle = 21
// values, padded to 24; intrinsics C x C upper triangle; rig 21).
template <int C>
struct TriSize {
  static constexpr int kN = C * (C + 1) / 2;
  static constexpr int kPad = (kN + 3) / 4 * 4;
};

template <typename R, int NR, int W>
__device__ __forceinline__ void schur_block(const R* J /*NR x W*/, const R* Jp /*NR x 3*/, const R* Vi, R* tri) {
  R Wt[W][3];
#pragma unroll
  for (int a = 0; a < W; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      R s = R(0);
#pragma unroll
      for (int i = 0; i < NR; ++i) s += J[i * W + a] * Jp[i * 3 + b];
      Wt[a][b] = s;
    }
  R T[W][3];
#pragma unroll
  for (int a = 0; a < W; ++a) sym3_mul(Vi, Wt[a], T[a]);
  int t = 0;
#pragma unroll
  for (int a = 0; a < W; ++a)
#pragma unroll
    for (int c = a; c < W; ++c) {
      R s = R(0);
#pragma unroll
      for (int i = 0; i < NR; ++i) s += J[i * W + a] * J[i * W + c];
      s -= T[a][0] * Wt[c][0] + T[a][1] * Wt[c][1] + T[a][2] * Wt[c][2];
      tri[t++] = s;
    }
}

template <typename R>
struct PrecondView {
  R* inst;   // [n_inst][24]
  R* rig;    // [n_rig][24]
  R* cam;    // [n_cam][CP] (CP = TriSize<CMAX>::kPad)
  int cam_stride;
};

// The right-hand side and preconditioner blocks, and the camera half of the
// implicit Schur product, are summed in shot-major order
// (solver_shot_major.cuh).

// ---------------------------------------------------------------------------
// Implicit Schur product, first half: zbuf_p += J_p^T (J_c x_c) per point.
// A is the arithmetic of the product: the working precision R for the PCG
// iterations, FP64 (on the same records) for the residual of iterative
// refinement.
template <typename R, typename A, int NR, int CMAX, bool RIG, typename Src>
__global__ void __launch_bounds__(256) schur_point_pass_kernel(SolveView<R> v, Src recs, const A* __restrict__ x,
                                                               A* __restrict__ zbuf) {
  using L = RecordLayout<NR, CMAX, RIG>;
  constexpr int NP = planes_of<R>(L::kWidth);
  constexpr int VN = Vec16<R>::kN;
  const SceneView<R>& s = v.scene;
  if (v.any_active && *v.any_active == 0) return;
  const int lane = int(threadIdx.x & 31u);
  const int64_t step = ((int64_t(gridDim.x) * blockDim.x) >> 5) * 32;
  int64_t base = ((int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5) * 32;
  // Software pipeline: the point index, shot and (stored) record of the
  // warp's next slot group are loaded while the current one is processed,
  // so only the L2-resident gathers (shot geometry, x) stay on the
  // iteration's critical path.
  // Batched solves skip the records of converged problems: there the record
  // is loaded only for active slots, not ahead.
  const bool prefetch = Src::kPrefetch && v.active == nullptr;
  int pt_n = -1, sh_n = 0;
  R rec_n[NP * VN];
  if (base < s.n_slots) {
    pt_n = s.obs_point[base + lane];
    sh_n = s.obs[base + lane].shot;
    if (prefetch) recs.point_major(v, base + lane, rec_n);
  }
  for (; base < s.n_slots; base += step) {
    const int64_t i = base + lane;
    const int pt = pt_n;
    const int sh = sh_n;
    R rec_r[NP * VN];
    if (prefetch) {
#pragma unroll
      for (int k = 0; k < NP * VN; ++k) rec_r[k] = rec_n[k];
    }
    if (base + step < s.n_slots) {
      pt_n = s.obs_point[base + step + lane];
      sh_n = s.obs[base + step + lane].shot;
      if (prefetch) recs.point_major(v, base + step + lane, rec_n);
    }
    const bool valid = pt >= 0 && slot_active(v, pt);
    A u[3] = {A(0), A(0), A(0)};
    if (valid) {
      if (!prefetch) recs.point_major(v, i, rec_r);
      A rec[NP * VN];
#pragma unroll
      for (int k = 0; k < NP * VN; ++k) rec[k] = A(rec_r[k]);
      int inst, cam, rig;
      shot_indices(s, sh, inst, cam, rig);
      CamGather<A, CMAX> g;
      gather_cam<A, CMAX, RIG>(x, v.cl, inst, cam, rig, g);
      A t[NR];
      apply_cam<A, NR, CMAX, RIG>(rec, g, t);
#pragma unroll
      for (int q = 0; q < NR; ++q) {
        u[0] += rec[L::kPt + q * 3] * t[q];
        u[1] += rec[L::kPt + q * 3 + 1] * t[q];
        u[2] += rec[L::kPt + q * 3 + 2] * t[q];
      }
    }
    const bool tail = warp_segment_sum<3, A>(valid ? pt : -1, u);
    if (tail && valid && v.point_free[pt]) red_add4(zbuf + 4 * int64_t(pt), u[0], u[1], u[2], A(0));
  }
}

// delta_p = V^-1 (-g_p - zbuf_p) for free points.
template <typename R>
__global__ void point_delta_kernel(int64_t n_points, const uint8_t* __restrict__ point_free, const R* __restrict__ Vinv,
                                   const R* __restrict__ gp, const R* __restrict__ zbuf, R* __restrict__ dp) {
  const int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (p >= n_points) return;
  R d[3] = {R(0), R(0), R(0)};
  if (point_free[p]) {
    R Vi[6], b[3];
#pragma unroll
    for (int k = 0; k < 6; ++k) Vi[k] = Vinv[8 * p + k];
#pragma unroll
    for (int k = 0; k < 3; ++k) b[k] = -gp[4 * p + k] - zbuf[4 * p + k];
    sym3_mul(Vi, b, d);
  }
  dp[4 * p] = d[0];
  dp[4 * p + 1] = d[1];
  dp[4 * p + 2] = d[2];
  dp[4 * p + 3] = R(0);
}

// FP64 block-wide sum into *out.
template <int BLOCK>
__device__ __forceinline__ void block_sum_add(double v, double* out) {
  __shared__ double red[BLOCK / 32];
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(kFullMask, v, d);
  if ((threadIdx.x & 31u) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    v = threadIdx.x < BLOCK / 32 ? red[threadIdx.x] : 0.0;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(kFullMask, v, d);
    if (threadIdx.x == 0) atomicAdd(out, v);
  }
  __syncthreads();
}

// Linear-model decrease  sum_o 0.5 (|f_o|^2 - |f_o + J_o delta|^2)  (FP64).
template <typename R, int NR, int CMAX, bool RIG, typename Src>
__global__ void __launch_bounds__(256) model_change_kernel(SolveView<R> v, Src recs, const R* __restrict__ dc_step,
                                                           const R* __restrict__ dp, double* __restrict__ out) {
  using L = RecordLayout<NR, CMAX, RIG>;
  constexpr int NP = planes_of<R>(L::kWidth);
  constexpr int VN = Vec16<R>::kN;
  const SceneView<R>& s = v.scene;
  double acc = 0.0;
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < s.n_slots; i += stride) {
    const int pt = s.obs_point[i];
    if (pt < 0) continue;
    R rec[NP * VN];
    recs.point_major(v, i, rec);
    int inst, cam, rig;
    shot_indices(s, shot_of(s, i), inst, cam, rig);
    CamGather<R, CMAX> g;
    gather_cam<R, CMAX, RIG>(dc_step, v.cl, inst, cam, rig, g);
    R t[NR];
    apply_cam<R, NR, CMAX, RIG>(rec, g, t);
    const R d0 = dp[4 * int64_t(pt)], d1 = dp[4 * int64_t(pt) + 1], d2 = dp[4 * int64_t(pt) + 2];
#pragma unroll
    for (int q = 0; q < NR; ++q) {
      const double r = double(rec[L::kR + q]);
      const double jd = double(t[q] + rec[L::kPt + q * 3] * d0 + rec[L::kPt + q * 3 + 1] * d1 +
                               rec[L::kPt + q * 3 + 2] * d2);
      // |r|^2 - |r + jd|^2 = -jd (2 r + jd)
      acc += -0.5 * jd * (2.0 * r + jd);
    }
  }
  block_sum_add<256>(acc, out);
}

// ---------------------------------------------------------------------------
// FP64 cost of a state: sum_o rho_o(|r_o|^2) / 2 with the IRLS weights, and
// the raw scaled residuals (for the reweighting and reprojection errors).
template <int M, int NR, int CMAX, bool RIG>
__global__ void __launch_bounds__(256) cost_kernel(SceneView<double> s, const float* __restrict__ wf,
                                                   const double* __restrict__ wd, int loss, double loss_a,
                                                   double* __restrict__ resid /* [n_slots][4] */,
                                                   double* __restrict__ out) {
  using L = RecordLayout<NR, CMAX, RIG>;
  __shared__ double s_cam[kSharedCameras * kMaxCameraParams];
  __shared__ int s_model[kSharedCameras];
  const int* models;
  const double* cams = stage_cameras(s, s_cam, s_model, models);
  double acc = 0.0;
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < s.n_slots; i += stride) {
    const int pt = s.obs_point[i];
    if (pt < 0) continue;
    ObsPack<double> ob;
    ldg_copy(s.obs + i, ob);
    ObsInputs<double> in;
    load_inputs<double, M>(s, ob, pt, cams, models, in);
    double rec[L::kWidth];
    eval_observation<double, M, NR, CMAX, RIG, false, true>(in, rec);
    double sq = 0.0;
#pragma unroll
    for (int q = 0; q < NR; ++q) sq += rec[q] * rec[q];
    const double w = wd ? wd[i] : double(wf[i]);
    double r0, r1, r2;
    robust_rho<double>(loss, loss_a, w, sq, r0, r1, r2);
    acc += 0.5 * r0;
    if (resid) {
#pragma unroll
      for (int q = 0; q < NR; ++q) resid[4 * i + q] = rec[q];
    }
  }
  block_sum_add<256>(acc, out);
}

// Points of the candidate state: X' = X + delta_p (FP64 master copy), and
// the working-precision copy of a state.
template <typename R>
__global__ void point_update_kernel(int64_t n, const Point4* __restrict__ X, const R* __restrict__ dp,
                                    Point4* __restrict__ Xc) {
  const int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const Point4 a = X[p];
  Xc[p] = Point4{a.x + double(dp[4 * p]), a.y + double(dp[4 * p + 1]), a.z + double(dp[4 * p + 2]), 0.0};
}

static __global__ void point_store_kernel(int64_t n, const Point4* __restrict__ X, PointF2* __restrict__ out) {
  const int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const Point4 a = X[p];
  out[p] = make_point_store(a.x, a.y, a.z, static_cast<float*>(nullptr));
}

// ---------------------------------------------------------------------------
// IRLS mixture statistics per error group (one group per shot plus GCP2D,
// bundle_adjuster.cc:559-562, and DEPTH, :599-602; mixture_reweighting.cc:
// 10-109, irls_helpers.cc:220-277).
//   stats pass:   S_g += w r r^T (upper triangle), W_g += w, N_g += 1
//   weight pass:  p_in = exp(-r^T Sigma^-1 r / 2) / sqrt((2 pi)^k det),
//                 w = clamp(p_in / (p_in + K), 1e-10, 1),
//                 LL_g += log(p_in + K), out_g += (w < 0.5)
struct IrlsGroupParams {
  double inv[6];     // Sigma^-1 upper triangle (k = 2 uses 0, 1, 3; k = 1 uses 0)
  double norm;       // 1 / sqrt((2 pi)^k det)
  double K;
  int active;        // group is being reweighted in this EM iteration
  int dim;
};

__device__ __forceinline__ int irls_group(const SceneView<double>& s, int64_t i, const uint8_t* gcp, int n_shots) {
  // groups: shots, then GCP2D (n_shots), then DEPTH (n_shots + 1)
  return gcp[i] == kSlotProjection ? s.obs[i].shot : n_shots + int(gcp[i]) - 1;
}

static __global__ void irls_stats_kernel(SceneView<double> s, const uint8_t* __restrict__ gcp, int n_shots,
                                         const double* __restrict__ resid, const float* __restrict__ wf,
                                         const double* __restrict__ wd, const int* __restrict__ group_dim,
                                         double* __restrict__ stats /* [groups][8] */) {
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < s.n_slots; i += stride) {
    if (s.obs_point[i] < 0) continue;
    const int g = irls_group(s, i, gcp, n_shots);
    const int k = group_dim[g];
    const double w = wd ? wd[i] : double(wf[i]);
    const double r0 = resid[4 * i], r1 = resid[4 * i + 1], r2 = resid[4 * i + 2];
    double* st = stats + 8 * int64_t(g);
    atomicAdd(st + 0, w * r0 * r0);
    atomicAdd(st + 1, w * r0 * r1);
    atomicAdd(st + 3, w * r1 * r1);
    if (k == 3) {
      atomicAdd(st + 2, w * r0 * r2);
      atomicAdd(st + 4, w * r1 * r2);
      atomicAdd(st + 5, w * r2 * r2);
    }
    atomicAdd(st + 6, w);
  }
}

static __global__ void irls_weight_kernel(SceneView<double> s, const uint8_t* __restrict__ gcp, int n_shots,
                                          const double* __restrict__ resid, const IrlsGroupParams* __restrict__ gp,
                                          float* __restrict__ wf, double* __restrict__ wd,
                                          double* __restrict__ ll /* [groups][2] */) {
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < s.n_slots; i += stride) {
    if (s.obs_point[i] < 0) continue;
    const int g = irls_group(s, i, gcp, n_shots);
    const IrlsGroupParams P = gp[g];
    if (!P.active) continue;
    const double r0 = resid[4 * i], r1 = resid[4 * i + 1], r2 = resid[4 * i + 2];
    double m;
    if (P.dim == 3) {
      m = P.inv[0] * r0 * r0 + P.inv[3] * r1 * r1 + P.inv[5] * r2 * r2 +
          2.0 * (P.inv[1] * r0 * r1 + P.inv[2] * r0 * r2 + P.inv[4] * r1 * r2);
    } else if (P.dim == 1) {
      m = P.inv[0] * r0 * r0;
    } else {
      m = P.inv[0] * r0 * r0 + 2.0 * P.inv[1] * r0 * r1 + P.inv[3] * r1 * r1;
    }
    const double p_in = exp(-0.5 * m) * P.norm;
    double w = p_in / (p_in + P.K);
    w = w < 1e-10 ? 1e-10 : (w > 1.0 ? 1.0 : w);
    if (wd) wd[i] = w;
    if (wf) wf[i] = float(w);
    atomicAdd(ll + 2 * int64_t(g), log(p_in + P.K));
    if (w < 0.5) atomicAdd(ll + 2 * int64_t(g) + 1, 1.0);
  }
}

}  // namespace gbba
