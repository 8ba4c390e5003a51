// Camera-side passes of the solver in shot-major order.
//
// Camera-side sums (gradient and column norms of the rig instances,
// intrinsics and rig cameras, the right-hand side and the Schur-Jacobi
// blocks of the reduced camera system, and the camera half of the implicit
// Schur product) accumulate many observations into few blocks: every
// observation of a shot adds into the same instance block, and usually all
// observations add into one intrinsics block.  Scattered per observation,
// those additions serialise on the same addresses.  These kernels instead
// read a second, shot-major copy of the records (sorted by rig instance,
// shot, point; written once per linearization by permute_records_kernel):
//   - each warp walks a contiguous run of slots, so its keys (instance,
//     camera, rig camera) change rarely;
//   - a warp sums its 32 lanes with shuffles and keeps a running per-key
//     total in registers (KeyCarry), flushed only when the key changes;
//   - at the end the warps of a block combine their remaining totals in
//     shared memory, so one block issues one atomic per value and key.
#pragma once

#include "solver_kernels.cuh"

namespace gbba {

constexpr int kShotMajorBlock = 256;
constexpr int kShotMajorWarps = kShotMajorBlock / 32;

// Shot-major views.
template <typename R>
struct ShotMajorView {
  const int* src;                  // [n_slots] point-major slot of each shot-major slot (-1: pad)
  const int* point;                // [n_slots] point index (-1: pad)
  const int* shot;                 // [n_slots]
  typename Vec16<R>::type* rec;    // [planes][n_slots] shot-major records
};

// Contiguous slot groups of 32 for the calling warp.
#define GB_WARP_CHUNK_LOOP(n_slots)                                                           \
  const int lane = int(threadIdx.x & 31u);                                                    \
  const int64_t warp_id = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;              \
  const int64_t n_warps = (int64_t(gridDim.x) * blockDim.x) >> 5;                             \
  const int64_t n_groups = (n_slots) >> 5;                                                    \
  const int64_t g_begin = warp_id * n_groups / n_warps;                                       \
  const int64_t g_end = (warp_id + 1) * n_groups / n_warps;                                   \
  for (int64_t base = g_begin * 32; base < g_end * 32; base += 32)

// Running per-key sum of K values held by a warp.  dest(key, k) gives the
// global address of value k of block `key`.  With CARRY false every warp
// iteration is flushed at once (for wide blocks whose running total would
// not fit in registers).
template <int K, typename R, bool CARRY>
struct KeyCarry {
  int key = -1;
  R v[CARRY ? K : 1];

  template <typename D>
  __device__ __forceinline__ void flush_lane0(int b, const R* x, D& dest) {
    if ((threadIdx.x & 31u) == 0) {
#pragma unroll
      for (int k = 0; k < K; ++k) red_add(dest(b, k), x[k]);
    }
  }

  // Adds every lane's x (lanes with lane_key < 0 add nothing).
  template <typename D>
  __device__ __forceinline__ void add(int lane_key, R (&x)[K], D& dest) {
    const int lead = __shfl_sync(kFullMask, lane_key, 0);
    if (__all_sync(kFullMask, lane_key == lead)) {
      if (lead < 0) return;
#pragma unroll
      for (int k = 0; k < K; ++k) {
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) x[k] += __shfl_xor_sync(kFullMask, x[k], d);
      }
      if constexpr (CARRY) {
        if (lead == key) {
#pragma unroll
          for (int k = 0; k < K; ++k) v[k] += x[k];
        } else {
          if (key >= 0) flush_lane0(key, v, dest);
          key = lead;
#pragma unroll
          for (int k = 0; k < K; ++k) v[k] = x[k];
        }
      } else {
        flush_lane0(lead, x, dest);
      }
      return;
    }
    // keys change inside the warp: segmented sums; the run ending at lane
    // 31 becomes the new carry (it usually continues in the next group)
    const bool tail = warp_segment_sum<K, R>(lane_key, x);
    const unsigned lane = threadIdx.x & 31u;
    if constexpr (CARRY) {
      if (key >= 0) flush_lane0(key, v, dest);
      if (tail && lane != 31u && lane_key >= 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) red_add(dest(lane_key, k), x[k]);
      }
      key = __shfl_sync(kFullMask, lane_key, 31);
#pragma unroll
      for (int k = 0; k < K; ++k) v[k] = __shfl_sync(kFullMask, x[k], 31);
    } else {
      if (tail && lane_key >= 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) red_add(dest(lane_key, k), x[k]);
      }
    }
  }

  // Combines the carries of the block's warps in shared memory and flushes
  // them: one atomic per value and distinct key.  Called by every thread.
  template <typename D>
  __device__ __forceinline__ void finish(D& dest, int* s_key, R* s_val) {
    if constexpr (CARRY) {
      const int w = int(threadIdx.x >> 5);
      if ((threadIdx.x & 31u) == 0) {
        s_key[w] = key;
#pragma unroll
        for (int k = 0; k < K; ++k) s_val[w * K + k] = v[k];
      }
      __syncthreads();
      for (int k = int(threadIdx.x); k < K; k += blockDim.x) {
        int cur = -1;
        R acc = R(0);
        for (int q = 0; q < kShotMajorWarps; ++q) {
          const int kq = s_key[q];
          if (kq < 0) continue;
          if (kq != cur) {
            if (cur >= 0) red_add(dest(cur, k), acc);
            cur = kq;
            acc = R(0);
          }
          acc += s_val[q * K + k];
        }
        if (cur >= 0) red_add(dest(cur, k), acc);
      }
      __syncthreads();
    }
  }
};

// Carry the intrinsics block in registers only while it stays small.
template <typename R, int K>
constexpr bool carry_fits() {
  return K * int(sizeof(R)) <= 256;
}

// Shared staging for KeyCarry::finish (the largest block of a kernel).
template <typename R, int K>
struct CarryStage {
  int key[kShotMajorWarps];
  R val[kShotMajorWarps * K];
};

// ---------------------------------------------------------------------------
// Copies the point-major records into shot-major order and accumulates the
// camera-side gradient J_c^T r and squared column norms of the linearization.
template <typename R, int NR, int CMAX, bool RIG, typename Src>
__global__ void __launch_bounds__(kShotMajorBlock) permute_records_kernel(SolveView<R> v, ShotMajorView<R> sm,
                                                                          Src recs, uint64_t plane_mask) {
  using L = RecordLayout<NR, CMAX, RIG>;
  constexpr int NP = planes_of<R>(L::kWidth);
  constexpr int VN = Vec16<R>::kN;
  // the gradient is summed in FP64 (near the optimum it is a small
  // difference of large sums); the column norms in the working precision
  const SceneView<R>& s = v.scene;
  double* gc = v.gc;
  R* dc = v.dc;
  const CamLayout cl = v.cl;
  auto g_inst = [gc](int b, int k) { return gc + 8 * b + k; };
  auto d_inst = [dc](int b, int k) { return dc + 8 * b + k; };
  auto g_cam = [gc, cl](int b, int k) { return gc + cl.cam_base + 16 * b + k; };
  auto d_cam = [dc, cl](int b, int k) { return dc + cl.cam_base + 16 * b + k; };
  auto g_rig = [gc, cl](int b, int k) { return gc + cl.rig_base + 8 * b + k; };
  auto d_rig = [dc, cl](int b, int k) { return dc + cl.rig_base + 8 * b + k; };
  KeyCarry<6, double, true> cg_inst;
  KeyCarry<6, R, true> cd_inst;
  KeyCarry<CMAX, double, carry_fits<double, CMAX>()> cg_cam;
  KeyCarry<CMAX, R, carry_fits<R, CMAX>()> cd_cam;
  KeyCarry<6, double, true> cg_rig;
  KeyCarry<6, R, true> cd_rig;
  GB_WARP_CHUNK_LOOP(s.n_slots) {
    const int64_t j = base + lane;
    const int src = sm.src[j];
    const bool valid = src >= 0;
    R rec[NP * VN];
    if (valid) {
      recs.point_major(v, src, rec);
    } else {
#pragma unroll
      for (int k = 0; k < NP * VN; ++k) rec[k] = R(0);
    }
#pragma unroll
    for (int p = 0; p < NP; ++p)
      if (plane_mask & (uint64_t(1) << p)) store_plane<R>(sm.rec + p * v.stride + j, rec + p * VN);
    int inst = 0, cam = 0, rig = -1;
    if (valid) shot_indices(s, sm.shot[j], inst, cam, rig);
    {
      double g6[6];
      R d6[6];
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        R gs = R(0), ds = R(0);
#pragma unroll
        for (int q = 0; q < NR; ++q) {
          const R jv = rec[L::kInst + q * 6 + k];
          gs += jv * rec[L::kR + q];
          ds += jv * jv;
        }
        g6[k] = double(gs);
        d6[k] = ds;
      }
      const int key = (valid && v.inst_free[inst]) ? inst : -1;
      cg_inst.add(key, g6, g_inst);
      cd_inst.add(key, d6, d_inst);
    }
    {
      const bool cvalid = valid && v.cam_free[cam];
      if (__any_sync(kFullMask, cvalid)) {
        double gcv[CMAX];
        R dcv[CMAX];
#pragma unroll
        for (int k = 0; k < CMAX; ++k) {
          R gs = R(0), ds = R(0);
#pragma unroll
          for (int q = 0; q < NR; ++q) {
            const R jv = rec[L::kCam + q * CMAX + k];
            gs += jv * rec[L::kR + q];
            ds += jv * jv;
          }
          gcv[k] = double(gs);
          dcv[k] = ds;
        }
        cg_cam.add(cvalid ? cam : -1, gcv, g_cam);
        cd_cam.add(cvalid ? cam : -1, dcv, d_cam);
      }
    }
    if constexpr (RIG) {
      const bool rvalid = valid && rig >= 0 && v.rig_free[rig];
      if (__any_sync(kFullMask, rvalid)) {
        double g6[6];
        R d6[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) {
          R gs = R(0), ds = R(0);
#pragma unroll
          for (int q = 0; q < NR; ++q) {
            const R jv = rec[L::kRig + q * 6 + k];
            gs += jv * rec[L::kR + q];
            ds += jv * jv;
          }
          g6[k] = double(gs);
          d6[k] = ds;
        }
        cg_rig.add(rvalid ? rig : -1, g6, g_rig);
        cd_rig.add(rvalid ? rig : -1, d6, d_rig);
      }
    }
  }
  constexpr int KS = CMAX > 6 ? CMAX : 6;
  __shared__ CarryStage<double, KS> sg;
  __shared__ CarryStage<R, KS> sd;
  cg_inst.finish(g_inst, sg.key, sg.val);
  cd_inst.finish(d_inst, sd.key, sd.val);
  cg_cam.finish(g_cam, sg.key, sg.val);
  cd_cam.finish(d_cam, sd.key, sd.val);
  if constexpr (RIG) {
    cg_rig.finish(g_rig, sg.key, sg.val);
    cd_rig.finish(d_rig, sd.key, sd.val);
  }
}

// ---------------------------------------------------------------------------
// Right-hand side sum_o J_c^T J_p V^-1 g_p and Schur-Jacobi blocks, shot-major.
template <typename R, int NR, int CMAX, bool RIG, typename Src>
__global__ void __launch_bounds__(kShotMajorBlock) schur_rhs_precond_sm_kernel(SolveView<R> v, ShotMajorView<R> sm,
                                                                               Src recs, double* __restrict__ rhs,
                                                                               PrecondView<R> pc) {
  using L = RecordLayout<NR, CMAX, RIG>;
  constexpr int NP = planes_of<R>(L::kWidth);
  constexpr int VN = Vec16<R>::kN;
  constexpr int T = TriSize<CMAX>::kN;
  // right-hand side summed in FP64 (it cancels against the gradient),
  // preconditioner blocks in the working precision
  const SceneView<R>& s = v.scene;
  const CamLayout cl = v.cl;
  auto b_inst = [rhs](int b, int k) { return rhs + 8 * b + k; };
  auto t_inst = [pc](int b, int k) { return pc.inst + 24 * int64_t(b) + k; };
  auto b_cam = [rhs, cl](int b, int k) { return rhs + cl.cam_base + 16 * b + k; };
  auto t_cam = [pc](int b, int k) { return pc.cam + int64_t(pc.cam_stride) * b + k; };
  auto b_rig = [rhs, cl](int b, int k) { return rhs + cl.rig_base + 8 * b + k; };
  auto t_rig = [pc](int b, int k) { return pc.rig + 24 * int64_t(b) + k; };
  KeyCarry<6, double, true> cb_inst;
  KeyCarry<21, R, carry_fits<R, 21>()> ct_inst;
  KeyCarry<CMAX, double, carry_fits<double, CMAX>()> cb_cam;
  KeyCarry<T, R, carry_fits<R, T>()> ct_cam;
  KeyCarry<6, double, true> cb_rig;
  KeyCarry<21, R, carry_fits<R, 21>()> ct_rig;
  GB_WARP_CHUNK_LOOP(s.n_slots) {
    const int64_t j = base + lane;
    const int pt = sm.point[j];
    const bool valid = pt >= 0;
    R rec[NP * VN];
    R e[NR], Vi[6];
    int inst = 0, cam = 0, rig = -1;
#pragma unroll
    for (int q = 0; q < NR; ++q) e[q] = R(0);
    if (valid) {
      recs.shot_major(v, j, sm.src[j], rec);
      shot_indices(s, sm.shot[j], inst, cam, rig);
#pragma unroll
      for (int k = 0; k < 6; ++k) Vi[k] = v.Vinv[8 * int64_t(pt) + k];
      R g[3] = {v.gp[4 * int64_t(pt)], v.gp[4 * int64_t(pt) + 1], v.gp[4 * int64_t(pt) + 2]};
      R q3[3];
      sym3_mul(Vi, g, q3);
#pragma unroll
      for (int q = 0; q < NR; ++q)
        e[q] = rec[L::kPt + q * 3] * q3[0] + rec[L::kPt + q * 3 + 1] * q3[1] + rec[L::kPt + q * 3 + 2] * q3[2];
    } else {
#pragma unroll
      for (int k = 0; k < NP * VN; ++k) rec[k] = R(0);
#pragma unroll
      for (int k = 0; k < 6; ++k) Vi[k] = R(0);
    }
    {
      // instance: rhs (6) + Schur-Jacobi block (21)
      double b6[6];
      R tri[21];
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        R t = R(0);
#pragma unroll
        for (int q = 0; q < NR; ++q) t += rec[L::kInst + q * 6 + k] * e[q];
        b6[k] = double(t);
      }
      schur_block<R, NR, 6>(rec + L::kInst, rec + L::kPt, Vi, tri);
      const int key = (valid && v.inst_free[inst]) ? inst : -1;
      cb_inst.add(key, b6, b_inst);
      ct_inst.add(key, tri, t_inst);
    }
    {
      const bool cvalid = valid && v.cam_free[cam];
      if (__any_sync(kFullMask, cvalid)) {
        double bc[CMAX];
        R tri[T];
#pragma unroll
        for (int k = 0; k < CMAX; ++k) {
          R t = R(0);
#pragma unroll
          for (int q = 0; q < NR; ++q) t += rec[L::kCam + q * CMAX + k] * e[q];
          bc[k] = double(t);
        }
        schur_block<R, NR, CMAX>(rec + L::kCam, rec + L::kPt, Vi, tri);
        cb_cam.add(cvalid ? cam : -1, bc, b_cam);
        ct_cam.add(cvalid ? cam : -1, tri, t_cam);
      }
    }
    if constexpr (RIG) {
      const bool rvalid = valid && rig >= 0 && v.rig_free[rig];
      if (__any_sync(kFullMask, rvalid)) {
        double b6[6];
        R tri[21];
#pragma unroll
        for (int k = 0; k < 6; ++k) {
          R t = R(0);
#pragma unroll
          for (int q = 0; q < NR; ++q) t += rec[L::kRig + q * 6 + k] * e[q];
          b6[k] = double(t);
        }
        schur_block<R, NR, 6>(rec + L::kRig, rec + L::kPt, Vi, tri);
        cb_rig.add(rvalid ? rig : -1, b6, b_rig);
        ct_rig.add(rvalid ? rig : -1, tri, t_rig);
      }
    }
  }
  constexpr int KB = CMAX > 6 ? CMAX : 6;
  constexpr int KT = T > 21 ? T : 21;
  __shared__ CarryStage<double, KB> sb;
  __shared__ CarryStage<R, KT> stt;
  cb_inst.finish(b_inst, sb.key, sb.val);
  ct_inst.finish(t_inst, stt.key, stt.val);
  cb_cam.finish(b_cam, sb.key, sb.val);
  ct_cam.finish(t_cam, stt.key, stt.val);
  if constexpr (RIG) {
    cb_rig.finish(b_rig, sb.key, sb.val);
    ct_rig.finish(t_rig, stt.key, stt.val);
  }
}

// ---------------------------------------------------------------------------
// Implicit Schur product, camera half, shot-major:
//   y_c += J_c^T (J_c x_c - J_p V^-1 zbuf_p).
// A is the arithmetic of the product (see schur_point_pass_kernel).
template <typename R, typename A, int NR, int CMAX, bool RIG, typename Src>
__global__ void __launch_bounds__(kShotMajorBlock) schur_camera_pass_sm_kernel(SolveView<R> v, ShotMajorView<R> sm,
                                                                               Src recs, const A* __restrict__ x,
                                                                               const A* __restrict__ zbuf,
                                                                               A* __restrict__ y) {
  using L = RecordLayout<NR, CMAX, RIG>;
  constexpr int NP = planes_of<R>(L::kWidth);
  constexpr int VN = Vec16<R>::kN;
  const SceneView<R>& s = v.scene;
  const CamLayout cl = v.cl;
  auto d_inst = [y](int b, int k) { return y + 8 * b + k; };
  auto d_cam = [y, cl](int b, int k) { return y + cl.cam_base + 16 * b + k; };
  auto d_rig = [y, cl](int b, int k) { return y + cl.rig_base + 8 * b + k; };
  if (v.any_active && *v.any_active == 0) return;  // uniform over the grid: no barrier is skipped by part of a block
  KeyCarry<6, A, true> c_inst;
  KeyCarry<CMAX, A, carry_fits<A, CMAX>()> c_cam;
  KeyCarry<6, A, true> c_rig;
  // Software pipeline (as in schur_point_pass_kernel): the next group's
  // point, shot and stored record are loaded one iteration ahead.
  // (batched solves load records only for active slots, not ahead)
  const bool prefetch = Src::kPrefetch && v.active == nullptr;
  int pt_n = -1, sh_n = 0;
  R rec_n[NP * VN];
  bool first = true;
  GB_WARP_CHUNK_LOOP(s.n_slots) {
    const int64_t j = base + lane;
    if (first) {
      pt_n = sm.point[j];
      sh_n = sm.shot[j];
      if (prefetch) recs.shot_major(v, j, 0, rec_n);
      first = false;
    }
    const int pt = pt_n;
    const int sh = sh_n;
    R rec_r[NP * VN];
    if (prefetch) {
#pragma unroll
      for (int k = 0; k < NP * VN; ++k) rec_r[k] = rec_n[k];
    }
    if (base + 32 < g_end * 32) {
      pt_n = sm.point[j + 32];
      sh_n = sm.shot[j + 32];
      if (prefetch) recs.shot_major(v, j + 32, 0, rec_n);
    }
    const bool valid = pt >= 0 && slot_active(v, pt);
    A rec[NP * VN];
    A e[NR];
    int inst = 0, cam = 0, rig = -1;
    if (valid) {
      if (!prefetch) recs.shot_major(v, j, sm.src[j], rec_r);
#pragma unroll
      for (int k = 0; k < NP * VN; ++k) rec[k] = A(rec_r[k]);
      shot_indices(s, sh, inst, cam, rig);
      CamGather<A, CMAX> g;
      gather_cam<A, CMAX, RIG>(x, v.cl, inst, cam, rig, g);
      apply_cam<A, NR, CMAX, RIG>(rec, g, e);
      A Vi[6], zb[3], z[3];
#pragma unroll
      for (int k = 0; k < 6; ++k) Vi[k] = A(v.Vinv[8 * int64_t(pt) + k]);
#pragma unroll
      for (int k = 0; k < 3; ++k) zb[k] = zbuf[4 * int64_t(pt) + k];
      sym3_mul(Vi, zb, z);
#pragma unroll
      for (int q = 0; q < NR; ++q)
        e[q] -= rec[L::kPt + q * 3] * z[0] + rec[L::kPt + q * 3 + 1] * z[1] + rec[L::kPt + q * 3 + 2] * z[2];
    } else {
#pragma unroll
      for (int k = 0; k < NP * VN; ++k) rec[k] = A(0);
#pragma unroll
      for (int q = 0; q < NR; ++q) e[q] = A(0);
    }
    {
      A a[6];
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        A t = A(0);
#pragma unroll
        for (int q = 0; q < NR; ++q) t += rec[L::kInst + q * 6 + k] * e[q];
        a[k] = t;
      }
      c_inst.add((valid && v.inst_free[inst]) ? inst : -1, a, d_inst);
    }
    {
      const bool cvalid = valid && v.cam_free[cam];
      if (__any_sync(kFullMask, cvalid)) {
        A c[CMAX];
#pragma unroll
        for (int k = 0; k < CMAX; ++k) {
          A t = A(0);
#pragma unroll
          for (int q = 0; q < NR; ++q) t += rec[L::kCam + q * CMAX + k] * e[q];
          c[k] = t;
        }
        c_cam.add(cvalid ? cam : -1, c, d_cam);
      }
    }
    if constexpr (RIG) {
      const bool rvalid = valid && rig >= 0 && v.rig_free[rig];
      if (__any_sync(kFullMask, rvalid)) {
        A a[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) {
          A t = A(0);
#pragma unroll
          for (int q = 0; q < NR; ++q) t += rec[L::kRig + q * 6 + k] * e[q];
          a[k] = t;
        }
        c_rig.add(rvalid ? rig : -1, a, d_rig);
      }
    }
  }
  constexpr int KS = CMAX > 6 ? CMAX : 6;
  __shared__ CarryStage<A, KS> st;
  c_inst.finish(d_inst, st.key, st.val);
  c_cam.finish(d_cam, st.key, st.val);
  if constexpr (RIG) c_rig.finish(d_rig, st.key, st.val);
}

}  // namespace gbba
