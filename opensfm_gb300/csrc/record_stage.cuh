// The two record passes of every PCG iteration (the implicit Schur product)
// with their stored records staged through shared memory.
//
// Each warp walks 32-slot groups.  While it works on one group, the record
// planes of its next group are copied into shared memory by cp.async (16
// bytes per lane and plane, L1 bypassed); the copy lands in the warp's
// other buffer and is waited for (cp.async.wait_group, a wait on the
// thread's own copies) after the slot's gathers (shot geometry, camera-side
// x, the point's blocks) have gone out.  Registers then hold one record,
// not two.  Arithmetic, summation order and results are those of
// schur_point_pass_kernel and schur_camera_pass_sm_kernel: only where the
// record comes from changes.
//
// Where it pays (mixed precision, PCG iteration of the Schur product):
//   * 8- to 10-plane records (Brown, 9 intrinsics): the 500-shot street
//     problem's iteration went from 0.194 to 0.144 ms;
//   * the 7-plane perspective record: 0.164 vs 0.170 ms on the 2.2M-
//     observation aerial problem, but 0.970 vs 0.897 ms on the 14.7M-
//     observation one, so records of up to 7 planes keep the register
//     pipeline.
//
// Shared memory: two buffers x NP planes x 256 threads x 16 bytes per block
// (80 KB for a 10-plane record), dynamic; solver setup raises the kernels'
// dynamic shared-memory limit.
#pragma once

#include <cuda_runtime.h>

#include "solver_kernels.cuh"
#include "solver_shot_major.cuh"

namespace gbba {

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

constexpr int kStagedBlock = 256;

template <typename R, int NP>
constexpr int staged_smem_bytes() {
  return 2 * NP * kStagedBlock * 16;
}

// Records of 8 to 10 planes are staged (two buffers of at most 80 KB per
// block); narrower ones do better with the register pipeline on large
// problems, wider ones (16 intrinsics columns) would leave one block per SM.
template <typename R, int NR, int CMAX, bool RIG>
constexpr bool staged_record_fits() {
  return planes_of<R>(RecordLayout<NR, CMAX, RIG>::kWidth) >= 8 &&
         planes_of<R>(RecordLayout<NR, CMAX, RIG>::kWidth) <= 10;
}

// Resident blocks per SM the register budget aims at (128 registers a
// thread: no spills for the staged records).
template <typename R, typename A, int NR, int CMAX, bool RIG>
constexpr int staged_min_blocks() {
  return 2;
}

// This thread's slot of plane p in buffer b.
template <typename R, int NP>
__device__ __forceinline__ typename Vec16<R>::type* stage_slot(unsigned char* base, int b, int p) {
  return reinterpret_cast<typename Vec16<R>::type*>(base) + (b * NP + p) * kStagedBlock + threadIdx.x;
}

// Issues the copies of slot i's record planes into buffer b.
template <typename R, int NP>
__device__ __forceinline__ void stage_record(unsigned char* base, int b, const typename Vec16<R>::type* planes,
                                             int64_t stride, int64_t i) {
#pragma unroll
  for (int p = 0; p < NP; ++p) cp_async16(stage_slot<R, NP>(base, b, p), planes + p * stride + i);
  cp_async_commit();
}

// This thread's record from buffer b (after the copies have landed).
template <typename R, int NP>
__device__ __forceinline__ void read_staged(unsigned char* base, int b, R* rec) {
  constexpr int VN = Vec16<R>::kN;
#pragma unroll
  for (int p = 0; p < NP; ++p) {
    const typename Vec16<R>::type q = *stage_slot<R, NP>(base, b, p);
    const R* e = reinterpret_cast<const R*>(&q);
#pragma unroll
    for (int k = 0; k < VN; ++k) rec[p * VN + k] = e[k];
  }
}

// zbuf_p += J_p^T (J_c x_c), point-major (single problem, stored records).
template <typename R, typename A, int NR, int CMAX, bool RIG>
__global__ void __launch_bounds__(kStagedBlock, (staged_min_blocks<R, A, NR, CMAX, RIG>()))
    staged_point_pass_kernel(SolveView<R> v, const typename Vec16<R>::type* __restrict__ planes, int64_t stride,
                             const A* __restrict__ x, A* __restrict__ zbuf) {
  using L = RecordLayout<NR, CMAX, RIG>;
  constexpr int NP = planes_of<R>(L::kWidth);
  constexpr int VN = Vec16<R>::kN;
  extern __shared__ __align__(16) unsigned char staged_smem[];
  const SceneView<R>& s = v.scene;
  const int lane = int(threadIdx.x & 31u);
  const int64_t step = ((int64_t(gridDim.x) * blockDim.x) >> 5) * 32;
  int64_t base = ((int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5) * 32;
  int pt_n = -1, sh_n = 0;
  int buf = 0;
  if (base < s.n_slots) {
    pt_n = s.obs_point[base + lane];
    sh_n = s.obs[base + lane].shot;
    stage_record<R, NP>(staged_smem, 0, planes, stride, base + lane);
  }
  for (; base < s.n_slots; base += step) {
    const int pt = pt_n;
    const int sh = sh_n;
    const bool more = base + step < s.n_slots;
    if (more) {
      pt_n = s.obs_point[base + step + lane];
      sh_n = s.obs[base + step + lane].shot;
      stage_record<R, NP>(staged_smem, buf ^ 1, planes, stride, base + step + lane);
    }
    const bool valid = pt >= 0;
    // the gathers (shot geometry, camera-side x) go out before the wait on
    // the record copies: their latency overlaps the copies'
    int inst = 0, cam = 0, rig = -1;
    CamGather<A, CMAX> g;
    if (valid) {
      shot_indices(s, sh, inst, cam, rig);
      gather_cam<A, CMAX, RIG>(x, v.cl, inst, cam, rig, g);
    }
    if (more) cp_async_wait<1>();  // this group's copies have landed; the next group's may not have
    else cp_async_wait<0>();
    R rec_r[NP * VN];
    read_staged<R, NP>(staged_smem, buf, rec_r);
    buf ^= 1;
    A u[3] = {A(0), A(0), A(0)};
    if (valid) {
      A rec[NP * VN];
#pragma unroll
      for (int k = 0; k < NP * VN; ++k) rec[k] = A(rec_r[k]);
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

// y_c = sum J_c^T (J_c x - J_p V^-1 zbuf), shot-major (single problem,
// stored records).
template <typename R, typename A, int NR, int CMAX, bool RIG>
__global__ void __launch_bounds__(kStagedBlock, (staged_min_blocks<R, A, NR, CMAX, RIG>()))
    staged_camera_pass_kernel(SolveView<R> v, ShotMajorView<R> sm, int64_t stride, const A* __restrict__ x,
                              const A* __restrict__ zbuf, A* __restrict__ y) {
  using L = RecordLayout<NR, CMAX, RIG>;
  constexpr int NP = planes_of<R>(L::kWidth);
  constexpr int VN = Vec16<R>::kN;
  extern __shared__ __align__(16) unsigned char staged_smem[];
  const SceneView<R>& s = v.scene;
  const CamLayout cl = v.cl;
  auto d_inst = [y](int b, int k) { return y + 8 * b + k; };
  auto d_cam = [y, cl](int b, int k) { return y + cl.cam_base + 16 * b + k; };
  auto d_rig = [y, cl](int b, int k) { return y + cl.rig_base + 8 * b + k; };
  KeyCarry<6, A, true> c_inst;
  KeyCarry<CMAX, A, carry_fits<A, CMAX>()> c_cam;
  KeyCarry<6, A, true> c_rig;
  int pt_n = -1, sh_n = 0;
  int buf = 0;
  bool first = true;
  GB_WARP_CHUNK_LOOP(s.n_slots) {
    const int64_t j = base + lane;
    if (first) {
      pt_n = sm.point[j];
      sh_n = sm.shot[j];
      stage_record<R, NP>(staged_smem, 0, sm.rec, stride, j);
      first = false;
    }
    const int pt = pt_n;
    const int sh = sh_n;
    const bool more = base + 32 < g_end * 32;
    if (more) {
      pt_n = sm.point[j + 32];
      sh_n = sm.shot[j + 32];
      stage_record<R, NP>(staged_smem, buf ^ 1, sm.rec, stride, j + 32);
    }
    const bool valid = pt >= 0;
    // the gathers (shot geometry, camera-side x, the point's V^-1 and zbuf)
    // go out before the wait on the record copies: their latency overlaps
    // the copies'
    int inst = 0, cam = 0, rig = -1;
    CamGather<A, CMAX> g;
    A Vi[6], zb[3];
    if (valid) {
      shot_indices(s, sh, inst, cam, rig);
      gather_cam<A, CMAX, RIG>(x, v.cl, inst, cam, rig, g);
#pragma unroll
      for (int k = 0; k < 6; ++k) Vi[k] = A(v.Vinv[8 * int64_t(pt) + k]);
#pragma unroll
      for (int k = 0; k < 3; ++k) zb[k] = zbuf[4 * int64_t(pt) + k];
    }
    if (more) cp_async_wait<1>();
    else cp_async_wait<0>();
    R rec_r[NP * VN];
    read_staged<R, NP>(staged_smem, buf, rec_r);
    buf ^= 1;
    A rec[NP * VN];
    A e[NR];
    if (valid) {
#pragma unroll
      for (int k = 0; k < NP * VN; ++k) rec[k] = A(rec_r[k]);
      apply_cam<A, NR, CMAX, RIG>(rec, g, e);
      A z[3];
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
  cp_async_wait<0>();
  constexpr int KS = CMAX > 6 ? CMAX : 6;
  __shared__ CarryStage<A, KS> st;
  c_inst.finish(d_inst, st.key, st.val);
  c_cam.finish(d_cam, st.key, st.val);
  if constexpr (RIG) c_rig.finish(d_rig, st.key, st.val);
}

}  // namespace gbba
