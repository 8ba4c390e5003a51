// Gauss-Newton blocks computed on the host (the orientation constraints):
// dense 8 x 8 blocks over padded camera-side coordinate groups (a rig
// instance at 8i, a rig camera at rig_base + 8r), stored for both (a, b) and
// (b, a).  Added to the implicit Schur product, the Schur-Jacobi
// preconditioner blocks and the explicit reduced camera system.
#pragma once

#include <cuda_runtime.h>

#include "solver_kernels.cuh"

namespace gbba {
namespace {

// y[row + r] += sum_c B[r][c] x[col + c], one thread per block row
template <typename A>
__global__ void host_block_spmv_kernel(int nb, const int2* __restrict__ base, const double* __restrict__ val,
                                       const A* __restrict__ x, A* __restrict__ y) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int b = t >> 3, r = t & 7;
  if (b >= nb) return;
  const int2 bs = base[b];
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < 8; ++c) s += val[64 * b + 8 * r + c] * double(x[bs.y + c]);
  if (s != 0.0) atomicAdd(y + bs.x + r, A(s));
}

// lower triangle of the dense system: each symmetric pair once
__global__ void host_block_dense_kernel(int nb, const int2* __restrict__ base, const double* __restrict__ val,
                                        const int* __restrict__ dmap, double* __restrict__ S, int lds) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int b = t >> 6, e = t & 63;
  if (b >= nb) return;
  const double v = val[64 * b + e];
  if (v == 0.0) return;
  const int dr = dmap[base[b].x + (e >> 3)], dc = dmap[base[b].y + (e & 7)];
  if (dr >= 0 && dc >= 0 && dr >= dc) atomicAdd(S + int64_t(dr) * lds + dc, v);
}

// diagonal blocks into the 6 x 6 preconditioner blocks (upper triangle)
template <typename R>
__global__ void host_block_precond_kernel(int nb, const int2* __restrict__ base, const double* __restrict__ val,
                                          CamLayout cl, R* __restrict__ tri_inst, R* __restrict__ tri_rig) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nb || base[b].x != base[b].y) return;
  const int g = base[b].x;
  R* tri = g < cl.rig_base ? tri_inst + 24 * int64_t(g / 8) : tri_rig + 24 * int64_t((g - cl.rig_base) / 8);
  int t = 0;
  for (int a = 0; a < 6; ++a)
    for (int c = a; c < 6; ++c) tri[t++] += R(val[64 * b + 8 * a + c]);
}

}  // namespace
}  // namespace gbba
