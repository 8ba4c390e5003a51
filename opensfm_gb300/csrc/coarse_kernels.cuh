// Device side of the two-level PCG preconditioner (coarse_space.h): probe
// vectors and the extraction of the Galerkin matrix E = Z^T A Z, its
// damping and symmetrization, and the coarse correction z += Z E^-1 Z^T r
// of every PCG iteration.  basis is [instance][6][7] (FP64), cluster the
// instance's cluster (-1: none); instance i owns entries 8 i .. 8 i + 5 of
// the camera-side vector.
#pragma once

#include <cstdint>

#include "solver_kernels.cuh"

namespace gbba {
namespace {

// v = sum over the clusters of colour k of their mode j (zero elsewhere).
template <typename R>
__global__ void coarse_probe_kernel(int n, int n_inst, const double* __restrict__ basis,
                                    const int* __restrict__ cluster, const int* __restrict__ colour, int k, int j,
                                    R* __restrict__ v) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  R val = R(0);
  if (t < 8 * n_inst) {
    const int s = t >> 3, a = t & 7;
    const int c = cluster[s];
    if (a < 6 && c >= 0 && colour[c] == k) val = R(basis[int64_t(s) * 42 + a * 7 + j]);
  }
  v[t] = val;
}

// The seven sums Z_c^T v over the instances of cluster c (one warp: each
// lane takes every 32nd instance, then a butterfly, so the order is fixed);
// every lane returns the totals.
template <typename R>
__device__ __forceinline__ void cluster_project(int c, const double* __restrict__ basis,
                                                const int* __restrict__ member_start, const int* __restrict__ members,
                                                const R* __restrict__ v, double (&out)[7]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int i = 0; i < 7; ++i) out[i] = 0.0;
  for (int q = member_start[c] + lane; q < member_start[c + 1]; q += 32) {
    const int s = members[q];
    const double* Z = basis + int64_t(s) * 42;
    double x[6];
#pragma unroll
    for (int a = 0; a < 6; ++a) x[a] = double(v[8 * s + a]);
#pragma unroll
    for (int a = 0; a < 6; ++a)
#pragma unroll
      for (int i = 0; i < 7; ++i) out[i] += Z[a * 7 + i] * x[a];
  }
#pragma unroll
  for (int i = 0; i < 7; ++i)
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) out[i] += __shfl_xor_sync(0xffffffffu, out[i], d);
}

// E[7 c + i][7 partner(c, k) + j] = (Z_c^T y)_i for the probe (k, j) (y = A v):
// one warp per cluster; each entry of E is written by one probe only.
template <typename R>
__global__ void coarse_extract_kernel(int n_clusters, int m, int n_colours, const double* __restrict__ basis,
                                      const int* __restrict__ member_start, const int* __restrict__ members,
                                      const int* __restrict__ partner, int k, int j, const R* __restrict__ y,
                                      double* __restrict__ E) {
  const int c1 = int((int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5);
  if (c1 >= n_clusters) return;  // whole warps
  const int c2 = partner[c1 * n_colours + k];
  if (c2 < 0) return;
  double out[7];
  cluster_project(c1, basis, member_start, members, y, out);
  const int lane = threadIdx.x & 31;
  if (lane < 7) {
    double val = out[0];
#pragma unroll
    for (int i = 1; i < 7; ++i)
      if (lane == i) val = out[i];
    E[int64_t(7 * c1 + lane) * m + 7 * c2 + j] = val;
  }
}

// W (lower triangle) = (E + E^T) / 2.
__global__ void coarse_symm_kernel(int m, const double* __restrict__ E, double* __restrict__ W) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= int64_t(m) * m) return;
  const int i = int(t / m), j = int(t - int64_t(i) * m);
  if (j > i) return;
  W[t] = 0.5 * (E[t] + E[int64_t(j) * m + i]);
}

// W += sum over the instances s of cluster c of Z_s^T diag(damp_s) Z_s, on
// the diagonal block of c (lower triangle); one thread per (c, i, j <= i).
template <typename R>
__global__ void coarse_damp_kernel(int n_clusters, int m, const double* __restrict__ basis,
                                   const int* __restrict__ member_start, const int* __restrict__ members,
                                   const R* __restrict__ damp, double* __restrict__ W) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 49 * n_clusters) return;
  const int c = t / 49, ij = t - 49 * c, i = ij / 7, j = ij - 7 * i;
  if (j > i) return;
  double acc = 0.0;
  for (int q = member_start[c]; q < member_start[c + 1]; ++q) {
    const int s = members[q];
    const double* Z = basis + int64_t(s) * 42;
#pragma unroll
    for (int a = 0; a < 6; ++a) acc += Z[a * 7 + i] * double(damp[8 * s + a]) * Z[a * 7 + j];
  }
  W[int64_t(7 * c + i) * m + 7 * c + j] += acc;
}

// A mode with no energy (all its coordinates locked) gets a unit diagonal
// and no coupling, so that W stays positive definite.
__global__ void coarse_unit_kernel(int m, double* __restrict__ W) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  if (W[int64_t(i) * m + i] > 0.0) return;
  for (int j = 0; j < i; ++j) W[int64_t(i) * m + j] = 0.0;
  for (int r = i + 1; r < m; ++r) W[int64_t(r) * m + i] = 0.0;
  W[int64_t(i) * m + i] = 1.0;
}

// w = Z^T r, one warp per cluster.
template <typename R>
__global__ void coarse_restrict_kernel(int n_clusters, const double* __restrict__ basis,
                                       const int* __restrict__ member_start, const int* __restrict__ members,
                                       const R* __restrict__ r, double* __restrict__ w) {
  const int c = int((int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5);
  if (c >= n_clusters) return;  // whole warps
  double out[7];
  cluster_project(c, basis, member_start, members, r, out);
  const int lane = threadIdx.x & 31;
  if (lane < 7) {
    double val = out[0];
#pragma unroll
    for (int i = 1; i < 7; ++i)
      if (lane == i) val = out[i];
    w[7 * c + lane] = val;
  }
}

// u = inv w for the m x m FP32 matrix inv (leading dimension ld, a multiple
// of 4, zero columns past m): one warp per row, w staged in shared memory
// as FP32.
constexpr int kCoarseGemvBlock = 256;
__global__ void __launch_bounds__(kCoarseGemvBlock) coarse_gemv_kernel(int m, int ld, const float* __restrict__ inv,
                                                                       const double* __restrict__ w,
                                                                       double* __restrict__ u) {
  extern __shared__ __align__(16) float ws[];
  for (int j = threadIdx.x; j < ld; j += kCoarseGemvBlock) ws[j] = j < m ? float(w[j]) : 0.f;
  __syncthreads();
  const int row = blockIdx.x * (kCoarseGemvBlock / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= m) return;
  const float4* a = reinterpret_cast<const float4*>(inv + int64_t(row) * ld);
  const float4* x = reinterpret_cast<const float4*>(ws);
  float acc = 0.f;
  for (int q = lane; q < ld / 4; q += 32) {
    const float4 av = a[q], xv = x[q];
    acc += av.x * xv.x + av.y * xv.y + av.z * xv.z + av.w * xv.w;
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, d);
  if (lane == 0) u[row] = double(acc);
}

// z += Z u and rz += r . (Z u) (u = E^-1 Z^T r).
template <typename R>
__global__ void coarse_prolong_kernel(int n_inst, const double* __restrict__ basis, const int* __restrict__ cluster,
                                      const double* __restrict__ u, const R* __restrict__ r, R* __restrict__ z,
                                      double* __restrict__ rz) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  double acc = 0.0;
  if (t < 8 * n_inst) {
    const int s = t >> 3, a = t & 7;
    const int c = cluster[s];
    if (a < 6 && c >= 0) {
      const double* Z = basis + int64_t(s) * 42 + a * 7;
      const double* uc = u + 7 * c;
      double add = 0.0;
#pragma unroll
      for (int i = 0; i < 7; ++i) add += Z[i] * uc[i];
      z[t] += R(add);
      acc = double(r[t]) * add;
    }
  }
  block_sum_add<256>(acc, rz);
}

}  // namespace
}  // namespace gbba
