// Dense SPD solver of the reduced camera system on GB300: a blocked
// left-looking Cholesky factorization with tensor-core block products, and
// FP64 conjugate gradients preconditioned by the factor.
//
// Factorization of the Jacobi-scaled FP32 matrix, tiles of 128 x 128, for
// every block column k:
//   update   A_ik -= sum_{j<k} L_ij L_kj^T   (i >= k; tensor cores, K = 128 k)
//   potrf    L_kk = chol(A_kk), Dinv_k = L_kk^-1   (one CTA, shared memory)
//   trsm     L_ik = A_ik Dinv_k^T               (i > k; tensor cores, K = 128)
// The block products use tcgen05.mma kind::tf32 with operands in shared
// memory (128-byte swizzled, K-major) and the FP32 accumulator in tensor
// memory.  Each FP32 operand is split into a TF32 high part and a TF32
// remainder; hi*hi + hi*lo + lo*hi restores FP32-level accuracy of every
// product ("3xTF32").  The solve is conjugate gradients in FP64 on the FP64
// matrix, preconditioned by the FP32 factor (flexible Polak-Ribiere form, as
// the FP32 triangular solves are not an exactly linear operator): one or two
// iterations when the scaled condition number times the FP32 unit roundoff
// is small, and still convergent where plain iterative refinement would
// stall (nearly singular gauge directions under small LM damping).  If the
// FP32 factorization meets a non-positive pivot, it is repeated with a
// growing diagonal shift; the shifted factor remains a valid preconditioner.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <vector>

#include "capi_util.h"
#include "dense_cholesky.h"

namespace gbba {
namespace {

constexpr int kTile = 128;                      // output tile rows = columns
constexpr int kKb = 32;                         // FP32 K values per stage: one 128-byte row
constexpr int kOpBytes = kTile * kKb * 4;       // one operand part per stage (16 KB)
constexpr int kStageBytes = 4 * kOpBytes;       // A hi, A lo, B hi, B lo
constexpr int kStages = 2;
constexpr int kGemmSmem = kStages * kStageBytes + 1024;  // + slack for 1024-byte alignment
constexpr int kGemmThreads = 128;               // four warps: one per 32 accumulator lanes
constexpr long long kSpinLimit = 1ll << 24;     // mbarrier polls before a wait gives up
constexpr int kTmemCols = 128;                  // FP32 accumulator: 128 lanes x 128 columns

// Instruction descriptor of tcgen05.mma kind::tf32: FP32 accumulator (bits
// 4-5 = 1), TF32 A and B (bits 7-9, 10-12 = 2), both K-major (bits 15, 16 =
// 0), N >> 3 at bits 17-22, M >> 4 at bits 24-28.
constexpr uint32_t kIdesc =
    (1u << 4) | (2u << 7) | (2u << 10) | (uint32_t(kTile >> 3) << 17) | (uint32_t(kTile >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor: K-major operand with the 128-byte
// swizzle, 8-row core groups 1024 bytes apart (stride byte offset), start
// address in 16-byte units, descriptor version 1 (bits 46-47), swizzle mode
// 2 = 128 bytes (bits 61-63).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = uint64_t((saddr >> 4) & 0x3FFFu);
  d |= uint64_t(1) << 16;
  d |= uint64_t(1024 >> 4) << 32;
  d |= uint64_t(1) << 46;
  d |= uint64_t(2) << 61;
  return d;
}

__device__ __forceinline__ float tf32_round(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
      "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (long long it = 0; it < kSpinLimit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 consecutive FP32 accumulator columns of this thread's lane.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// A 128 x 32 FP32 block (rows of `src`, columns k0..k0+31) into registers:
// eight 16-byte pieces per thread, rows of 128 bytes read by 8 consecutive
// threads.
__device__ __forceinline__ void load_block(const float* src, int ld, int k0, float4 (&x)[8], int tid) {
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int f = tid + q * kGemmThreads;
    const int r = f >> 3, c = f & 7;
    x[q] = *reinterpret_cast<const float4*>(src + int64_t(r) * ld + k0 + c * 4);
  }
}

// Splits a block into TF32 high and remainder parts and stores both in the
// 128-byte swizzled K-major layout: row r at byte r * 128, its 16-byte chunk
// c at position c ^ (r & 7).
__device__ __forceinline__ void split_store(const float4 (&x)[8], uint8_t* hi, uint8_t* lo, int tid) {
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int f = tid + q * kGemmThreads;
    const int r = f >> 3, c = f & 7;
    float4 h, l;
    h.x = tf32_round(x[q].x);
    h.y = tf32_round(x[q].y);
    h.z = tf32_round(x[q].z);
    h.w = tf32_round(x[q].w);
    l.x = tf32_round(x[q].x - h.x);
    l.y = tf32_round(x[q].y - h.y);
    l.z = tf32_round(x[q].z - h.z);
    l.w = tf32_round(x[q].w - h.w);
    const int off = r * 128 + ((c ^ (r & 7)) << 4);
    *reinterpret_cast<float4*>(hi + off) = h;
    *reinterpret_cast<float4*>(lo + off) = l;
  }
}

struct GemmArgs {
  const float* a;    // A rows of tile row 0
  int lda;
  const float* b;    // B rows of tile column 0
  int ldb;
  float* c;          // C tile (0, 0)
  int ldc;
  const float* cin;  // C = cin - A B^T (cin laid out as C), else null
  int k;             // multiple of kKb, > 0
  int k_chunk;       // K range of one CTA (blockIdx.z), a multiple of kKb
  int subtract;      // 1: C -= A B^T with atomic adds (split K), 0: store
  int* status;
};

// One 128 x 128 tile of C = A B^T (or cin - A B^T, or C -= A B^T) per CTA:
// tile row blockIdx.x, tile column blockIdx.y, K range blockIdx.z.  A and C
// may alias (the in-place triangular solve, a single K range): every A row of
// the tile is read before the epilogue writes C.  The next stage's operands
// are loaded into registers while the current stage is split, stored and
// multiplied.
__global__ void __launch_bounds__(kGemmThreads, 1) tc_gemm_nt_kernel(GemmArgs g) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t bars[kStages];
  __shared__ uint32_t tmem_holder;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t raw = smem_u32(smem_raw);
  uint8_t* smem = smem_raw + ((1024u - (raw & 1023u)) & 1023u);
  const uint32_t sbase = smem_u32(smem);
  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars[s])));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_holder)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_holder;

  const int k0 = int(blockIdx.z) * g.k_chunk;
  const float* A = g.a + int64_t(blockIdx.x) * kTile * g.lda + k0;
  const float* B = g.b + int64_t(blockIdx.y) * kTile * g.ldb + k0;
  const int nkb = max(0, min(g.k_chunk, g.k - k0)) / kKb;
  bool ok = true;
  int committed = 0;  // stages whose products were issued
  float4 na[8], nb[8];
  if (nkb > 0) {
    load_block(A, g.lda, 0, na, tid);
    load_block(B, g.ldb, 0, nb, tid);
  }
  for (int kb = 0; kb < nkb; ++kb) {
    const int s = kb & 1;
    float4 ca[8], cb[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      ca[q] = na[q];
      cb[q] = nb[q];
    }
    if (kb + 1 < nkb) {
      load_block(A, g.lda, (kb + 1) * kKb, na, tid);
      load_block(B, g.ldb, (kb + 1) * kKb, nb, tid);
    }
    if (kb >= kStages) {
      // the products of stage kb - 2 have finished reading buffer s
      const bool w = mbar_wait(smem_u32(&bars[s]), uint32_t((kb >> 1) - 1) & 1u);
      ok = __syncthreads_and(w ? 1 : 0) != 0;
      if (!ok) break;
    }
    uint8_t* st = smem + s * kStageBytes;
    split_store(ca, st, st + kOpBytes, tid);
    split_store(cb, st + 2 * kOpBytes, st + 3 * kOpBytes, tid);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
      const uint32_t a_hi = sbase + uint32_t(s * kStageBytes);
      const uint32_t a_lo = a_hi + kOpBytes, b_hi = a_hi + 2 * kOpBytes, b_lo = a_hi + 3 * kOpBytes;
#pragma unroll
      for (int kk = 0; kk < kKb / 8; ++kk) {
        const uint32_t off = uint32_t(kk * 32);  // 8 TF32 values = 32 bytes along K
        mma_tf32(tmem, sw128_desc(a_lo + off), sw128_desc(b_hi + off), (kb | kk) != 0 ? 1u : 0u);
        mma_tf32(tmem, sw128_desc(a_hi + off), sw128_desc(b_lo + off), 1u);
        mma_tf32(tmem, sw128_desc(a_hi + off), sw128_desc(b_hi + off), 1u);
      }
      mma_commit(smem_u32(&bars[s]));
    }
    committed = kb + 1;
  }
  if (committed > 0) {
    // a commit tracks every earlier product of the issuing thread: waiting
    // for the last one covers all (also after a timeout, so that tensor
    // memory is not released under running products)
    const int last = committed - 1;
    const bool w = mbar_wait(smem_u32(&bars[last & 1]), uint32_t(last >> 1) & 1u);
    ok = (__syncthreads_and(w ? 1 : 0) != 0) && ok;
  }
  tc_fence_after();
  if (ok && committed == nkb && nkb > 0) {
    const int row = warp * 32 + lane;
    float* C = g.c + int64_t(blockIdx.x) * kTile * g.ldc + int64_t(blockIdx.y) * kTile + int64_t(row) * g.ldc;
    const float* Cin =
        g.cin ? g.cin + int64_t(blockIdx.x) * kTile * g.ldc + int64_t(blockIdx.y) * kTile + int64_t(row) * g.ldc
              : nullptr;
#pragma unroll 1
    for (int cc = 0; cc < kTile / 32; ++cc) {
      float v[32];
      tmem_ld32(tmem + (uint32_t(warp * 32) << 16) + uint32_t(cc * 32), v);
      if (g.subtract) {
#pragma unroll
        for (int q = 0; q < 32; ++q) atomicAdd(C + cc * 32 + q, -v[q]);
      } else {
#pragma unroll
        for (int q = 0; q < 32; q += 4) {
          float4 o = make_float4(v[q], v[q + 1], v[q + 2], v[q + 3]);
          if (Cin) {
            const float4 ci = *reinterpret_cast<const float4*>(Cin + cc * 32 + q);
            o = make_float4(ci.x - o.x, ci.y - o.y, ci.z - o.z, ci.w - o.w);
          }
          *reinterpret_cast<float4*>(C + cc * 32 + q) = o;
        }
      }
    }
  } else if (nkb > 0 && tid == 0) {
    atomicExch(g.status, 2);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
  }
}

// ---------------------------------------------------------------------------
// Diagonal tile: L_kk = chol(A_kk) and Dinv_k = L_kk^-1, in shared memory,
// in eight 16-column panels.  Per panel: one warp factors the 16 x 16
// diagonal block (lane = row, warp-synchronous), one thread per row solves
// the rows below it against that block, and all threads update the rest of
// the tile.  The inverse: one warp per diagonal block, then the blocks below
// the diagonal, block row by block row: X_ij = -X_ii sum_{j<=m<i} L_im X_mj.
constexpr int kPotrfThreads = 512;
constexpr int kLdS = kTile + 1;
constexpr int kPanel = 16;
constexpr int kPotrfSmem = (2 * kTile * kLdS + (kTile / kPanel - 1) * kPanel * kPanel) * 4;

__global__ void __launch_bounds__(kPotrfThreads) potrf_tile_kernel(float* L, int ld, int k, float* dinv,
                                                                   int* status) {
  extern __shared__ float sm[];
  float* a = sm;                   // the tile, then its factor (lower)
  float* x = a + kTile * kLdS;     // the inverse of the factor (lower)
  float* tmp = x + kTile * kLdS;   // [3][32][32] partial sums of the inverse
  __shared__ int bad;
  __shared__ float rdiag[kTile];  // 1 / L_jj
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  float* tile = L + int64_t(k) * kTile * ld + int64_t(k) * kTile;
  for (int t = tid; t < kTile * kTile; t += kPotrfThreads) {
    const int i = t >> 7, j = t & (kTile - 1);
    a[i * kLdS + j] = tile[int64_t(i) * ld + j];
    x[i * kLdS + j] = 0.f;
  }
  if (tid == 0) bad = 0;
  __syncthreads();
  for (int p = 0; p < kTile / kPanel; ++p) {
    const int c0 = kPanel * p;
    if (warp == 0) {
      // the diagonal block, warp-synchronous: lane = row (lanes beyond the
      // panel only take part in the warp's collective steps)
      const bool act = lane < kPanel;
      const int i = c0 + (act ? lane : kPanel - 1);
      for (int j = 0; j < kPanel; ++j) {
        const int jj = c0 + j;
        float d = a[jj * kLdS + jj];
        if (!(d > 0.f) || !isfinite(d)) {
          if (lane == 0) bad = 1;
          d = 1.f;
        }
        // the factor only preconditions FP64 conjugate gradients: the fast
        // reciprocal square root is accurate enough
        const float inv = rsqrtf(d);
        const float l = d * inv;
        __syncwarp();
        if (lane == j) {
          a[jj * kLdS + jj] = l;
          rdiag[jj] = inv;
        }
        if (act && lane > j) a[i * kLdS + jj] *= inv;
        __syncwarp();
        // all loads first (constant offsets, so they issue back to back),
        // then the predicated updates of this lane's row
        const float lij = a[i * kLdS + jj];
        float lc[kPanel], ar[kPanel];
#pragma unroll
        for (int c = 0; c < kPanel; ++c) {
          lc[c] = a[(c0 + c) * kLdS + jj];
          ar[c] = a[i * kLdS + c0 + c];
        }
#pragma unroll
        for (int c = 0; c < kPanel; ++c)
          if (act && c > j && c <= lane) a[i * kLdS + c0 + c] = ar[c] - lij * lc[c];
        __syncwarp();
      }
    }
    __syncthreads();
    for (int i = c0 + kPanel + tid; i < kTile; i += kPotrfThreads) {
      // row i of the panel in registers, solved against the diagonal block
      float row[kPanel];
#pragma unroll
      for (int j = 0; j < kPanel; ++j) row[j] = a[i * kLdS + c0 + j];
#pragma unroll
      for (int j = 0; j < kPanel; ++j) {
        float v = row[j];
#pragma unroll
        for (int m = 0; m < j; ++m) v -= row[m] * a[(c0 + j) * kLdS + c0 + m];
        row[j] = v * rdiag[c0 + j];
      }
#pragma unroll
      for (int j = 0; j < kPanel; ++j) a[i * kLdS + c0 + j] = row[j];
    }
    __syncthreads();
    const int r0 = c0 + kPanel;
    for (int i = r0 + (tid >> 4); i < kTile; i += kPotrfThreads / 16) {
      for (int c = r0 + (tid & 15); c <= i; c += 16) {
        float v = 0.f;
#pragma unroll 8
        for (int m = 0; m < kPanel; ++m) v += a[i * kLdS + c0 + m] * a[c * kLdS + c0 + m];
        a[i * kLdS + c] -= v;
      }
    }
    __syncthreads();
  }
  // inverse of the diagonal 32 x 32 blocks: warp w inverts block w, lane = column
  if (warp < kTile / kPanel) {
    // lane c holds column c of the block's inverse in registers
    const int b0 = kPanel * warp, c = lane < kPanel ? lane : kPanel - 1;
    float col[kPanel];
#pragma unroll
    for (int i = 0; i < kPanel; ++i) {
      float v = i == c ? 1.f : 0.f;
#pragma unroll
      for (int m = 0; m < i; ++m) v -= a[(b0 + i) * kLdS + b0 + m] * col[m];
      col[i] = i >= c ? v * rdiag[b0 + i] : 0.f;
    }
    if (lane < kPanel) {
#pragma unroll
      for (int i = 0; i < kPanel; ++i) x[(b0 + i) * kLdS + b0 + c] = col[i];
    }
  }
  __syncthreads();
  for (int bi = 1; bi < kTile / kPanel; ++bi) {
    for (int e = tid; e < bi * kPanel * kPanel; e += kPotrfThreads) {
      const int j = e / (kPanel * kPanel), r = (e / kPanel) % kPanel, c = e % kPanel;
      float v = 0.f;
      for (int kk = j; kk < bi; ++kk)
#pragma unroll 8
        for (int m = 0; m < kPanel; ++m)
          v += a[(kPanel * bi + r) * kLdS + kPanel * kk + m] * x[(kPanel * kk + m) * kLdS + kPanel * j + c];
      tmp[e] = v;
    }
    __syncthreads();
    for (int e = tid; e < bi * kPanel * kPanel; e += kPotrfThreads) {
      const int j = e / (kPanel * kPanel), r = (e / kPanel) % kPanel, c = e % kPanel;
      float v = 0.f;
      for (int m = 0; m <= r; ++m)
        v += x[(kPanel * bi + r) * kLdS + kPanel * bi + m] * tmp[j * kPanel * kPanel + m * kPanel + c];
      x[(kPanel * bi + r) * kLdS + kPanel * j + c] = -v;
    }
    __syncthreads();
  }
  float* dk = dinv + int64_t(k) * kTile * kTile;
  for (int t = tid; t < kTile * kTile; t += kPotrfThreads) {
    const int i = t >> 7, j = t & (kTile - 1);
    tile[int64_t(i) * ld + j] = j <= i ? a[i * kLdS + j] : 0.f;
    dk[t] = j <= i ? x[i * kLdS + j] : 0.f;
  }
  if (tid == 0 && bad) atomicExch(status + 1, 1);
}

// ---------------------------------------------------------------------------
// Scaling and conversion.
__global__ void jacobi_scale_kernel(int n, const double* __restrict__ A, int lda, double* __restrict__ d,
                                    int* status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double a = A[int64_t(i) * lda + i];
  if (!(a > 0.0) || !isfinite(a)) {
    atomicExch(status, 1);
    d[i] = 1.0;
  } else {
    d[i] = 1.0 / sqrt(a);
  }
}

// L = fp32(D A D) on the lower triangle (identity on the padding), zero
// above; A's upper triangle becomes the mirror of its lower triangle.
__global__ void load_scaled_kernel(int n, int n_pad, double* A, int lda, const double* __restrict__ d,
                                   float* __restrict__ L, double shift) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= int64_t(n_pad) * n_pad) return;
  const int i = int(t / n_pad), j = int(t % n_pad);
  float v = 0.f;
  if (i < n && j < n) {
    if (j <= i) {
      const double a = A[int64_t(i) * lda + j];
      v = float(a * d[i] * d[j] + (i == j ? shift : 0.0));
      if (j < i) A[int64_t(j) * lda + i] = a;
    }
  } else if (i == j) {
    v = 1.f;
  }
  L[t] = v;
}

__device__ __forceinline__ float warp_sum_f(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_sum_d(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---------------------------------------------------------------------------
// Triangular solves with the tiled factor, one launch per tile step with one
// CTA per tile it touches.  Forward, step k: y_k = Dinv_k b_k (CTA 0 stores
// it) and b_i -= L_ik y_k for i > k (CTA i - k).  Backward, step k: x_k =
// Dinv_k^T y_k (CTA k stores it) and y_i -= L_ki^T x_k for i < k (CTA i).
// Each CTA recomputes the 128-long diagonal product instead of waiting for
// another CTA.
constexpr int kTsThreads = 256;

__global__ void ts_init_kernel(int n, int n_pad, const float* __restrict__ rs, float* __restrict__ b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n_pad) b[i] = i < n ? rs[i] : 0.f;
}

__global__ void __launch_bounds__(kTsThreads) fwd_step_kernel(const float* __restrict__ L, int ld,
                                                              const float* __restrict__ dinv, int k,
                                                              float* __restrict__ b, float* __restrict__ y) {
  __shared__ __align__(16) float bk[kTile];
  __shared__ __align__(16) float yk[kTile];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid < kTile) bk[tid] = b[k * kTile + tid];
  __syncthreads();
  const float4 bv = reinterpret_cast<const float4*>(bk)[lane];
  const float* D = dinv + int64_t(k) * kTile * kTile;
  for (int r = warp; r < kTile; r += kTsThreads / 32) {
    const float4 dv = reinterpret_cast<const float4*>(D + r * kTile)[lane];
    const float s = warp_sum_f(dv.x * bv.x + dv.y * bv.y + dv.z * bv.z + dv.w * bv.w);
    if (lane == 0) yk[r] = s;
  }
  __syncthreads();
  if (blockIdx.x == 0) {
    if (tid < kTile) y[k * kTile + tid] = yk[tid];
    return;
  }
  const int i = k + int(blockIdx.x);
  const float4 yv = reinterpret_cast<const float4*>(yk)[lane];
  for (int r = warp; r < kTile; r += kTsThreads / 32) {
    const float4 lv = reinterpret_cast<const float4*>(L + int64_t(i * kTile + r) * ld + k * kTile)[lane];
    const float s = warp_sum_f(lv.x * yv.x + lv.y * yv.y + lv.z * yv.z + lv.w * yv.w);
    if (lane == 0) b[i * kTile + r] -= s;
  }
}

__global__ void __launch_bounds__(kTsThreads) bwd_step_kernel(const float* __restrict__ L, int ld,
                                                              const float* __restrict__ dinv, int k,
                                                              float* __restrict__ y, float* __restrict__ xv) {
  __shared__ float tk[kTile], xk[kTile], part[2][kTile];
  const int tid = threadIdx.x, c = tid & (kTile - 1), h = tid >> 7;
  if (tid < kTile) tk[tid] = y[k * kTile + tid];
  __syncthreads();
  const float* D = dinv + int64_t(k) * kTile * kTile;
  float s = 0.f;
#pragma unroll 8
  for (int r = h * 64; r < h * 64 + 64; ++r) s += D[r * kTile + c] * tk[r];
  part[h][c] = s;
  __syncthreads();
  if (tid < kTile) xk[tid] = part[0][tid] + part[1][tid];
  __syncthreads();
  const int i = int(blockIdx.x);
  if (i == k) {
    if (tid < kTile) xv[k * kTile + tid] = xk[tid];
    return;
  }
  float s2 = 0.f;
#pragma unroll 8
  for (int r = h * 64; r < h * 64 + 64; ++r) s2 += L[int64_t(k * kTile + r) * ld + i * kTile + c] * xk[r];
  part[h][c] = s2;
  __syncthreads();
  if (tid < kTile) y[i * kTile + tid] -= part[0][tid] + part[1][tid];
}

// z = D x (back to the unscaled unknowns, FP64)
__global__ void ts_finish_kernel(int n, const double* __restrict__ d, const float* __restrict__ xv,
                                 double* __restrict__ z) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) z[i] = d[i] * double(xv[i]);
}

// Flexible preconditioned conjugate gradients in FP64.  Scalars live on the
// device: rz = r.z, pq = p.(A p), rr = |D r|^2, rz_new = r.z_new, rz_mix =
// r.z_old (Polak-Ribiere beta = (rz_new - rz_mix) / rz), bb = |D b|^2.  The
// residual is measured after the Jacobi scaling D, which makes the
// tolerance independent of the units of the unknowns.
enum { kRz = 0, kPq = 1, kRr = 2, kRzNew = 3, kRzMix = 4, kBb = 5, kNumScal = 6 };

__device__ __forceinline__ void block_add(double v, double* out) {
  __shared__ double wsum[32];
  v = warp_sum_d(v);
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) wsum[w] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int k = 0; k < int(blockDim.x >> 5); ++k) s += wsum[k];
    atomicAdd(out, s);
  }
  __syncthreads();
}

// x = 0, r = b, rs = fp32(D b), bb = |b|^2
__global__ void cg_init_kernel(int n, const double* __restrict__ b, const double* __restrict__ d,
                               double* __restrict__ x, double* __restrict__ r, float* __restrict__ rs,
                               double* __restrict__ scal) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double e = 0.0;
  if (i < n) {
    const double v = b[i];
    x[i] = 0.0;
    r[i] = v;
    const double sv = d[i] * v;
    rs[i] = float(sv);
    e = sv * sv;
  }
  block_add(e, scal + kBb);
}

// q = A p (full FP64 matrix, one warp per row), pq += p.q
__global__ void symv_kernel(int n, const double* __restrict__ A, int lda, const double* __restrict__ p,
                            double* __restrict__ q, double* __restrict__ scal) {
  const int row = int((int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  double e = 0.0;
  if (row < n) {
    const double* ar = A + int64_t(row) * lda;
    double s = 0.0;
    for (int j = lane; j < n; j += 32) s += ar[j] * p[j];
    s = warp_sum_d(s);
    if (lane == 0) {
      q[row] = s;
      e = s * p[row];
    }
  }
  block_add(e, scal + kPq);
}

// alpha = rz / pq; x += alpha p; r -= alpha q; rs = fp32(D r); rr += |r|^2
__global__ void cg_update_kernel(int n, const double* __restrict__ p, const double* __restrict__ q,
                                 const double* __restrict__ d, double* __restrict__ x, double* __restrict__ r,
                                 float* __restrict__ rs, double* __restrict__ scal) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const double pq = scal[kPq];
  const double alpha = pq > 0.0 ? scal[kRz] / pq : 0.0;
  double e = 0.0;
  if (i < n) {
    x[i] += alpha * p[i];
    const double v = r[i] - alpha * q[i];
    r[i] = v;
    const double sv = d[i] * v;
    rs[i] = float(sv);
    e = sv * sv;
  }
  block_add(e, scal + kRr);
}

// rz_new += r.z_new, rz_mix += r.z_old (z_old null: first direction)
__global__ void cg_dots_kernel(int n, const double* __restrict__ r, const double* __restrict__ z,
                               const double* __restrict__ z_old, double* __restrict__ scal) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double a = 0.0, b = 0.0;
  if (i < n) {
    a = r[i] * z[i];
    if (z_old) b = r[i] * z_old[i];
  }
  block_add(a, scal + kRzNew);
  if (z_old) block_add(b, scal + kRzMix);
}

// p = z + beta p (beta = 0 on the first direction)
__global__ void cg_dir_kernel(int n, const double* __restrict__ z, double* __restrict__ p,
                              const double* __restrict__ scal, int first) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double rz = scal[kRz];
  const double beta = first || !(rz != 0.0) ? 0.0 : (scal[kRzNew] - scal[kRzMix]) / rz;
  p[i] = z[i] + beta * p[i];
}

__global__ void cg_rotate_kernel(double* scal) {
  scal[kRz] = scal[kRzNew];
  scal[kPq] = 0.0;
  scal[kRr] = 0.0;
  scal[kRzNew] = 0.0;
  scal[kRzMix] = 0.0;
}

// ---- batched columns (inverse_columns): K right-hand sides in lockstep,
// vectors stored [n_pad][K] row-major so that a warp reads one row's K
// values.  Per-column scalars at mscal[c * kNumScal + ...].
constexpr int kRhs = DenseSpdSolver::kInverseBatch;

// Adds v to out[c] for the column c of each thread: a shared-memory sum per
// block, then one global atomic per column.
__device__ __forceinline__ void column_add(double v, int c, int K, double* out, int which) {
  __shared__ double cs[kRhs];
  if (threadIdx.x < kRhs) cs[threadIdx.x] = 0.0;
  __syncthreads();
  if (c >= 0 && v != 0.0) atomicAdd(&cs[c], v);
  __syncthreads();
  if (threadIdx.x < K && cs[threadIdx.x] != 0.0) atomicAdd(&out[threadIdx.x * kNumScal + which], cs[threadIdx.x]);
}

// x = 0, r = e_{unit[c]}, rs = fp32(D r) (rows n .. n_pad - 1 zero), bb = |D e|^2
__global__ void mcg_init_kernel(int n, int n_pad, int K, const int* __restrict__ unit, const double* __restrict__ d,
                                double* __restrict__ X, double* __restrict__ R, float* __restrict__ RS,
                                double* __restrict__ scal) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= int64_t(n_pad) * K) return;
  const int i = int(t / K), c = int(t % K);
  const double b = (i < n && i == unit[c]) ? 1.0 : 0.0;
  X[t] = 0.0;
  R[t] = b;
  RS[t] = i < n ? float(d[i] * b) : 0.f;
  if (b != 0.0) scal[c * kNumScal + kBb] = d[i] * d[i];
}

// Triangular steps with K <= 32 right-hand sides.  A CTA stages a 128 x 128
// factor tile in shared memory (Ms[j][r], rows padded to 132 floats) and the
// 128 x 32 right-hand block (Vs[j][c]); thread (tr, tc) = (tid / 8, tid % 8)
// computes the 4 x 4 outputs Out[4 tr + a][4 tc + b] = sum_j Ms[j][4 tr + a]
// Vs[j][4 tc + b] from float4 reads.  Columns c >= K are zero.
constexpr int kMsLd = kTile + 4;
constexpr int kMsteps = (kTile * kMsLd + 2 * kTile * kRhs) * int(sizeof(float));  // dynamic shared bytes

// Ms[j][r] = M[r][j] (transpose) or M[j][r], M a 128 x 128 tile at m with
// leading dimension ld
__device__ __forceinline__ void load_tile(float* Ms, const float* __restrict__ m, int64_t ld, bool transpose) {
  for (int e = threadIdx.x; e < kTile * kTile / 4; e += kTsThreads) {
    const int row = e / (kTile / 4), col = (e % (kTile / 4)) * 4;
    const float4 v = *reinterpret_cast<const float4*>(m + row * ld + col);
    if (transpose) {
      Ms[(col + 0) * kMsLd + row] = v.x;
      Ms[(col + 1) * kMsLd + row] = v.y;
      Ms[(col + 2) * kMsLd + row] = v.z;
      Ms[(col + 3) * kMsLd + row] = v.w;
    } else {
      *reinterpret_cast<float4*>(Ms + row * kMsLd + col) = v;
    }
  }
}

// Vs[j][c] = V[j * ldv + c] for c < K, else 0 (128 rows)
__device__ __forceinline__ void load_rhs(float* Vs, const float* __restrict__ v, int K, int ldv) {
  for (int e = threadIdx.x; e < kTile * kRhs; e += kTsThreads) {
    const int j = e / kRhs, c = e % kRhs;
    Vs[e] = c < K ? v[int64_t(j) * ldv + c] : 0.f;
  }
}

__device__ __forceinline__ void tile_product(const float* Ms, const float* Vs, float (&acc)[4][4]) {
  const int r0 = (threadIdx.x >> 3) * 4, c0 = (threadIdx.x & 7) * 4;
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0.f;
#pragma unroll 8
  for (int j = 0; j < kTile; ++j) {
    const float4 m = *reinterpret_cast<const float4*>(Ms + j * kMsLd + r0);
    const float4 v = *reinterpret_cast<const float4*>(Vs + j * kRhs + c0);
    const float mv[4] = {m.x, m.y, m.z, m.w}, vv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b) acc[a][b] += mv[a] * vv[b];
  }
}

// Forward step k: Y_k = Dinv_k B_k (CTA 0 stores it), B_i -= L_ik Y_k for
// i = k + blockIdx.x > k.  B and Y are [n_pad][ldb] row-major; CTA column
// blockIdx.y takes the K columns from 32 blockIdx.y.
__global__ void __launch_bounds__(kTsThreads) mfwd_step_kernel(const float* __restrict__ L, int ld,
                                                               const float* __restrict__ dinv, int k, int K,
                                                               int ldb, float* __restrict__ B,
                                                               float* __restrict__ Y) {
  extern __shared__ __align__(16) float msm[];
  float* Ms = msm;
  float* Vs = Ms + kTile * kMsLd;
  float* Os = Vs + kTile * kRhs;
  const int r0 = (threadIdx.x >> 3) * 4, c0 = (threadIdx.x & 7) * 4;
  const int col = int(blockIdx.y) * kRhs;
  B += col;
  Y += col;
  load_tile(Ms, dinv + int64_t(k) * kTile * kTile, kTile, true);
  load_rhs(Vs, B + int64_t(k) * kTile * ldb, K, ldb);
  __syncthreads();
  float acc[4][4];
  tile_product(Ms, Vs, acc);
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) Os[(r0 + a) * kRhs + c0 + b] = acc[a][b];
  if (blockIdx.x == 0) {
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b)
        if (c0 + b < K) Y[(int64_t(k) * kTile + r0 + a) * ldb + c0 + b] = acc[a][b];
    return;
  }
  const int i = k + int(blockIdx.x);
  __syncthreads();  // Ms free, Os complete
  load_tile(Ms, L + int64_t(i) * kTile * ld + int64_t(k) * kTile, ld, true);
  __syncthreads();
  tile_product(Ms, Os, acc);
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b)
      if (c0 + b < K) B[(int64_t(i) * kTile + r0 + a) * ldb + c0 + b] -= acc[a][b];
}

// Backward step k: X_k = Dinv_k^T Y_k (CTA k stores it), Y_i -= L_ki^T X_k
// for i = blockIdx.x < k; columns as in the forward step.
__global__ void __launch_bounds__(kTsThreads) mbwd_step_kernel(const float* __restrict__ L, int ld,
                                                               const float* __restrict__ dinv, int k, int K,
                                                               int ldb, float* __restrict__ Y,
                                                               float* __restrict__ X) {
  extern __shared__ __align__(16) float msm[];
  float* Ms = msm;
  float* Vs = Ms + kTile * kMsLd;
  float* Os = Vs + kTile * kRhs;
  const int r0 = (threadIdx.x >> 3) * 4, c0 = (threadIdx.x & 7) * 4;
  const int col = int(blockIdx.y) * kRhs;
  Y += col;
  X += col;
  load_tile(Ms, dinv + int64_t(k) * kTile * kTile, kTile, false);
  load_rhs(Vs, Y + int64_t(k) * kTile * ldb, K, ldb);
  __syncthreads();
  float acc[4][4];
  tile_product(Ms, Vs, acc);
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) Os[(r0 + a) * kRhs + c0 + b] = acc[a][b];
  const int i = int(blockIdx.x);
  if (i == k) {
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 4; ++b)
        if (c0 + b < K) X[(int64_t(k) * kTile + r0 + a) * ldb + c0 + b] = acc[a][b];
    return;
  }
  __syncthreads();
  load_tile(Ms, L + int64_t(k) * kTile * ld + int64_t(i) * kTile, ld, false);
  __syncthreads();
  tile_product(Ms, Os, acc);
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b)
      if (c0 + b < K) Y[(int64_t(i) * kTile + r0 + a) * ldb + c0 + b] -= acc[a][b];
}

// Z = D X (FP64, rows < n)
__global__ void mts_finish_kernel(int n, int K, const double* __restrict__ d, const float* __restrict__ X,
                                  double* __restrict__ Z) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= int64_t(n) * K) return;
  Z[t] = d[t / K] * double(X[t]);
}

// Q += A P over the column range of blockIdx.y (two halves, so that about
// 2 n / 32 CTAs share the FP64 pipes), and pq += P.Q per column.  32 rows x
// K columns per CTA; thread (row r = tid / 8, columns 4 (tid % 8) .. + 3).
constexpr int kSymmRows = 32, kSymmK = 32;
__global__ void __launch_bounds__(256) msymm_kernel(int n, int K, const double* __restrict__ A, int lda,
                                                    const double* __restrict__ P, double* __restrict__ Q,
                                                    double* __restrict__ scal) {
  __shared__ double As[kSymmRows][kSymmK + 1];
  __shared__ double Ps[kSymmK][kRhs];
  const int tid = threadIdx.x, r = tid >> 3, cg = (tid & 7) * 4;
  const int row0 = blockIdx.x * kSymmRows;
  const int half = (n + 1) / 2;
  const int j_begin = blockIdx.y == 0 ? 0 : half, j_end = blockIdx.y == 0 ? half : n;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int j0 = j_begin; j0 < j_end; j0 += kSymmK) {
    for (int e = tid; e < kSymmRows * kSymmK; e += 256) {
      const int rr = e / kSymmK, jj = e % kSymmK;
      const int gi = row0 + rr, gj = j0 + jj;
      As[rr][jj] = (gi < n && gj < j_end) ? A[int64_t(gi) * lda + gj] : 0.0;
    }
    for (int e = tid; e < kSymmK * kRhs; e += 256) {
      const int jj = e / kRhs, c = e % kRhs;
      const int gj = j0 + jj;
      Ps[jj][c] = (gj < j_end && c < K) ? P[int64_t(gj) * K + c] : 0.0;
    }
    __syncthreads();
#pragma unroll 4
    for (int jj = 0; jj < kSymmK; ++jj) {
      const double a = As[r][jj];
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[q] += a * Ps[jj][cg + q];
    }
    __syncthreads();
  }
  const int gi = row0 + r;
  double pq[4] = {0.0, 0.0, 0.0, 0.0};
  if (gi < n) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int c = cg + q;
      if (c < K) {
        atomicAdd(&Q[int64_t(gi) * K + c], acc[q]);
        pq[q] = acc[q] * P[int64_t(gi) * K + c];
      }
    }
  }
  __shared__ double cs[kRhs];
  if (tid < kRhs) cs[tid] = 0.0;
  __syncthreads();
#pragma unroll
  for (int q = 0; q < 4; ++q)
    if (pq[q] != 0.0) atomicAdd(&cs[cg + q], pq[q]);
  __syncthreads();
  if (tid < K && cs[tid] != 0.0) atomicAdd(&scal[tid * kNumScal + kPq], cs[tid]);
}

// alpha_c = rz_c / pq_c; X += alpha P; R -= alpha Q; RS = fp32(D R); rr += |D R|^2
__global__ void mcg_update_kernel(int n, int K, const double* __restrict__ P, const double* __restrict__ Q,
                                  const double* __restrict__ d, double* __restrict__ X, double* __restrict__ R,
                                  float* __restrict__ RS, double* __restrict__ scal) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  int c = -1;
  double e = 0.0;
  if (t < int64_t(n) * K) {
    c = int(t % K);
    const double pq = scal[c * kNumScal + kPq];
    const double alpha = pq > 0.0 ? scal[c * kNumScal + kRz] / pq : 0.0;
    X[t] += alpha * P[t];
    const double v = R[t] - alpha * Q[t];
    R[t] = v;
    const double sv = d[t / K] * v;
    RS[t] = float(sv);
    e = sv * sv;
  }
  column_add(e, c, K, scal, kRr);
}

// rz_new += R.Z_new, rz_mix += R.Z_old per column (Z_old null: first direction)
__global__ void mcg_dots_kernel(int n, int K, const double* __restrict__ R, const double* __restrict__ Zn,
                                const double* __restrict__ Zo, double* __restrict__ scal) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  int c = -1;
  double a = 0.0, b = 0.0;
  if (t < int64_t(n) * K) {
    c = int(t % K);
    a = R[t] * Zn[t];
    if (Zo) b = R[t] * Zo[t];
  }
  column_add(a, c, K, scal, kRzNew);
  if (Zo) column_add(b, c, K, scal, kRzMix);
}

// P = Z + beta_c P (beta = 0 on the first direction)
__global__ void mcg_dir_kernel(int n, int K, const double* __restrict__ Z, double* __restrict__ P,
                               const double* __restrict__ scal, int first) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= int64_t(n) * K) return;
  const int c = int(t % K);
  const double rz = scal[c * kNumScal + kRz];
  const double beta = first || !(rz != 0.0) ? 0.0 : (scal[c * kNumScal + kRzNew] - scal[c * kNumScal + kRzMix]) / rz;
  P[t] = Z[t] + beta * P[t];
}

__global__ void mcg_rotate_kernel(int K, double* scal) {
  const int c = threadIdx.x;
  if (c >= K) return;
  double* s = scal + c * kNumScal;
  s[kRz] = s[kRzNew];
  s[kPq] = 0.0;
  s[kRr] = 0.0;
  s[kRzNew] = 0.0;
  s[kRzMix] = 0.0;
}

// out[6 c + k] = X[gather[6 c + k], c] (-1: 0)
__global__ void mgather_kernel(int K, const int* __restrict__ gather, const double* __restrict__ X,
                               double* __restrict__ out) {
  const int t = threadIdx.x;
  if (t >= 6 * K) return;
  const int c = t / 6, g = gather[t];
  out[t] = g >= 0 ? X[int64_t(g) * K + c] : 0.0;
}

void set_smem(const void* f, int bytes) {
  GB_CUDA(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
}

void launch_gemm(const GemmArgs& g, int tiles_m, int tiles_n, int splits = 1) {
  static bool configured = false;
  if (!configured) {
    set_smem(reinterpret_cast<const void*>(tc_gemm_nt_kernel), kGemmSmem);
    configured = true;
  }
  tc_gemm_nt_kernel<<<dim3(tiles_m, tiles_n, splits), kGemmThreads, kGemmSmem>>>(g);
}

// Splits K so that a launch fills about one wave of CTAs (152 SMs), with at
// least four stages of 32 per CTA.
int k_splits(int tiles, int k) {
  const int by_sms = (152 + tiles - 1) / tiles;
  const int by_k = std::max(1, k / (4 * kKb));
  return std::max(1, std::min(by_sms, by_k));
}

double seconds_now() {
  using clk = std::chrono::steady_clock;
  return std::chrono::duration<double>(clk::now().time_since_epoch()).count();
}

}  // namespace

void tc_gemm_nt(const float* A, int lda, const float* B, int ldb, float* C, int ldc, int m, int n, int k,
                int* status) {
  if (m % kTile || n % kTile || k % kKb || k <= 0 || lda % 4 || ldb % 4 || ldc % 4)
    throw std::invalid_argument("tc_gemm_nt: m, n must be multiples of 128, k a positive multiple of 32");
  GemmArgs g{A, lda, B, ldb, C, ldc, nullptr, k, k, 0, status};
  launch_gemm(g, m / kTile, n / kTile);
  GB_CUDA(cudaGetLastError());
}

int DenseSpdSolver::factor(double* A, int n, int lda) {
  n_ = n;
  A_ = A;
  lda_ = lda;
  nt_ = (n + kTile - 1) / kTile;
  n_pad_ = nt_ * kTile;
  shift_ = 0.0;
  if (n <= 0) return 0;
  static bool configured = false;
  if (!configured) {
    set_smem(reinterpret_cast<const void*>(potrf_tile_kernel), kPotrfSmem);
    configured = true;
  }
  if (n_pad_ > 32768) throw std::invalid_argument("dense solver: system larger than 32768 unknowns");
  L_.resize(size_t(n_pad_) * n_pad_);
  dinv_.resize(size_t(nt_) * kTile * kTile);
  rs_.resize(n_pad_);
  ts_.resize(3 * size_t(n_pad_));
  dscale_.resize(n_pad_);
  r_.resize(4 * size_t(n_pad_));  // r, p, q and the second preconditioned residual
  z_.resize(n_pad_);
  scal_.resize(kNumScal);
  // status: [0] non-positive diagonal, [1] non-positive pivot, [2] wait timed out
  status_.resize(3);
  status_.zero();
  jacobi_scale_kernel<<<(n + 255) / 256, 256>>>(n, A, lda, dscale_.get(), status_.get());
  int st[3] = {0, 0, 0};
  GB_CUDA(cudaMemcpy(st, status_.get(), sizeof(st), cudaMemcpyDeviceToHost));
  if (st[0]) return 1;
  // the scaled matrix has a unit diagonal: the shifts are relative to it
  static const double kShifts[] = {0.0, 1e-6, 1e-4, 1e-2, 1.0};
  for (double shift : kShifts) {
    const int64_t total = int64_t(n_pad_) * n_pad_;
    load_scaled_kernel<<<int((total + 255) / 256), 256>>>(n, n_pad_, A, lda, dscale_.get(), L_.get(), shift);
    float* L = L_.get();
    const int ld = n_pad_;
    for (int k = 0; k < nt_; ++k) {
      float* rowk = L + int64_t(k) * kTile * ld;
      if (k > 0) {
        // A_ik -= L_i,0:k L_k,0:k^T, K split across CTAs (atomic subtraction)
        const int K = k * kTile;
        const int splits = k_splits(nt_ - k, K);
        const int chunk = (K / kKb + splits - 1) / splits * kKb;
        GemmArgs g{rowk, ld, rowk, ld, rowk + int64_t(k) * kTile, ld, nullptr, K, chunk, 1, status_.get() + 2};
        launch_gemm(g, nt_ - k, 1, (K + chunk - 1) / chunk);
      }
      potrf_tile_kernel<<<1, kPotrfThreads, kPotrfSmem>>>(L, ld, k, dinv_.get(), status_.get());
      if (k + 1 < nt_) {
        float* below = L + int64_t(k + 1) * kTile * ld + int64_t(k) * kTile;
        GemmArgs g{below, ld, dinv_.get() + int64_t(k) * kTile * kTile, kTile, below, ld, nullptr, kTile, kTile,
                   0, status_.get() + 2};
        launch_gemm(g, nt_ - k - 1, 1);
      }
    }
    GB_CUDA(cudaGetLastError());
    GB_CUDA(cudaMemcpy(st, status_.get(), sizeof(st), cudaMemcpyDeviceToHost));
    if (st[2]) return 2;
    shift_ = shift;
    if (!st[1]) return 0;
    GB_CUDA(cudaMemset(status_.get() + 1, 0, sizeof(int)));
  }
  return 1;
}

int DenseSpdSolver::solve(const double* b, double* x, double tol, int max_iterations, DenseSolveStats* stats) {
  DenseSolveStats out;
  if (n_ <= 0) {
    if (stats) *stats = out;
    return 0;
  }
  const int n = n_;
  const int eg = (n + 255) / 256;
  const int rows_per_block = 8;
  const int mg = (n + rows_per_block - 1) / rows_per_block;
  double* r = r_.get();
  double* p = r + n_pad_;
  double* q = p + n_pad_;
  double* z_new = q + n_pad_;
  double* z_old = z_.get();
  double* scal = scal_.get();
  float* tb = ts_.get();
  float* ty = tb + n_pad_;
  float* tx = ty + n_pad_;
  // z = D (L L^T)^-1 rs, rs = fp32(D r)
  auto precondition = [&](double* z) {
    ts_init_kernel<<<(n_pad_ + 255) / 256, 256>>>(n, n_pad_, rs_.get(), tb);
    for (int k = 0; k < nt_; ++k)
      fwd_step_kernel<<<nt_ - k, kTsThreads>>>(L_.get(), n_pad_, dinv_.get(), k, tb, ty);
    for (int k = nt_ - 1; k >= 0; --k)
      bwd_step_kernel<<<k + 1, kTsThreads>>>(L_.get(), n_pad_, dinv_.get(), k, ty, tx);
    ts_finish_kernel<<<eg, 256>>>(n, dscale_.get(), tx, z);
  };
  scal_.zero();
  cg_init_kernel<<<eg, 256>>>(n, b, dscale_.get(), x, r, rs_.get(), scal);
  precondition(z_old);
  cg_dots_kernel<<<eg, 256>>>(n, r, z_old, nullptr, scal);
  cg_dir_kernel<<<eg, 256>>>(n, z_old, p, scal, 1);
  cg_rotate_kernel<<<1, 1>>>(scal);
  GB_CUDA(cudaGetLastError());
  double bb = 0.0;
  GB_CUDA(cudaMemcpy(&bb, scal + kBb, sizeof(double), cudaMemcpyDeviceToHost));
  if (!(bb > 0.0)) {
    if (stats) *stats = out;
    return 0;
  }
  out.status = 3;
  for (int it = 0; it < max_iterations; ++it) {
    symv_kernel<<<mg, 32 * rows_per_block>>>(n, A_, lda_, p, q, scal);
    cg_update_kernel<<<eg, 256>>>(n, p, q, dscale_.get(), x, r, rs_.get(), scal);
    double s2[2];  // pq, rr
    GB_CUDA(cudaMemcpy(s2, scal + kPq, sizeof(s2), cudaMemcpyDeviceToHost));
    ++out.refinements;
    const double rel = std::sqrt(s2[1] / bb);
    out.rel_residual = rel;
    if (!(s2[0] > 0.0)) {
      out.status = std::isfinite(s2[0]) ? 1 : 3;  // p . A p <= 0: not positive definite
      break;
    }
    if (!std::isfinite(rel)) break;
    if (rel <= tol) {
      out.status = 0;
      break;
    }
    precondition(z_new);
    cg_dots_kernel<<<eg, 256>>>(n, r, z_new, z_old, scal);
    cg_dir_kernel<<<eg, 256>>>(n, z_new, p, scal, 0);
    cg_rotate_kernel<<<1, 1>>>(scal);
    std::swap(z_new, z_old);
  }
  GB_CUDA(cudaGetLastError());
  if (stats) *stats = out;
  return out.status;
}

// B = D (identity) on the first n columns of the [n_pad][ldb] matrix
__global__ void unit_rhs_kernel(int n, int n_pad, int ldb, const double* __restrict__ d, float* __restrict__ B) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= int64_t(n_pad) * ldb) return;
  const int row = int(t / ldb), c = int(t - int64_t(row) * ldb);
  B[t] = (row == c && row < n) ? float(d[row]) : 0.f;
}

// inv[row][c] = d[row] X[row][c] for rows and columns < n
__global__ void inverse_store_kernel(int n, int ldb, const double* __restrict__ d, const float* __restrict__ X,
                                     float* __restrict__ inv, int ld) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= int64_t(n) * n) return;
  const int row = int(t / n), c = int(t - int64_t(row) * n);
  inv[int64_t(row) * ld + c] = float(d[row] * double(X[int64_t(row) * ldb + c]));
}

// inv = (inv + inv^T) / 2
__global__ void symmetrize_kernel(int n, float* __restrict__ inv, int ld) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= int64_t(n) * n) return;
  const int i = int(t / n), j = int(t - int64_t(i) * n);
  if (j >= i) return;
  const float a = inv[int64_t(i) * ld + j], b = inv[int64_t(j) * ld + i];
  const float v = 0.5f * (a + b);
  inv[int64_t(i) * ld + j] = v;
  inv[int64_t(j) * ld + i] = v;
}

void DenseSpdSolver::explicit_inverse(float* inv, int ld) {
  if (n_ <= 0) return;
  const int n = n_;
  const int ldb = (n + kRhs - 1) / kRhs * kRhs;
  const int batches = ldb / kRhs;
  const size_t vk = size_t(n_pad_) * ldb;
  mts_.resize(3 * vk);
  static bool configured = false;
  if (!configured) {
    set_smem(reinterpret_cast<const void*>(mfwd_step_kernel), kMsteps);
    set_smem(reinterpret_cast<const void*>(mbwd_step_kernel), kMsteps);
    configured = true;
  }
  float* TB = mts_.get();
  float* TY = TB + vk;
  float* TX = TY + vk;
  unit_rhs_kernel<<<int((int64_t(vk) + 255) / 256), 256>>>(n, n_pad_, ldb, dscale_.get(), TB);
  // every column batch in the same launch (blockIdx.y)
  for (int k = 0; k < nt_; ++k)
    mfwd_step_kernel<<<dim3(nt_ - k, batches), kTsThreads, kMsteps>>>(L_.get(), n_pad_, dinv_.get(), k, kRhs, ldb,
                                                                     TB, TY);
  for (int k = nt_ - 1; k >= 0; --k)
    mbwd_step_kernel<<<dim3(k + 1, batches), kTsThreads, kMsteps>>>(L_.get(), n_pad_, dinv_.get(), k, kRhs, ldb, TY,
                                                                   TX);
  inverse_store_kernel<<<int((int64_t(n) * n + 255) / 256), 256>>>(n, ldb, dscale_.get(), TX, inv, ld);
  symmetrize_kernel<<<int((int64_t(n) * n + 255) / 256), 256>>>(n, inv, ld);
  GB_CUDA(cudaGetLastError());
}

int DenseSpdSolver::inverse_columns(const int* unit, int m, const int* gather, double* out, double tol,
                                    int max_iterations) {
  if (n_ <= 0 || m <= 0) return 0;
  const int n = n_;
  const size_t nk = size_t(n_pad_) * kRhs;
  mv_.resize(6 * nk);
  mts_.resize(4 * nk);
  mscal_.resize(size_t(kRhs) * kNumScal);
  mout_.resize(6 * kRhs);
  munit_.resize(kRhs);
  mgather_.resize(6 * kRhs);
  static bool configured = false;
  if (!configured) {
    set_smem(reinterpret_cast<const void*>(mfwd_step_kernel), kMsteps);
    set_smem(reinterpret_cast<const void*>(mbwd_step_kernel), kMsteps);
    configured = true;
  }
  int failed = 0;
  std::vector<double> s2(size_t(kRhs) * kNumScal), bb(kRhs);
  for (int c0 = 0; c0 < m && !failed; c0 += kRhs) {
    const int K = std::min(kRhs, m - c0);
    const size_t vk = size_t(n_pad_) * K;
    double* X = mv_.get();
    double* R = X + vk;
    double* P = R + vk;
    double* Q = P + vk;
    double* Zn = Q + vk;
    double* Zo = Zn + vk;
    float* RS = mts_.get();
    float* TB = RS + vk;
    float* TY = TB + vk;
    float* TX = TY + vk;
    double* scal = mscal_.get();
    munit_.upload(unit + c0, K);
    mgather_.upload(gather + 6 * size_t(c0), 6 * size_t(K));
    const int ge = int((int64_t(n_pad_) * K + 255) / 256);
    const int gn = int((int64_t(n) * K + 255) / 256);
    // Z = D (L L^T)^-1 RS, K columns
    auto precondition = [&](double* Z) {
      GB_CUDA(cudaMemcpyAsync(TB, RS, vk * sizeof(float), cudaMemcpyDeviceToDevice));
      for (int k = 0; k < nt_; ++k)
        mfwd_step_kernel<<<nt_ - k, kTsThreads, kMsteps>>>(L_.get(), n_pad_, dinv_.get(), k, K, K, TB, TY);
      for (int k = nt_ - 1; k >= 0; --k)
        mbwd_step_kernel<<<k + 1, kTsThreads, kMsteps>>>(L_.get(), n_pad_, dinv_.get(), k, K, K, TY, TX);
      mts_finish_kernel<<<gn, 256>>>(n, K, dscale_.get(), TX, Z);
    };
    mscal_.zero();
    mcg_init_kernel<<<ge, 256>>>(n, n_pad_, K, munit_.get(), dscale_.get(), X, R, RS, scal);
    precondition(Zo);
    mcg_dots_kernel<<<gn, 256>>>(n, K, R, Zo, nullptr, scal);
    mcg_dir_kernel<<<gn, 256>>>(n, K, Zo, P, scal, 1);
    GB_CUDA(cudaMemcpy(s2.data(), scal, sizeof(double) * K * kNumScal, cudaMemcpyDeviceToHost));
    for (int c = 0; c < K; ++c) bb[c] = s2[c * kNumScal + kBb];
    mcg_rotate_kernel<<<1, kRhs>>>(K, scal);
    GB_CUDA(cudaGetLastError());
    bool done = false;
    for (int it = 0; it < max_iterations && !done; ++it) {
      GB_CUDA(cudaMemsetAsync(Q, 0, vk * sizeof(double)));
      msymm_kernel<<<dim3((n + kSymmRows - 1) / kSymmRows, 2), 256>>>(n, K, A_, lda_, P, Q, scal);
      mcg_update_kernel<<<gn, 256>>>(n, K, P, Q, dscale_.get(), X, R, RS, scal);
      GB_CUDA(cudaMemcpy(s2.data(), scal, sizeof(double) * K * kNumScal, cudaMemcpyDeviceToHost));
      done = true;
      for (int c = 0; c < K; ++c) {
        const double pq = s2[c * kNumScal + kPq], rr = s2[c * kNumScal + kRr];
        const double rel = bb[c] > 0.0 ? std::sqrt(rr / bb[c]) : 0.0;
        if (!std::isfinite(rel)) failed = 1;
        if (rel > tol) {
          done = false;
          if (!(pq > 0.0)) failed = 1;  // p . A p <= 0 before convergence: not positive definite
        }
      }
      if (failed) break;
      if (done) break;
      precondition(Zn);
      mcg_dots_kernel<<<gn, 256>>>(n, K, R, Zn, Zo, scal);
      mcg_dir_kernel<<<gn, 256>>>(n, K, Zn, P, scal, 0);
      mcg_rotate_kernel<<<1, kRhs>>>(K, scal);
      std::swap(Zn, Zo);
    }
    if (!done) failed = 1;
    mgather_kernel<<<1, 6 * kRhs>>>(K, mgather_.get(), X, mout_.get());
    GB_CUDA(cudaGetLastError());
    mout_.download(out + 6 * size_t(c0), 6 * size_t(K));
    GB_CUDA(cudaDeviceSynchronize());
  }
  return failed;
}

}  // namespace gbba

// ---------------------------------------------------------------------------
// C ABI (include/gbba.h)
extern "C" int gbba_dense_spd_solve(const double* a, int n, const double* b, double* x, double tol,
                                    int max_refinements, gbba_dense_stats_t* stats) {
  return gbba::guarded([&] {
    if (!a || !b || !x || n < 0 || max_refinements < 1 || !(tol > 0.0))
      throw gbba::ApiError(GBBA_ERR_INVALID_ARGUMENT, "gbba_dense_spd_solve: invalid argument");
    gbba::DeviceArray<double> A, B, X;
    A.upload(a, size_t(n) * n);
    B.upload(b, size_t(n));
    X.resize(size_t(std::max(n, 1)));
    gbba::DenseSpdSolver solver;
    GB_CUDA(cudaDeviceSynchronize());
    const double t0 = gbba::seconds_now();
    gbba::DenseSolveStats st;
    st.status = solver.factor(A.get(), n, n);
    GB_CUDA(cudaDeviceSynchronize());
    const double t1 = gbba::seconds_now();
    if (st.status == 0) solver.solve(B.get(), X.get(), tol, max_refinements, &st);
    GB_CUDA(cudaDeviceSynchronize());
    const double t2 = gbba::seconds_now();
    X.download(x, size_t(n));
    GB_CUDA(cudaDeviceSynchronize());
    if (stats) {
      stats->status = st.status;
      stats->refinements = st.refinements;
      stats->rel_residual = st.rel_residual;
      stats->factor_seconds = t1 - t0;
      stats->solve_seconds = t2 - t1;
    }
  });
}

extern "C" int gbba_dense_gemm_nt(const float* a, const float* b, float* c, int m, int n, int k) {
  return gbba::guarded([&] {
    if (!a || !b || !c || m <= 0 || n <= 0 || k <= 0 || m % 128 || n % 128 || k % 32)
      throw gbba::ApiError(GBBA_ERR_INVALID_ARGUMENT,
                           "gbba_dense_gemm_nt: m, n must be positive multiples of 128 and k of 32");
    gbba::DeviceArray<float> A, B, C;
    gbba::DeviceArray<int> status(1);
    A.upload(a, size_t(m) * k);
    B.upload(b, size_t(n) * k);
    C.resize(size_t(m) * n);
    status.zero();
    gbba::tc_gemm_nt(A.get(), k, B.get(), k, C.get(), n, m, n, k, status.get());
    int st = 0;
    status.download(&st, 1);
    C.download(c, size_t(m) * n);
    GB_CUDA(cudaDeviceSynchronize());
    if (st != 0) throw gbba::ApiError(GBBA_ERR_CUDA, "gbba_dense_gemm_nt: a device wait timed out");
  });
}
