// Post-solve outlier selection on the device, as
// sfm::BAHelpers::RemoveOutliers (ba_helpers.cc:1847-1975) selects it:
//
//   threshold  FIXED: the configured value.  AUTO: over all observations'
//              2D errors e, the componentwise medians m (the element of
//              rank n/2, as std::nth_element at size()/2), the robust
//              deviation s = 1.486 * median_i |e_i - m|, and threshold =
//              auto_ratio * |(m_x + s, m_y + s)|.
//   outlier    |e|^2 > threshold^2, or IRLS weight < weight_threshold.
//   removed    points that lose an observation and keep fewer than two.
//
// The medians are exact: a radix selection over the FP64 bit patterns
// (mapped to order-preserving unsigned keys, 11-bit digits, one histogram
// pass per digit for both error columns at once, the digit found by a
// one-block scan on the device; after the third digit only the keys that
// still match are read) returns the element of the requested rank, so the
// threshold is the one a sort would give.  The whole selection runs
// on the stream without a host synchronization.  Products and sums that decide a
// comparison are rounded without contraction (__dmul_rn / __dadd_rn), as
// the host computes them.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "capi_util.h"
#include "outliers.h"

namespace gbba {
namespace {

constexpr int kDigitBits = 11;
constexpr int kBins = 1 << kDigitBits;

__device__ __forceinline__ uint64_t order_key(double v) {
  const uint64_t b = static_cast<uint64_t>(__double_as_longlong(v));
  return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}

__device__ __forceinline__ double key_to_double(uint64_t k) {
  const uint64_t b = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
  return __longlong_as_double(static_cast<long long>(b));
}

// Radix selection state of one column: the digits fixed so far (prefix
// under mask) and the rank still sought among the keys that match them.
struct SelectState {
  unsigned long long prefix, mask;
  long long rank;
};

// Histogram of one digit of the keys of column c (c < n_cols <= 2) of
// v[i * stride + c] whose higher digits match the column's prefix.
__global__ void digit_histogram_kernel(int64_t n, const double* __restrict__ v, int stride, int n_cols,
                                       const SelectState* __restrict__ st, int shift, uint32_t digit_mask,
                                       unsigned* __restrict__ hist) {
  __shared__ unsigned h[2][kBins];
  for (int b = threadIdx.x; b < n_cols * kBins; b += blockDim.x) h[b / kBins][b % kBins] = 0u;
  __syncthreads();
  const uint64_t p0 = st[0].prefix, m0 = st[0].mask;
  const uint64_t p1 = n_cols > 1 ? st[1].prefix : 0, m1 = n_cols > 1 ? st[1].mask : 0;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const uint64_t k0 = order_key(v[i * stride]);
    if ((k0 & m0) == p0) atomicAdd(&h[0][uint32_t(k0 >> shift) & digit_mask], 1u);
    if (n_cols > 1) {
      const uint64_t k1 = order_key(v[i * stride + 1]);
      if ((k1 & m1) == p1) atomicAdd(&h[1][uint32_t(k1 >> shift) & digit_mask], 1u);
    }
  }
  __syncthreads();
  for (int b = threadIdx.x; b < n_cols * kBins; b += blockDim.x)
    if (h[b / kBins][b % kBins]) atomicAdd(&hist[b], h[b / kBins][b % kBins]);
}

// The same histogram that also copies the keys it counts (those matching the
// column's prefix) to the column's candidate list cand[c * cap ..], with a
// warp-aggregated append; later digits then read only the candidates.
__global__ void digit_histogram_compact_kernel(int64_t n, const double* __restrict__ v, int stride, int n_cols,
                                               const SelectState* __restrict__ st, int shift, uint32_t digit_mask,
                                               unsigned* __restrict__ hist, uint64_t* __restrict__ cand,
                                               int64_t cap, unsigned long long* __restrict__ count) {
  __shared__ unsigned h[2][kBins];
  for (int b = threadIdx.x; b < n_cols * kBins; b += blockDim.x) h[b / kBins][b % kBins] = 0u;
  __syncthreads();
  const unsigned lane = threadIdx.x & 31u;
  const int64_t step = int64_t(gridDim.x) * blockDim.x;
  // i - lane is the same for the whole warp, so the loop is warp-uniform
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i - lane < n; i += step) {
    const bool valid = i < n;
    for (int c = 0; c < n_cols; ++c) {
      const uint64_t k = valid ? order_key(v[i * stride + c]) : 0ull;
      const bool match = valid && (k & st[c].mask) == st[c].prefix;
      if (match) atomicAdd(&h[c][uint32_t(k >> shift) & digit_mask], 1u);
      const unsigned ballot = __ballot_sync(0xffffffffu, match);
      if (ballot) {
        const int leader = __ffs(ballot) - 1;
        unsigned long long base = 0;
        if (int(lane) == leader) base = atomicAdd(&count[c], static_cast<unsigned long long>(__popc(ballot)));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (match) cand[c * cap + int64_t(base) + __popc(ballot & ((1u << lane) - 1u))] = k;
      }
    }
  }
  __syncthreads();
  for (int b = threadIdx.x; b < n_cols * kBins; b += blockDim.x)
    if (h[b / kBins][b % kBins]) atomicAdd(&hist[b], h[b / kBins][b % kBins]);
}

// Histogram of one digit over the candidate keys of each column.
__global__ void candidate_histogram_kernel(const uint64_t* __restrict__ cand, int64_t cap,
                                           const unsigned long long* __restrict__ count, int n_cols,
                                           const SelectState* __restrict__ st, int shift, uint32_t digit_mask,
                                           unsigned* __restrict__ hist) {
  __shared__ unsigned h[2][kBins];
  for (int b = threadIdx.x; b < n_cols * kBins; b += blockDim.x) h[b / kBins][b % kBins] = 0u;
  __syncthreads();
  const int64_t step = int64_t(gridDim.x) * blockDim.x;
  for (int c = 0; c < n_cols; ++c) {
    const int64_t m = int64_t(count[c]);
    const uint64_t p = st[c].prefix, mk = st[c].mask;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < m; i += step) {
      const uint64_t k = cand[c * cap + i];
      if ((k & mk) == p) atomicAdd(&h[c][uint32_t(k >> shift) & digit_mask], 1u);
    }
  }
  __syncthreads();
  for (int b = threadIdx.x; b < n_cols * kBins; b += blockDim.x)
    if (h[b / kBins][b % kBins]) atomicAdd(&hist[b], h[b / kBins][b % kBins]);
}

// The digit of the sought rank in each column's histogram, appended to the
// column's prefix: one block of 256 threads per column, 8 bins a thread, a
// block-wide exclusive scan of the thread sums; the thread whose bins hold
// the rank writes the digit.
constexpr int kSelectThreads = 256;
constexpr int kBinsPerThread = kBins / kSelectThreads;

__global__ void __launch_bounds__(kSelectThreads)
    digit_select_kernel(const unsigned* __restrict__ hist, SelectState* __restrict__ st, int shift,
                        uint32_t digit_mask) {
  const int c = blockIdx.x, t = threadIdx.x;
  const long long rank = st[c].rank;  // read by every thread before the writer's update
  const unsigned* hc = hist + c * kBins;
  long long local[kBinsPerThread];
  long long sum = 0;
#pragma unroll
  for (int k = 0; k < kBinsPerThread; ++k) {
    local[k] = hc[t * kBinsPerThread + k];
    sum += local[k];
  }
  long long incl = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const long long v = __shfl_up_sync(0xffffffffu, incl, o);
    if ((t & 31) >= o) incl += v;
  }
  __shared__ long long warp_sums[kSelectThreads / 32];
  if ((t & 31) == 31) warp_sums[t >> 5] = incl;
  __syncthreads();
  long long excl = incl - sum;
  for (int w = 0; w < (t >> 5); ++w) excl += warp_sums[w];
  long long total = 0;
  for (int w = 0; w < kSelectThreads / 32; ++w) total += warp_sums[w];
  int digit = -1;
  long long cum = excl;
  if (excl <= rank && rank < excl + sum) {
    for (int k = 0; k < kBinsPerThread; ++k) {
      if (cum + local[k] > rank) {
        digit = t * kBinsPerThread + k;
        break;
      }
      cum += local[k];
    }
  } else if (t == kSelectThreads - 1 && rank >= total) {
    digit = 0;  // no key of that rank (cannot happen for rank < n): digit 0, as a sequential scan leaves it
    cum = total;
  }
  if (digit >= 0) {
    st[c].rank = rank - cum;
    st[c].prefix |= static_cast<unsigned long long>(uint32_t(digit) & digit_mask) << shift;
    st[c].mask |= static_cast<unsigned long long>(digit_mask) << shift;
  }
}

// |e_i - m| for the 2D errors, m the selected medians.
__global__ void deviation_kernel(int64_t n, const double* __restrict__ e, int stride,
                                 const SelectState* __restrict__ st, double* __restrict__ dev) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double mx = key_to_double(st[0].prefix), my = key_to_double(st[1].prefix);
  const double dx = __dadd_rn(e[i * stride], -mx);
  const double dy = __dadd_rn(e[i * stride + 1], -my);
  dev[i] = sqrt(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
}

// AUTO threshold = ratio * |(m_x + s, m_y + s)|, s = 1.486 * the median
// deviation; writes the threshold and its square.
__global__ void auto_threshold_kernel(const SelectState* __restrict__ st, double ratio, double* __restrict__ thr) {
  const double mx = key_to_double(st[0].prefix), my = key_to_double(st[1].prefix);
  const double robust_std = __dmul_rn(1.486, key_to_double(st[2].prefix));
  const double ax = __dadd_rn(mx, robust_std), ay = __dadd_rn(my, robust_std);
  const double t = __dmul_rn(ratio, sqrt(__dadd_rn(__dmul_rn(ax, ax), __dmul_rn(ay, ay))));
  thr[0] = t;
  thr[1] = __dmul_rn(t, t);
}

// Adds the warp's count of `pred` to *counter with one atomic (every lane
// of the warp calls it).
__device__ __forceinline__ void warp_count(bool pred, unsigned long long* counter) {
  const unsigned m = __ballot_sync(0xffffffffu, pred);
  if ((threadIdx.x & 31) == 0 && m) atomicAdd(counter, static_cast<unsigned long long>(__popc(m)));
}

// Outlier flags and per-point counts of observations and outliers.  Each
// thread takes kFlagPerThread observations a block width apart (coalesced)
// and issues all of their loads before the first comparison, so a warp has
// that many rows in flight; the per-point counters are plain reductions to
// L2 (2.46M points: 20 MB).  Measured at 14.7M observations: 0.48 ms with
// one observation per thread and the weight read behind the error test,
// 0.23 ms with eight per thread.  The total is counted per warp: one atomic
// on the shared counter per warp.
constexpr int kFlagPerThread = 8;
constexpr int kFlagBlock = 256;

__global__ void __launch_bounds__(kFlagBlock) flag_kernel(int64_t n, const double* __restrict__ e, int stride,
                                                          const double* __restrict__ w,
                                                          const int32_t* __restrict__ obs_point,
                                                          const double* __restrict__ thr, double weight_threshold,
                                                          uint8_t* __restrict__ flags, unsigned* __restrict__ point_obs,
                                                          unsigned* __restrict__ point_out,
                                                          unsigned long long* __restrict__ n_out) {
  const int64_t base = int64_t(blockIdx.x) * (kFlagBlock * kFlagPerThread) + threadIdx.x;
  double x[kFlagPerThread], y[kFlagPerThread], wt[kFlagPerThread];
  int p[kFlagPerThread];
#pragma unroll
  for (int k = 0; k < kFlagPerThread; ++k) {
    const int64_t i = base + int64_t(k) * kFlagBlock;
    p[k] = -1;
    if (i < n) {
      x[k] = e[i * stride];
      y[k] = e[i * stride + 1];
      wt[k] = w[i];
      p[k] = obs_point[i];
    }
  }
  const double thr_sqr = thr[1];
  unsigned n_mine = 0;
#pragma unroll
  for (int k = 0; k < kFlagPerThread; ++k) {
    if (p[k] < 0) continue;
    const int64_t i = base + int64_t(k) * kFlagBlock;
    const double sq = __dadd_rn(__dmul_rn(x[k], x[k]), __dmul_rn(y[k], y[k]));
    const bool out = (sq > thr_sqr) | (wt[k] < weight_threshold);
    flags[i] = out ? 1 : 0;
    atomicAdd(&point_obs[p[k]], 1u);
    if (out) atomicAdd(&point_out[p[k]], 1u);
    n_mine += out ? 1u : 0u;
  }
  unsigned s = n_mine;
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0 && s) atomicAdd(n_out, static_cast<unsigned long long>(s));
}

__global__ void removed_kernel(int64_t n_points, const unsigned* __restrict__ point_obs,
                               const unsigned* __restrict__ point_out, uint8_t* __restrict__ removed,
                               unsigned long long* __restrict__ n_removed) {
  const int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  bool r = false;
  if (p < n_points) {
    r = point_out[p] > 0 && point_obs[p] - point_out[p] < 2;
    removed[p] = r ? 1 : 0;
  }
  warp_count(r, n_removed);
}

// Host arithmetic rounded operation by operation (no fused multiply-add
// contraction), as the device kernels and a plain host restatement round it.
double mul_rn(double a, double b) {
  volatile double r = a * b;
  return r;
}

int grid_for(int64_t n, int block = 256, int cap = 152 * 8) {
  return int(std::max<int64_t>(1, std::min<int64_t>(cap, (n + block - 1) / block)));
}

// Radix selection of the element of rank st[c].rank (0-based, ascending)
// of each column c < n_cols of v[i * stride + c], i < n: six passes of an
// 11-bit digit (the last 9 bits wide), each a histogram and a one-block
// scan on the device, no host synchronization.  The first two passes read
// every row; the third also copies the keys that still match (those that
// share the selected sign, exponent and top mantissa bits: a small set
// unless many values are nearly equal) to the candidate lists
// cand[c * n ..], and the last three read only those.  The selected keys
// are left in st[c].prefix.
void select_ranks(const double* v, int stride, int n_cols, int64_t n, SelectState* st, DeviceArray<unsigned>& hist,
                  uint64_t* cand, unsigned long long* count) {
  int top = 64;
  int pass = 0;
  GB_CUDA(cudaMemsetAsync(count, 0, 2 * sizeof(unsigned long long)));
  while (top > 0) {
    const int width = top >= kDigitBits ? kDigitBits : top;
    const int shift = top - width;
    const uint32_t dmask = (1u << width) - 1u;
    hist.zero();
    if (pass < 2)
      digit_histogram_kernel<<<grid_for(n), 256>>>(n, v, stride, n_cols, st, shift, dmask, hist.get());
    else if (pass == 2)
      digit_histogram_compact_kernel<<<grid_for(n), 256>>>(n, v, stride, n_cols, st, shift, dmask, hist.get(), cand,
                                                           n, count);
    else
      candidate_histogram_kernel<<<grid_for(n), 256>>>(cand, n, count, n_cols, st, shift, dmask, hist.get());
    digit_select_kernel<<<n_cols, kSelectThreads>>>(hist.get(), st, shift, dmask);
    GB_CUDA(cudaGetLastError());
    top = shift;
    ++pass;
  }
}

}  // namespace

OutlierResult find_outliers(const double* errors, int stride, const double* weights, const int32_t* obs_point,
                            int64_t n, int64_t n_points, const OutlierConfig& cfg, uint8_t* flags,
                            uint8_t* point_removed) {
  OutlierResult res;
  if (stride < 2) throw std::invalid_argument("find_outliers: errors need at least two columns");
  for (int64_t p = 0; p < n_points; ++p) point_removed[p] = 0;
  if (n <= 0) return res;
  for (int64_t i = 0; i < n; ++i)
    if (obs_point[i] < 0 || obs_point[i] >= n_points)
      throw std::out_of_range("find_outliers: observation point index out of range");
  DeviceArray<double> e, w, dev;
  DeviceArray<int32_t> op;
  e.upload(errors, size_t(n) * stride);
  w.upload(weights, size_t(n));
  op.upload(obs_point, size_t(n));
  // every buffer is allocated before the timed span starts
  const size_t n_pts = static_cast<size_t>(std::max<int64_t>(1, n_points));
  DeviceArray<double> thr(2);
  DeviceArray<unsigned> hist, pobs(n_pts), pout(n_pts);
  DeviceArray<SelectState> st;
  DeviceArray<uint64_t> cand;                 // AUTO: candidate keys, n per column
  DeviceArray<unsigned long long> ccount(2);  // AUTO: candidates per column
  DeviceArray<uint8_t> f(static_cast<size_t>(n)), rem(n_pts);
  DeviceArray<unsigned long long> counts(2);
  if (cfg.filter_type == 0) {
    const double t[2] = {cfg.fixed_threshold, mul_rn(cfg.fixed_threshold, cfg.fixed_threshold)};
    thr.upload(t, 2);
  } else {
    hist.resize(2 * kBins);
    dev.resize(size_t(n));
    cand.resize(2 * size_t(n));
    const long long mid = static_cast<long long>(n / 2);
    const SelectState init[3] = {{0ull, 0ull, mid}, {0ull, 0ull, mid}, {0ull, 0ull, mid}};
    st.upload(init, 3);
  }
  cudaEvent_t ev[2];
  for (cudaEvent_t& x : ev) GB_CUDA(cudaEventCreate(&x));
  GB_CUDA(cudaEventRecord(ev[0]));
  if (cfg.filter_type != 0) {
    // medians of the two error columns (one pass per digit for both), then
    // the median deviation, all on the device
    select_ranks(e.get(), stride, 2, n, st.get(), hist, cand.get(), ccount.get());
    deviation_kernel<<<int((n + 255) / 256), 256>>>(n, e.get(), stride, st.get(), dev.get());
    GB_CUDA(cudaGetLastError());
    select_ranks(dev.get(), 1, 1, n, st.get() + 2, hist, cand.get(), ccount.get());
    auto_threshold_kernel<<<1, 1>>>(st.get(), cfg.auto_ratio, thr.get());
    GB_CUDA(cudaGetLastError());
  }
  pobs.zero();
  pout.zero();
  counts.zero();
  const int64_t per_block = int64_t(kFlagBlock) * kFlagPerThread;
  flag_kernel<<<int((n + per_block - 1) / per_block), kFlagBlock>>>(n, e.get(), stride, w.get(), op.get(), thr.get(),
                                                                     cfg.weight_threshold, f.get(), pobs.get(),
                                                                     pout.get(), counts.get());
  if (n_points > 0)
    removed_kernel<<<int((n_points + 255) / 256), 256>>>(n_points, pobs.get(), pout.get(), rem.get(),
                                                         counts.get() + 1);
  GB_CUDA(cudaGetLastError());
  GB_CUDA(cudaEventRecord(ev[1]));
  unsigned long long c[2];
  double t[2];
  counts.download(c, 2);
  thr.download(t, 2);
  f.download(flags, size_t(n));
  if (n_points > 0) rem.download(point_removed, size_t(n_points));
  GB_CUDA(cudaDeviceSynchronize());
  float ms = 0.0f;
  GB_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
  for (cudaEvent_t& x : ev) GB_CUDA(cudaEventDestroy(x));
  res.threshold = t[0];
  res.n_outliers = int64_t(c[0]);
  res.n_removed_points = int64_t(c[1]);
  res.device_seconds = 1e-3 * double(ms);
  return res;
}

}  // namespace gbba

extern "C" int gbba_find_outliers(const double* errors, int stride, const double* weights, const int32_t* obs_point,
                                  int64_t n, int64_t n_points, const gbba_outlier_config_t* config, uint8_t* flags,
                                  uint8_t* point_removed, gbba_outlier_result_t* result) {
  return gbba::guarded([&] {
    if (!config || (n > 0 && (!errors || !weights || !obs_point || !flags)) || (n_points > 0 && !point_removed) ||
        n < 0 || n_points < 0 || (config->filter_type != 0 && config->filter_type != 1))
      throw gbba::ApiError(GBBA_ERR_INVALID_ARGUMENT, "gbba_find_outliers: invalid argument");
    gbba::OutlierConfig cfg;
    cfg.filter_type = config->filter_type;
    cfg.fixed_threshold = config->fixed_threshold;
    cfg.auto_ratio = config->auto_ratio;
    cfg.weight_threshold = config->weight_threshold;
    gbba::OutlierResult r;
    try {
      r = gbba::find_outliers(errors, stride, weights, obs_point, n, n_points, cfg, flags, point_removed);
    } catch (const std::out_of_range& e) {
      throw gbba::ApiError(GBBA_ERR_OUT_OF_RANGE, e.what());
    } catch (const std::invalid_argument& e) {
      throw gbba::ApiError(GBBA_ERR_INVALID_ARGUMENT, e.what());
    }
    if (result) {
      result->threshold = r.threshold;
      result->n_outliers = r.n_outliers;
      result->n_removed_points = r.n_removed_points;
      result->device_seconds = r.device_seconds;
    }
  });
}
