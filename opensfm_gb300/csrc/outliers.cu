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
// pass per digit) returns the element of the requested rank, so the
// threshold is the one a sort would give.  Products and sums that decide a
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

double key_value(uint64_t k) {
  const uint64_t b = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
  double v;
  std::memcpy(&v, &b, sizeof(v));
  return v;
}

// Histogram of one digit of the keys of v[i * stride] whose higher bits
// match the selected prefix.
__global__ void digit_histogram_kernel(int64_t n, const double* __restrict__ v, int stride, uint64_t prefix,
                                       uint64_t prefix_mask, int shift, uint32_t digit_mask,
                                       unsigned* __restrict__ hist) {
  __shared__ unsigned h[kBins];
  for (int b = threadIdx.x; b < kBins; b += blockDim.x) h[b] = 0u;
  __syncthreads();
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const uint64_t k = order_key(v[i * stride]);
    if ((k & prefix_mask) == prefix) atomicAdd(&h[uint32_t(k >> shift) & digit_mask], 1u);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < kBins; b += blockDim.x)
    if (h[b]) atomicAdd(&hist[b], h[b]);
}

// |e_i - m| for the 2D errors.
__global__ void deviation_kernel(int64_t n, const double* __restrict__ e, int stride, double mx, double my,
                                 double* __restrict__ dev) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double dx = __dadd_rn(e[i * stride], -mx);
  const double dy = __dadd_rn(e[i * stride + 1], -my);
  dev[i] = sqrt(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
}

// Outlier flags and per-point counts of observations and outliers.
__global__ void flag_kernel(int64_t n, const double* __restrict__ e, int stride, const double* __restrict__ w,
                            const int32_t* __restrict__ obs_point, double thr_sqr, double weight_threshold,
                            uint8_t* __restrict__ flags, unsigned* __restrict__ point_obs,
                            unsigned* __restrict__ point_out, unsigned long long* __restrict__ n_out) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double x = e[i * stride], y = e[i * stride + 1];
  const double sq = __dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y));
  const bool out = sq > thr_sqr || w[i] < weight_threshold;
  flags[i] = out ? 1 : 0;
  const int p = obs_point[i];
  atomicAdd(&point_obs[p], 1u);
  if (out) {
    atomicAdd(&point_out[p], 1u);
    atomicAdd(n_out, 1ull);
  }
}

__global__ void removed_kernel(int64_t n_points, const unsigned* __restrict__ point_obs,
                               const unsigned* __restrict__ point_out, uint8_t* __restrict__ removed,
                               unsigned long long* __restrict__ n_removed) {
  const int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (p >= n_points) return;
  const bool r = point_out[p] > 0 && point_obs[p] - point_out[p] < 2;
  removed[p] = r ? 1 : 0;
  if (r) atomicAdd(n_removed, 1ull);
}

// Host arithmetic rounded operation by operation (no fused multiply-add
// contraction), as the device kernels and a plain host restatement round it.
double mul_rn(double a, double b) {
  volatile double r = a * b;
  return r;
}
double add_rn(double a, double b) {
  volatile double r = a + b;
  return r;
}

int grid_for(int64_t n, int block = 256, int cap = 152 * 8) {
  return int(std::max<int64_t>(1, std::min<int64_t>(cap, (n + block - 1) / block)));
}

// The element of rank `rank` (0-based, ascending) of v[i * stride], i < n.
double select_rank(const double* v, int stride, int64_t n, int64_t rank, DeviceArray<unsigned>& hist) {
  uint64_t prefix = 0, mask = 0;
  std::vector<unsigned> h(kBins);
  int top = 64;
  while (top > 0) {
    const int width = top >= kDigitBits ? kDigitBits : top;
    const int shift = top - width;
    const uint32_t dmask = (1u << width) - 1u;
    hist.zero();
    digit_histogram_kernel<<<grid_for(n), 256>>>(n, v, stride, prefix, mask, shift, dmask, hist.get());
    GB_CUDA(cudaGetLastError());
    hist.download(h.data(), kBins);
    GB_CUDA(cudaDeviceSynchronize());
    int64_t cum = 0;
    uint32_t digit = 0;
    for (uint32_t b = 0; b <= dmask; ++b) {
      if (cum + int64_t(h[b]) > rank) {
        digit = b;
        break;
      }
      cum += h[b];
    }
    rank -= cum;
    prefix |= uint64_t(digit) << shift;
    mask |= uint64_t(dmask) << shift;
    top = shift;
  }
  return key_value(prefix);
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
  cudaEvent_t ev[2];
  for (cudaEvent_t& x : ev) GB_CUDA(cudaEventCreate(&x));
  GB_CUDA(cudaEventRecord(ev[0]));
  double threshold = 1.0;
  if (cfg.filter_type == 0) {
    threshold = cfg.fixed_threshold;
  } else {
    DeviceArray<unsigned> hist(kBins);
    const int64_t mid = n / 2;
    const double mx = select_rank(e.get(), stride, n, mid, hist);
    const double my = select_rank(e.get() + 1, stride, n, mid, hist);
    dev.resize(size_t(n));
    deviation_kernel<<<int((n + 255) / 256), 256>>>(n, e.get(), stride, mx, my, dev.get());
    GB_CUDA(cudaGetLastError());
    const double robust_std = mul_rn(1.486, select_rank(dev.get(), 1, n, mid, hist));
    const double ax = add_rn(mx, robust_std), ay = add_rn(my, robust_std);
    threshold = mul_rn(cfg.auto_ratio, std::sqrt(add_rn(mul_rn(ax, ax), mul_rn(ay, ay))));
  }
  res.threshold = threshold;
  DeviceArray<uint8_t> f{static_cast<size_t>(n)}, rem{static_cast<size_t>(std::max<int64_t>(1, n_points))};
  DeviceArray<unsigned> pobs{static_cast<size_t>(std::max<int64_t>(1, n_points))},
      pout{static_cast<size_t>(std::max<int64_t>(1, n_points))};
  DeviceArray<unsigned long long> counts(2);
  pobs.zero();
  pout.zero();
  counts.zero();
  flag_kernel<<<int((n + 255) / 256), 256>>>(n, e.get(), stride, w.get(), op.get(), mul_rn(threshold, threshold),
                                             cfg.weight_threshold, f.get(), pobs.get(), pout.get(), counts.get());
  if (n_points > 0)
    removed_kernel<<<int((n_points + 255) / 256), 256>>>(n_points, pobs.get(), pout.get(), rem.get(),
                                                         counts.get() + 1);
  GB_CUDA(cudaGetLastError());
  GB_CUDA(cudaEventRecord(ev[1]));
  unsigned long long c[2];
  counts.download(c, 2);
  f.download(flags, size_t(n));
  if (n_points > 0) rem.download(point_removed, size_t(n_points));
  GB_CUDA(cudaDeviceSynchronize());
  float ms = 0.0f;
  GB_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
  for (cudaEvent_t& x : ev) GB_CUDA(cudaEventDestroy(x));
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
