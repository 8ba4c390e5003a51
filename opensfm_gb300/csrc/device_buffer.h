// Small RAII helpers for device memory and CUDA error propagation in the
// host layer.  Errors become gbba::CudaError exceptions inside C++; the
// C-ABI boundary converts them to status codes and never throws.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace gbba {

struct CudaError : std::runtime_error {
  explicit CudaError(const std::string& m) : std::runtime_error(m) {}
};

inline void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    throw CudaError(std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e));
  }
}
#define GB_CUDA(call) ::gbba::cuda_check((call), #call)

template <typename T>
class DeviceArray {
 public:
  DeviceArray() = default;
  explicit DeviceArray(size_t n) { resize(n); }
  ~DeviceArray() { release(); }
  DeviceArray(const DeviceArray&) = delete;
  DeviceArray& operator=(const DeviceArray&) = delete;
  DeviceArray(DeviceArray&& o) noexcept : ptr_(o.ptr_), n_(o.n_) {
    o.ptr_ = nullptr;
    o.n_ = 0;
  }
  DeviceArray& operator=(DeviceArray&& o) noexcept {
    if (this != &o) {
      release();
      ptr_ = o.ptr_;
      n_ = o.n_;
      o.ptr_ = nullptr;
      o.n_ = 0;
    }
    return *this;
  }
  void resize(size_t n) {
    if (n == n_) return;
    release();
    if (n) GB_CUDA(cudaMalloc(reinterpret_cast<void**>(&ptr_), n * sizeof(T)));
    n_ = n;
  }
  void release() {
    if (ptr_) cudaFree(ptr_);
    ptr_ = nullptr;
    n_ = 0;
  }
  void upload(const T* h, size_t n, cudaStream_t s = 0) {
    resize(n);
    if (n) GB_CUDA(cudaMemcpyAsync(ptr_, h, n * sizeof(T), cudaMemcpyHostToDevice, s));
  }
  void upload(const std::vector<T>& h, cudaStream_t s = 0) { upload(h.data(), h.size(), s); }
  void download(T* h, size_t n, cudaStream_t s = 0) const {
    if (n) GB_CUDA(cudaMemcpyAsync(h, ptr_, n * sizeof(T), cudaMemcpyDeviceToHost, s));
  }
  void zero(cudaStream_t s = 0) {
    if (n_) GB_CUDA(cudaMemsetAsync(ptr_, 0, n_ * sizeof(T), s));
  }
  T* get() { return ptr_; }
  const T* get() const { return ptr_; }
  size_t size() const { return n_; }
  size_t bytes() const { return n_ * sizeof(T); }

 private:
  T* ptr_ = nullptr;
  size_t n_ = 0;
};

}  // namespace gbba
