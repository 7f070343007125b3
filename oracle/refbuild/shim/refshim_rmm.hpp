// Stand-ins for the RMM names the reference's sources use, written from
// their names and call signatures only.  RMM's default device resource is a
// plain cudaMalloc / cudaFree resource, so device_uvector and device_scalar
// allocate with cudaMalloc and free with cudaFree (which synchronises the
// device), as the reference does when no pool resource is installed.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <new>
#include <stdexcept>
#include <string>
#include <utility>

namespace rmm {

namespace refshim {
inline void check(cudaError_t e, const char *what) {
  if (e != cudaSuccess) {
    cudaGetLastError();
    if (e == cudaErrorMemoryAllocation) throw std::bad_alloc();
    throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
  }
}
}  // namespace refshim

class cuda_stream_view {
 public:
  constexpr cuda_stream_view() = default;
  constexpr cuda_stream_view(cudaStream_t s) : s_(s) {}
  constexpr cudaStream_t value() const { return s_; }
  constexpr operator cudaStream_t() const { return s_; }

 private:
  cudaStream_t s_ = nullptr;
};

inline constexpr cuda_stream_view cuda_stream_default{};

template <typename T>
class device_uvector {
 public:
  device_uvector(std::size_t n, cuda_stream_view) : n_(n) {
    if (n) refshim::check(cudaMalloc(&p_, n * sizeof(T)), "rmm::device_uvector");
  }
  device_uvector(const device_uvector &) = delete;
  device_uvector &operator=(const device_uvector &) = delete;
  device_uvector(device_uvector &&o) noexcept
      : p_(std::exchange(o.p_, nullptr)), n_(std::exchange(o.n_, 0)) {}
  device_uvector &operator=(device_uvector &&o) noexcept {
    if (this != &o) {
      release();
      p_ = std::exchange(o.p_, nullptr);
      n_ = std::exchange(o.n_, 0);
    }
    return *this;
  }
  ~device_uvector() { release(); }
  T *data() { return p_; }
  const T *data() const { return p_; }
  std::size_t size() const { return n_; }

 private:
  void release() {
    if (p_) cudaFree(p_);
    p_ = nullptr;
  }
  T *p_ = nullptr;
  std::size_t n_ = 0;
};

// One device element; the reference constructs every scalar with a zero
// value and reads it back with explicit copies.
template <typename T>
class device_scalar {
 public:
  device_scalar(T v, cuda_stream_view s) : init_(v) {
    refshim::check(cudaMalloc(&p_, sizeof(T)), "rmm::device_scalar");
    bool zero = true;
    const unsigned char *b = reinterpret_cast<const unsigned char *>(&init_);
    for (std::size_t i = 0; i < sizeof(T); ++i) zero = zero && b[i] == 0;
    if (zero) {
      // a zero value is set with a stream-ordered memset (no host sync)
      refshim::check(cudaMemsetAsync(p_, 0, sizeof(T), s.value()), "rmm::device_scalar");
    } else {
      refshim::check(cudaMemcpyAsync(p_, &init_, sizeof(T), cudaMemcpyHostToDevice, s.value()),
                     "rmm::device_scalar");
      // the host value must stay readable until the copy runs
      refshim::check(cudaStreamSynchronize(s.value()), "rmm::device_scalar");
    }
  }
  device_scalar(const device_scalar &) = delete;
  device_scalar &operator=(const device_scalar &) = delete;
  ~device_scalar() {
    if (p_) cudaFree(p_);
  }
  T *data() { return p_; }
  const T *data() const { return p_; }
  T value(cuda_stream_view s) const {
    T out{};
    refshim::check(cudaMemcpyAsync(&out, p_, sizeof(T), cudaMemcpyDeviceToHost, s.value()),
                   "rmm::device_scalar::value");
    refshim::check(cudaStreamSynchronize(s.value()), "rmm::device_scalar::value");
    return out;
  }

 private:
  T *p_ = nullptr;
  T init_{};
};

namespace mr {
class device_memory_resource {};
inline device_memory_resource *get_current_device_resource() {
  static device_memory_resource r;
  return &r;
}
}  // namespace mr

}  // namespace rmm
