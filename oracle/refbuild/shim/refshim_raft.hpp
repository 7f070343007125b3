// Stand-ins for the handful of RAFT names the reference's sources use
// (containers, views, a copy, warp constants and the error macro), written
// from their names and call signatures only, so that the unmodified reference
// compiles with nvcc for sm_103a without the RAPIDS stack.
//
// Semantics kept: device containers are plain cudaMalloc allocations (RAFT's
// default device resource), host containers are uninitialised host memory,
// pinned containers come from cudaMallocHost, `copy` is one cudaMemcpyAsync
// with cudaMemcpyDefault on the given stream, and RAFT_CUDA_TRY throws a
// std::runtime_error carrying the CUDA error string.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <new>
#include <stdexcept>
#include <string>
#include <utility>

#include "refshim_rmm.hpp"

#ifndef RAFT_CUDA_TRY
#define RAFT_CUDA_TRY(call)                                                      \
  do {                                                                           \
    cudaError_t refshim_status_ = (call);                                        \
    if (refshim_status_ != cudaSuccess) {                                        \
      cudaGetLastError();                                                        \
      throw std::runtime_error(std::string("CUDA error: ") +                     \
                               cudaGetErrorString(refshim_status_) + " at " +    \
                               __FILE__ + ":" + std::to_string(__LINE__));       \
    }                                                                            \
  } while (0)
#endif

namespace raft {

struct row_major {};
struct col_major {};

// The reference only passes a resources object through to the factories.
class resources {
 public:
  resources() = default;
  resources(const resources &) = delete;
  resources &operator=(const resources &) = delete;
};

__host__ __device__ constexpr int warp_size() { return 32; }
__host__ __device__ constexpr unsigned warp_full_mask() { return 0xffffffffu; }

template <typename A, typename B>
__host__ __device__ constexpr auto ceildiv(A a, B b) -> decltype(a + b) {
  return (a + b - 1) / b;
}

template <typename T>
void copy(T *dst, const T *src, std::size_t n, rmm::cuda_stream_view stream) {
  if (n == 0) return;
  RAFT_CUDA_TRY(cudaMemcpyAsync(dst, src, n * sizeof(T), cudaMemcpyDefault, stream.value()));
}

// Non-owning row-major matrix view.
template <typename T, typename I, typename L = row_major>
class device_matrix_view {
 public:
  device_matrix_view() = default;
  __host__ __device__ device_matrix_view(T *p, I rows, I cols) : p_(p), rows_(rows), cols_(cols) {}
  __host__ __device__ T *data_handle() const { return p_; }
  __host__ __device__ I extent(int dim) const { return dim == 0 ? rows_ : cols_; }
  __host__ __device__ std::size_t size() const { return (std::size_t)rows_ * (std::size_t)cols_; }

 private:
  T *p_ = nullptr;
  I rows_ = 0, cols_ = 0;
};

template <typename T, typename I, typename L = row_major>
device_matrix_view<T, I, L> make_device_matrix_view(T *p, I rows, I cols) {
  return device_matrix_view<T, I, L>(p, rows, cols);
}

namespace refshim {

enum class Where { device, host, pinned };

// Owning buffer of n elements of a trivially copyable T, not constructed
// (RAFT's containers leave their storage uninitialised as well).
template <typename T, Where W>
class buffer {
 public:
  buffer() = default;
  explicit buffer(std::size_t n) : n_(n) {
    if (n == 0) return;
    const std::size_t bytes = n * sizeof(T);
    void *p = nullptr;
    if (W == Where::device) {
      RAFT_CUDA_TRY(cudaMalloc(&p, bytes));
    } else if (W == Where::pinned) {
      RAFT_CUDA_TRY(cudaMallocHost(&p, bytes));
    } else {
      p = std::malloc(bytes);
      if (!p) throw std::bad_alloc();
    }
    p_ = static_cast<T *>(p);
  }
  buffer(const buffer &) = delete;
  buffer &operator=(const buffer &) = delete;
  buffer(buffer &&o) noexcept : p_(std::exchange(o.p_, nullptr)), n_(std::exchange(o.n_, 0)) {}
  buffer &operator=(buffer &&o) noexcept {
    if (this != &o) {
      release();
      p_ = std::exchange(o.p_, nullptr);
      n_ = std::exchange(o.n_, 0);
    }
    return *this;
  }
  ~buffer() { release(); }
  T *data() const { return p_; }
  std::size_t size() const { return n_; }

 private:
  void release() {
    if (!p_) return;
    if (W == Where::device) {
      cudaFree(p_);
    } else if (W == Where::pinned) {
      cudaFreeHost(p_);
    } else {
      std::free(p_);
    }
    p_ = nullptr;
  }
  T *p_ = nullptr;
  std::size_t n_ = 0;
};

template <typename T, typename I, Where W>
class matrix {
 public:
  matrix(I rows, I cols) : buf_((std::size_t)rows * (std::size_t)cols), rows_(rows), cols_(cols) {}
  matrix(matrix &&) noexcept = default;
  matrix &operator=(matrix &&) noexcept = default;
  T *data_handle() const { return buf_.data(); }
  I extent(int dim) const { return dim == 0 ? rows_ : cols_; }
  std::size_t size() const { return buf_.size(); }
  device_matrix_view<T, I, row_major> view() const { return {buf_.data(), rows_, cols_}; }

 private:
  buffer<T, W> buf_;
  I rows_, cols_;
};

template <typename T, typename I, Where W>
class vector {
 public:
  explicit vector(I n) : buf_((std::size_t)n), n_(n) {}
  vector(vector &&) noexcept = default;
  vector &operator=(vector &&) noexcept = default;
  T *data_handle() const { return buf_.data(); }
  I extent(int) const { return n_; }
  std::size_t size() const { return buf_.size(); }

 private:
  buffer<T, W> buf_;
  I n_;
};

}  // namespace refshim

template <typename T, typename I = std::size_t, typename L = row_major>
using device_matrix = refshim::matrix<T, I, refshim::Where::device>;
template <typename T, typename I = std::size_t, typename L = row_major>
using host_matrix = refshim::matrix<T, I, refshim::Where::host>;
template <typename T, typename I = std::size_t, typename L = row_major>
using pinned_matrix = refshim::matrix<T, I, refshim::Where::pinned>;
template <typename T, typename I = std::size_t>
using device_vector = refshim::vector<T, I, refshim::Where::device>;
template <typename T, typename I = std::size_t>
using host_vector = refshim::vector<T, I, refshim::Where::host>;
template <typename T, typename I = std::size_t>
using pinned_vector = refshim::vector<T, I, refshim::Where::pinned>;

template <typename T, typename I = std::size_t, typename L = row_major>
device_matrix<T, I, L> make_device_matrix(const resources &, I rows, I cols) {
  return device_matrix<T, I, L>(rows, cols);
}
template <typename T, typename I = std::size_t, typename L = row_major>
host_matrix<T, I, L> make_host_matrix(const resources &, I rows, I cols) {
  return host_matrix<T, I, L>(rows, cols);
}
template <typename T, typename I = std::size_t, typename L = row_major>
host_matrix<T, I, L> make_host_matrix(I rows, I cols) {
  return host_matrix<T, I, L>(rows, cols);
}
template <typename T, typename I = std::size_t, typename L = row_major>
pinned_matrix<T, I, L> make_pinned_matrix(const resources &, I rows, I cols) {
  return pinned_matrix<T, I, L>(rows, cols);
}
template <typename T, typename I = std::size_t>
device_vector<T, I> make_device_vector(const resources &, I n) {
  return device_vector<T, I>(n);
}
template <typename T, typename I = std::size_t>
host_vector<T, I> make_host_vector(const resources &, I n) {
  return host_vector<T, I>(n);
}
template <typename T, typename I = std::size_t>
pinned_vector<T, I> make_pinned_vector(const resources &, I n) {
  return pinned_vector<T, I>(n);
}

}  // namespace raft
