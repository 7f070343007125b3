// gm_op_sgd_noalloc: the SGD operator of gm_op_sgd with its scratch in a
// fixed device array instead of cudaMalloc'd buffers.
//
// Who needs it: callers that must not allocate device memory while they run
// -- a host framework whose own memory pool owns the GPU's memory (a
// cudaMalloc from a library beside it can fail or fragment that pool), and
// latency-bound loops where cudaFree's implicit device-wide synchronisation
// would stall every other stream.  Such callers pass only their inputs and
// outputs; the scratch lives in g_sgd_scratch below.
//
// The array is a file-scope __device__ variable: every GPU that loads this
// library holds its 8 MiB (plus 128 bytes) until the process exits.  Host
// code sees the name g_sgd_scratch only as a host-side stand-in, so the
// device address is looked up with cudaGetSymbolAddress, once per device,
// with that device current, on the first call made on it.
#include <cstdint>
#include <mutex>
#include <string>

#include "gm_kernels.h"
#include "../../include/gpumap_gb300_ops.h"

namespace gm {
int set_last_error(int code, const char *msg);
}

namespace {

constexpr int64_t kMaxEdges = GM_SGD_NOALLOC_MAX_EDGES;
constexpr int kMaxDevices = 64;

// Layout: next_s[kMaxEdges] | next_n[kMaxEdges] | 16 int scalars | 16 float scalars.
static __device__ __align__(256) float g_sgd_scratch[2 * kMaxEdges + 32];

std::mutex g_addr_mu;
float *g_addr[kMaxDevices] = {};

// Writes every scalar slot the epoch kernel reads (the rest to zero), so
// nothing from the previous call's contents survives into this one.
__global__ void k_noalloc_scalars(int *iscal, float *fscal, int nnz, int n, float rounding) {
  const int t = threadIdx.x;
  if (t < 16) {
    iscal[t] = t == 2 ? nnz : (t == gm::kIscalN ? n : 0);
    fscal[t] = t == 2 ? rounding : 0.0f;
  }
}

int scratch_address(float **out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return gm::set_last_error(GM_ERR_CUDA, cudaGetErrorString(e));
  }
  if (dev < 0 || dev >= kMaxDevices) return gm::set_last_error(GM_ERR_INVALID, "device ordinal out of range");
  std::lock_guard<std::mutex> g(g_addr_mu);
  if (!g_addr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_sgd_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return gm::set_last_error(GM_ERR_CUDA, (std::string("cudaGetSymbolAddress of the SGD scratch: ") +
                                              cudaGetErrorString(e)).c_str());
    }
    g_addr[dev] = (float *)p;
  }
  *out = g_addr[dev];
  return GM_OK;
}

}  // namespace

extern "C" int gm_op_sgd_noalloc(float *emb, int64_t n, const int32_t *head, const int32_t *tail,
                                 const float *eps, int64_t nnz, float rounding, float alpha0,
                                 float gamma, float a, float b, int32_t n_epochs,
                                 int32_t negative_sample_rate, uint64_t seed, void *stream) {
  if (n < 1 || nnz < 0 || n_epochs < 0) return gm::set_last_error(GM_ERR_INVALID, "bad sizes");
  if (nnz > kMaxEdges)
    return gm::set_last_error(GM_ERR_INVALID,
                              "gm_op_sgd_noalloc: nnz exceeds its fixed scratch of 1048576 edges; "
                              "use gm_op_sgd for larger edge lists");
  if (n > INT32_MAX) return gm::set_last_error(GM_ERR_INVALID, "n exceeds int32 range");
  if ((uintptr_t)emb % 8 != 0) return gm::set_last_error(GM_ERR_INVALID, "emb must be 8-byte aligned");
  float *base = nullptr;
  const int rc = scratch_address(&base);
  if (rc != GM_OK) return rc;
  if (nnz == 0 || n_epochs == 0) return gm::set_last_error(GM_OK, "");
  cudaStream_t s = (cudaStream_t)stream;
  float *next_s = base;
  float *next_n = base + kMaxEdges;
  int *iscal = (int *)(base + 2 * kMaxEdges);
  float *fscal = base + 2 * kMaxEdges + 16;
  k_noalloc_scalars<<<1, 32, 0, s>>>(iscal, fscal, (int)nnz, (int)n, rounding);
  gm::note_launch();
  gm::launch_epoch_init(eps, (int)nnz, negative_sample_rate, next_s, next_n, s);
  gm::launch_sgd(emb, head, tail, eps, next_s, next_n, iscal, fscal, (int)((nnz + 255) / 256), alpha0,
                 gamma, a, b, n_epochs, negative_sample_rate, seed, s);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return gm::set_last_error(GM_ERR_CUDA, cudaGetErrorString(e));
  return gm::set_last_error(GM_OK, "");
}
