// Test-infrastructure driver: runs the reference's own embedding step
// (jjmmwon/gpumap cpp/src/kernels/embedding_kernel.cuh, compiled in place
// from the installed reference sources) on a published k-NN table and an
// initial embedding read from a file, and writes the embedding it produces,
// so that this build's embedding can be compared with the reference's on the
// same inputs.
//
// Steps, in the reference's own order for a batch of every row
// (impl.cuh:380-475): prepend_self_knn_kernel, compute_fuzzy_graph, then
// run_optimize_layout (maximum weight, trim_graph,
// make_epochs_per_sample_kernel, compute_rounding_factor and its per-epoch
// optimize_batch_kernel loop, seed 42, gamma 1).  Every row is in the batch,
// so the reposition step for unselected rows does not run; no noise is added.
//
// Input  (little endian): int32 n, k, euclidean, n_epochs, negative_sample_rate;
//        float alpha, a, b; uint32 pub_idx[n*(k+1)]; float pub_dist[n*(k+1)];
//        float embedding[n*2].
// Output: float embedding[n*2].
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "kernels/embedding_kernel.cuh"

namespace {

#define CK(x)                                                                       \
  do {                                                                              \
    cudaError_t e_ = (x);                                                           \
    if (e_ != cudaSuccess) {                                                        \
      std::fprintf(stderr, "%s:%d %s\n", __FILE__, __LINE__, cudaGetErrorString(e_)); \
      std::exit(2);                                                                 \
    }                                                                               \
  } while (0)

template <typename T>
void rd(std::FILE *f, T *p, size_t n) {
  if (n && std::fread(p, sizeof(T), n, f) != n) {
    std::fprintf(stderr, "short read\n");
    std::exit(2);
  }
}
template <typename T>
T *dev(size_t n) {
  T *p = nullptr;
  CK(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)));
  return p;
}

}  // namespace

int main(int argc, char **argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: %s in.bin out.bin\n", argv[0]);
    return 1;
  }
  std::FILE *in = std::fopen(argv[1], "rb");
  if (!in) return 1;
  int n, k, eucl, n_epochs, nsr;
  float alpha, a, b;
  rd(in, &n, 1), rd(in, &k, 1), rd(in, &eucl, 1), rd(in, &n_epochs, 1), rd(in, &nsr, 1);
  rd(in, &alpha, 1), rd(in, &a, 1), rd(in, &b, 1);
  const size_t w = (size_t)k + 1;
  std::vector<uint32_t> pidx((size_t)n * w);
  std::vector<float> pdist((size_t)n * w), emb((size_t)n * 2);
  rd(in, pidx.data(), pidx.size());
  rd(in, pdist.data(), pdist.size());
  rd(in, emb.data(), emb.size());
  std::fclose(in);

  cudaStream_t s;
  CK(cudaStreamCreate(&s));
  uint32_t *d_pidx = dev<uint32_t>(pidx.size());
  float *d_pdist = dev<float>(pdist.size());
  float *d_emb = dev<float>(emb.size());
  std::vector<uint32_t> batch(n);
  for (int i = 0; i < n; ++i) batch[i] = (uint32_t)i;
  uint32_t *d_batch = dev<uint32_t>(n);
  CK(cudaMemcpy(d_pidx, pidx.data(), pidx.size() * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_pdist, pdist.data(), pdist.size() * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_emb, emb.data(), emb.size() * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_batch, batch.data(), (size_t)n * 4, cudaMemcpyHostToDevice));

  // embed-time k-NN with self in column 0 (impl.cuh:397-412)
  uint32_t *e_idx = dev<uint32_t>((size_t)n * k);
  float *e_dist = dev<float>((size_t)n * k);
  {
    const int total = n * k, tpb = 256;
    gpumap::prepend_self_knn_kernel<uint32_t><<<(total + tpb - 1) / tpb, tpb, 0, s>>>(
        d_pidx, (int)w, d_pdist, (int)w, e_idx, e_dist, n, k, eucl != 0);
    CK(cudaGetLastError());
  }
  const int max_nnz = 2 * n * k;
  int *cr = dev<int>(max_nnz), *cc = dev<int>(max_nnz);
  float *cv = dev<float>(max_nnz);
  float *sg = dev<float>(n), *rh = dev<float>(n);
  const int nnz = gpumap::compute_fuzzy_graph<uint32_t>(e_idx, k, e_dist, k, n, k, d_batch, n, cr, cc,
                                                        cv, s, sg, rh);
  gpumap::run_optimize_layout(d_emb, n, cr, cc, cv, nnz, alpha, 1.0f, a, b, n_epochs, nsr, 42ULL, s);
  CK(cudaStreamSynchronize(s));
  CK(cudaMemcpy(emb.data(), d_emb, emb.size() * 4, cudaMemcpyDeviceToHost));

  std::FILE *out = std::fopen(argv[2], "wb");
  if (!out) return 1;
  std::fwrite(emb.data(), 4, emb.size(), out);
  std::fclose(out);
  std::printf("nnz %d\n", nnz);
  return 0;
}
