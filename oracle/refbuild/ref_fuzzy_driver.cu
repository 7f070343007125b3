// Test-infrastructure driver: runs the reference's own embed-time fuzzy
// simplicial set and edge scheduling (jjmmwon/gpumap
// cpp/src/kernels/embedding_kernel.cuh, compiled in place from the installed
// reference sources) on a published k-NN table read from a file, and writes
// what they produce, so the CPU oracle can be pinned to the reference.
//
// Steps, in the reference's own order (impl.cuh:380-420, embedding_kernel.cuh
// :650-770): prepend_self_knn_kernel, compute_fuzzy_graph (mean distance,
// smooth_knn_dist, membership strengths, symmetrise and expand), then
// reduce_max_kernel, trim_graph, make_epochs_per_sample_kernel and
// compute_rounding_factor.  No SGD is run.
//
// Input  (little endian): int32 n, k, euclidean, nb, n_epochs; float alpha;
//        uint32 pub_idx[n*(k+1)]; float pub_dist[n*(k+1)]; int32 batch[nb].
// Output: int32 nnz, extras, nnz_trim; float max_w, rounding;
//         float sigma[n], rho[n]; int32 coo_row[nnz], coo_col[nnz];
//         float coo_val[nnz]; int32 t_row[nnz_trim], t_col[nnz_trim];
//         float t_eps[nnz_trim].
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
void wr(std::FILE *f, const T *p, size_t n) {
  if (n) std::fwrite(p, sizeof(T), n, f);
}
template <typename T>
T *dev(size_t n) {
  T *p = nullptr;
  CK(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)));
  return p;
}
template <typename T>
std::vector<T> back(const T *d, size_t n) {
  std::vector<T> h(n);
  if (n) CK(cudaMemcpy(h.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost));
  return h;
}

}  // namespace

int main(int argc, char **argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: %s in.bin out.bin\n", argv[0]);
    return 1;
  }
  std::FILE *in = std::fopen(argv[1], "rb");
  if (!in) return 1;
  int n, k, eucl, nb, n_epochs;
  float alpha;
  rd(in, &n, 1), rd(in, &k, 1), rd(in, &eucl, 1), rd(in, &nb, 1), rd(in, &n_epochs, 1);
  rd(in, &alpha, 1);
  const size_t w = (size_t)k + 1;
  std::vector<uint32_t> pidx((size_t)n * w);
  std::vector<float> pdist((size_t)n * w);
  std::vector<uint32_t> batch(nb);
  rd(in, pidx.data(), pidx.size());
  rd(in, pdist.data(), pdist.size());
  rd(in, batch.data(), batch.size());
  std::fclose(in);

  cudaStream_t s;
  CK(cudaStreamCreate(&s));
  uint32_t *d_pidx = dev<uint32_t>(pidx.size());
  float *d_pdist = dev<float>(pdist.size());
  uint32_t *d_batch = dev<uint32_t>(nb);
  CK(cudaMemcpy(d_pidx, pidx.data(), pidx.size() * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_pdist, pdist.data(), pdist.size() * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_batch, batch.data(), (size_t)nb * 4, cudaMemcpyHostToDevice));

  // embed-time k-NN with self in column 0 (impl.cuh:397-412)
  uint32_t *e_idx = dev<uint32_t>((size_t)n * k);
  float *e_dist = dev<float>((size_t)n * k);
  {
    const int total = n * k, tpb = 256;
    gpumap::prepend_self_knn_kernel<uint32_t><<<(total + tpb - 1) / tpb, tpb, 0, s>>>(
        d_pidx, (int)w, d_pdist, (int)w, e_idx, e_dist, n, k, eucl != 0);
    CK(cudaGetLastError());
  }
  const int max_nnz = 2 * nb * k;
  int *cr = dev<int>(max_nnz), *cc = dev<int>(max_nnz);
  float *cv = dev<float>(max_nnz);
  float *sg = dev<float>(n), *rh = dev<float>(n);
  const int nnz = gpumap::compute_fuzzy_graph<uint32_t>(e_idx, k, e_dist, k, n, k, d_batch, nb, cr, cc,
                                                        cv, s, sg, rh);
  CK(cudaStreamSynchronize(s));
  std::vector<int> h_cr = back(cr, nnz), h_cc = back(cc, nnz);
  std::vector<float> h_cv = back(cv, nnz), h_sg = back(sg, n), h_rh = back(rh, n);

  // scheduling, the first steps of run_optimize_layout (embedding_kernel.cuh:726-781)
  float max_w = 0.0f, rounding = 1.0f;
  int nnz2 = 0;
  std::vector<int> h_tr, h_tc;
  std::vector<float> h_te;
  if (nnz > 0) {
    const int tpb = 256;
    float *d_max = dev<float>(1);
    CK(cudaMemsetAsync(d_max, 0, 4, s));
    gpumap::reduce_max_kernel<<<(nnz + tpb - 1) / tpb, tpb, tpb * sizeof(float), s>>>(cv, nnz, d_max);
    CK(cudaMemcpyAsync(&max_w, d_max, 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (max_w > 0.0f) {
      nnz2 = gpumap::trim_graph(cr, cc, cv, nnz, max_w, n_epochs, s);
      if (nnz2 > 0) {
        gpumap::make_epochs_per_sample_kernel<<<(nnz2 + tpb - 1) / tpb, tpb, 0, s>>>(cv, nnz2, max_w,
                                                                                    n_epochs);
        rounding = gpumap::compute_rounding_factor(cr, nnz2, n, alpha, s);
      }
    }
    CK(cudaStreamSynchronize(s));
    h_tr = back(cr, nnz2), h_tc = back(cc, nnz2), h_te = back(cv, nnz2);
  }
  const int extras = nnz - nb * k;

  std::FILE *out = std::fopen(argv[2], "wb");
  if (!out) return 1;
  wr(out, &nnz, 1), wr(out, &extras, 1), wr(out, &nnz2, 1), wr(out, &max_w, 1), wr(out, &rounding, 1);
  wr(out, h_sg.data(), n), wr(out, h_rh.data(), n);
  wr(out, h_cr.data(), nnz), wr(out, h_cc.data(), nnz), wr(out, h_cv.data(), nnz);
  wr(out, h_tr.data(), nnz2), wr(out, h_tc.data(), nnz2), wr(out, h_te.data(), nnz2);
  std::fclose(out);
  std::printf("nnz %d extras %d trimmed %d max_w %g rounding %g\n", nnz, extras, nnz2, max_w, rounding);
  return 0;
}
