// Single Hamiltonian elements H_IJ = <I|H|J> of the determinant space.
//
// Reference: POLYQUANT_DETSET::operator()(i, j) (src/ci/determinant_set.hpp:139)
// returns Slater_Condon(i, j) (src/ci/detset/slater_condon.cpp:4-100) for any
// pair, whatever an explicit matrix built by create_ham may have pruned
// (explicit_ham.cpp:79).  Here an element is found among the connections of
// determinant I, enumerated exactly as the sigma kernels and the explicit
// matrix enumerate them (ci_conn.cuh for one species, two_conn_visit in
// ci_two.cu for two), so it is exact FP64 and independent of any screening.
// One warp per pair for one species (the connection list of one determinant
// is walked lane-strided), one thread per pair for two species.
#include <algorithm>

#include "ci_conn.cuh"
#include "pq_internal.h"

namespace pq {

__global__ void elements_one_kernel(ConnArgs a, int64_t n, const int32_t *ia, const int32_t *ib, const int64_t *J,
                                    double *out) {
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= n) return;  // whole warps leave together (blockDim is a multiple of 32)
  const ConnRow r = conn_row(a, ia[w], ib[w]);
  const int64_t tot = r.total(), target = J[w];
  double found = 0.0;
  bool hit = false;
  for (int64_t t = lane; t < tot; t += 32) {
    double v;
    if (conn_elem(a, r, t, &v) == target) {
      found = v;
      hit = true;
    }
  }
  const unsigned m = __ballot_sync(0xffffffffu, hit);
  if (m) found = __shfl_sync(0xffffffffu, found, __ffs(m) - 1);
  if (lane == 0) out[w] = m ? found : 0.0;
}

pq_status ci_elements(pq_ci_handle *h, int64_t n, const int64_t *I, const int64_t *J, double *out) {
  for (int64_t k = 0; k < n; k++)
    if (I[k] < 0 || I[k] >= h->n_dets || J[k] < 0 || J[k] >= h->n_dets) {
      set_error("pq_ci_elements: pair %lld = (%lld, %lld) outside 0..%lld", (long long)k, (long long)I[k],
                (long long)J[k], (long long)h->n_dets - 1);
      return PQ_ERR_ARG;
    }
  if (n == 0) return PQ_OK;
  cudaStream_t st = h->stream;
  std::vector<int64_t> vi(I, I + n), vj(J, J + n);
  DevBuf dI, dJ, dout;
  PQ_TRY(upload(dJ, vj, st));
  PQ_TRY(dout.alloc(sizeof(double) * (size_t)n));
  if (h->n_species == 2) {
    std::vector<int32_t> t4((size_t)4 * n);
    for (int64_t k = 0; k < n; k++) ci_unfold2_one(h, I[k], t4.data() + 4 * k);
    DevBuf dt;
    PQ_TRY(upload(dt, t4, st));
    PQ_TRY(upload(dI, vi, st));
    PQ_TRY(ci_elements2(h, n, dt.as<int32_t>(), dI.as<int64_t>(), dJ.as<int64_t>(), dout.as<double>()));
    PQ_CUDA_TRY(cudaMemcpyAsync(out, dout.ptr, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, st));
    PQ_CUDA_TRY(cudaStreamSynchronize(st));  // the index buffers are freed on return
    return PQ_OK;
  }
  // one species: determinant I = rowoff[ia] + ib
  std::vector<int32_t> ia(n), ib(n);
  for (int64_t k = 0; k < n; k++) {
    const int64_t r = (int64_t)(std::upper_bound(h->rowoff.begin(), h->rowoff.end(), I[k]) - h->rowoff.begin()) - 1;
    ia[k] = (int32_t)r;
    ib[k] = (int32_t)(I[k] - h->rowoff[r]);
  }
  DevBuf dia, dib;
  PQ_TRY(upload(dia, ia, st));
  PQ_TRY(upload(dib, ib, st));
  const ConnArgs a = make_conn_args(h);
  const int64_t threads = 32 * n;
  elements_one_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(a, n, dia.as<int32_t>(), dib.as<int32_t>(),
                                                                       dJ.as<int64_t>(), dout.as<double>());
  PQ_CUDA_TRY(cudaGetLastError());
  PQ_CUDA_TRY(cudaMemcpyAsync(out, dout.ptr, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, st));
  PQ_CUDA_TRY(cudaStreamSynchronize(st));
  return PQ_OK;
}

}  // namespace pq

using namespace pq;

extern "C" {

pq_status pq_ci_elements(pq_ci_handle *h, int64_t n, const int64_t *I, const int64_t *J, double *out) {
  clear_error();
  if (!h || n < 0 || (n > 0 && (!I || !J || !out))) {
    set_error("pq_ci_elements: NULL argument or negative count");
    return PQ_ERR_ARG;
  }
  if (n > (int64_t)1 << 26) {
    set_error("pq_ci_elements: %lld pairs in one call (at most 2^26)", (long long)n);
    return PQ_ERR_ARG;
  }
  return ci_elements(h, n, I, J, out);
}

pq_status pq_ci_element(pq_ci_handle *h, int64_t i, int64_t j, double *out) {
  clear_error();
  if (!h || !out) {
    set_error("pq_ci_element: NULL argument");
    return PQ_ERR_ARG;
  }
  return ci_elements(h, 1, &i, &j, out);
}

}  // extern "C"
