// Explicit sparse Hamiltonian (the reference's build_matrix path):
// POLYQUANT_DETSET::create_ham (src/ci/detset/explicit_ham.cpp:51-84) with
// single_species_create_ham (explicit_ham_singleparticle.cpp) assembles the
// upper triangle of H as an Eigen row-major sparse matrix from the same
// Slater-Condon elements, drops exact zeros, prunes |H_IJ| <= threshold when a
// screening threshold is set, and the solver multiplies with
// Spectra::SparseSymMatProd (epci.cpp:623-668).
//
// Here the matrix is built on the device in CSR with both triangles (rows are
// gathered without atomics): one thread per determinant counts its kept
// connections, a host prefix sum gives the row offsets, and a second pass
// writes (column, value).  The elements come from the shared connection
// enumerator (ci_conn.cuh).  sigma with the explicit matrix is a warp-per-row
// gather over the interleaved vectors.  pq_ci_ham_csr exports the reference's
// layout (upper triangle with the diagonal, columns ascending) or the full
// matrix.  FP64.  A two-species (electron-positron) space uses the same
// count/fill passes over the product-space enumerator of ci_two.cu
// (two_species_create_ham, explicit_ham_mixedparticle.cpp:190-553).
#include <algorithm>
#include <numeric>

#include "ci_conn.cuh"
#include "pq_internal.h"

namespace pq {

__device__ __forceinline__ bool keep_elem(int64_t J, int64_t I, double v, double thr) {
  if (J < 0) return false;
  if (thr > 0.0) return fabs(v) > thr;
  return J == I || v != 0.0;
}

// grid (alpha strings, beta blocks of 128): thread <-> determinant (ia, ib)
template <bool FILL>
__global__ void __launch_bounds__(128) ham_rows_kernel(ConnArgs a, int na, double thr, int32_t *cnt,
                                                       const int64_t *row_ptr, int32_t *col, double *val) {
  const int ia = blockIdx.x;
  if (ia >= na) return;
  for (int ib = blockIdx.y * blockDim.x + threadIdx.x; ib < a.rowlen[ia]; ib += gridDim.y * blockDim.x) {
    const ConnRow r = conn_row(a, ia, ib);
    const int64_t tot = r.total();
    int64_t w = FILL ? row_ptr[r.I] : 0;
    int32_t c = 0;
    for (int64_t t = 0; t < tot; t++) {
      double v;
      const int64_t J = conn_elem(a, r, t, &v);
      if (!keep_elem(J, r.I, v, thr)) continue;
      if (FILL) {
        col[w] = (int32_t)J;
        val[w] = v;
        w++;
      } else {
        c++;
      }
    }
    if (!FILL) cnt[r.I] = c;
  }
}

// Y[I][v] = sum_k val[k] X[col[k]][v], warp per row, interleaved vectors (nvp per det)
template <int NV>
__global__ void __launch_bounds__(256) ham_spmv_kernel(const int64_t *row_ptr, const int32_t *col, const double *val,
                                                       int64_t n, const double *X, double *Y) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t I = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); I < n; I += warps) {
    double acc[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) acc[v] = 0.0;
    for (int64_t k = row_ptr[I] + lane; k < row_ptr[I + 1]; k += 32) {
      const double h = val[k];
      const double *x = X + (int64_t)col[k] * NV;
#pragma unroll
      for (int v = 0; v < NV; v++) acc[v] += h * x[v];
    }
#pragma unroll
    for (int v = 0; v < NV; v++)
      for (int o = 16; o; o >>= 1) acc[v] += __shfl_xor_sync(0xffffffffu, acc[v], o);
    if (lane == 0)
#pragma unroll
      for (int v = 0; v < NV; v++) Y[I * NV + v] = acc[v];
  }
}

pq_status ci_ham_spmv(pq_ci_handle *h, const void *X, void *Y, int nvp) {
  const int64_t n = h->n_dets;
  const unsigned grid = (unsigned)std::min<int64_t>((n + 7) / 8, 152 * 64);
  const int64_t *rp = h->d_hrow.as<int64_t>();
  const int32_t *cl = h->d_hcol.as<int32_t>();
  const double *vl = h->d_hval.as<double>();
  if (nvp == 1)
    ham_spmv_kernel<1><<<grid, 256, 0, h->stream>>>(rp, cl, vl, n, (const double *)X, (double *)Y);
  else if (nvp == 2)
    ham_spmv_kernel<2><<<grid, 256, 0, h->stream>>>(rp, cl, vl, n, (const double *)X, (double *)Y);
  else if (nvp == 3)
    ham_spmv_kernel<3><<<grid, 256, 0, h->stream>>>(rp, cl, vl, n, (const double *)X, (double *)Y);
  else if (nvp == 4)
    ham_spmv_kernel<4><<<grid, 256, 0, h->stream>>>(rp, cl, vl, n, (const double *)X, (double *)Y);
  else {
    set_error("explicit sigma: %d interleaved vectors", nvp);
    return PQ_ERR_ARG;
  }
  PQ_CUDA_TRY(cudaGetLastError());
  return PQ_OK;
}

static pq_status ham_build(pq_ci_handle *h, double thr) {
  if (h->n_dets > 0x7fffffffLL) {
    set_error("pq_ci_ham_build: %lld determinants exceed 32-bit column indices", (long long)h->n_dets);
    return PQ_ERR_ARG;
  }
  const int64_t n = h->n_dets;
  cudaStream_t st = h->stream;
  const bool two = h->n_species == 2;
  const ConnArgs a = two ? ConnArgs{} : make_conn_args(h);
  const int na = (int)h->rowlen.size();
  const int maxlen = *std::max_element(h->rowlen.begin(), h->rowlen.end());
  const dim3 grid((unsigned)na, (unsigned)std::min((maxlen + 127) / 128, 65535));
  DevBuf dcnt;
  PQ_TRY(dcnt.alloc(sizeof(int32_t) * (n + 1)));
  if (two) {
    PQ_TRY(ci_ham_rows2(h, thr, dcnt.as<int32_t>(), nullptr, nullptr, nullptr));
  } else {
    ham_rows_kernel<false><<<grid, 128, 0, st>>>(a, na, thr, dcnt.as<int32_t>(), nullptr, nullptr, nullptr);
    PQ_CUDA_TRY(cudaGetLastError());
  }
  std::vector<int32_t> cnt(n);
  PQ_CUDA_TRY(cudaMemcpyAsync(cnt.data(), dcnt.ptr, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st));
  PQ_CUDA_TRY(cudaStreamSynchronize(st));
  std::vector<int64_t> rp(n + 1, 0);
  for (int64_t i = 0; i < n; i++) rp[i + 1] = rp[i] + cnt[i];
  const int64_t nnz = rp[n];
  PQ_TRY(upload(h->d_hrow, rp, st));
  PQ_TRY(h->d_hcol.alloc(sizeof(int32_t) * (nnz + 1)));
  PQ_TRY(h->d_hval.alloc(sizeof(double) * (nnz + 1)));
  if (two) {
    PQ_TRY(ci_ham_rows2(h, thr, nullptr, h->d_hrow.as<int64_t>(), h->d_hcol.as<int32_t>(), h->d_hval.as<double>()));
  } else {
    ham_rows_kernel<true><<<grid, 128, 0, st>>>(a, na, thr, nullptr, h->d_hrow.as<int64_t>(),
                                                h->d_hcol.as<int32_t>(), h->d_hval.as<double>());
    PQ_CUDA_TRY(cudaGetLastError());
  }
  PQ_CUDA_TRY(cudaStreamSynchronize(st));
  h->h_nnz = nnz;
  return PQ_OK;
}

}  // namespace pq

using namespace pq;

extern "C" {

pq_status pq_ci_ham_build(pq_ci_handle *h, double screening_threshold, int32_t use_for_sigma, int64_t *nnz) {
  clear_error();
  if (!h || screening_threshold < 0.0) {
    set_error("pq_ci_ham_build: bad arguments");
    return PQ_ERR_ARG;
  }
  h->use_explicit = false;
  PQ_TRY(ham_build(h, screening_threshold));
  h->use_explicit = use_for_sigma != 0;
  if (nnz) *nnz = h->h_nnz;
  return PQ_OK;
}

pq_status pq_ci_ham_release(pq_ci_handle *h) {
  if (!h) return PQ_OK;
  cudaStreamSynchronize(h->stream);
  h->use_explicit = false;
  h->h_nnz = 0;
  h->d_hrow.release();
  h->d_hcol.release();
  h->d_hval.release();
  return PQ_OK;
}

// Host copy of the explicit matrix: upper != 0 gives the reference's layout
// (upper triangle with the diagonal, row-major, columns ascending), else the
// full symmetric matrix.  Pass NULL arrays to query *nnz only.
pq_status pq_ci_ham_csr(pq_ci_handle *h, int32_t upper, int64_t *nnz, int64_t *row_ptr, int32_t *col, double *val) {
  clear_error();
  if (!h || !nnz) {
    set_error("pq_ci_ham_csr: NULL argument");
    return PQ_ERR_ARG;
  }
  if (!h->d_hrow.ptr) {
    set_error("pq_ci_ham_csr: call pq_ci_ham_build first");
    return PQ_ERR_STATE;
  }
  const int64_t n = h->n_dets, m = h->h_nnz;
  std::vector<int64_t> rp(n + 1);
  std::vector<int32_t> cl(m);
  std::vector<double> vl(m);
  PQ_CUDA_TRY(cudaMemcpyAsync(rp.data(), h->d_hrow.ptr, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost, h->stream));
  PQ_CUDA_TRY(cudaMemcpyAsync(cl.data(), h->d_hcol.ptr, sizeof(int32_t) * m, cudaMemcpyDeviceToHost, h->stream));
  PQ_CUDA_TRY(cudaMemcpyAsync(vl.data(), h->d_hval.ptr, sizeof(double) * m, cudaMemcpyDeviceToHost, h->stream));
  PQ_CUDA_TRY(cudaStreamSynchronize(h->stream));
  int64_t k = 0;
  std::vector<std::pair<int32_t, double>> row;
  if (row_ptr) row_ptr[0] = 0;
  for (int64_t i = 0; i < n; i++) {
    row.clear();
    for (int64_t e = rp[i]; e < rp[i + 1]; e++)
      if (!upper || cl[e] >= i) row.emplace_back(cl[e], vl[e]);
    std::sort(row.begin(), row.end(), [](const auto &x, const auto &y) { return x.first < y.first; });
    if (col && val)
      for (size_t e = 0; e < row.size(); e++) {
        col[k + e] = row[e].first;
        val[k + e] = row[e].second;
      }
    k += (int64_t)row.size();
    if (row_ptr) row_ptr[i + 1] = k;
  }
  *nnz = k;
  return PQ_OK;
}

}  // extern "C"
