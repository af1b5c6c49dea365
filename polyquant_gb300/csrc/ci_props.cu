// Properties of CI vectors on the device (one species): <S^2> of each state
// and the one-particle reduced density matrix of one state and spin.
//
// <S^2> follows POLYQUANT_DETSET::evaluate_s2 (src/ci/detset/s2.cpp:4-123):
// diagonal n_a + s_z (s_z - 1) from the open shells of each determinant
// (n_a open-shell alpha electrons, s_z = n_a - n_open / 2), and for every
// alpha single h_a -> p_a paired with the beta single p_a -> h_a (a spin
// flip) the term -phase_a phase_b C_I C_J.
// The 1-RDM follows create_1rdm (src/ci/detset/rdm1.cpp:4-72): C_I^2 on the
// occupied orbitals of the chosen spin, and phase C_I C_J on (k, l) and
// (l, k) for each single of that spin between I and an earlier J (hole k in
// I, particle l).
// Thread <-> determinant (grid: alpha strings x beta blocks), per-block
// reduction in shared memory, then one atomic per block and entry.
#include <algorithm>

#include "ci_conn.cuh"
#include "pq_internal.h"

namespace pq {

constexpr int PROP_THREADS = 128;
constexpr int S2_MAXV = 8;

__global__ void __launch_bounds__(PROP_THREADS) s2_kernel(ConnArgs a, int na, const double *C, int64_t ldc, int nvec,
                                                          double *out) {
  __shared__ double red[S2_MAXV][PROP_THREADS / 32];
  const int ia = blockIdx.x;
  double acc[S2_MAXV];
#pragma unroll
  for (int v = 0; v < S2_MAXV; v++) acc[v] = 0.0;
  for (int ib = blockIdx.y * blockDim.x + threadIdx.x; ia < na && ib < a.rowlen[ia]; ib += gridDim.y * blockDim.x) {
    const ConnRow r = conn_row(a, ia, ib);
    double cI[S2_MAXV];
#pragma unroll
    for (int v = 0; v < S2_MAXV; v++) cI[v] = v < nvec ? C[r.I + v * ldc] : 0.0;
    const uint64_t open = r.am ^ r.bm;
    const int n_open = __popcll(open), n_a = __popcll(open & r.am);
    const double sz = n_a - 0.5 * n_open;
    const double d = n_a + sz * (sz - 1.0);
#pragma unroll
    for (int v = 0; v < S2_MAXV; v++) acc[v] += cI[v] * cI[v] * d;
    for (int s = 0; s < r.n1a; s++) {
      const int Ja = a.a1_J[r.a1b + s], infa = a.a1_info[r.a1b + s];
      const uint64_t jam = a.astr[Ja];
      const int ha = __ffsll((long long)(r.am & ~jam)) - 1, pa = __ffsll((long long)(jam & ~r.am)) - 1;
      if (!((r.bm >> pa) & 1ULL) || ((r.bm >> ha) & 1ULL)) continue;
      const uint64_t jbm = r.bm ^ (1ULL << pa) ^ (1ULL << ha);
      for (int q = 0; q < r.n1b; q++) {
        const int Jb = a.b1_J[r.b1b + q];
        if (a.bstr[Jb] != jbm) continue;
        if (Jb < a.rowlen[Ja]) {
          const int64_t J = a.rowoff[Ja] + Jb;
          const double ph = ((infa ^ a.b1_info[r.b1b + q]) & 1) ? -1.0 : 1.0;
#pragma unroll
          for (int v = 0; v < S2_MAXV; v++)
            if (v < nvec) acc[v] -= ph * cI[v] * C[J + v * ldc];
        }
        break;
      }
    }
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int v = 0; v < S2_MAXV; v++) {
    double x = acc[v];
    for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) red[v][w] = x;
  }
  __syncthreads();
  if (threadIdx.x < nvec) {
    double x = 0.0;
    for (int i = 0; i < PROP_THREADS / 32; i++) x += red[threadIdx.x][i];
    atomicAdd(out + threadIdx.x, x);
  }
}

// rdm[k + l * n] (column-major n x n), spin 0 = alpha, 1 = beta
__global__ void __launch_bounds__(PROP_THREADS) rdm1_kernel(ConnArgs a, int na, int n, int spin, const double *C,
                                                            double *rdm) {
  extern __shared__ double acc[];  // n x n
  for (int i = threadIdx.x; i < n * n; i += blockDim.x) acc[i] = 0.0;
  __syncthreads();
  const int ia = blockIdx.x;
  for (int ib = blockIdx.y * blockDim.x + threadIdx.x; ia < na && ib < a.rowlen[ia]; ib += gridDim.y * blockDim.x) {
    const ConnRow r = conn_row(a, ia, ib);
    const double cI = C[r.I];
    const uint64_t mine = spin == 0 ? r.am : r.bm;
    const double c2 = cI * cI;
    if (fabs(c2) > 1e-16)
      for (uint64_t m = mine; m; m &= m - 1) {
        const int o = __ffsll((long long)m) - 1;
        atomicAdd(acc + o * (n + 1), c2);
      }
    const int ns = spin == 0 ? r.n1a : r.n1b;
    for (int s = 0; s < ns; s++) {
      int64_t J = -1;
      int info;
      uint64_t jm;
      if (spin == 0) {
        const int Ja = a.a1_J[r.a1b + s];
        info = a.a1_info[r.a1b + s];
        jm = a.astr[Ja];
        if (r.ib < a.rowlen[Ja]) J = a.rowoff[Ja] + r.ib;
      } else {
        const int Jb = a.b1_J[r.b1b + s];
        info = a.b1_info[r.b1b + s];
        jm = a.bstr[Jb];
        if (Jb < a.rowlen[r.ia]) J = a.rowoff[r.ia] + Jb;
      }
      if (J < 0 || J > r.I) continue;  // each pair once, from the later determinant
      const double c = ((info & 1) ? -cI : cI) * C[J];
      if (fabs(c) <= 1e-16) continue;
      const int k = __ffsll((long long)(mine & ~jm)) - 1, l = __ffsll((long long)(jm & ~mine)) - 1;
      atomicAdd(acc + k + l * n, c);
      atomicAdd(acc + l + k * n, c);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n * n; i += blockDim.x)
    if (acc[i] != 0.0) atomicAdd(rdm + i, acc[i]);
}

static pq_status props_check(const pq_ci_handle *h, const char *what) {
  if (h->n_species != 1) {
    set_error("%s: one species only", what);
    return PQ_ERR_ARG;
  }
  return PQ_OK;
}

}  // namespace pq

using namespace pq;

extern "C" {

pq_status pq_ci_s2(pq_ci_handle *h, const double *C, int64_t ldc, int32_t nvec, double *s2) {
  clear_error();
  if (!h || !C || !s2 || nvec < 1 || ldc < (h ? h->n_dets : 0)) {
    set_error("pq_ci_s2: bad arguments");
    return PQ_ERR_ARG;
  }
  PQ_TRY(props_check(h, "pq_ci_s2"));
  const ConnArgs a = make_conn_args(h);
  const int na = (int)h->rowlen.size();
  const int maxlen = *std::max_element(h->rowlen.begin(), h->rowlen.end());
  const dim3 grid((unsigned)na, (unsigned)std::min((maxlen + PROP_THREADS - 1) / PROP_THREADS, 65535));
  DevBuf out;
  PQ_TRY(out.alloc(sizeof(double) * S2_MAXV));
  for (int v0 = 0; v0 < nvec; v0 += S2_MAXV) {
    const int c = std::min(S2_MAXV, nvec - v0);
    PQ_CUDA_TRY(cudaMemsetAsync(out.ptr, 0, sizeof(double) * S2_MAXV, h->stream));
    s2_kernel<<<grid, PROP_THREADS, 0, h->stream>>>(a, na, C + (size_t)v0 * ldc, ldc, c, out.as<double>());
    PQ_CUDA_TRY(cudaGetLastError());
    PQ_CUDA_TRY(cudaMemcpyAsync(s2 + v0, out.ptr, sizeof(double) * c, cudaMemcpyDeviceToHost, h->stream));
  }
  PQ_CUDA_TRY(cudaStreamSynchronize(h->stream));
  return PQ_OK;
}

pq_status pq_ci_rdm1(pq_ci_handle *h, const double *C, int32_t spin, double *rdm) {
  clear_error();
  if (!h || !C || !rdm || spin < 0 || spin > 1) {
    set_error("pq_ci_rdm1: bad arguments");
    return PQ_ERR_ARG;
  }
  PQ_TRY(props_check(h, "pq_ci_rdm1"));
  const int n = h->n_orb[0];
  const ConnArgs a = make_conn_args(h);
  const int na = (int)h->rowlen.size();
  const int maxlen = *std::max_element(h->rowlen.begin(), h->rowlen.end());
  const dim3 grid((unsigned)na, (unsigned)std::min((maxlen + PROP_THREADS - 1) / PROP_THREADS, 65535));
  DevBuf out;
  PQ_TRY(out.alloc(sizeof(double) * n * n));
  PQ_CUDA_TRY(cudaMemsetAsync(out.ptr, 0, sizeof(double) * n * n, h->stream));
  const size_t smem = sizeof(double) * n * n;
  if (smem > 48 * 1024) PQ_CUDA_TRY(cudaFuncSetAttribute(rdm1_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  rdm1_kernel<<<grid, PROP_THREADS, smem, h->stream>>>(a, na, n, spin, C, out.as<double>());
  PQ_CUDA_TRY(cudaGetLastError());
  PQ_CUDA_TRY(cudaMemcpyAsync(rdm, out.ptr, sizeof(double) * n * n, cudaMemcpyDeviceToHost, h->stream));
  PQ_CUDA_TRY(cudaStreamSynchronize(h->stream));
  return PQ_OK;
}

}  // extern "C"
