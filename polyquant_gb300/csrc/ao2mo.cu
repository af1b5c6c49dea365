// AO->MO two-electron integral transform (pq_ao2mo) and one-body transform
// (pq_mo1).
//
// Reference: src/integral/integral.cpp:207-477 (transform_mo_2_body_integrals):
// four quarter transforms, output (npair_a x npair_b) at [idx2(i,j), idx2(k,l)].
// Here the four quarters run as two pair-symmetric half transforms, each a
// batch of small GEMMs C^T M C over unpacked symmetric slices:
//   half 1: for every AO ket pair (la si): H1[la si][ij] = (C_a^T M_{la si} C_a)[i][j]
//   half 2: for every MO bra pair (ij):    E[ij][kl]    = (C_b^T N_{ij} C_b)[k][l]
// where M_{la si}[mu][nu] = (mu nu|la si) and N_{ij}[la][si] = H1[la si][ij].
// Work = 4 n_ao^3 npair + 4 n_ao^3 npair flops for equal sizes.
//
// PQ_XFORM_FP64 issues the batched GEMMs through cuBLAS (plain FP64 library
// GEMMs); the split-precision tensor-core modes are in ao2mo_tc.cu.
#include <cublas_v2.h>

#include <algorithm>

#include "pq_internal.h"

namespace pq {

#define PQ_CUBLAS_TRY2(call)                                                        \
  do {                                                                              \
    cublasStatus_t cs_ = (call);                                                    \
    if (cs_ != CUBLAS_STATUS_SUCCESS) {                                             \
      set_error("%s failed: cublas status %d (%s:%d)", #call, (int)cs_, __FILE__, __LINE__); \
      return PQ_ERR_CUDA;                                                           \
    }                                                                               \
  } while (0)

__device__ __forceinline__ int64_t tri(int64_t i, int64_t j) { return i > j ? i * (i + 1) / 2 + j : j * (j + 1) / 2 + i; }

// out[b][mu + nu*n] = source pair-matrix element (idx2(mu,nu), ket0 + b)
// layout PACKED8: src[tri(tri(mu,nu), ket)]; PAIRS: src[tri(mu,nu) + ket*ld]
__global__ void unpack_slices_kernel(const double *src, int layout, int64_t ld, int n, int64_t ket0, int nb,
                                     double *out) {
  int64_t total = (int64_t)nb * n * n;
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (; i < total; i += stride) {
    int64_t b = i / ((int64_t)n * n);
    int64_t r = i - b * n * n;
    int nu = (int)(r / n), mu = (int)(r - (int64_t)nu * n);
    int64_t bra = tri(mu, nu), ket = ket0 + b;
    out[i] = layout == PQ_AO_PACKED8 ? src[tri(bra, ket)] : src[bra + ket * ld];
  }
}

// dst[(ket0 + b) * npair_mo + tri(i,j)] = slices[b][i + j*m] for i >= j
__global__ void pack_slices_kernel(const double *slices, int m, int64_t ket0, int nb, double *dst) {
  int64_t np = (int64_t)m * (m + 1) / 2;
  int64_t total = (int64_t)nb * np;
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (; t < total; t += stride) {
    int64_t b = t / np, p = t - b * np;
    int i = (int)((sqrt(8.0 * (double)p + 1.0) - 1.0) * 0.5);
    while ((int64_t)i * (i + 1) / 2 > p) i--;
    while ((int64_t)(i + 1) * (i + 2) / 2 <= p) i++;
    int j = (int)(p - (int64_t)i * (i + 1) / 2);
    dst[(ket0 + b) * np + p] = slices[b * (int64_t)m * m + i + (int64_t)j * m];
  }
}

// tiled transpose: out[c * rows + r] = in[r * cols + c]
__global__ void transpose_kernel(const double *in, int64_t rows, int64_t cols, double *out) {
  __shared__ double tile[32][33];
  int64_t r0 = (int64_t)blockIdx.y * 32, c0 = (int64_t)blockIdx.x * 32;
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    int64_t r = r0 + y, c = c0 + threadIdx.x;
    if (r < rows && c < cols) tile[y][threadIdx.x] = in[r * cols + c];
  }
  __syncthreads();
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    int64_t c = c0 + y, r = r0 + threadIdx.x;
    if (r < rows && c < cols) out[c * rows + r] = tile[threadIdx.x][y];
  }
}

static pq_status transpose(const double *in, int64_t rows, int64_t cols, double *out, cudaStream_t st) {
  dim3 grid((unsigned)((cols + 31) / 32), (unsigned)((rows + 31) / 32));
  if (grid.y > 65535) {
    set_error("transpose: %lld rows exceed the grid limit", (long long)rows);
    return PQ_ERR_ARG;
  }
  transpose_kernel<<<grid, dim3(32, 8), 0, st>>>(in, rows, cols, out);
  PQ_CUDA_TRY(cudaGetLastError());
  return PQ_OK;
}

// One half transform: for each of nket slices S_b (n x n, symmetric, unpacked
// from src), dst[b][tri(i,j)] = (C^T S_b C)[i][j].
static pq_status half_transform_fp64(cublasHandle_t cb, const double *src, int layout, int64_t ld, int n,
                                     int64_t nket, const double *C, int64_t ldc, int m, double *dst,
                                     cudaStream_t st) {
  const int64_t slice = (int64_t)n * n;
  int64_t bt = std::max<int64_t>(1, std::min<int64_t>(nket, (int64_t)(512LL << 20) / (sizeof(double) * slice)));
  DevBuf S, T, H;
  PQ_TRY(S.alloc(sizeof(double) * slice * bt));
  PQ_TRY(T.alloc(sizeof(double) * (int64_t)n * m * bt));
  PQ_TRY(H.alloc(sizeof(double) * (int64_t)m * m * bt));
  const double one = 1.0, zero = 0.0;
  for (int64_t k0 = 0; k0 < nket; k0 += bt) {
    int nb = (int)std::min(bt, nket - k0);
    unsigned g = (unsigned)std::min<int64_t>((slice * nb + 255) / 256, 152 * 32);
    unpack_slices_kernel<<<g, 256, 0, st>>>(src, layout, ld, n, k0, nb, S.as<double>());
    PQ_CUDA_TRY(cudaGetLastError());
    // T_b = S_b C   (n x m);  H_b = C^T T_b   (m x m)
    PQ_CUBLAS_TRY2(cublasDgemmStridedBatched(cb, CUBLAS_OP_N, CUBLAS_OP_N, n, m, n, &one, S.as<double>(), n, slice, C,
                                             (int)ldc, 0, &zero, T.as<double>(), n, (int64_t)n * m, nb));
    PQ_CUBLAS_TRY2(cublasDgemmStridedBatched(cb, CUBLAS_OP_T, CUBLAS_OP_N, m, m, n, &one, C, (int)ldc, 0,
                                             T.as<double>(), n, (int64_t)n * m, &zero, H.as<double>(), m,
                                             (int64_t)m * m, nb));
    int64_t np = (int64_t)m * (m + 1) / 2;
    unsigned g2 = (unsigned)std::min<int64_t>((np * nb + 255) / 256, 152 * 32);
    pack_slices_kernel<<<g2, 256, 0, st>>>(H.as<double>(), m, k0, nb, dst);
    PQ_CUDA_TRY(cudaGetLastError());
  }
  return PQ_OK;
}

pq_status ao2mo_fp64(const double *eri_ao, int layout, int64_t n_ao_a, int64_t n_ao_b, const double *Ca, int64_t lda,
                     int64_t nmo_a, const double *Cb, int64_t ldb, int64_t nmo_b, double *eri_mo, cudaStream_t st) {
  cublasHandle_t cb;
  if (cublasCreate(&cb) != CUBLAS_STATUS_SUCCESS) {
    set_error("cublasCreate failed");
    return PQ_ERR_CUDA;
  }
  struct Guard {
    cublasHandle_t h;
    ~Guard() { cublasDestroy(h); }
  } guard{cb};
  PQ_CUBLAS_TRY2(cublasSetStream(cb, st));
  const int64_t npa = n_ao_a * (n_ao_a + 1) / 2, npb = n_ao_b * (n_ao_b + 1) / 2;
  const int64_t nma = nmo_a * (nmo_a + 1) / 2, nmb = nmo_b * (nmo_b + 1) / 2;
  // half 1 over ket AO pairs: H1[ket][ij]  (npb x nma, row-major)
  DevBuf H1, H1t, Erow;
  PQ_TRY(H1.alloc(sizeof(double) * npb * nma));
  PQ_TRY(half_transform_fp64(cb, eri_ao, layout, npa, (int)n_ao_a, npb, Ca, lda, (int)nmo_a, H1.as<double>(), st));
  // H1t[ij][ket]
  PQ_TRY(H1t.alloc(sizeof(double) * npb * nma));
  PQ_TRY(transpose(H1.as<double>(), npb, nma, H1t.as<double>(), st));
  H1.release();
  // half 2 over bra MO pairs: slices of H1t rows are packed (la si) -> PAIRS layout with ld = npb over "bra"
  // unpack_slices with PAIRS reads src[tri(mu,nu) + ket*ld]: here mu,nu = la,si and ket = ij, ld = npb.
  PQ_TRY(Erow.alloc(sizeof(double) * nma * nmb));
  PQ_TRY(half_transform_fp64(cb, H1t.as<double>(), PQ_AO_PAIRS, npb, (int)n_ao_b, nma, Cb, ldb, (int)nmo_b,
                             Erow.as<double>(), st));
  H1t.release();
  // Erow[ij][kl] (row-major) -> reference column-major eri_mo[ij + kl*nma]
  PQ_TRY(transpose(Erow.as<double>(), nma, nmb, eri_mo, st));
  PQ_CUDA_TRY(cudaStreamSynchronize(st));
  return PQ_OK;
}

pq_status ao2mo_tc(const double *eri_ao, int layout, int64_t n_ao, const double *Ca, int64_t lda, int64_t nmo,
                   int mode, double *eri_mo, cudaStream_t st);

}  // namespace pq

using namespace pq;

extern "C" pq_status pq_ao2mo(const double *eri_ao, int32_t layout, int64_t n_ao_a, int64_t n_ao_b, const double *C_a,
                              int64_t ldc_a, int64_t n_mo_a, const double *C_b, int64_t ldc_b, int64_t n_mo_b,
                              int32_t mode, double *eri_mo, void *stream) {
  clear_error();
  if (!eri_ao || !C_a || !C_b || !eri_mo || n_ao_a < 1 || n_ao_b < 1 || n_mo_a < 1 || n_mo_b < 1 ||
      n_mo_a > n_ao_a || n_mo_b > n_ao_b || ldc_a < n_ao_a || ldc_b < n_ao_b) {
    set_error("pq_ao2mo: bad arguments");
    return PQ_ERR_ARG;
  }
  if (layout != PQ_AO_PACKED8 && layout != PQ_AO_PAIRS) {
    set_error("pq_ao2mo: unknown layout %d", layout);
    return PQ_ERR_ARG;
  }
  if (layout == PQ_AO_PACKED8 && n_ao_a != n_ao_b) {
    set_error("pq_ao2mo: PACKED8 needs one species (n_ao_a == n_ao_b)");
    return PQ_ERR_ARG;
  }
  if (n_ao_a > 1024 || n_ao_b > 1024) {
    set_error("pq_ao2mo: n_ao above 1024 is not supported");
    return PQ_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  if (mode == PQ_XFORM_FP64)
    return ao2mo_fp64(eri_ao, layout, n_ao_a, n_ao_b, C_a, ldc_a, n_mo_a, C_b, ldc_b, n_mo_b, eri_mo, st);
  if (mode == PQ_XFORM_BF16X3 || mode == PQ_XFORM_TF32X3) {
    if (n_ao_a != n_ao_b || n_mo_a != n_mo_b || C_a != C_b) {
      set_error("pq_ao2mo: split-precision modes transform one species block (C_a == C_b)");
      return PQ_ERR_ARG;
    }
    return ao2mo_tc(eri_ao, layout, n_ao_a, C_a, ldc_a, n_mo_a, mode, eri_mo, st);
  }
  set_error("pq_ao2mo: unknown mode %d", mode);
  return PQ_ERR_ARG;
}

extern "C" pq_status pq_mo1(const double *F_ao, int64_t n_ao, const double *C, int64_t ldc, int64_t n_mo,
                            double *h_mo, void *stream) {
  clear_error();
  if (!F_ao || !C || !h_mo || n_ao < 1 || n_mo < 1 || ldc < n_ao) {
    set_error("pq_mo1: bad arguments");
    return PQ_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  cublasHandle_t cb;
  if (cublasCreate(&cb) != CUBLAS_STATUS_SUCCESS) {
    set_error("cublasCreate failed");
    return PQ_ERR_CUDA;
  }
  struct Guard {
    cublasHandle_t h;
    ~Guard() { cublasDestroy(h); }
  } guard{cb};
  PQ_CUBLAS_TRY2(cublasSetStream(cb, st));
  DevBuf T;
  PQ_TRY(T.alloc(sizeof(double) * n_ao * n_mo));
  const double one = 1.0, zero = 0.0;
  PQ_CUBLAS_TRY2(cublasDgemm(cb, CUBLAS_OP_N, CUBLAS_OP_N, (int)n_ao, (int)n_mo, (int)n_ao, &one, F_ao, (int)n_ao, C,
                             (int)ldc, &zero, T.as<double>(), (int)n_ao));
  PQ_CUBLAS_TRY2(cublasDgemm(cb, CUBLAS_OP_T, CUBLAS_OP_N, (int)n_mo, (int)n_mo, (int)n_ao, &one, C, (int)ldc,
                             T.as<double>(), (int)n_ao, &zero, h_mo, (int)n_mo));
  PQ_CUDA_TRY(cudaStreamSynchronize(st));
  return PQ_OK;
}
