// Block Davidson eigensolver on the GPU for the lowest roots of H.
//
// Replaces the reference's use of Spectra::DavidsonSymEigsSolver
// (src/ci/epci.cpp:589-608): initial subspace = unit vectors at the smallest
// diagonal elements, diagonal preconditioner (theta - H_II)^-1, convergence
// when every residual norm is below convergence_E, subspace limits
// initial = num_subspace_vec and max = max(2*initial, 10*num_states).
// Spectra itself is not part of the reference tree; this solver is pinned by
// the converged energies only.
//
// All subspace algebra (Gram-Schmidt, projections, Ritz vectors, residual
// norms, preconditioner denominators) is FP64 on the device through cuBLAS;
// the Rayleigh matrix eigenproblem (at most a few hundred rows) is solved on
// the host in FP64.  With precision = PQ_FP32 the sigma vectors of new search
// directions come from the FP32 kernel applied to (H - s) with s the current
// lowest Ritz value, and every restart recomputes the Ritz vectors' sigma in
// FP64 ("residual refinement"), so reported energies and residual norms are
// always exact FP64 Rayleigh quotients and residuals.
#include <cublas_v2.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <numeric>
#include <vector>

#include "pq_internal.h"

namespace pq {

#define PQ_CUBLAS_TRY(call)                                                          \
  do {                                                                               \
    cublasStatus_t cs_ = (call);                                                     \
    if (cs_ != CUBLAS_STATUS_SUCCESS) {                                              \
      set_error("%s failed: cublas status %d (%s:%d)", #call, (int)cs_, __FILE__, __LINE__); \
      return PQ_ERR_CUDA;                                                            \
    }                                                                                \
  } while (0)

// Cyclic Jacobi eigensolver for a small symmetric matrix (column-major n x n).
// Eigenvalues ascending in w, eigenvectors in the columns of Z.
static void jacobi_eigh(int n, std::vector<double> A, std::vector<double> &w, std::vector<double> &Z) {
  Z.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; i++) Z[i + (size_t)i * n] = 1.0;
  auto a = [&](int i, int j) -> double & { return A[i + (size_t)j * n]; };
  for (int sweep = 0; sweep < 100; sweep++) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < n; i++)
      for (int j = 0; j < n; j++) {
        tot += a(i, j) * a(i, j);
        if (i != j) off += a(i, j) * a(i, j);
      }
    if (off <= 1e-30 * std::max(tot, 1e-300)) break;
    for (int p = 0; p < n - 1; p++)
      for (int q = p + 1; q < n; q++) {
        double apq = a(p, q);
        if (std::fabs(apq) < 1e-300) continue;
        double theta = (a(q, q) - a(p, p)) / (2.0 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; k++) {
          double akp = a(k, p), akq = a(k, q);
          a(k, p) = c * akp - s * akq;
          a(k, q) = s * akp + c * akq;
        }
        for (int k = 0; k < n; k++) {
          double apk = a(p, k), aqk = a(q, k);
          a(p, k) = c * apk - s * aqk;
          a(q, k) = s * apk + c * aqk;
        }
        for (int k = 0; k < n; k++) {
          double zkp = Z[k + (size_t)p * n], zkq = Z[k + (size_t)q * n];
          Z[k + (size_t)p * n] = c * zkp - s * zkq;
          Z[k + (size_t)q * n] = s * zkp + c * zkq;
        }
      }
  }
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::sort(order.begin(), order.end(), [&](int x, int y) { return a(x, x) < a(y, y); });
  std::vector<double> Zs((size_t)n * n);
  w.resize(n);
  for (int j = 0; j < n; j++) {
    w[j] = a(order[j], order[j]);
    for (int i = 0; i < n; i++) Zs[i + (size_t)j * n] = Z[i + (size_t)order[j] * n];
  }
  Z.swap(Zs);
}

// C[:, j] = op(A) B[:, j] for j < q, one DGEMV per column.  A is the tall
// n x m block of V or W (n up to ~1e9 rows, m <= a few dozen columns): DGEMV
// streams it at the FP64 FMA rate, while DGEMM on these shapes runs an order
// of magnitude slower.
static pq_status tall_skinny(cublasHandle_t cb, cublasOperation_t op, int64_t n, int m, const double *A,
                             const double *B, int64_t ldb, int q, double *C, int64_t ldc) {
  const double one = 1.0, zero = 0.0;
  for (int j = 0; j < q; j++)
    PQ_CUBLAS_TRY(cublasDgemv(cb, op, (int)n, m, &one, A, (int)n, B + (size_t)j * ldb, 1, &zero, C + (size_t)j * ldc, 1));
  return PQ_OK;
}

__global__ void unit_vectors_kernel(double *V, int64_t n, const int64_t *idx, int m) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (; i < n * m; i += stride) {
    int64_t c = i / n, r = i - c * n;
    V[i] = (idx[c] == r) ? 1.0 : 0.0;
  }
}

// Selection of the m smallest diagonal elements in the order (value, index), one element per pass: pass j
// finds the smallest pair above the pair of pass j-1 (block minima, then one block over the block minima).
constexpr int SEL_BLOCKS = 152 * 4, SEL_THREADS = 256;

struct ValIdx {
  double v;
  int64_t i;
};
__device__ __forceinline__ bool vi_less(double a, int64_t ia, double b, int64_t ib) { return a < b || (a == b && ia < ib); }
__device__ __forceinline__ ValIdx vi_min_block(ValIdx x) {
  __shared__ ValIdx red[SEL_THREADS / 32];
  for (int o = 16; o; o >>= 1) {
    const double v = __shfl_xor_sync(0xffffffffu, x.v, o);
    const int64_t i = __shfl_xor_sync(0xffffffffu, x.i, o);
    if (vi_less(v, i, x.v, x.i)) x = {v, i};
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
  __syncthreads();
  if (threadIdx.x < 32) {
    x = threadIdx.x < SEL_THREADS / 32 ? red[threadIdx.x] : ValIdx{INFINITY, INT64_MAX};
    for (int o = 16; o; o >>= 1) {
      const double v = __shfl_xor_sync(0xffffffffu, x.v, o);
      const int64_t i = __shfl_xor_sync(0xffffffffu, x.i, o);
      if (vi_less(v, i, x.v, x.i)) x = {v, i};
    }
  }
  return x;
}

// block minima of the pairs (D[i], i) above sel[j - 1] (every pair for j = 0)
__global__ void __launch_bounds__(SEL_THREADS) select_pass_kernel(const double *D, int64_t n, const ValIdx *sel, int j,
                                                                  ValIdx *blk) {
  const ValIdx prev = j > 0 ? sel[j - 1] : ValIdx{-INFINITY, -1};
  ValIdx best{INFINITY, INT64_MAX};
  for (int64_t i = (int64_t)blockIdx.x * SEL_THREADS + threadIdx.x; i < n; i += (int64_t)gridDim.x * SEL_THREADS) {
    const double v = D[i];
    if (vi_less(prev.v, prev.i, v, i) && vi_less(v, i, best.v, best.i)) best = {v, i};
  }
  best = vi_min_block(best);
  if (threadIdx.x == 0) blk[blockIdx.x] = best;
}
__global__ void __launch_bounds__(SEL_THREADS) select_final_kernel(const ValIdx *blk, int nblk, ValIdx *sel, int j) {
  ValIdx best{INFINITY, INT64_MAX};
  for (int b = threadIdx.x; b < nblk; b += SEL_THREADS)
    if (vi_less(blk[b].v, blk[b].i, best.v, best.i)) best = blk[b];
  best = vi_min_block(best);
  if (threadIdx.x == 0) sel[j] = best;
}

// T[:, j] = R[:, j] / (theta_j - D)   (diagonal preconditioner)
__global__ void precondition_kernel(const double *R, const double *D, const double *theta, int64_t n, int k,
                                    double *T) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (; i < n * k; i += stride) {
    int64_t c = i / n, r = i - c * n;
    double den = theta[c] - D[r];
    if (fabs(den) < 1e-8) den = den < 0 ? -1e-8 : 1e-8;
    T[i] = R[i] / den;
  }
}

// W[:, j] = Y_il[:, j] + s * V[:, j] from the interleaved FP32 sigma of (H - s)
__global__ void unshift_kernel(const float *Y, int nvp, int nv, const double *V, int64_t ldv, double s, int64_t n,
                               double *W, int64_t ldw) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (; i < n; i += stride)
    for (int v = 0; v < nv; v++) W[i + v * ldw] = (double)Y[i * nvp + v] + s * V[i + v * ldv];
}

// One Davidson solve as a step-wise state machine: init() and advance() stop
// whenever sigma vectors are needed (a SigmaRequest), so one driver can serve a
// single problem and a lockstep batch of problems with one sigma launch per
// iteration.
pq_status DavidsonRun::init(pq_ci_handle *hh, const pq_davidson_params &pp, ::cublasContext *shared_cb) {
  t_start = std::chrono::steady_clock::now();
  h = hh;
  p = pp;
  n = h->n_dets;
  k = p.num_states;
  st = h->stream;
  if (k < 1 || n < 1) {
    set_error("davidson: num_states=%d, n_dets=%lld", k, (long long)n);
    return PQ_ERR_ARG;
  }
  if (p.precision != PQ_FP64 && p.precision != PQ_FP32) {
    set_error("davidson: precision must be PQ_FP64 or PQ_FP32");
    return PQ_ERR_ARG;
  }
  if (n > 0x7fffffffLL) {
    set_error("davidson: n_dets beyond the 32-bit cuBLAS dimension limit");
    return PQ_ERR_ARG;
  }
  m0 = std::max(p.num_subspace_vec, k);
  mmax = p.max_subspace > 0 ? p.max_subspace : std::max(2 * p.num_subspace_vec, 10 * k);
  mmax = std::max(mmax, m0 + k);
  if ((int64_t)m0 > n) m0 = (int)n;
  if ((int64_t)mmax > n) mmax = (int)n;
  if (k > m0) {
    set_error("davidson: num_states %d exceeds the space dimension %lld", k, (long long)n);
    return PQ_ERR_ARG;
  }
  iter_max = p.iteration_max > 0 ? p.iteration_max : 500;
  tol = p.convergence_E > 0 ? p.convergence_E : 1e-6;
  switch_tol = std::max(tol, 1e-5);
  phase32 = p.precision == PQ_FP32;
  if (shared_cb) {
    cb = shared_cb;
  } else {
    if (cublasCreate(&cb) != CUBLAS_STATUS_SUCCESS) {
      set_error("cublasCreate failed");
      return PQ_ERR_CUDA;
    }
    own_cb = true;
    PQ_CUBLAS_TRY(cublasSetStream(cb, st));
  }
  PQ_TRY(V.alloc(sizeof(double) * (size_t)n * mmax));
  PQ_TRY(W.alloc(sizeof(double) * (size_t)n * mmax));
  PQ_TRY(X.alloc(sizeof(double) * (size_t)n * k));
  PQ_TRY(R.alloc(sizeof(double) * (size_t)n * k));
  PQ_TRY(T.alloc(sizeof(double) * (size_t)n * std::max(k, m0)));
  PQ_TRY(dth.alloc(sizeof(double) * std::max(k, 8)));
  theta.assign(k, 0.0);
  rnorm.assign(k, 0.0);
  // initial subspace: unit vectors at the m0 smallest diagonal elements (ties by index), selected on the device
  std::vector<int64_t> idx(m0);
  {
    const int nblk = (int)std::min<int64_t>(SEL_BLOCKS, (n + SEL_THREADS - 1) / SEL_THREADS);
    PQ_TRY(tmp.ensure(sizeof(ValIdx) * (size_t)(nblk + m0)));
    ValIdx *blk = tmp.as<ValIdx>(), *sel = blk + nblk;
    for (int j = 0; j < m0; j++) {
      select_pass_kernel<<<nblk, SEL_THREADS, 0, st>>>(h->d_diag.as<double>(), n, sel, j, blk);
      select_final_kernel<<<1, SEL_THREADS, 0, st>>>(blk, nblk, sel, j);
    }
    PQ_CUDA_TRY(cudaGetLastError());
    std::vector<ValIdx> hs(m0);
    PQ_CUDA_TRY(cudaMemcpyAsync(hs.data(), sel, sizeof(ValIdx) * m0, cudaMemcpyDeviceToHost, st));
    PQ_CUDA_TRY(cudaStreamSynchronize(st));
    for (int j = 0; j < m0; j++) idx[j] = hs[j].i;
    shift = hs[0].v;
  }
  PQ_TRY(upload(didx, idx, st));
  unit_vectors_kernel<<<grid(), 256, 0, st>>>(V.as<double>(), n, didx.as<int64_t>(), m0);
  PQ_CUDA_TRY(cudaGetLastError());
  if (h->n_species == 1) {
    // sigma of a unit vector is a column of H: exact FP64 from its connections
    PQ_TRY(ci_unit_columns(h, idx, W.as<double>()));
    pending = false;
    stage = AFTER_INIT;
  } else {
    request(V.as<double>(), W.as<double>(), m0, PQ_FP64, 0.0, AFTER_INIT);
  }
  return PQ_OK;
}

void DavidsonRun::request(const double *src, double *dst, int cnt, int prec, double s, Stage next) {
  req = SigmaRequest{src, dst, cnt, prec, s};
  pending = true;
  stage = next;
  if (prec == PQ_FP64)
    rep.sigma_calls_fp64++;
  else
    rep.sigma_calls_fp32++;
}

pq_status DavidsonRun::advance() {
  pending = false;
  switch (stage) {
    case AFTER_INIT:
      m = m0;
      exact = true;
      break;
    case AFTER_REFINE:
      exact = true;
      just_refined = true;
      m = r_restart;
      g_valid = 0;
      break;
    case AFTER_NEW:
      if (req.precision == PQ_FP32) exact = false;
      m += req.cnt;
      break;
    default:
      break;
  }
  std::vector<double> G, w;
  while (true) {
    it++;
    if (it > iter_max) {
      it = iter_max;
      return finish_state(PQ_NOT_CONVERGED);
    }
    PQ_TRY(rayleigh(m, G));
    jacobi_eigh(m, G, w, Z);
    for (int i = 0; i < k; i++) theta[i] = w[i];
    PQ_TRY(tmp.ensure(sizeof(double) * (size_t)m * k));
    std::vector<double> Yk(Z.begin(), Z.begin() + (size_t)m * k);
    PQ_CUDA_TRY(cudaMemcpyAsync(tmp.ptr, Yk.data(), sizeof(double) * m * k, cudaMemcpyHostToDevice, st));
    // X = V Y, R = W Y - X theta
    PQ_TRY(tall_skinny(cb, CUBLAS_OP_N, n, m, V.as<double>(), tmp.as<double>(), m, k, X.as<double>(), n));
    PQ_TRY(tall_skinny(cb, CUBLAS_OP_N, n, m, W.as<double>(), tmp.as<double>(), m, k, R.as<double>(), n));
    double maxr = 0.0;
    for (int i = 0; i < k; i++) {
      double mt = -theta[i];
      PQ_CUBLAS_TRY(cublasDaxpy(cb, (int)n, &mt, X.as<double>() + (size_t)i * n, 1, R.as<double>() + (size_t)i * n, 1));
      PQ_CUBLAS_TRY(cublasDnrm2(cb, (int)n, R.as<double>() + (size_t)i * n, 1, &rnorm[i]));
      maxr = std::max(maxr, rnorm[i]);
    }
    if (p.verbose) {
      printf("davidson it %3d  m %3d  %s  t %8.3f s  sigma %8.3f s", it, m, exact ? "fp64" : "mixd",
             std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count(), rep.sigma_seconds);
      for (int i = 0; i < k; i++) printf("  E%d % .12f r %.2e", i, theta[i] + p.energy_shift, rnorm[i]);
      printf("\n");
    }
    rep.max_residual = maxr;
    if (maxr < tol && exact) return finish_state(PQ_OK);
    // Mixed precision: FP32 sigma for new directions.  The FP32 phase drives
    // the (inexact) residual to a fraction of the target so that a single
    // FP64 refinement usually finishes the solve; it refines early when the
    // inexact residual stops improving (the FP32 noise floor), and switches to
    // FP64 directions only when two refinements in a row made no progress.
    if (phase32 && exact && just_refined) {
      if (maxr > 0.5 * last_refined) phase32 = false;
      last_refined = maxr;
      best32 = 1e300;
      stall32 = 0;
    }
    if (phase32 && !exact) {
      if (maxr < 0.9 * best32) {
        best32 = maxr;
        stall32 = 0;
      } else {
        stall32++;
      }
    }
    just_refined = false;
    const bool refine = !exact && (!phase32 || maxr < 0.3 * switch_tol || stall32 >= 3 || force_refine);
    const bool need_restart = (m + k > mmax) || refine;
    force_refine = false;
    if (need_restart) {
      // a refinement restarts from the k Ritz vectors (one FP64 sigma call
      // for the k roots); a restart for subspace size keeps min(m0, m)
      // vectors and rotates W with V, inexact FP32 columns included (the
      // next refinement replaces them)
      int r = refine ? k : std::min(m0, m);
      r = std::max(r, k);
      // V[:, 0:r] = V Z[:, 0:r]; W likewise (via the temporary T)
      PQ_TRY(tmp.ensure(sizeof(double) * (size_t)m * r));
      std::vector<double> Zr(Z.begin(), Z.begin() + (size_t)m * r);
      PQ_CUDA_TRY(cudaMemcpyAsync(tmp.ptr, Zr.data(), sizeof(double) * m * r, cudaMemcpyHostToDevice, st));
      PQ_TRY(T.ensure(sizeof(double) * (size_t)n * r));
      PQ_TRY(tall_skinny(cb, CUBLAS_OP_N, n, m, V.as<double>(), tmp.as<double>(), m, r, T.as<double>(), n));
      PQ_CUDA_TRY(cudaMemcpyAsync(V.ptr, T.ptr, sizeof(double) * n * r, cudaMemcpyDeviceToDevice, st));
      if (refine) {
        // FP64 residual refinement: exact sigma of the restart vectors
        r_restart = r;
        request(V.as<double>(), W.as<double>(), r, PQ_FP64, 0.0, AFTER_REFINE);
        return PQ_OK;
      }
      PQ_TRY(tall_skinny(cb, CUBLAS_OP_N, n, m, W.as<double>(), tmp.as<double>(), m, r, T.as<double>(), n));
      PQ_CUDA_TRY(cudaMemcpyAsync(W.ptr, T.ptr, sizeof(double) * n * r, cudaMemcpyDeviceToDevice, st));
      // the rotated Rayleigh matrix Z_r^T G Z_r is diag(w) (Z diagonalises G)
      for (int j = 0; j < r; j++)
        for (int i = 0; i < r; i++) Gk[i + (size_t)j * mmax] = i == j ? w[i] : 0.0;
      g_valid = r;
      m = r;
      continue;
    }
    // corrections for unconverged roots
    int nt = 0;
    std::vector<double> th_u;
    for (int i = 0; i < k; i++) {
      if (rnorm[i] < tol) continue;
      PQ_CUDA_TRY(cudaMemcpyAsync(T.as<double>() + (size_t)nt * n, R.as<double>() + (size_t)i * n, sizeof(double) * n,
                                  cudaMemcpyDeviceToDevice, st));
      th_u.push_back(theta[i]);
      nt++;
    }
    PQ_CUDA_TRY(cudaMemcpyAsync(dth.ptr, th_u.data(), sizeof(double) * nt, cudaMemcpyHostToDevice, st));
    precondition_kernel<<<grid(), 256, 0, st>>>(T.as<double>(), h->d_diag.as<double>(), dth.as<double>(), n, nt,
                                                T.as<double>());
    PQ_CUDA_TRY(cudaGetLastError());
    int added = 0;
    PQ_TRY(orthonormalize_append(m, nt, &added));
    if (added == 0) {
      // no new direction: the subspace is invariant to working precision
      if (exact) return finish_state(PQ_OK);
      force_refine = true;
      continue;
    }
    shift = theta[0];
    const int prec = phase32 ? PQ_FP32 : PQ_FP64;
    request(V.as<double>() + (size_t)m * n, W.as<double>() + (size_t)m * n, added, prec, shift, AFTER_NEW);
    return PQ_OK;
  }
}

pq_status DavidsonRun::finish_state(pq_status r) {
  done = true;
  result = r;
  rep.iterations = it;
  rep.converged = r == PQ_OK;
  return PQ_OK;
}

pq_status DavidsonRun::outputs(double *energies, double *vecs) {
  for (int i = 0; i < k; i++) energies[i] = theta[i] + p.energy_shift;
  if (vecs) PQ_CUDA_TRY(cudaMemcpyAsync(vecs, X.ptr, sizeof(double) * n * k, cudaMemcpyDeviceToDevice, st));
  PQ_CUDA_TRY(cudaStreamSynchronize(st));
  rep.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
  return PQ_OK;
}

DavidsonRun::~DavidsonRun() {
  if (cb && own_cb) cublasDestroy(cb);
}

// G = V[:, 0:m]^T W[:, 0:m] on the host, kept across iterations in Gk
// (leading dimension mmax): only the columns added since the last call are
// computed, B = V[:, 0:m]^T W[:, g_valid:m], and mirrored into the rows, so
// the matrix is symmetric by construction.
pq_status DavidsonRun::rayleigh(int mm, std::vector<double> &G) {
  if ((int)Gk.size() < mmax * mmax) Gk.assign((size_t)mmax * mmax, 0.0);
  if (g_valid < mm) {
    const int c0 = g_valid, nc = mm - c0;
    PQ_TRY(tmp.ensure(sizeof(double) * (size_t)mm * nc));
    PQ_TRY(tall_skinny(cb, CUBLAS_OP_T, n, mm, V.as<double>(), W.as<double>() + (size_t)c0 * n, n, nc,
                       tmp.as<double>(), mm));
    std::vector<double> B((size_t)mm * nc);
    PQ_CUDA_TRY(cudaMemcpyAsync(B.data(), tmp.ptr, sizeof(double) * mm * nc, cudaMemcpyDeviceToHost, st));
    PQ_CUDA_TRY(cudaStreamSynchronize(st));
    for (int j = 0; j < nc; j++)
      for (int i = 0; i < mm; i++) {
        double v = B[i + (size_t)j * mm];
        if (i >= c0 && i - c0 < j) continue;                                   // lower part of the new block
        if (i >= c0 && i - c0 > j) v = 0.5 * (v + B[(c0 + j) + (size_t)(i - c0) * mm]);  // new x new: average
        Gk[i + (size_t)(c0 + j) * mmax] = Gk[(c0 + j) + (size_t)i * mmax] = v;
      }
    g_valid = mm;
  }
  G.resize((size_t)mm * mm);
  for (int j = 0; j < mm; j++)
    for (int i = 0; i < mm; i++) G[i + (size_t)j * mm] = Gk[i + (size_t)j * mmax];
  return PQ_OK;
}

// Orthonormalise columns T[:, 0:kk] against V[:, 0:mm] and each other (two
// classical Gram-Schmidt passes); accepted columns are appended to V.
pq_status DavidsonRun::orthonormalize_append(int mm0, int kk, int *added) {
  const double one = 1.0, mone = -1.0, zero = 0.0;
  PQ_TRY(coef.ensure(sizeof(double) * (size_t)(mm0 + kk) * 2));
  int mm = mm0;
  for (int j = 0; j < kk; j++) {
    double *t = T.as<double>() + (size_t)j * n;
    double nrm0 = 0.0;
    PQ_CUBLAS_TRY(cublasDnrm2(cb, (int)n, t, 1, &nrm0));
    if (!(nrm0 > 0.0) || !std::isfinite(nrm0)) continue;
    // classical Gram-Schmidt, repeated once unless the first pass kept at
    // least 1/sqrt(2) of the norm (then t is orthogonal to working precision)
    double nrm = nrm0;
    for (int pass = 0; pass < 2; pass++) {
      const double before = nrm;
      PQ_CUBLAS_TRY(cublasDgemv(cb, CUBLAS_OP_T, (int)n, mm, &one, V.as<double>(), (int)n, t, 1, &zero, coef.as<double>(), 1));
      PQ_CUBLAS_TRY(cublasDgemv(cb, CUBLAS_OP_N, (int)n, mm, &mone, V.as<double>(), (int)n, coef.as<double>(), 1, &one, t, 1));
      PQ_CUBLAS_TRY(cublasDnrm2(cb, (int)n, t, 1, &nrm));
      if (nrm >= 0.70710678118654752 * before) break;
    }
    if (!(nrm > 1e-8 * nrm0) || nrm < 1e-300) continue;
    double inv = 1.0 / nrm;
    PQ_CUBLAS_TRY(cublasDscal(cb, (int)n, &inv, t, 1));
    PQ_CUDA_TRY(cudaMemcpyAsync(V.as<double>() + (size_t)mm * n, t, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    mm++;
  }
  *added = mm - mm0;
  return PQ_OK;
}

// sigma of a request for one problem: column-major FP64 in and out; the FP32
// path applies (H - shift) and adds shift * src back in FP64
pq_status sigma_request_single(pq_ci_handle *h, const SigmaRequest &r) {
  const int64_t n = h->n_dets;
  const unsigned g = (unsigned)std::min<int64_t>((n + 255) / 256, 152 * 16);
  for (int v0 = 0; v0 < r.cnt; v0 += 4) {
    const int c = std::min(4, r.cnt - v0), nvp = il_width(h, c, r.precision);
    const size_t esz = r.precision == PQ_FP64 ? sizeof(double) : sizeof(float);
    PQ_TRY(h->x_il.ensure(esz * nvp * (size_t)(n + 1)));
    PQ_TRY(h->y_il.ensure(esz * nvp * (size_t)(n + 1)));
    PQ_TRY(ci_to_il(h, r.src, n, v0, c, nvp, r.precision, h->x_il.ptr));
    PQ_TRY(ci_sigma_il(h, h->x_il.ptr, h->y_il.ptr, nvp, r.precision, r.precision == PQ_FP64 ? 0.0 : r.shift));
    if (r.precision == PQ_FP64) {
      PQ_TRY(ci_from_il(h, h->y_il.ptr, v0, c, nvp, PQ_FP64, r.dst, n));
    } else {
      unshift_kernel<<<g, 256, 0, h->stream>>>((const float *)h->y_il.ptr, nvp, c, r.src + (size_t)v0 * n, n, r.shift, n,
                                               r.dst + (size_t)v0 * n, n);
      PQ_CUDA_TRY(cudaGetLastError());
    }
  }
  return PQ_OK;
}

pq_status ci_davidson(pq_ci_handle *h, const pq_davidson_params *p, double *energies, double *vecs,
                      pq_davidson_report *rep_out) {
  DavidsonRun D;
  PQ_TRY(D.init(h, *p));
  while (!D.done) {
    if (D.pending) {
      const auto t0 = std::chrono::steady_clock::now();
      PQ_TRY(sigma_request_single(h, D.req));
      PQ_CUDA_TRY(cudaStreamSynchronize(h->stream));
      D.rep.sigma_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    PQ_TRY(D.advance());
  }
  PQ_TRY(D.outputs(energies, vecs));
  if (rep_out) *rep_out = D.rep;
  if (D.result != PQ_OK)
    set_error("davidson: not converged after %d iterations (max residual %.3e)", D.iter_max, D.rep.max_residual);
  return D.result;
}

}  // namespace pq
