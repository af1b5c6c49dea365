/*
 * pq_ci.h -- C ABI of the GB300 CI sigma library (libpq_gb300.so).
 *
 * Drop-in replacement for the determinant-space operator that polyquant's
 * Davidson driver calls.  Reference interfaces replaced (paths inside the
 * polyquant project):
 *
 *   POLYQUANT_DETSET<uint64_t>::rows()/cols()        src/ci/determinant_set.hpp:127-134
 *   POLYQUANT_DETSET<uint64_t>::operator()(i, i)     src/ci/determinant_set.hpp:139
 *   POLYQUANT_DETSET<uint64_t>::operator*(X)         src/ci/determinant_set.hpp:170, src/ci/detset/direct.cpp:5-18
 *   POLYQUANT_DETSET<uint64_t>::create_sigma         src/ci/detset/direct.cpp:21-33
 *   POLYQUANT_DETSET<uint64_t>::precompute_diagonal_Slater_Condon  src/ci/detset/slater_condon.cpp:102-153
 *   POLYQUANT_EPCI::setup_determinants               src/ci/epci.cpp:334-388
 *   Spectra::DavidsonSymEigsSolver<DETSET>::compute  (driver call site src/ci/epci.cpp:589-608)
 *
 * Conventions: every function returns a pq_status; nothing calls exit().  The
 * message of the last failure on the calling thread is pq_last_error().  Host
 * buffers belong to the caller, device buffers created by the library belong
 * to the handle.  Calls on one handle are ordered on its CUDA stream; a handle
 * is used by one host thread at a time.  Sizes are int64.
 */
#ifndef PQ_CI_H
#define PQ_CI_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t pq_status;
enum {
  PQ_OK = 0,
  PQ_ERR_ARG = 1,         /* invalid argument or unsupported problem */
  PQ_ERR_CUDA = 2,        /* a CUDA runtime or library call failed */
  PQ_ERR_OOM = 3,         /* device allocation failed */
  PQ_NOT_CONVERGED = 4,   /* Davidson hit its iteration limit; results are the last iterate */
  PQ_TIMEOUT = 5,         /* a bounded device wait gave up */
  PQ_ERR_STATE = 6        /* call out of order (e.g. no GPU, handle destroyed) */
};

enum { PQ_FP64 = 0, PQ_FP32 = 1 };

/* Message of the last failing call on this host thread ("" if none). */
const char *pq_last_error(void);
/* Library version string. */
const char *pq_version(void);

/*
 * One CI problem, in the reference's conventions.
 *  n_orb        active orbitals per species (POLYQUANT_DETSET::max_orb), 1..128;
 *               strings of more than 64 orbitals are held as two words
 *  n_alpha/beta active particles per spin (frozen core already removed)
 *  restricted   1: one spin block of integrals (the reference's `1 % size` rule)
 *  charge       species charge; cross-species terms carry charge[0]*charge[1]
 *  ex_level     {alpha max, beta max, total max} per species
 *               (POLYQUANT_EPCI::excitation_level, ci_keywords "excitation_level")
 *  max_collective  limit on the summed excitation of all species
 *  h1[s][spin]  n_orb x n_orb MO one-body integrals (column-major, host)
 *  eri[a][sa][b][sb]  (npair_a x npair_b) MO ERIs, column-major, element
 *               [idx2(i,j) + idx2(k,l)*npair_a] = (ij|kl), b >= a, host
 *               (POLYQUANT_INTEGRAL::mo_two_body_ints, integral.cpp:479-516)
 * Pointers of the spin index 1 may be NULL for restricted species.
 */
typedef struct {
  int32_t n_species;
  int32_t n_orb[2];
  int32_t n_alpha[2];
  int32_t n_beta[2];
  int32_t restricted[2];
  double charge[2];
  int32_t ex_level[2][3];
  int32_t max_collective;
  const double *h1[2][2];
  const double *eri[2][2][2][2];
} pq_ci_desc;

typedef struct pq_ci_handle pq_ci_handle;

/* Build strings, excitation tables, determinant addressing and the diagonal
 * on the device (replaces setup_determinants + precompute_diagonal).
 * stream: a cudaStream_t, or NULL for the default stream. */
pq_status pq_ci_create(const pq_ci_desc *desc, void *stream, pq_ci_handle **out);
/* Selected-string space (an extension with no reference counterpart: heat-bath
 * selected CI over strings, polyquant_gb300/heatbath.py): the determinants are
 * the full product of caller-chosen string lists, in list order (species 0
 * alpha outermost).  strings[2 s + spin] holds n_strings[2 s + spin]
 * occupation masks (bit o = orbital o; at most 64 orbitals; each with the
 * species' particle count for that spin; no duplicates).  desc supplies the
 * orbitals, particle counts, integrals and charges; its excitation levels and
 * collective limit are ignored.  Everything else (sigma, Davidson, explicit H,
 * elements, properties) works on the handle as on any other. */
pq_status pq_ci_create_selected(const pq_ci_desc *desc, const uint64_t *const *strings, const int64_t *n_strings,
                                void *stream, pq_ci_handle **out);
pq_status pq_ci_destroy(pq_ci_handle *h);

/* rows() == cols() == number of determinants. */
pq_status pq_ci_num_dets(const pq_ci_handle *h, int64_t *n_dets);
/* Strings of one species/spin in the reference layout: n_words per string,
 * word 0 holds the highest orbitals (determinant_creation.cpp:13, 62-68).
 * words == NULL queries n_strings and n_words only. */
pq_status pq_ci_strings(const pq_ci_handle *h, int32_t species, int32_t spin, uint64_t *words, int64_t *n_strings,
                        int32_t *n_words);
/* Unfolded string indices of every determinant, n_dets x (2*n_species), host
 * buffer (det_idx_unfold, determinant_creation.cpp:378-388). */
pq_status pq_ci_det_unfold(const pq_ci_handle *h, int32_t *out);
/* Diagonal H_II (operator()(i,i)); out is a DEVICE buffer of n_dets doubles. */
pq_status pq_ci_diag(pq_ci_handle *h, double *out_device);

/* sigma = H C for nvec vectors (operator*).  C and S are DEVICE buffers,
 * column-major n_dets x nvec with leading dimensions ldc, lds (the Eigen layout
 * the reference passes).  precision: PQ_FP64 or PQ_FP32 (FP32 tables and
 * arithmetic, inputs/outputs still FP64). */
pq_status pq_ci_sigma(pq_ci_handle *h, const double *C, int64_t ldc, int32_t nvec, double *S, int64_t lds,
                      int32_t precision);
/* Same with HOST buffers (blocking).  Page-locked buffers (cudaHostAlloc or
 * cudaHostRegister) are read and written in place by the layout-conversion
 * kernels, so C streams straight from host memory into the interleaved work
 * vectors and sigma straight back.  Pageable buffers are staged: the device
 * copies of C and sigma are kept by the handle and reused by later calls
 * (released with the handle). */
pq_status pq_ci_sigma_host(pq_ci_handle *h, const double *C, int64_t ldc, int32_t nvec, double *S, int64_t lds,
                           int32_t precision);

/* Same as pq_ci_sigma, but allocates nothing: no reference counterpart (the
 * reference's operator* allocates its result on every call).  For callers
 * that may not call cudaMalloc/cudaFree while computing (a host whose device
 * memory is pre-reserved by its own pool, a latency-critical loop that must
 * not hit the implicit synchronisation of cudaMalloc/cudaFree, an iteration
 * recorded into a CUDA graph).  The work vectors live in a fixed 2 x 16 MiB
 * array compiled into the library, so n_dets * w * sizeof(T) must not exceed
 * 16 MiB, where w = 4 for nvec >= 3 (else nvec) and T is double (PQ_FP64) or
 * float (PQ_FP32); larger problems return PQ_ERR_ARG.  The array's device
 * address is looked up on the first call in each CUDA context (make that call
 * before any stream capture) and kept for that context; do not use the
 * library across a cudaDeviceReset, which can move the array.  All calls
 * share the array: calls that overlap on the GPU race and must be serialised
 * by the caller. */
pq_status pq_ci_sigma_noalloc(pq_ci_handle *h, const double *C, int64_t ldc, int32_t nvec, double *S, int64_t lds,
                              int32_t precision);

/* Hamiltonian elements H_IJ = <I|H|J> for any pair of determinant indices
 * (POLYQUANT_DETSET::operator()(i, j) = Slater_Condon(i, j),
 * src/ci/determinant_set.hpp:139, src/ci/detset/slater_condon.cpp:4-100).
 * Exact FP64, computed from the connections of I as sigma applies them, so an
 * explicit matrix built with a screening threshold does not change them.
 * pq_ci_elements: I, J, out are HOST arrays of n entries (n <= 2^26); indices
 * outside 0..n_dets-1 return PQ_ERR_ARG.  Blocking. */
pq_status pq_ci_element(pq_ci_handle *h, int64_t i, int64_t j, double *out);
pq_status pq_ci_elements(pq_ci_handle *h, int64_t n, const int64_t *I, const int64_t *J, double *out);

/* Native-layout sigma on DEVICE buffers interleaved by determinant:
 * X[det * nvec + v].  T = double (precision PQ_FP64) or float (PQ_FP32).
 * diag_shift is subtracted from H_II (sigma = (H - shift*1) X). */
pq_status pq_ci_sigma_interleaved(pq_ci_handle *h, const void *X, void *Y, int32_t nvec, int32_t precision,
                                  double diag_shift);

/* Diagnostic, no reference counterpart: device bytes the handle holds as
 * grow-on-demand work memory (the interleaved vectors of pq_ci_sigma, the
 * host-sigma staging copies, the transposed copies, tensor-core tables and
 * same-spin GEMM buffers of the FP32 full-CI sigma).  Meant for tests. */
pq_status pq_debug_scratch_bytes(const pq_ci_handle *h, int64_t *bytes);

/* Block Davidson on the GPU (replaces Spectra::DavidsonSymEigsSolver with the
 * reference's parameters: initial = num_subspace_vec, max = max(2*initial,
 * 10*num_states), epci.cpp:589-590). */
typedef struct {
  int32_t num_states;
  int32_t num_subspace_vec;
  int32_t max_subspace;      /* <= 0: max(2*num_subspace_vec, 10*num_states) */
  int32_t iteration_max;     /* ci_keywords "iteration_max" (default 500) */
  double convergence_E;      /* residual-norm tolerance (ci_keywords "convergence_E") */
  int32_t precision;         /* PQ_FP64, or PQ_FP32 = FP32 sigma with FP64 refinement */
  double energy_shift;       /* added to eigenvalues (E_nuc + frozen-core energy) */
  int32_t verbose;           /* 1: per-iteration table on stdout */
} pq_davidson_params;

typedef struct {
  int32_t iterations;
  int32_t sigma_calls_fp64;
  int32_t sigma_calls_fp32;
  int32_t converged;
  double max_residual;
  double seconds;
  double sigma_seconds;      /* wall time of the sigma evaluations (layout conversion included) */
} pq_davidson_report;

/* energies: host, num_states doubles (shift included).  vecs: DEVICE buffer
 * n_dets x num_states column-major, or NULL. */
pq_status pq_ci_davidson(pq_ci_handle *h, const pq_davidson_params *p, double *energies, double *vecs,
                         pq_davidson_report *report);

/* ---- explicit sparse Hamiltonian ------------------------------------------
 * Replaces POLYQUANT_DETSET::create_ham (src/ci/detset/explicit_ham.cpp:51-84,
 * explicit_ham_singleparticle.cpp, explicit_ham_mixedparticle.cpp; the
 * reference's default build_matrix path) and its use through
 * Spectra::SparseSymMatProd (src/ci/epci.cpp:623-668).  Builds H on the device
 * (one species or an electron-positron product space, FP64); exact zeros are
 * dropped and,
 * for screening_threshold > 0, every |H_IJ| <= threshold (the reference's
 * ham.prune(threshold, 1.0)).  use_for_sigma != 0 makes FP64 sigma calls
 * (pq_ci_sigma*, pq_ci_davidson's FP64 requests) multiply with the matrix;
 * FP32 requests keep the direct kernels.  *nnz: stored entries (both
 * triangles). */
pq_status pq_ci_ham_build(pq_ci_handle *h, double screening_threshold, int32_t use_for_sigma, int64_t *nnz);
pq_status pq_ci_ham_release(pq_ci_handle *h);

/* Host copy in CSR: upper != 0 gives the reference's storage (upper triangle
 * with the diagonal, row-major, columns ascending), else both triangles.
 * row_ptr: n_dets + 1 entries; col/val: *nnz entries.  Pass NULL arrays to
 * query *nnz first. */
pq_status pq_ci_ham_csr(pq_ci_handle *h, int32_t upper, int64_t *nnz, int64_t *row_ptr, int32_t *col, double *val);

/* ---- properties of CI vectors ----------------------------------------------
 * <S^2> of nvec states for every species: replaces
 * POLYQUANT_DETSET::evaluate_s2 (src/ci/detset/s2.cpp:4-123).  C: DEVICE,
 * n_dets x nvec column-major; s2: host, nvec x n_species values, state-major
 * (s2[v * n_species + s]). */
pq_status pq_ci_s2(pq_ci_handle *h, const double *C, int64_t ldc, int32_t nvec, double *s2);

/* One-particle density matrix of one state, species and spin (0 alpha,
 * 1 beta): replaces create_1rdm (src/ci/detset/rdm1.cpp:4-72).  C: DEVICE,
 * n_dets values; rdm: host, n_orb[species] x n_orb[species] column-major. */
pq_status pq_ci_rdm1(pq_ci_handle *h, const double *C, int32_t species, int32_t spin, double *rdm);

/* ---- batches of independent problems -------------------------------------
 * Many small CI problems of uneven size solved together: one persistent sigma
 * kernel per Davidson iteration covers every active problem (work units
 * pulled from a device counter in descending cost order, FP64 and FP32
 * problems in the same launch), and the per-iteration launch sequence is a
 * CUDA graph replayed each iteration.  The reference runs one
 * POLYQUANT_EPCI::run (src/ci/epci.cpp:575-686) per problem; these calls solve
 * the same eigenproblems with the same sigma terms
 * (src/ci/direct_singleparticle.cpp:238-372,
 * src/ci/direct_mixedparticle.cpp:269-611).
 *
 * Every problem must be a full product of complete string spaces (full CI of
 * species 0, optionally times full CI of species 1 with at most 40
 * determinants); other problems are rejected with PQ_ERR_ARG.  stream may be
 * NULL: the batch then owns a non-blocking stream and synchronises the device
 * on entry to each call. */
typedef struct pq_ci_batch pq_ci_batch;

/* descs: n problem descriptions (integral pointers are read during the call only). */
pq_status pq_ci_batch_create(const pq_ci_desc *descs, int32_t n, void *stream, pq_ci_batch **out);
pq_status pq_ci_batch_destroy(pq_ci_batch *b);
pq_status pq_ci_batch_num_dets(const pq_ci_batch *b, int32_t i, int64_t *n_dets);

/* sigma = H C for every problem: C[i], S[i] DEVICE pointers to n_dets(i) x nvec
 * column-major FP64 (ldc / lds may be NULL; else each entry must equal n_dets). */
pq_status pq_ci_batch_sigma(pq_ci_batch *b, const double *const *C, const int64_t *ldc, int32_t nvec,
                            double *const *S, const int64_t *lds, int32_t precision);

/* Launch shape chosen by the autotuner on the first sigma or Davidson call
 * (0, 0 before that). */
pq_status pq_ci_batch_tuning(const pq_ci_batch *b, int32_t *warps_per_cta, int32_t *rows_per_unit);

/* Block Davidson for every problem with the same parameters.  Problems are
 * processed in groups whose Davidson buffers fit workspace_bytes (0: 80% of
 * the free device memory).  energies: host, n x num_states; reports: host, n
 * entries or NULL.  Returns PQ_NOT_CONVERGED if any problem did not converge. */
pq_status pq_ci_batch_davidson(pq_ci_batch *b, const pq_davidson_params *p, size_t workspace_bytes,
                               double *energies, pq_davidson_report *reports);

#ifdef __cplusplus
}
#endif
#endif
