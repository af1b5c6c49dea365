// Internal declarations shared by the CUDA translation units of libpq_gb300.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <chrono>
#include <memory>
#include <string>
#include <vector>

#include "pq_ci.h"
#include "pq_ints.h"

struct cublasContext;  // cuBLAS handle type (cublasHandle_t)

// Orbitals per species: strings are held as at most two 64-bit words.
#define PQ_MAX_ORB 128

namespace pq {

// Thread-local error message behind pq_last_error().
void set_error(const char *fmt, ...);
void clear_error();

#define PQ_CUDA_TRY(call)                                                                                  \
  do {                                                                                                     \
    cudaError_t e_ = (call);                                                                               \
    if (e_ != cudaSuccess) {                                                                               \
      pq::set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__);           \
      return e_ == cudaErrorMemoryAllocation ? PQ_ERR_OOM : PQ_ERR_CUDA;                                   \
    }                                                                                                      \
  } while (0)

#define PQ_TRY(expr)                   \
  do {                                 \
    pq_status s_ = (expr);             \
    if (s_ != PQ_OK) return s_;        \
  } while (0)

// Device buffer owned by a handle.
struct DevBuf {
  void *ptr = nullptr;
  size_t bytes = 0;
  ~DevBuf() { release(); }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
  }
  pq_status alloc(size_t n);
  // grow-only allocation used for scratch; contents are not preserved
  pq_status ensure(size_t n) { return n <= bytes ? PQ_OK : alloc(n); }
  template <typename T> T *as() const { return static_cast<T *>(ptr); }
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
};

template <typename T> pq_status upload(DevBuf &b, const std::vector<T> &v, cudaStream_t s) {
  PQ_TRY(b.alloc(v.size() * sizeof(T) + 16));
  if (!v.empty()) PQ_CUDA_TRY(cudaMemcpyAsync(b.ptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
  return PQ_OK;
}

// Excitation tables of one spin list of one species (CSR over strings).
// Single entries: J (string index), info = (pair << 1) | (phase < 0), and the
// same-spin part of the element F = h_hp + sum_{k in occ(I)} ((hp|kk) - (hk|kp)).
// Double entries: J and the full same-spin element value.
struct SpinTablesDev {
  int64_t n_str = 0;
  int64_t n1 = 0, n2 = 0;  // total entries
  int32_t max1 = 0, max2 = 0;
  DevBuf str;              // uint64 occupation masks, bit o = orbital o (orbitals 0..63)
  DevBuf str_hi;           // orbitals 64..127, bit o - 64 (allocated only for wide strings)
  DevBuf s1_off, s1_J, s1_info, s1_F64, s1_F32;
  DevBuf s2_off, s2_J, s2_D64, s2_D32;
  DevBuf e_same64;         // per-string same-spin energy (diagonal part)
};

struct SameSpinGemm;  // ci_sigma32_ss.cu
void ss_delete(SameSpinGemm *g);

}  // namespace pq

struct pq_ci_handle {
  pq_ci_desc desc{};
  cudaStream_t stream = nullptr;
  int n_species = 1;
  int n_orb[2] = {0, 0};
  int npair[2] = {0, 0};
  int n_words = 1;     // words per string in the reference layout, (max n_orb >> 6) + 1
  bool wide = false;   // some species has more than 64 orbitals: strings keep a second word
  bool selected = false;  // strings given by the caller (pq_ci_create_selected): full product, no levels
  int n_blocks[2] = {1, 1};  // spin blocks of integrals per species
  // host strings (occupation masks, reference order) and their levels
  std::vector<uint64_t> str[2][2];
  std::vector<uint64_t> str_hi[2][2];  // orbitals 64..127 of each string (wide only)
  std::vector<int32_t> lvl[2][2];
  // determinant addressing over species-0 alpha strings (single species)
  int64_t n_dets = 0;
  bool full = false;  // every (alpha, beta) pair present
  std::vector<int64_t> rowoff;
  std::vector<int32_t> rowlen;
  pq::DevBuf d_rowoff, d_rowlen;
  pq::SpinTablesDev tab[2][2];
  // cross-spin ERI block (pair_alpha | pair_beta), row-major, per precision
  pq::DevBuf d_eab64, d_eab32;
  pq::DevBuf d_diag;
  // scratch for layout conversion
  pq::DevBuf x_il, y_il;
  // device staging of pq_ci_sigma_host (column-major C and sigma)
  pq::DevBuf host_c, host_s;
  // scratch of the FP32 full-CI sigma (transposed copies) and the transposed cross block
  pq::DevBuf x_t, z_t, d_eba32;
  bool fp32_v2 = false;  // FP32 sigma uses ci_sigma32.cu
  // FP32 alpha-beta doubles on the tensor cores (ci_sigma32_tc.cu): beta scatter table, scale of the
  // integrals, error word and max |X|
  pq::DevBuf tc_btab, tc_aux;
  pq::DevBuf tc_toff, tc_tinfo;  // per tile of 32 beta strings: scatter targets and their contributions
  float tc_sw = 1.0f;
  int tc_sms = 0;
  bool tc_ready = false;
  bool fp32_tc = false;  // the FP32 full-CI sigma uses the tensor-core alpha-beta path
  bool fp32_ss = false;  // ... and the same-spin doubles as tensor-core GEMMs (ci_sigma32_ss.cu)
  std::unique_ptr<pq::SameSpinGemm, void (*)(pq::SameSpinGemm *)> ss{nullptr, pq::ss_delete};
  // two species: addressing of the product space (see ci_two.cu)
  std::vector<int32_t> e_a, e_b;        // species-0 (alpha, beta) string pair of each kept pair ie
  std::vector<int64_t> ebase;           // first determinant of pair ie's species-1 block
  std::vector<int32_t> elev;            // allowed species-1 level of pair ie (-1: empty block)
  int lcap = 0;
  std::vector<int64_t> psize;           // species-1 block size per level
  std::vector<int32_t> prowoff, prowlen;  // (lcap+1) x n_str[1][0]
  std::vector<int64_t> pfirst;          // offset of level L's (a, b) list
  std::vector<int32_t> pdet_a, pdet_b;  // species-1 (alpha, beta) of block entry q, per level
  pq::DevBuf d_e_a, d_e_b, d_ebase, d_elev, d_prowoff, d_prowlen, d_pfirst, d_psize, d_pdet_a, d_pdet_b;
  pq::DevBuf d_ie_first;  // species-0 pair holding the first determinant of each 128-determinant block
  bool full2 = false;     // full product of complete string spaces (arithmetic addressing)
  // integral blocks, row-major: [s] same-species alpha|beta, [se][sp] electron|positron
  pq::DevBuf d_eabs64[2], d_eabs32[2], d_ep64[2][2], d_ep32[2][2];
  pq::DevBuf d_epc64[2][2], d_epc32[2][2];  // cross blocks times charge[0] * charge[1]
  // explicit Hamiltonian (ci_explicit.cu): CSR with both triangles, FP64
  pq::DevBuf d_hrow, d_hcol, d_hval;
  int64_t h_nnz = 0;
  bool use_explicit = false;  // FP64 sigma multiplies with the explicit matrix
};

namespace pq {
// ci_setup.cu
pq_status ci_build(pq_ci_handle *h);
pq_status make_strings(int n_orb, int n_e, int ex_max, std::vector<uint64_t> &out, std::vector<int32_t> &lvl,
                       std::vector<uint64_t> *out_hi = nullptr);
pq_status build_spin_tables(pq_ci_handle *h, int s, int sp, const double *h1_host, const double *eri_host);
// ci_two.cu (electron + positron product space)
pq_status ci_build2(pq_ci_handle *h);
pq_status ci_sigma2_il(pq_ci_handle *h, const void *X, void *Y, int nvp, int precision, double shift);
pq_status ci_unfold2(const pq_ci_handle *h, int32_t *out);
// exact H_IJ of listed pairs: device arrays (t4 = string indices of each I), and the host unfold of one
// determinant of a two-species space
pq_status ci_elements2(pq_ci_handle *h, int64_t n, const int32_t *t4, const int64_t *I, const int64_t *J, double *out);
void ci_unfold2_one(const pq_ci_handle *h, int64_t I, int32_t *t);
// explicit-H rows of a two-species space: counts when cnt != NULL, else fills col/val at row_ptr
pq_status ci_ham_rows2(pq_ci_handle *h, double thr, int32_t *cnt, const int64_t *row_ptr, int32_t *col, double *val);
// ci_sigma.cu
// allow_scratch = false keeps sigma on kernels that need no work memory beyond X and Y
pq_status ci_sigma_il(pq_ci_handle *h, const void *X, void *Y, int nvec, int precision, double shift,
                      bool allow_scratch = true);
// ci_explicit.cu: sigma with the explicit matrix (FP64, interleaved vectors)
pq_status ci_ham_spmv(pq_ci_handle *h, const void *X, void *Y, int nvp);
// exact FP64 columns H[:, dets[c]] into column-major W (one species)
pq_status ci_unit_columns(pq_ci_handle *h, const std::vector<int64_t> &dets, double *W);
// ci_element.cu: exact H_IJ of n pairs (host index arrays, host output)
pq_status ci_elements(pq_ci_handle *h, int64_t n, const int64_t *I, const int64_t *J, double *out);
// interleave width of a block of nv <= 4 vectors: 1, 2 or 4; two-species spaces take 3 in FP64 (their FP64
// sigma is bound by the FP64 pipe, so a padded fourth root would only add FMAs), while in FP32 four roots
// load as one 16-byte vector
inline int il_width(const pq_ci_handle *h, int nv, int precision) {
  if (nv == 3 && h->n_species == 2 && precision == PQ_FP64) return 3;
  return nv == 1 ? 1 : (nv == 2 ? 2 : 4);
}
// ci_sigma32.cu
bool sigma32_v2_applicable(const pq_ci_handle *h);
pq_status ci_sigma32_v2(pq_ci_handle *h, const void *X, void *Y, int nvp, double shift);
// ci_sigma32_tc.cu: Y += alpha-beta doubles of X (FP32, interleaved), on the tensor cores
bool sigma32_tc_applicable(const pq_ci_handle *h);
pq_status ci_sigma32_ab_tc(pq_ci_handle *h, const void *X, void *Y, int nvp);
// ci_sigma32_ss.cu
bool sigma32_ss_applicable(const pq_ci_handle *h);
pq_status ci_sigma32_same_spin_tc(pq_ci_handle *h, const float *X, float *Y);
pq_status ci_sigma32_ss_prepare(pq_ci_handle *h);
const float *ci_sigma32_ss_coulomb(const pq_ci_handle *h, int spin_row);
size_t ci_sigma32_ss_bytes(const pq_ci_handle *h);  // device bytes of the same-spin GEMM state (0 before use)
pq_status ci_to_il(pq_ci_handle *h, const double *C, int64_t ldc, int v0, int nv, int nvp, int precision, void *X);
pq_status ci_from_il(pq_ci_handle *h, const void *Y, int v0, int nv, int nvp, int precision, double *S, int64_t lds);
// ci_davidson.cu
pq_status ci_davidson(pq_ci_handle *h, const pq_davidson_params *p, double *energies, double *vecs,
                      pq_davidson_report *rep);

// A pending sigma evaluation of a Davidson run: dst = H src for cnt columns
// (column-major, leading dimension n_dets); FP32 requests use (H - shift) in
// FP32 and add shift * src back in FP64.
struct SigmaRequest {
  const double *src;
  double *dst;
  int cnt;
  int precision;
  double shift;
};
pq_status sigma_request_single(pq_ci_handle *h, const SigmaRequest &r);

class DavidsonRun {
 public:
  enum Stage { NONE, AFTER_INIT, AFTER_REFINE, AFTER_NEW };
  // shared_cb: a cuBLAS handle bound to h->stream that the run borrows (else it creates its own)
  pq_status init(pq_ci_handle *h, const pq_davidson_params &p, ::cublasContext *shared_cb = nullptr);
  pq_status advance();  // after the pending request was evaluated
  pq_status outputs(double *energies, double *vecs);
  ~DavidsonRun();
  bool pending = false, done = false;
  SigmaRequest req{};
  pq_status result = PQ_NOT_CONVERGED;
  pq_davidson_report rep{};
  std::vector<double> theta, rnorm;
  int iter_max = 500;
  pq_ci_handle *h = nullptr;
  int64_t n = 0;

 private:
  void request(const double *src, double *dst, int cnt, int prec, double s, Stage next);
  pq_status finish_state(pq_status r);
  pq_status rayleigh(int m, std::vector<double> &G);
  pq_status orthonormalize_append(int m, int k, int *added);
  unsigned grid() const { return (unsigned)((n + 255) / 256 < 152 * 16 ? (n + 255) / 256 : 152 * 16); }
  pq_davidson_params p{};
  cudaStream_t st = nullptr;
  ::cublasContext *cb = nullptr;
  bool own_cb = false;
  DevBuf V, W, X, R, T, tmp, dth, didx, coef;
  std::vector<double> Z, Gk;  // Ritz rotation; Rayleigh matrix (mmax x mmax, first g_valid columns valid)
  int g_valid = 0;
  int k = 0, m0 = 0, mmax = 0, m = 0, it = 0, r_restart = 0;
  double tol = 1e-6, switch_tol = 1e-5, shift = 0.0, last_refined = 1e300, best32 = 1e300;
  int stall32 = 0;
  bool exact = true, phase32 = false, just_refined = false, force_refine = false;
  Stage stage = NONE;
  std::chrono::steady_clock::time_point t_start;
};
}  // namespace pq
