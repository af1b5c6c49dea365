// extern "C" entry points of libpq_gb300 (declared in include/pq_ci.h and
// include/pq_ints.h).  Argument checking, error reporting and handle lifetime
// live here; the work is in the .cu translation units.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>

#include "pq_internal.h"

namespace pq {
static thread_local char g_err[1024] = "";

void set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}
void clear_error() { g_err[0] = 0; }

static pq_status check_device() {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    set_error("no CUDA device available (%s)", e == cudaSuccess ? "0 devices" : cudaGetErrorString(e));
    return PQ_ERR_STATE;
  }
  return PQ_OK;
}
}  // namespace pq

using namespace pq;

extern "C" {

const char *pq_last_error(void) { return g_err; }
const char *pq_version(void) { return "polyquant-gb300 0.1 (sm_103a)"; }

pq_status pq_ci_create(const pq_ci_desc *desc, void *stream, pq_ci_handle **out) {
  clear_error();
  if (!desc || !out) {
    set_error("pq_ci_create: NULL argument");
    return PQ_ERR_ARG;
  }
  *out = nullptr;
  PQ_TRY(check_device());
  pq_ci_handle *h = new (std::nothrow) pq_ci_handle();
  if (!h) {
    set_error("host allocation failed");
    return PQ_ERR_OOM;
  }
  h->desc = *desc;
  h->stream = (cudaStream_t)stream;
  pq_status s = ci_build(h);
  if (s != PQ_OK) {
    delete h;
    return s;
  }
  *out = h;
  return PQ_OK;
}

pq_status pq_ci_create_selected(const pq_ci_desc *desc, const uint64_t *const *strings, const int64_t *n_strings,
                                void *stream, pq_ci_handle **out) {
  clear_error();
  if (!desc || !strings || !n_strings || !out || desc->n_species < 1 || desc->n_species > 2) {
    set_error("pq_ci_create_selected: bad arguments");
    return PQ_ERR_ARG;
  }
  *out = nullptr;
  // check the lists before anything touches the device
  for (int s = 0; s < desc->n_species; s++) {
    const int no = desc->n_orb[s];
    if (no < 1 || no > 64) {
      set_error("pq_ci_create_selected: n_orb[%d]=%d outside 1..64", s, no);
      return PQ_ERR_ARG;
    }
    const int ne[2] = {desc->n_alpha[s], desc->n_beta[s]};
    for (int sp = 0; sp < 2; sp++) {
      const int64_t n = n_strings[2 * s + sp];
      const uint64_t *w = strings[2 * s + sp];
      if (n < 1 || n > INT32_MAX / 2 || !w) {
        set_error("pq_ci_create_selected: species %d spin %d: %lld strings", s, sp, (long long)n);
        return PQ_ERR_ARG;
      }
      const uint64_t outside = no >= 64 ? 0ULL : ~((1ULL << no) - 1ULL);
      std::vector<uint64_t> sorted(w, w + n);
      for (uint64_t m : sorted)
        if ((m & outside) || __builtin_popcountll(m) != ne[sp]) {
          set_error("pq_ci_create_selected: species %d spin %d: string %#llx is not %d of %d orbitals", s, sp,
                    (unsigned long long)m, ne[sp], no);
          return PQ_ERR_ARG;
        }
      std::sort(sorted.begin(), sorted.end());
      if (std::adjacent_find(sorted.begin(), sorted.end()) != sorted.end()) {
        set_error("pq_ci_create_selected: species %d spin %d: a string appears twice", s, sp);
        return PQ_ERR_ARG;
      }
    }
  }
  PQ_TRY(check_device());
  pq_ci_handle *h = new (std::nothrow) pq_ci_handle();
  if (!h) {
    set_error("host allocation failed");
    return PQ_ERR_OOM;
  }
  h->desc = *desc;
  // every string at level 0 and no level limits: the determinant list is the full product, in list order
  for (int s = 0; s < desc->n_species; s++)
    for (int t = 0; t < 3; t++) h->desc.ex_level[s][t] = INT32_MAX / 4;
  h->desc.max_collective = INT32_MAX / 4;
  h->selected = true;
  for (int s = 0; s < desc->n_species; s++)
    for (int sp = 0; sp < 2; sp++) {
      const int64_t n = n_strings[2 * s + sp];
      h->str[s][sp].assign(strings[2 * s + sp], strings[2 * s + sp] + n);
      h->lvl[s][sp].assign(n, 0);
    }
  h->stream = (cudaStream_t)stream;
  pq_status st = ci_build(h);
  if (st != PQ_OK) {
    delete h;
    return st;
  }
  *out = h;
  return PQ_OK;
}

pq_status pq_ci_destroy(pq_ci_handle *h) {
  if (!h) return PQ_OK;
  cudaStreamSynchronize(h->stream);
  delete h;
  return PQ_OK;
}

pq_status pq_ci_num_dets(const pq_ci_handle *h, int64_t *n) {
  if (!h || !n) {
    set_error("pq_ci_num_dets: NULL argument");
    return PQ_ERR_ARG;
  }
  *n = h->n_dets;
  return PQ_OK;
}

pq_status pq_ci_strings(const pq_ci_handle *h, int32_t species, int32_t spin, uint64_t *words, int64_t *n_strings,
                        int32_t *n_words) {
  if (!h || species < 0 || species >= h->n_species || spin < 0 || spin > 1) {
    set_error("pq_ci_strings: bad handle/species/spin");
    return PQ_ERR_ARG;
  }
  const std::vector<uint64_t> &s = h->str[species][spin];
  if (n_strings) *n_strings = (int64_t)s.size();
  if (n_words) *n_words = h->n_words;
  if (words) {
    // reference layout: orbital o lives in word n_words-1-(o>>6), bit o&63
    const std::vector<uint64_t> &hi = h->str_hi[species][spin];
    int nw = h->n_words;
    for (size_t i = 0; i < s.size(); i++) {
      for (int w = 0; w < nw; w++) words[i * nw + w] = 0;
      words[i * nw + (nw - 1)] = s[i];
      if (h->wide) words[i * nw + (nw - 2)] = hi[i];
    }
  }
  return PQ_OK;
}

pq_status pq_ci_det_unfold(const pq_ci_handle *h, int32_t *out) {
  if (!h || !out) {
    set_error("pq_ci_det_unfold: NULL argument");
    return PQ_ERR_ARG;
  }
  if (h->n_species == 2) return ci_unfold2(h, out);
  int64_t k = 0;
  for (size_t ia = 0; ia < h->rowlen.size(); ia++)
    for (int32_t ib = 0; ib < h->rowlen[ia]; ib++) {
      out[2 * k] = (int32_t)ia;
      out[2 * k + 1] = ib;
      k++;
    }
  return PQ_OK;
}

pq_status pq_ci_diag(pq_ci_handle *h, double *out_device) {
  if (!h || !out_device) {
    set_error("pq_ci_diag: NULL argument");
    return PQ_ERR_ARG;
  }
  if (h->n_dets)
    PQ_CUDA_TRY(cudaMemcpyAsync(out_device, h->d_diag.ptr, sizeof(double) * h->n_dets, cudaMemcpyDeviceToDevice,
                                h->stream));
  PQ_CUDA_TRY(cudaStreamSynchronize(h->stream));
  return PQ_OK;
}

static pq_status sigma_device(pq_ci_handle *h, const double *C, int64_t ldc, int32_t nvec, double *S, int64_t lds,
                              int32_t precision) {
  if (!h || !C || !S || nvec < 1 || ldc < h->n_dets || lds < h->n_dets) {
    set_error("pq_ci_sigma: bad arguments (nvec=%d, ldc=%lld, lds=%lld, n_dets=%lld)", nvec, (long long)ldc,
              (long long)lds, (long long)(h ? h->n_dets : 0));
    return PQ_ERR_ARG;
  }
  if (precision != PQ_FP64 && precision != PQ_FP32) {
    set_error("pq_ci_sigma: precision must be PQ_FP64 or PQ_FP32");
    return PQ_ERR_ARG;
  }
  size_t esz = precision == PQ_FP64 ? sizeof(double) : sizeof(float);
  for (int v0 = 0; v0 < nvec; v0 += 4) {
    int nv = nvec - v0 < 4 ? nvec - v0 : 4;
    int nvp = il_width(h, nv, precision);
    size_t bytes = esz * (size_t)nvp * (size_t)(h->n_dets + 1);
    PQ_TRY(h->x_il.ensure(bytes));
    PQ_TRY(h->y_il.ensure(bytes));
    PQ_TRY(ci_to_il(h, C, ldc, v0, nv, nvp, precision, h->x_il.ptr));
    PQ_TRY(ci_sigma_il(h, h->x_il.ptr, h->y_il.ptr, nvp, precision, 0.0));
    PQ_TRY(ci_from_il(h, h->y_il.ptr, v0, nv, nvp, precision, S, lds));
  }
  return PQ_OK;
}

pq_status pq_ci_sigma(pq_ci_handle *h, const double *C, int64_t ldc, int32_t nvec, double *S, int64_t lds,
                      int32_t precision) {
  clear_error();
  return sigma_device(h, C, ldc, nvec, S, lds, precision);
}

// Device address of a page-locked (pinned or registered) host buffer; NULL for pageable memory.
static const void *mapped_host(const void *p) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();  // clear the sticky-free error of an unknown pointer
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

pq_status pq_ci_sigma_host(pq_ci_handle *h, const double *C, int64_t ldc, int32_t nvec, double *S, int64_t lds,
                           int32_t precision) {
  clear_error();
  if (!h || !C || !S || nvec < 1 || ldc < h->n_dets || lds < h->n_dets) {
    set_error("pq_ci_sigma_host: bad arguments (nvec=%d, ldc=%lld, lds=%lld, n_dets=%lld)", nvec, (long long)ldc,
              (long long)lds, (long long)(h ? h->n_dets : 0));
    return PQ_ERR_ARG;
  }
  int64_t n = h->n_dets;
  // Page-locked buffers are read and written in place: the layout conversions around sigma load C from host
  // memory and store sigma back to it (over NVLink-C2C on Grace), so nothing is staged and the transfers run
  // on all SMs instead of one copy engine.
  const void *mc = mapped_host(C), *ms = mapped_host(S);
  if (mc && ms && getenv("PQ_SIGMA_HOST_STAGED") == nullptr) {
    PQ_TRY(sigma_device(h, (const double *)mc, ldc, nvec, (double *)ms, lds, precision));
    PQ_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return PQ_OK;
  }
  // pageable buffers: device copies of C and sigma stay with the handle (grow-only), so repeated calls
  // allocate nothing; with ldc == n (and lds == n) each block moves in one copy
  const size_t bytes = sizeof(double) * (size_t)n * nvec + 16;
  PQ_TRY(h->host_c.ensure(bytes));
  PQ_TRY(h->host_s.ensure(bytes));
  double *dc = h->host_c.as<double>(), *ds = h->host_s.as<double>();
  if (ldc == n) {
    PQ_CUDA_TRY(cudaMemcpyAsync(dc, C, sizeof(double) * (size_t)n * nvec, cudaMemcpyHostToDevice, h->stream));
  } else {
    for (int v = 0; v < nvec; v++)
      PQ_CUDA_TRY(cudaMemcpyAsync(dc + (size_t)v * n, C + (size_t)v * ldc, sizeof(double) * n, cudaMemcpyHostToDevice,
                                  h->stream));
  }
  PQ_TRY(sigma_device(h, dc, n, nvec, ds, n, precision));
  if (lds == n) {
    PQ_CUDA_TRY(cudaMemcpyAsync(S, ds, sizeof(double) * (size_t)n * nvec, cudaMemcpyDeviceToHost, h->stream));
  } else {
    for (int v = 0; v < nvec; v++)
      PQ_CUDA_TRY(cudaMemcpyAsync(S + (size_t)v * lds, ds + (size_t)v * n, sizeof(double) * n, cudaMemcpyDeviceToHost,
                                  h->stream));
  }
  PQ_CUDA_TRY(cudaStreamSynchronize(h->stream));
  return PQ_OK;
}

pq_status pq_ci_sigma_interleaved(pq_ci_handle *h, const void *X, void *Y, int32_t nvec, int32_t precision,
                                  double diag_shift) {
  clear_error();
  if (!h || !X || !Y) {
    set_error("pq_ci_sigma_interleaved: NULL argument");
    return PQ_ERR_ARG;
  }
  return ci_sigma_il(h, X, Y, nvec, precision, diag_shift);
}

pq_status pq_debug_scratch_bytes(const pq_ci_handle *h, int64_t *bytes) {
  if (!h || !bytes) {
    set_error("pq_debug_scratch_bytes: NULL argument");
    return PQ_ERR_ARG;
  }
  *bytes = (int64_t)(h->x_il.bytes + h->y_il.bytes + h->x_t.bytes + h->z_t.bytes + h->tc_btab.bytes + h->tc_aux.bytes +
                     h->tc_toff.bytes + h->tc_tinfo.bytes + h->host_c.bytes + h->host_s.bytes + ci_sigma32_ss_bytes(h));
  return PQ_OK;
}

pq_status pq_ci_davidson(pq_ci_handle *h, const pq_davidson_params *p, double *energies, double *vecs,
                         pq_davidson_report *report) {
  clear_error();
  if (!h || !p || !energies) {
    set_error("pq_ci_davidson: NULL argument");
    return PQ_ERR_ARG;
  }
  return ci_davidson(h, p, energies, vecs, report);
}

}  // extern "C"
