// Reference-faithful restatement of the one-species sigma build -- TEST AND
// BASELINE INFRASTRUCTURE ONLY (never linked into the product library).
//
// Keeps the data structures and loop order of
// POLYQUANT_DETSET::sigma_one_species_class_singleshot
// (src/ci/detset/direct_singleparticle.cpp:238-372) so that its CPU cost can be
// measured: the determinant index is a hash map from the string-index tuple
// to the global index (determinant_set.hpp:100), det_idx_unfold is a linear
// search of that map for the value (determinant_creation.cpp:378-388) and is
// called by every thread for every determinant before the thread filter,
// single/double maps are per-string index lists, each thread accumulates
// into a private N x k sigma, and the private copies are summed in a critical
// section.  Each connected pair (I, J) with J's string index >= I's is
// visited once and updates sigma_I and sigma_J; exact-zero elements are
// skipped.  The Slater-Condon elements are the C oracle's
// (orc_same_part_ham_single/double, restating slater_condon_singleparticle.cpp)
// and the diagonal is orc_diagonal.
#include <omp.h>

#include <cstdint>
#include <cstring>
#include <unordered_map>
#include <vector>

extern "C" {
#include "pq_oracle.h"
}

namespace {

struct TupleHash {
  size_t operator()(const std::vector<int> &v) const {
    size_t h = 1469598103934665603ull;
    for (int x : v) h = (h ^ (size_t)(uint32_t)x) * 1099511628211ull;
    return h;
  }
};

struct RefDetset {
  orc_detset *ds = nullptr;  // strings, maps, elements and diagonal of the C oracle
  int64_t n = 0;
  std::unordered_map<std::vector<int>, int, TupleHash> dets;
  std::vector<std::vector<size_t>> singles[2], doubles[2];
  const double *diag = nullptr;

  std::vector<int> unfold(int64_t i) const {
    for (const auto &kv : dets)
      if (kv.second == i) return kv.first;
    return {};
  }
};

}  // namespace

extern "C" {

void *refalg_create(const orc_desc *d) {
  if (d->n_species != 1) return nullptr;
  orc_detset *ds = orc_detset_create(d, 0);
  if (!ds) return nullptr;
  RefDetset *r = new RefDetset();
  r->ds = ds;
  r->n = orc_n_dets(ds);
  const int32_t *u = orc_unfold(ds);
  r->dets.reserve((size_t)r->n);
  for (int64_t i = 0; i < r->n; i++) r->dets[{u[2 * i], u[2 * i + 1]}] = (int)i;
  for (int sp = 0; sp < 2; sp++) {
    int64_t ns = orc_n_strings(ds, 0, sp);
    r->singles[sp].resize(ns);
    r->doubles[sp].resize(ns);
    for (int64_t s = 0; s < ns; s++) {
      const int32_t *l;
      int64_t m = orc_singles(ds, 0, sp, s, &l);
      r->singles[sp][s].assign(l, l + m);
      m = orc_doubles(ds, 0, sp, s, &l);
      r->doubles[sp][s].assign(l, l + m);
    }
  }
  r->diag = orc_diagonal(ds);
  return r;
}

void refalg_destroy(void *p) {
  RefDetset *r = (RefDetset *)p;
  if (!r) return;
  orc_detset_destroy(r->ds);
  delete r;
}

int64_t refalg_n_dets(const void *p) { return ((const RefDetset *)p)->n; }

// S = H C for nvec column-major vectors (ldc, lds >= n_dets).
void refalg_sigma(void *p, const double *C, int64_t ldc, int nvec, double *S, int64_t lds, int nthreads) {
  RefDetset *r = (RefDetset *)p;
  const int64_t n = r->n;
  if (nthreads <= 0) nthreads = omp_get_max_threads();
  for (int v = 0; v < nvec; v++) std::memset(S + v * lds, 0, sizeof(double) * n);
#pragma omp parallel num_threads(nthreads)
  {
    const int nt = omp_get_num_threads(), tid = omp_get_thread_num();
    std::vector<double> priv((size_t)n * nvec, 0.0);
    auto pair = [&](int64_t i, int64_t j, double h) {
      if (h == 0.0) return;
      for (int v = 0; v < nvec; v++) {
        priv[(size_t)v * n + i] += h * C[j + v * ldc];
        priv[(size_t)v * n + j] += h * C[i + v * ldc];
      }
    };
    for (int64_t i = 0; i < n; i++) {
      const std::vector<int> iu = r->unfold(i);  // every thread, every determinant
      if (i % nt != tid) continue;
      const int ia = iu[0], ib = iu[1];
      const int32_t I[4] = {ia, ib, 0, 0};
      for (int v = 0; v < nvec; v++) priv[(size_t)v * n + i] += r->diag[i] * C[i + v * ldc];
      for (size_t ja : r->singles[0][ia]) {
        if ((int)ja < ia) continue;
        auto it = r->dets.find({(int)ja, ib});
        if (it != r->dets.end()) {
          const int32_t J[4] = {(int32_t)ja, ib, 0, 0};
          pair(i, it->second, orc_same_part_ham_single(r->ds, 0, I, J));
        }
        for (size_t jb : r->singles[1][ib]) {
          auto it2 = r->dets.find({(int)ja, (int)jb});
          if (it2 != r->dets.end()) {
            const int32_t J[4] = {(int32_t)ja, (int32_t)jb, 0, 0};
            pair(i, it2->second, orc_same_part_ham_double(r->ds, 0, I, J));
          }
        }
      }
      for (size_t jb : r->singles[1][ib]) {
        if ((int)jb < ib) continue;
        auto it = r->dets.find({ia, (int)jb});
        if (it != r->dets.end()) {
          const int32_t J[4] = {ia, (int32_t)jb, 0, 0};
          pair(i, it->second, orc_same_part_ham_single(r->ds, 0, I, J));
        }
      }
      for (size_t ja : r->doubles[0][ia]) {
        if ((int)ja < ia) continue;
        auto it = r->dets.find({(int)ja, ib});
        if (it != r->dets.end()) {
          const int32_t J[4] = {(int32_t)ja, ib, 0, 0};
          pair(i, it->second, orc_same_part_ham_double(r->ds, 0, I, J));
        }
      }
      for (size_t jb : r->doubles[1][ib]) {
        if ((int)jb < ib) continue;
        auto it = r->dets.find({ia, (int)jb});
        if (it != r->dets.end()) {
          const int32_t J[4] = {ia, (int32_t)jb, 0, 0};
          pair(i, it->second, orc_same_part_ham_double(r->ds, 0, I, J));
        }
      }
    }
#pragma omp critical
    for (int v = 0; v < nvec; v++)
      for (int64_t i = 0; i < n; i++) S[i + v * lds] += priv[(size_t)v * n + i];
  }
}

}  // extern "C"
