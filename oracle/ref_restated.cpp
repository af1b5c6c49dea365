// Reference-faithful restatement of the sigma builds -- TEST AND BASELINE
// INFRASTRUCTURE ONLY (never linked into the product library).
//
// Keeps the data structures and loop order of
// POLYQUANT_DETSET::sigma_one_species_class_singleshot
// (src/ci/detset/direct_singleparticle.cpp:238-372) and
// sigma_two_species_class_singleshot (direct_mixedparticle.cpp:269-611) so
// that their CPU cost can be measured: the determinant index is a hash map
// from the string-index tuple to the global index (determinant_set.hpp:100),
// det_idx_unfold is a linear search of that map for the value
// (determinant_creation.cpp:378-388) -- called by every thread for every
// determinant before the thread filter in the one-species builder, after it
// in the two-species one -- single/double maps are per-string index lists,
// each thread accumulates into a private N x k sigma, and the private copies
// are summed in a critical section.  Each connected pair (I, J) whose first
// changed string index grows from I to J is visited once and updates sigma_I
// and sigma_J; exact-zero elements are skipped.  The Slater-Condon elements
// are the C oracle's (orc_same_part_ham_* and orc_mixed_part_ham_*, restating
// slater_condon_{single,mixed}particle.cpp, cross terms times charge[0] *
// charge[1]) and the diagonal is orc_diagonal.
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
  int ns = 1;
  double cf = 0.0;  // charge[0] * charge[1]
  std::unordered_map<std::vector<int>, int, TupleHash> dets;
  std::vector<std::vector<size_t>> singles[2][2], doubles[2][2];  // [species][spin][string]
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
  if (d->n_species != 1 && d->n_species != 2) return nullptr;
  orc_detset *ds = orc_detset_create(d, 0);
  if (!ds) return nullptr;
  RefDetset *r = new RefDetset();
  r->ds = ds;
  r->ns = d->n_species;
  r->cf = d->n_species == 2 ? d->charge[0] * d->charge[1] : 0.0;
  r->n = orc_n_dets(ds);
  const int nt = 2 * r->ns;
  const int32_t *u = orc_unfold(ds);
  r->dets.reserve((size_t)r->n);
  for (int64_t i = 0; i < r->n; i++) r->dets[std::vector<int>(u + nt * i, u + nt * (i + 1))] = (int)i;
  for (int sp = 0; sp < r->ns; sp++)
    for (int spin = 0; spin < 2; spin++) {
      int64_t nstr = orc_n_strings(ds, sp, spin);
      r->singles[sp][spin].resize(nstr);
      r->doubles[sp][spin].resize(nstr);
      for (int64_t s = 0; s < nstr; s++) {
        const int32_t *l;
        int64_t m = orc_singles(ds, sp, spin, s, &l);
        r->singles[sp][spin][s].assign(l, l + m);
        m = orc_doubles(ds, sp, spin, s, &l);
        r->doubles[sp][spin][s].assign(l, l + m);
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

static void sigma_two(RefDetset *r, const double *C, int64_t ldc, int nvec, double *S, int64_t lds, int nthreads);

// S = H C for nvec column-major vectors (ldc, lds >= n_dets).
void refalg_sigma(void *p, const double *C, int64_t ldc, int nvec, double *S, int64_t lds, int nthreads) {
  RefDetset *r = (RefDetset *)p;
  if (r->ns == 2) {
    sigma_two(r, C, ldc, nvec, S, lds, nthreads);
    return;
  }
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
      for (size_t ja : r->singles[0][0][ia]) {
        if ((int)ja < ia) continue;
        auto it = r->dets.find({(int)ja, ib});
        if (it != r->dets.end()) {
          const int32_t J[4] = {(int32_t)ja, ib, 0, 0};
          pair(i, it->second, orc_same_part_ham_single(r->ds, 0, I, J));
        }
        for (size_t jb : r->singles[0][1][ib]) {
          auto it2 = r->dets.find({(int)ja, (int)jb});
          if (it2 != r->dets.end()) {
            const int32_t J[4] = {(int32_t)ja, (int32_t)jb, 0, 0};
            pair(i, it2->second, orc_same_part_ham_double(r->ds, 0, I, J));
          }
        }
      }
      for (size_t jb : r->singles[0][1][ib]) {
        if ((int)jb < ib) continue;
        auto it = r->dets.find({ia, (int)jb});
        if (it != r->dets.end()) {
          const int32_t J[4] = {ia, (int32_t)jb, 0, 0};
          pair(i, it->second, orc_same_part_ham_single(r->ds, 0, I, J));
        }
      }
      for (size_t ja : r->doubles[0][0][ia]) {
        if ((int)ja < ia) continue;
        auto it = r->dets.find({(int)ja, ib});
        if (it != r->dets.end()) {
          const int32_t J[4] = {(int32_t)ja, ib, 0, 0};
          pair(i, it->second, orc_same_part_ham_double(r->ds, 0, I, J));
        }
      }
      for (size_t jb : r->doubles[0][1][ib]) {
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

// sigma_two_species_class_singleshot: slots A, B, C, D = (species 0 alpha,
// species 0 beta, species 1 alpha, species 1 beta).  For each slot s, singles
// with a larger string index (same-species single + cf * cross single), then
// those singles combined with singles of every later slot (same-species
// alpha-beta double + cf * cross double, or cf * cross double across the
// species), then same-spin doubles with a larger string index.
static void sigma_two(RefDetset *r, const double *C, int64_t ldc, int nvec, double *S, int64_t lds, int nthreads) {
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
      if (i % nt != tid) continue;
      const std::vector<int> iu = r->unfold(i);
      const int32_t I[4] = {iu[0], iu[1], iu[2], iu[3]};
      for (int v = 0; v < nvec; v++) priv[(size_t)v * n + i] += r->diag[i] * C[i + v * ldc];
      for (int slot = 0; slot < 4; slot++) {
        const int sp = slot >> 1, spin = slot & 1;
        for (size_t js : r->singles[sp][spin][iu[slot]]) {
          if ((int)js < iu[slot]) continue;
          std::vector<int> ju = iu;
          ju[slot] = (int)js;
          auto it = r->dets.find(ju);
          if (it != r->dets.end()) {
            const int32_t J[4] = {ju[0], ju[1], ju[2], ju[3]};
            const double h = orc_same_part_ham_single(r->ds, sp, I, J) + r->cf * orc_mixed_part_ham_single(r->ds, 0, 1, I, J);
            pair(i, it->second, h);
          }
          for (int slot2 = slot + 1; slot2 < 4; slot2++) {
            const int sp2 = slot2 >> 1, spin2 = slot2 & 1;
            for (size_t js2 : r->singles[sp2][spin2][iu[slot2]]) {
              std::vector<int> ku = ju;
              ku[slot2] = (int)js2;
              auto it2 = r->dets.find(ku);
              if (it2 == r->dets.end()) continue;
              const int32_t K[4] = {ku[0], ku[1], ku[2], ku[3]};
              double h = r->cf * orc_mixed_part_ham_double(r->ds, 0, 1, I, K);
              if (sp2 == sp) h += orc_same_part_ham_double(r->ds, sp, I, K);
              pair(i, it2->second, h);
            }
          }
        }
      }
      for (int slot = 0; slot < 4; slot++) {
        const int sp = slot >> 1, spin = slot & 1;
        for (size_t js : r->doubles[sp][spin][iu[slot]]) {
          if ((int)js < iu[slot]) continue;
          std::vector<int> ju = iu;
          ju[slot] = (int)js;
          auto it = r->dets.find(ju);
          if (it == r->dets.end()) continue;
          const int32_t J[4] = {ju[0], ju[1], ju[2], ju[3]};
          pair(i, it->second, orc_same_part_ham_double(r->ds, sp, I, J));
        }
      }
    }
#pragma omp critical
    for (int v = 0; v < nvec; v++)
      for (int64_t i = 0; i < n; i++) S[i + v * lds] += priv[(size_t)v * n + i];
  }
}
