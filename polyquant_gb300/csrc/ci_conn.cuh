// Enumeration of the determinants connected to one determinant (one species,
// FP64): the diagonal, alpha and beta singles, same-spin doubles and
// alpha-beta doubles, in that order, with their Hamiltonian elements
// (same_part_ham_diag/single/double, slater_condon_singleparticle.cpp:4-175,
// through the excitation tables of ci_setup.cu).  Shared by the exact
// unit-vector columns and the explicit sparse Hamiltonian.
#pragma once
#include "pq_bits.cuh"
#include "pq_internal.h"

namespace pq {

struct ConnArgs {
  const uint64_t *astr, *bstr;
  const uint64_t *astr_hi, *bstr_hi;  // orbitals 64..127 (NULL for one-word strings)
  const int64_t *a1_off, *a2_off, *b1_off, *b2_off;
  const int32_t *a1_J, *a1_info, *a2_J, *b1_J, *b1_info, *b2_J;
  const double *a1_F, *a2_D, *b1_F, *b2_D;
  const int64_t *rowoff;
  const int32_t *rowlen;
  const double *eab;  // (pair_alpha | pair_beta) row-major
  const double *diag;
  int npair;
};

inline ConnArgs make_conn_args(const pq_ci_handle *h) {
  ConnArgs a{};
  const SpinTablesDev &A = h->tab[0][0], &B = h->tab[0][1];
  a.astr = A.str.as<uint64_t>();
  a.bstr = B.str.as<uint64_t>();
  a.astr_hi = A.str_hi.as<uint64_t>();
  a.bstr_hi = B.str_hi.as<uint64_t>();
  a.a1_off = A.s1_off.as<int64_t>();
  a.a2_off = A.s2_off.as<int64_t>();
  a.b1_off = B.s1_off.as<int64_t>();
  a.b2_off = B.s2_off.as<int64_t>();
  a.a1_J = A.s1_J.as<int32_t>();
  a.a1_info = A.s1_info.as<int32_t>();
  a.a2_J = A.s2_J.as<int32_t>();
  a.b1_J = B.s1_J.as<int32_t>();
  a.b1_info = B.s1_info.as<int32_t>();
  a.b2_J = B.s2_J.as<int32_t>();
  a.a1_F = A.s1_F64.as<double>();
  a.a2_D = A.s2_D64.as<double>();
  a.b1_F = B.s1_F64.as<double>();
  a.b2_D = B.s2_D64.as<double>();
  a.rowoff = h->d_rowoff.as<int64_t>();
  a.rowlen = h->d_rowlen.as<int32_t>();
  a.eab = h->d_eab64.as<double>();
  a.diag = h->d_diag.as<double>();
  a.npair = h->npair[0];
  return a;
}

// Offsets and counts of one determinant's connection classes.
struct ConnRow {
  int ia, ib;
  int64_t I, a1b, a2b, b1b, b2b;
  int n1a, n2a, n1b, n2b;
  uint64_t am, bm, amh, bmh;  // occupation words (lo, hi) of the alpha and beta strings
  __device__ __forceinline__ int64_t total() const { return 1 + (int64_t)n1a + n1b + n2a + n2b + (int64_t)n1a * n1b; }
};

__device__ __forceinline__ ConnRow conn_row(const ConnArgs &a, int ia, int ib) {
  ConnRow r;
  r.ia = ia;
  r.ib = ib;
  r.I = a.rowoff[ia] + ib;
  r.a1b = a.a1_off[ia];
  r.a2b = a.a2_off[ia];
  r.b1b = a.b1_off[ib];
  r.b2b = a.b2_off[ib];
  r.n1a = (int)(a.a1_off[ia + 1] - r.a1b);
  r.n2a = (int)(a.a2_off[ia + 1] - r.a2b);
  r.n1b = (int)(a.b1_off[ib + 1] - r.b1b);
  r.n2b = (int)(a.b2_off[ib + 1] - r.b2b);
  r.am = a.astr[ia];
  r.bm = a.bstr[ib];
  r.amh = hiword(a.astr_hi, ia);
  r.bmh = hiword(a.bstr_hi, ib);
  return r;
}

// Connection t (0 <= t < r.total()) of determinant r: returns the partner's
// index, or -1 when the partner is not in the determinant list, and its
// Hamiltonian element in *v.
__device__ __forceinline__ int64_t conn_elem(const ConnArgs &a, const ConnRow &r, int64_t t, double *v) {
  int64_t J = -1;
  double x = 0.0;
  if (t == 0) {
    J = r.I;
    x = a.diag[r.I];
  } else if ((t -= 1) < r.n1a) {
    const int Ja = a.a1_J[r.a1b + t], info = a.a1_info[r.a1b + t], ph = info >> 1;
    double f = a.a1_F[r.a1b + t];
    for_occ(r.bm, r.bmh, [&](int k) { f += a.eab[(int64_t)ph * a.npair + k * (k + 3) / 2]; });
    x = (info & 1) ? -f : f;
    if (r.ib < a.rowlen[Ja]) J = a.rowoff[Ja] + r.ib;
  } else if ((t -= r.n1a) < r.n1b) {
    const int Jb = a.b1_J[r.b1b + t], info = a.b1_info[r.b1b + t], ph = info >> 1;
    double f = a.b1_F[r.b1b + t];
    for_occ(r.am, r.amh, [&](int k) { f += a.eab[(int64_t)(k * (k + 3) / 2) * a.npair + ph]; });
    x = (info & 1) ? -f : f;
    if (Jb < a.rowlen[r.ia]) J = a.rowoff[r.ia] + Jb;
  } else if ((t -= r.n1b) < r.n2a) {
    const int Ja = a.a2_J[r.a2b + t];
    x = a.a2_D[r.a2b + t];
    if (r.ib < a.rowlen[Ja]) J = a.rowoff[Ja] + r.ib;
  } else if ((t -= r.n2a) < r.n2b) {
    const int Jb = a.b2_J[r.b2b + t];
    x = a.b2_D[r.b2b + t];
    if (Jb < a.rowlen[r.ia]) J = a.rowoff[r.ia] + Jb;
  } else {
    t -= r.n2b;
    const int s = (int)(t / r.n1b), q = (int)(t - (int64_t)s * r.n1b);
    const int Ja = a.a1_J[r.a1b + s], ia_ = a.a1_info[r.a1b + s];
    const int Jb = a.b1_J[r.b1b + q], ib_ = a.b1_info[r.b1b + q];
    const double e = a.eab[(int64_t)(ia_ >> 1) * a.npair + (ib_ >> 1)];
    x = ((ia_ ^ ib_) & 1) ? -e : e;
    if (Jb < a.rowlen[Ja]) J = a.rowoff[Ja] + Jb;
  }
  *v = x;
  return J;
}

}  // namespace pq
