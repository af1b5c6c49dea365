// Two-species (e.g. electron + positron) determinant space and sigma = H C.
//
// Reference behaviour (paths inside the polyquant project):
//   det list        src/ci/detset/determinant_creation.cpp:148-206 (four nested
//                   loops; species-0 pair kept if its excitation <= total[0],
//                   species-1 pair if <= total[1] and the sum <= max_collective)
//   diagonal        src/ci/detset/slater_condon.cpp:102-153 (cross term once)
//   cross elements  src/ci/detset/slater_condon_mixedparticle.cpp:4-236,
//                   multiplied by charge[0]*charge[1]
//   sigma           src/ci/detset/direct_mixedparticle.cpp:269-611
//                   (sigma_two_species_class_singleshot)
//
// Addressing: species-0 (alpha, beta) pairs are kept as prefix rows exactly as
// for one species; each kept pair ie owns a contiguous block of species-1
// pairs whose allowed level L = min(total[1], max_collective - level(ie))
// depends only on ie, and the blocks of one level share one prefix-row layout:
//   det(ea, eb, pa, pb) = ebase[ie] + prowoff[L][pa] + pb  (pb < prowlen[L][pa]).
// This reproduces the reference's sequential numbering of the nested loops.
//
// Kernel: one CTA per species-0 pair, threads over the determinants of its
// block; each thread gathers H_IJ C_J over every connection class of the
// reference's singleshot builder (singles of each of the four spin lists with
// their same-species and cross-species Coulomb terms, same-spin doubles,
// alpha-beta doubles within a species, single x single cross doubles).
#include <algorithm>
#include <type_traits>

#include "pq_bits.cuh"
#include "pq_internal.h"

namespace pq {

__device__ __forceinline__ int tri2(int i, int j) { return i > j ? i * (i + 1) / 2 + j : j * (j + 1) / 2 + i; }

template <typename T> struct List2 {
  const uint64_t *str, *str_hi;  // str_hi: orbitals 64..127 (NULL for one-word strings)
  const int64_t *s1_off;
  const int32_t *s1_J;
  const int32_t *s1_info;
  const T *s1_F;
  const int64_t *s2_off;
  const int32_t *s2_J;
  const T *s2_D;
};

template <typename T> struct Args2 {
  List2<T> l[4];  // slots: species0 alpha, species0 beta, species1 alpha, species1 beta
  int npair[2];
  int npa1;       // number of species-1 alpha strings (row length of the per-level tables)
  const T *eab[2];      // [species] (pair_alpha | pair_beta) row-major
  const T *ep[2][2];    // [spin block of species 0][spin block of species 1] (pair_0 | pair_1) row-major
  const T *epc[2][2];   // the same blocks times charge[0] * charge[1] (the cross doubles' coefficient)
  int blk[2][2];        // [species][spin] -> spin block index
  T cf;                 // charge[0] * charge[1]
  const int32_t *rowoff0, *rowlen0;
  const int32_t *e_a, *e_b, *elev;
  const int64_t *ebase;
  const int32_t *prowoff, *prowlen;
  const int64_t *pfirst, *psize;
  const int32_t *pdet_a, *pdet_b;
  const double *diag;
  double shift;
  const T *X;
  T *Y;
  // full product of complete string spaces: det(t) = ((t0 * nst[1] + t1) * nst[2] + t2) * nst[3] + t3
  int nst[4];
};

template <typename T, bool FULL = false>
__device__ __forceinline__ int64_t lookup2(const Args2<T> &p, const int (&t)[4]) {
  if (FULL) return (((int64_t)t[0] * p.nst[1] + t[1]) * p.nst[2] + t[2]) * p.nst[3] + t[3];
  if (t[1] >= p.rowlen0[t[0]]) return -1;
  const int ie = p.rowoff0[t[0]] + t[1];
  const int L = p.elev[ie];
  if (L < 0) return -1;
  const int64_t r = (int64_t)L * p.npa1 + t[2];
  if (t[3] >= p.prowlen[r]) return -1;
  return p.ebase[ie] + p.prowoff[r] + t[3];
}

template <typename T, int NV> __device__ __forceinline__ void axpy_gather(T (&acc)[NV], T c, const T *X, int64_t j) {
#pragma unroll
  for (int v = 0; v < NV; v++) acc[v] = fma(c, __ldg(X + j * NV + v), acc[v]);
}
// four FP32 roots: one 16-byte load (the interleaved rows are 16-byte aligned)
template <> __device__ __forceinline__ void axpy_gather<float, 4>(float (&acc)[4], float c, const float *X, int64_t j) {
  const float4 x = __ldg(reinterpret_cast<const float4 *>(X) + j);
  acc[0] = fmaf(c, x.x, acc[0]);
  acc[1] = fmaf(c, x.y, acc[1]);
  acc[2] = fmaf(c, x.z, acc[2]);
  acc[3] = fmaf(c, x.w, acc[3]);
}

// sum over occupied orbitals k of the string (m, mh) of M[row * ld + tri(k,k)] (row fixed) or
// M[tri(k,k) * ld + col]
template <typename T> __device__ __forceinline__ T coul_row(const T *M, int ld, int row, uint64_t m, uint64_t mh) {
  T s = 0;
  for_occ(m, mh, [&](int k) { s += __ldg(M + (int64_t)row * ld + tri2(k, k)); });
  return s;
}
template <typename T> __device__ __forceinline__ T coul_col(const T *M, int ld, int col, uint64_t m, uint64_t mh) {
  T s = 0;
  for_occ(m, mh, [&](int k) { s += __ldg(M + (int64_t)tri2(k, k) * ld + col); });
  return s;
}

// occupation words (lo, hi) of the four strings of determinant t
template <typename T>
__device__ __forceinline__ void load_words(const Args2<T> &p, const int (&t)[4], uint64_t (&m)[4], uint64_t (&mh)[4]) {
#pragma unroll
  for (int s = 0; s < 4; s++) {
    m[s] = p.l[s].str[t[s]];
    mh[s] = hiword(p.l[s].str_hi, t[s]);
  }
}

// v or -v selected by the low bit of `neg`, on the integer pipe (a negation would be an FP64 instruction)
__device__ __forceinline__ float flip2(float v, uint32_t neg) { return __int_as_float(__float_as_int(v) ^ (int)(neg << 31)); }
__device__ __forceinline__ double flip2(double v, uint32_t neg) {
  return __hiloint2double(__double2hiint(v) ^ (int)(neg << 31), __double2loint(v));
}

// Every off-diagonal connection of determinant t (string indices per slot,
// occupation words m, mh) in the classes of the reference's singleshot builder: singles of
// each of the four spin lists with their same-species and cross-species
// Coulomb terms, alpha-beta doubles within a species, single x single cross
// doubles, same-spin doubles.  f(J, H_IJ) is called for each partner J that is
// in the determinant list; each partner appears once.
// FULL: the space is a full product of complete string spaces (every lookup is arithmetic).
template <bool FULL = false, typename T, typename F>
__device__ __forceinline__ void two_conn_visit(const Args2<T> &p, const int (&t)[4], const uint64_t (&m)[4],
                                               const uint64_t (&mh)[4], F &&f) {
  // FP32: the slot loops are unrolled, so slots are constants and the string-index arrays stay in registers
  // (34 % faster on the PsH-like space); the FP64 kernel is bound by its FP64 pipe and keeps the compact
  // loops and its register count
  constexpr bool UNROLL = std::is_same<T, float>::value;
  // the connections of one slot s (its singles, their single x single partners in later slots, its
  // same-spin doubles)
  auto slot = [&](const int s) {
    const int sp = s >> 1, spin = s & 1, other = s ^ 1;
    const List2<T> &ls = p.l[s];
    const int np = p.npair[sp];
    const int64_t o0 = ls.s1_off[t[s]], o1 = ls.s1_off[t[s] + 1];
    for (int64_t e = o0; e < o1; e++) {
      const int info = __ldg(ls.s1_info + e);
      const int pr = info >> 1;
      const uint32_t neg = (uint32_t)(info & 1);
      int tj[4] = {t[0], t[1], t[2], t[3]};
      tj[s] = __ldg(ls.s1_J + e);
      // single in slot s
      const int64_t j = lookup2<T, FULL>(p, tj);
      if (j >= 0) {
        T h = __ldg(ls.s1_F + e);
        h += spin == 0 ? coul_row(p.eab[sp], np, pr, m[other], mh[other])
                       : coul_col(p.eab[sp], np, pr, m[other], mh[other]);
        T x = 0;
        if (sp == 0) {
          x += coul_row(p.ep[p.blk[0][spin]][p.blk[1][0]], p.npair[1], pr, m[2], mh[2]);
          x += coul_row(p.ep[p.blk[0][spin]][p.blk[1][1]], p.npair[1], pr, m[3], mh[3]);
        } else {
          x += coul_col(p.ep[p.blk[0][0]][p.blk[1][spin]], p.npair[1], pr, m[0], mh[0]);
          x += coul_col(p.ep[p.blk[0][1]][p.blk[1][spin]], p.npair[1], pr, m[1], mh[1]);
        }
        h += p.cf * x;
        h = flip2(h, neg);
        f(j, h);
      }
      // single x single in a later slot r
      auto pair_with = [&](const int r) {
        const List2<T> &lr = p.l[r];
        const int64_t q0 = lr.s1_off[t[r]], q1 = lr.s1_off[t[r] + 1];
        for (int64_t g = q0; g < q1; g++) {
          int tk[4] = {tj[0], tj[1], tj[2], tj[3]};
          tk[r] = __ldg(lr.s1_J + g);
          const int64_t k = lookup2<T, FULL>(p, tk);
          if (k < 0) continue;
          const int info2 = __ldg(lr.s1_info + g);
          const int pr2 = info2 >> 1;
          T c;
          if ((r >> 1) == sp) {  // alpha-beta double within one species
            c = __ldg(p.eab[sp] + (int64_t)pr * np + pr2);
          } else {                // cross-species double: species-0 slot s, species-1 slot r
            c = __ldg(p.epc[p.blk[0][spin]][p.blk[1][r & 1]] + (int64_t)pr * p.npair[1] + pr2);
          }
          c = flip2(c, neg ^ (uint32_t)(info2 & 1));
          f(k, c);
        }
      };
      if constexpr (UNROLL) {
#pragma unroll
        for (int r = s + 1; r < 4; r++) pair_with(r);
      } else {
        for (int r = s + 1; r < 4; r++) pair_with(r);
      }
    }
    // same-spin doubles in slot s
    const int64_t d0 = ls.s2_off[t[s]], d1 = ls.s2_off[t[s] + 1];
    for (int64_t e = d0; e < d1; e++) {
      int tj[4] = {t[0], t[1], t[2], t[3]};
      tj[s] = __ldg(ls.s2_J + e);
      const int64_t j = lookup2<T, FULL>(p, tj);
      if (j >= 0) f(j, __ldg(ls.s2_D + e));
    }
  };
  if constexpr (UNROLL) {
#pragma unroll
    for (int s = 0; s < 4; s++) slot(s);
  } else {
    for (int s = 0; s < 4; s++) slot(s);
  }
}

// Thread per determinant over the flat determinant list (every thread busy, whatever the block sizes).
// FULL: string indices by division; otherwise the species-0 pair holding I is found from the pair at
// which the CTA's first determinant lies (a few steps forward through the sorted block bases).
// WIDE: strings of more than 64 orbitals (two words); one-word spaces keep the hi words at compile-time zero.
template <typename T, int NV, bool FULL, bool WIDE>
__global__ void __launch_bounds__(128) sigma_two_species_kernel(Args2<T> p, int64_t n_dets, const int32_t *ie_first) {
  const int64_t I = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= n_dets) return;
  int t[4];
  if (FULL) {
    int64_t r = I;
    t[3] = (int)(r % p.nst[3]);
    r /= p.nst[3];
    t[2] = (int)(r % p.nst[2]);
    r /= p.nst[2];
    t[1] = (int)(r % p.nst[1]);
    t[0] = (int)(r / p.nst[1]);
  } else {
    int ie = ie_first[blockIdx.x];
    int L = p.elev[ie];
    while (L < 0 || I >= p.ebase[ie] + p.psize[L]) L = p.elev[++ie];
    const int64_t q = I - p.ebase[ie];
    t[0] = p.e_a[ie];
    t[1] = p.e_b[ie];
    t[2] = p.pdet_a[p.pfirst[L] + q];
    t[3] = p.pdet_b[p.pfirst[L] + q];
  }
  uint64_t m[4], mh[4];
  if (WIDE) {
    load_words(p, t, m, mh);
  } else {
#pragma unroll
    for (int s = 0; s < 4; s++) {
      m[s] = p.l[s].str[t[s]];
      mh[s] = 0;
    }
  }
  T acc[NV];
  const T dI = (T)(p.diag[I] - p.shift);
#pragma unroll
  for (int v = 0; v < NV; v++) acc[v] = dI * __ldg(p.X + I * NV + v);
  two_conn_visit<FULL>(p, t, m, mh, [&](int64_t j, T h) { axpy_gather<T, NV>(acc, h, p.X, j); });
#pragma unroll
  for (int v = 0; v < NV; v++) p.Y[I * NV + v] = acc[v];
}

// Rows of the explicit Hamiltonian (two_species_create_ham,
// explicit_ham_mixedparticle.cpp:190-553): the diagonal, then every kept
// off-diagonal element; exact zeros are dropped and |H_IJ| <= thr pruned when
// thr > 0, as ham.prune(thr, 1.0) does (explicit_ham.cpp:79-81).  FILL = false
// counts the kept elements of each row, FILL = true writes them at row_ptr.
template <bool FILL>
__global__ void __launch_bounds__(128) ham_rows_two_kernel(Args2<double> p, double thr, int32_t *cnt,
                                                           const int64_t *row_ptr, int32_t *col, double *val) {
  const int ie = blockIdx.x;
  const int L = p.elev[ie];
  if (L < 0) return;
  const int64_t nq = p.psize[L];
  for (int64_t q = threadIdx.x; q < nq; q += blockDim.x) {
    const int64_t I = p.ebase[ie] + q;
    const int t[4] = {p.e_a[ie], p.e_b[ie], p.pdet_a[p.pfirst[L] + q], p.pdet_b[p.pfirst[L] + q]};
    uint64_t m[4], mh[4];
    load_words(p, t, m, mh);
    int64_t w = FILL ? row_ptr[I] : 0;
    int32_t c = 0;
    auto emit = [&](int64_t j, double h) {
      const bool keep = thr > 0.0 ? fabs(h) > thr : (j == I || h != 0.0);
      if (!keep) return;
      if (FILL) {
        col[w] = (int32_t)j;
        val[w] = h;
        w++;
      } else {
        c++;
      }
    };
    emit(I, p.diag[I]);
    two_conn_visit(p, t, m, mh, emit);
    if (!FILL) cnt[I] = c;
  }
}

// Diagonal: same-species energies of both species plus charge[0]*charge[1]
// times the cross Coulomb sum over every pair of occupied orbitals.
__global__ void __launch_bounds__(128) diag_two_kernel(Args2<double> p, const double *es0, const double *es1,
                                                       const double *es2, const double *es3, double *diag) {
  const int ie = blockIdx.x;
  const int L = p.elev[ie];
  if (L < 0) return;
  const int64_t nq = p.psize[L];
  const double *es[4] = {es0, es1, es2, es3};
  for (int64_t q = threadIdx.x; q < nq; q += blockDim.x) {
    const int t[4] = {p.e_a[ie], p.e_b[ie], p.pdet_a[p.pfirst[L] + q], p.pdet_b[p.pfirst[L] + q]};
    uint64_t m[4], mh[4];
    load_words(p, t, m, mh);
    double e = 0.0;
    for (int s = 0; s < 4; s++) e += es[s][t[s]];
    for (int sp = 0; sp < 2; sp++)
      for_occ(m[2 * sp], mh[2 * sp], [&](int i) {
        e += coul_row(p.eab[sp], p.npair[sp], tri2(i, i), m[2 * sp + 1], mh[2 * sp + 1]);
      });
    double x = 0.0;
    for (int se = 0; se < 2; se++)
      for (int spn = 0; spn < 2; spn++)
        for_occ(m[se], mh[se], [&](int i) {
          x += coul_row(p.ep[p.blk[0][se]][p.blk[1][spn]], p.npair[1], tri2(i, i), m[2 + spn], mh[2 + spn]);
        });
    diag[p.ebase[ie] + q] = e + p.cf * x;
  }
}

// ---------------------------------------------------------------------------
template <typename T> static Args2<T> make_args(pq_ci_handle *h);

static List2<double> view64(const SpinTablesDev &t) {
  return {t.str.as<uint64_t>(), t.str_hi.as<uint64_t>(), t.s1_off.as<int64_t>(), t.s1_J.as<int32_t>(),
          t.s1_info.as<int32_t>(), t.s1_F64.as<double>(), t.s2_off.as<int64_t>(), t.s2_J.as<int32_t>(), t.s2_D64.as<double>()};
}
static List2<float> view32(const SpinTablesDev &t) {
  return {t.str.as<uint64_t>(), t.str_hi.as<uint64_t>(), t.s1_off.as<int64_t>(), t.s1_J.as<int32_t>(),
          t.s1_info.as<int32_t>(), t.s1_F32.as<float>(), t.s2_off.as<int64_t>(), t.s2_J.as<int32_t>(), t.s2_D32.as<float>()};
}

template <typename T> static Args2<T> make_args(pq_ci_handle *h) {
  constexpr bool dbl = std::is_same<T, double>::value;
  Args2<T> a{};
  for (int s = 0; s < 4; s++) {
    const SpinTablesDev &tb = h->tab[s >> 1][s & 1];
    if constexpr (dbl)
      a.l[s] = view64(tb);
    else
      a.l[s] = view32(tb);
  }
  for (int sp = 0; sp < 2; sp++) {
    a.npair[sp] = h->npair[sp];
    a.eab[sp] = (const T *)(dbl ? h->d_eabs64[sp].ptr : h->d_eabs32[sp].ptr);
    for (int spin = 0; spin < 2; spin++) a.blk[sp][spin] = spin % h->n_blocks[sp];
  }
  for (int x = 0; x < 2; x++)
    for (int y = 0; y < 2; y++) {
      a.ep[x][y] = (const T *)(dbl ? h->d_ep64[x][y].ptr : h->d_ep32[x][y].ptr);
      a.epc[x][y] = (const T *)(dbl ? h->d_epc64[x][y].ptr : h->d_epc32[x][y].ptr);
    }
  a.npa1 = (int)h->str[1][0].size();
  a.cf = (T)(h->desc.charge[0] * h->desc.charge[1]);
  a.rowoff0 = h->d_rowoff.as<int32_t>();
  a.rowlen0 = h->d_rowlen.as<int32_t>();
  a.e_a = h->d_e_a.as<int32_t>();
  a.e_b = h->d_e_b.as<int32_t>();
  a.elev = h->d_elev.as<int32_t>();
  a.ebase = h->d_ebase.as<int64_t>();
  a.prowoff = h->d_prowoff.as<int32_t>();
  a.prowlen = h->d_prowlen.as<int32_t>();
  a.pfirst = h->d_pfirst.as<int64_t>();
  a.psize = h->d_psize.as<int64_t>();
  a.pdet_a = h->d_pdet_a.as<int32_t>();
  a.pdet_b = h->d_pdet_b.as<int32_t>();
  a.diag = h->d_diag.as<double>();
  for (int s = 0; s < 4; s++) a.nst[s] = (int)h->str[s >> 1][s & 1].size();
  return a;
}

// row-major FP64 and FP32 copies of a column-major block, times `scale`; the uploads are synchronised here
// because the host vectors are released on return
static pq_status upload_rm(DevBuf &b64, DevBuf &b32, const double *colmajor, int rows, int cols, cudaStream_t st,
                           double scale = 1.0) {
  std::vector<double> rm((size_t)rows * cols);
  for (int r = 0; r < rows; r++)
    for (int c = 0; c < cols; c++) rm[(size_t)r * cols + c] = scale * colmajor[(size_t)r + (size_t)c * rows];
  PQ_TRY(upload(b64, rm, st));
  std::vector<float> f(rm.begin(), rm.end());
  PQ_TRY(upload(b32, f, st));
  PQ_CUDA_TRY(cudaStreamSynchronize(st));
  return PQ_OK;
}

pq_status ci_build2(pq_ci_handle *h) {
  const pq_ci_desc &d = h->desc;
  cudaStream_t st = h->stream;
  int maxorb = 0;
  for (int s = 0; s < 2; s++) {
    if (d.n_orb[s] < 1 || d.n_orb[s] > PQ_MAX_ORB) {
      set_error("n_orb[%d]=%d outside 1..%d", s, d.n_orb[s], PQ_MAX_ORB);
      return PQ_ERR_ARG;
    }
    if (d.n_alpha[s] < 0 || d.n_beta[s] < 0 || d.n_alpha[s] > d.n_orb[s] || d.n_beta[s] > d.n_orb[s]) {
      set_error("particle counts of species %d do not fit %d orbitals", s, d.n_orb[s]);
      return PQ_ERR_ARG;
    }
    h->n_orb[s] = d.n_orb[s];
    h->npair[s] = d.n_orb[s] * (d.n_orb[s] + 1) / 2;
    h->n_blocks[s] = d.restricted[s] ? 1 : 2;
    maxorb = std::max(maxorb, d.n_orb[s]);
  }
  h->n_words = (maxorb >> 6) + 1;
  h->wide = maxorb > 64;
  if (h->selected && h->wide) {
    set_error("selected string lists hold at most 64 orbitals per species");
    return PQ_ERR_ARG;
  }
  for (int s = 0; s < 2 && !h->selected; s++) {
    int ne[2] = {d.n_alpha[s], d.n_beta[s]};
    for (int sp = 0; sp < 2; sp++)
      PQ_TRY(make_strings(d.n_orb[s], ne[sp], d.ex_level[s][sp], h->str[s][sp], h->lvl[s][sp],
                          h->wide ? &h->str_hi[s][sp] : nullptr));
  }
  // integral blocks
  for (int s = 0; s < 2; s++) {
    const int A = 0, B = 1 % h->n_blocks[s];
    const double *h1a = d.h1[s][A], *h1b = d.h1[s][B];
    const double *eaa = d.eri[s][A][s][A], *ebb = d.eri[s][B][s][B], *eab = d.eri[s][A][s][B];
    if (!h1a || !h1b || !eaa || !ebb || !eab) {
      set_error("missing integral block of species %d", s);
      return PQ_ERR_ARG;
    }
    PQ_TRY(build_spin_tables(h, s, 0, h1a, eaa));
    PQ_TRY(build_spin_tables(h, s, 1, h1b, ebb));
    PQ_TRY(upload_rm(h->d_eabs64[s], h->d_eabs32[s], eab, h->npair[s], h->npair[s], st));
  }
  for (int x = 0; x < 2; x++)
    for (int y = 0; y < 2; y++) {
      const int bx = x % h->n_blocks[0], by = y % h->n_blocks[1];
      const double *ep = d.eri[0][bx][1][by];
      if (!ep) {
        set_error("missing cross-species integral block eri[0][%d][1][%d]", bx, by);
        return PQ_ERR_ARG;
      }
      PQ_TRY(upload_rm(h->d_ep64[x][y], h->d_ep32[x][y], ep, h->npair[0], h->npair[1], st));
      PQ_TRY(upload_rm(h->d_epc64[x][y], h->d_epc32[x][y], ep, h->npair[0], h->npair[1], st,
                       d.charge[0] * d.charge[1]));
    }
  // addressing
  const std::vector<int32_t> &l0a = h->lvl[0][0], &l0b = h->lvl[0][1], &l1a = h->lvl[1][0], &l1b = h->lvl[1][1];
  const int64_t n0a = (int64_t)l0a.size(), n0b = (int64_t)l0b.size(), n1a = (int64_t)l1a.size(), n1b = (int64_t)l1b.size();
  const int tot0 = d.ex_level[0][2], tot1 = d.ex_level[1][2], mc = d.max_collective;
  auto prefix = [](const std::vector<int32_t> &lv, int lim) {
    int32_t c = 0;
    while (lim >= 0 && c < (int32_t)lv.size() && lv[c] <= lim) c++;
    return c;
  };
  h->rowoff.assign(n0a, 0);
  h->rowlen.assign(n0a, 0);
  std::vector<int32_t> rowoff32(n0a);
  int64_t ne = 0;
  for (int64_t i = 0; i < n0a; i++) {
    rowoff32[i] = (int32_t)ne;
    h->rowoff[i] = ne;
    h->rowlen[i] = prefix(l0b, tot0 - l0a[i]);
    ne += h->rowlen[i];
  }
  h->lcap = std::min(l1a.back() + l1b.back(), 63);
  const int lcap = h->lcap;
  h->psize.assign(lcap + 1, 0);
  h->prowoff.assign((size_t)(lcap + 1) * n1a, 0);
  h->prowlen.assign((size_t)(lcap + 1) * n1a, 0);
  h->pfirst.assign(lcap + 2, 0);
  h->pdet_a.clear();
  h->pdet_b.clear();
  for (int L = 0; L <= lcap; L++) {
    int64_t acc = 0;
    h->pfirst[L] = (int64_t)h->pdet_a.size();
    for (int64_t k = 0; k < n1a; k++) {
      int32_t len = prefix(l1b, L - l1a[k]);
      h->prowoff[(size_t)L * n1a + k] = (int32_t)acc;
      h->prowlen[(size_t)L * n1a + k] = len;
      for (int32_t l = 0; l < len; l++) {
        h->pdet_a.push_back((int32_t)k);
        h->pdet_b.push_back(l);
      }
      acc += len;
    }
    h->psize[L] = acc;
  }
  h->e_a.assign(ne, 0);
  h->e_b.assign(ne, 0);
  h->ebase.assign(ne, 0);
  h->elev.assign(ne, -1);
  int64_t nd = 0;
  for (int64_t i = 0; i < n0a; i++)
    for (int32_t j = 0; j < h->rowlen[i]; j++) {
      int64_t ie = h->rowoff[i] + j;
      h->e_a[ie] = (int32_t)i;
      h->e_b[ie] = j;
      h->ebase[ie] = nd;
      int e0 = l0a[i] + l0b[j];
      int L = std::min(tot1, mc - e0);
      L = std::min(L, lcap);
      h->elev[ie] = L;
      if (L >= 0) nd += h->psize[L];
    }

  if (ne > INT32_MAX || nd <= 0) {
    set_error("two-species space: %lld species-0 pairs, %lld determinants", (long long)ne, (long long)nd);
    return PQ_ERR_ARG;
  }
  h->n_dets = nd;
  h->full = false;
  // the pair holding the first determinant of every 128-determinant block of the flat list
  {
    std::vector<int32_t> first((size_t)((nd + 127) / 128));
    int64_t ie = 0;
    for (size_t b = 0; b < first.size(); b++) {
      const int64_t I = (int64_t)b * 128;
      while (h->elev[ie] < 0 || I >= h->ebase[ie] + h->psize[h->elev[ie]]) ie++;
      first[b] = (int32_t)ie;
    }
    PQ_TRY(upload(h->d_ie_first, first, st));
  }
  // a full product of complete string spaces: every species-0 pair kept with the whole species-1 space
  {
    bool full = ne == n0a * n0b;
    const int64_t n1 = n1a * n1b;
    for (int64_t ie = 0; full && ie < ne; ie++) full = h->elev[ie] >= 0 && h->psize[h->elev[ie]] == n1;
    h->full2 = full && nd == ne * n1;
  }
  PQ_TRY(upload(h->d_rowoff, rowoff32, st));
  PQ_TRY(upload(h->d_rowlen, h->rowlen, st));
  PQ_TRY(upload(h->d_e_a, h->e_a, st));
  PQ_TRY(upload(h->d_e_b, h->e_b, st));
  PQ_TRY(upload(h->d_ebase, h->ebase, st));
  PQ_TRY(upload(h->d_elev, h->elev, st));
  PQ_TRY(upload(h->d_prowoff, h->prowoff, st));
  PQ_TRY(upload(h->d_prowlen, h->prowlen, st));
  PQ_TRY(upload(h->d_pfirst, h->pfirst, st));
  PQ_TRY(upload(h->d_psize, h->psize, st));
  PQ_TRY(upload(h->d_pdet_a, h->pdet_a, st));
  PQ_TRY(upload(h->d_pdet_b, h->pdet_b, st));
  PQ_TRY(h->d_diag.alloc(sizeof(double) * (nd + 1)));
  Args2<double> a = make_args<double>(h);
  a.cf = h->desc.charge[0] * h->desc.charge[1];
  diag_two_kernel<<<(unsigned)ne, 128, 0, st>>>(a, h->tab[0][0].e_same64.as<double>(), h->tab[0][1].e_same64.as<double>(),
                                               h->tab[1][0].e_same64.as<double>(), h->tab[1][1].e_same64.as<double>(),
                                               h->d_diag.as<double>());
  PQ_CUDA_TRY(cudaGetLastError());
  PQ_CUDA_TRY(cudaStreamSynchronize(st));
  return PQ_OK;
}

template <typename T, int NV>
static pq_status launch2(pq_ci_handle *h, const void *X, void *Y, double shift) {
  Args2<T> a = make_args<T>(h);
  a.shift = shift;
  a.X = (const T *)X;
  a.Y = (T *)Y;
  const unsigned grid = (unsigned)((h->n_dets + 127) / 128);
  // wide strings take the searched addressing, which holds for full products too
  if (h->wide)
    sigma_two_species_kernel<T, NV, false, true><<<grid, 128, 0, h->stream>>>(a, h->n_dets, h->d_ie_first.as<int32_t>());
  else if (h->full2)
    sigma_two_species_kernel<T, NV, true, false><<<grid, 128, 0, h->stream>>>(a, h->n_dets, nullptr);
  else
    sigma_two_species_kernel<T, NV, false, false><<<grid, 128, 0, h->stream>>>(a, h->n_dets, h->d_ie_first.as<int32_t>());
  PQ_CUDA_TRY(cudaGetLastError());
  return PQ_OK;
}

pq_status ci_sigma2_il(pq_ci_handle *h, const void *X, void *Y, int nvp, int precision, double shift) {
  if (precision == PQ_FP64) {
    if (nvp == 1) return launch2<double, 1>(h, X, Y, shift);
    if (nvp == 2) return launch2<double, 2>(h, X, Y, shift);
    if (nvp == 3) return launch2<double, 3>(h, X, Y, shift);
    if (nvp == 4) return launch2<double, 4>(h, X, Y, shift);
  } else if (precision == PQ_FP32) {
    if (nvp == 1) return launch2<float, 1>(h, X, Y, shift);
    if (nvp == 2) return launch2<float, 2>(h, X, Y, shift);
    if (nvp == 3) return launch2<float, 3>(h, X, Y, shift);
    if (nvp == 4) return launch2<float, 4>(h, X, Y, shift);
  }
  set_error("unsupported interleave width %d / precision %d", nvp, precision);
  return PQ_ERR_ARG;
}

pq_status ci_ham_rows2(pq_ci_handle *h, double thr, int32_t *cnt, const int64_t *row_ptr, int32_t *col, double *val) {
  const Args2<double> a = make_args<double>(h);
  const unsigned ne = (unsigned)h->e_a.size();
  if (cnt)
    ham_rows_two_kernel<false><<<ne, 128, 0, h->stream>>>(a, thr, cnt, nullptr, nullptr, nullptr);
  else
    ham_rows_two_kernel<true><<<ne, 128, 0, h->stream>>>(a, thr, nullptr, row_ptr, col, val);
  PQ_CUDA_TRY(cudaGetLastError());
  return PQ_OK;
}

// H_IJ for a list of pairs, thread per pair: the diagonal element, or the
// partner J among the connections of I (the same elements as sigma and the
// explicit matrix); pairs that are not connected give 0.
__global__ void elements_two_kernel(Args2<double> p, int64_t n, const int32_t *t4, const int64_t *I, const int64_t *J,
                                    double *out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t target = J[i];
  double v = 0.0;
  if (I[i] == target) {
    v = p.diag[target];
  } else {
    const int t[4] = {t4[4 * i], t4[4 * i + 1], t4[4 * i + 2], t4[4 * i + 3]};
    uint64_t m[4], mh[4];
    load_words(p, t, m, mh);
    two_conn_visit(p, t, m, mh, [&](int64_t j, double h) {
      if (j == target) v = h;
    });
  }
  out[i] = v;
}

pq_status ci_elements2(pq_ci_handle *h, int64_t n, const int32_t *t4, const int64_t *I, const int64_t *J, double *out) {
  const Args2<double> a = make_args<double>(h);
  const unsigned grid = (unsigned)((n + 127) / 128);
  if (grid) elements_two_kernel<<<grid, 128, 0, h->stream>>>(a, n, t4, I, J, out);
  PQ_CUDA_TRY(cudaGetLastError());
  return PQ_OK;
}

// String indices (species-0 alpha, beta, species-1 alpha, beta) of one
// determinant: the species-0 pair whose block holds I, then its block entry.
void ci_unfold2_one(const pq_ci_handle *h, int64_t I, int32_t *t) {
  const int64_t ie = (int64_t)(std::upper_bound(h->ebase.begin(), h->ebase.end(), I) - h->ebase.begin()) - 1;
  // empty blocks share their successor's base: step back to the block that holds I
  int64_t k = ie;
  while (k > 0 && (h->elev[k] < 0 || h->ebase[k] + h->psize[h->elev[k]] <= I)) k--;
  const int L = h->elev[k];
  const int64_t q = I - h->ebase[k];
  t[0] = h->e_a[k];
  t[1] = h->e_b[k];
  t[2] = h->pdet_a[h->pfirst[L] + q];
  t[3] = h->pdet_b[h->pfirst[L] + q];
}

pq_status ci_unfold2(const pq_ci_handle *h, int32_t *out) {
  int64_t k = 0;
  for (size_t ie = 0; ie < h->e_a.size(); ie++) {
    int L = h->elev[ie];
    if (L < 0) continue;
    for (int64_t q = 0; q < h->psize[L]; q++) {
      out[4 * k + 0] = h->e_a[ie];
      out[4 * k + 1] = h->e_b[ie];
      out[4 * k + 2] = h->pdet_a[h->pfirst[L] + q];
      out[4 * k + 3] = h->pdet_b[h->pfirst[L] + q];
      k++;
    }
  }
  return PQ_OK;
}

}  // namespace pq
