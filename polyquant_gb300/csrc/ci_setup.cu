// Determinant-space setup on the GPU: string enumeration (host, reference
// order), prefix-row determinant addressing, single/double replacement tables
// with phases (device, popcount bit arithmetic) and the diagonal H_II.
//
// Reference behaviour restated (paths inside the polyquant project):
//   strings      src/ci/detset/determinant_creation.cpp:6-72,139-146; src/ci/epci.cpp:341-380
//   det list     src/ci/detset/determinant_creation.cpp:148-206
//   replacement  src/ci/detset/determinant_creation.cpp:209-351 (maps),
//                src/ci/detset/determinant_operations.cpp:17-116 (holes, particles, phase)
//   elements     src/ci/detset/slater_condon_singleparticle.cpp:4-175
//   diagonal     src/ci/detset/slater_condon.cpp:102-153
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>

#include "pq_bits.cuh"
#include "pq_internal.h"

namespace pq {

pq_status DevBuf::alloc(size_t n) {
  release();
  if (n == 0) n = 16;
  cudaError_t e = cudaMalloc(&ptr, n);
  if (e != cudaSuccess) {
    ptr = nullptr;
    set_error("cudaMalloc(%zu) failed: %s", n, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? PQ_ERR_OOM : PQ_ERR_CUDA;
  }
  bytes = n;
  return PQ_OK;
}

__host__ __device__ inline int idx2(int i, int j) { return i > j ? i * (i + 1) / 2 + j : j * (j + 1) / 2 + i; }

// bits 0 .. k-1 of a 64-bit word (k in 0..64)
__host__ __device__ inline uint64_t low_bits(int k) { return k <= 0 ? 0ULL : (k >= 64 ? ~0ULL : ((1ULL << k) - 1ULL)); }

// Occupied orbitals of the string (dl: orbitals 0..63, dh: 64..127) strictly between lo and hi (lo < hi).
__host__ __device__ inline int between_count(uint64_t dl, uint64_t dh, int lo, int hi) {
  if (hi - lo <= 1) return 0;
  const uint64_t ml = low_bits(hi) & ~low_bits(lo + 1);
  const uint64_t mh = low_bits(hi - 64) & ~low_bits(lo + 1 - 64);
#ifdef __CUDA_ARCH__
  return __popcll(dl & ml) + __popcll(dh & mh);
#else
  return __builtin_popcountll(dl & ml) + __builtin_popcountll(dh & mh);
#endif
}

// ---------------------------------------------------------------------------
// host: strings in the reference's order.  HF string first, then for each
// level k: k-subsets of the occupied HF orbitals (lexicographic, outer) x
// k-subsets of the virtual orbitals (lexicographic, inner).
static bool next_comb(std::vector<int> &c, int n) {
  int k = (int)c.size();
  int i = k - 1;
  while (i >= 0 && c[i] == n - k + i) i--;
  if (i < 0) return false;
  c[i]++;
  for (int j = i + 1; j < k; j++) c[j] = c[j - 1] + 1;
  return true;
}

pq_status make_strings(int n_orb, int n_e, int ex_max, std::vector<uint64_t> &out, std::vector<int32_t> &lvl,
                       std::vector<uint64_t> *out_hi) {
  out.clear();
  lvl.clear();
  if (out_hi) out_hi->clear();
  if (n_orb > 64 && !out_hi) {
    set_error("make_strings: %d orbitals need two words", n_orb);
    return PQ_ERR_ARG;
  }
  typedef unsigned __int128 u128;
  auto push = [&](u128 t, int k) {
    out.push_back((uint64_t)t);
    if (out_hi) out_hi->push_back((uint64_t)(t >> 64));
    lvl.push_back(k);
  };
  u128 hf = 0;
  for (int i = 0; i < n_e; i++) hf |= (u128)1 << i;
  push(hf, 0);
  int n_virt = n_orb - n_e;
  for (int k = 1; k <= ex_max; k++) {
    if (k > n_virt) {
      set_error("excitation level %d exceeds the %d virtual orbitals", k, n_virt);
      return PQ_ERR_ARG;
    }
    if (k > n_e) continue;
    std::vector<int> co(k), cv(k);
    std::iota(co.begin(), co.end(), 0);
    do {
      std::iota(cv.begin(), cv.end(), 0);
      do {
        u128 t = hf;
        for (int i = 0; i < k; i++) t &= ~((u128)1 << co[i]);
        for (int i = 0; i < k; i++) t |= (u128)1 << (n_e + cv[i]);
        push(t, k);
      } while (next_comb(cv, n_virt));
    } while (next_comb(co, n_e));
    if (out.size() > (size_t)INT32_MAX) {
      set_error("string list too long");
      return PQ_ERR_ARG;
    }
  }
  return PQ_OK;
}

// ---------------------------------------------------------------------------
// device: replacement tables.  One thread per string.
// index of the string (kl, kh) among strings sorted by (hi word, lo word); -1 when absent
__device__ inline int64_t find_string(const uint64_t *sorted, const uint64_t *sorted_hi, const int32_t *perm, int64_t n,
                                      uint64_t kl, uint64_t kh) {
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    int64_t mid = (lo + hi) >> 1;
    const uint64_t mh = hiword(sorted_hi, mid);
    if (mh < kh || (mh == kh && sorted[mid] < kl))
      lo = mid + 1;
    else
      hi = mid;
  }
  return (lo < n && sorted[lo] == kl && hiword(sorted_hi, lo) == kh) ? perm[lo] : -1;
}

struct TableArgs {
  int64_t n_str;
  const uint64_t *masks, *masks_hi;
  const uint64_t *sorted, *sorted_hi;
  const int32_t *perm;
  int n_orb, npair;
  const double *h1;   // n x n column-major
  const double *eri;  // npair x npair column-major, same-spin block
  int32_t *cnt1, *cnt2;
  const int64_t *off1, *off2;
  int32_t *J1, *info1;
  double *F1;
  int32_t *J2;
  double *D2;
  double *esame;
};

template <bool COUNT>
__global__ void __launch_bounds__(128) spin_tables_kernel(TableArgs a) {
  int64_t I = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= a.n_str) return;
  const uint64_t m = a.masks[I], mh = hiword(a.masks_hi, I);
  const int n = a.n_orb;
  int occ[128], vir[128];
  int no = 0, nv = 0;
  for (int o = 0; o < n; o++) {
    if (occupied(m, mh, o))
      occ[no++] = o;
    else
      vir[nv++] = o;
  }
  // flip orbital o of the string (jl, jh)
  auto flip = [](uint64_t &jl, uint64_t &jh, int o) {
    if (o < 64)
      jl ^= 1ULL << o;
    else
      jh ^= 1ULL << (o - 64);
  };
  auto E = [&](int r, int c) { return a.eri[(int64_t)r + (int64_t)c * a.npair]; };
  int32_t c1 = 0, c2 = 0;
  int64_t w1 = COUNT ? 0 : a.off1[I], w2 = COUNT ? 0 : a.off2[I];
  // singles: hole h (occupied in I), particle p (empty in I)
  for (int x = 0; x < no; x++) {
    int hh = occ[x];
    for (int y = 0; y < nv; y++) {
      int pp = vir[y];
      uint64_t jm = m, jh = mh;
      flip(jm, jh, hh);
      flip(jm, jh, pp);
      int64_t J = find_string(a.sorted, a.sorted_hi, a.perm, a.n_str, jm, jh);
      if (J < 0) continue;
      if (COUNT) {
        c1++;
        continue;
      }
      int lo = hh < pp ? hh : pp, hi = hh < pp ? pp : hh;
      int neg = between_count(m, mh, lo, hi) & 1;
      int php = idx2(hh, pp);
      double f = a.h1[hh + (int64_t)pp * n];
      for (int z = 0; z < no; z++) {
        int k = occ[z];
        f += E(php, idx2(k, k)) - E(idx2(hh, k), idx2(k, pp));
      }
      a.J1[w1] = (int32_t)J;
      a.info1[w1] = (php << 1) | neg;
      a.F1[w1] = f;
      w1++;
    }
  }
  // same-spin doubles: holes h0 < h1, particles p0 < p1
  for (int x0 = 0; x0 < no; x0++)
    for (int x1 = x0 + 1; x1 < no; x1++) {
      int h0 = occ[x0], h1 = occ[x1];
      for (int y0 = 0; y0 < nv; y0++)
        for (int y1 = y0 + 1; y1 < nv; y1++) {
          int p0 = vir[y0], p1 = vir[y1];
          uint64_t jm = m, jh = mh;
          flip(jm, jh, h0);
          flip(jm, jh, h1);
          flip(jm, jh, p0);
          flip(jm, jh, p1);
          int64_t J = find_string(a.sorted, a.sorted_hi, a.perm, a.n_str, jm, jh);
          if (J < 0) continue;
          if (COUNT) {
            c2++;
            continue;
          }
          // phase: pairs (h0,p0), (h1,p1) after sorting holes and particles
          int a0 = h0 < p0 ? h0 : p0, b0 = h0 < p0 ? p0 : h0;
          int a1 = h1 < p1 ? h1 : p1, b1 = h1 < p1 ? p1 : h1;
          int nperm = between_count(m, mh, a0, b0) + between_count(m, mh, a1, b1);
          if (a0 < a1 && a1 < b0 && b0 < b1) nperm++;
          double v = E(idx2(h0, p0), idx2(h1, p1)) - E(idx2(h0, p1), idx2(h1, p0));
          a.J2[w2] = (int32_t)J;
          a.D2[w2] = (nperm & 1) ? -v : v;
          w2++;
        }
    }
  if (COUNT) {
    a.cnt1[I] = c1;
    a.cnt2[I] = c2;
    // same-spin diagonal energy of the string
    double e = 0.0;
    for (int x = 0; x < no; x++) e += a.h1[occ[x] + (int64_t)occ[x] * n];
    for (int x = 0; x < no; x++)
      for (int y = 0; y < no; y++) {
        int i = occ[x], j = occ[y];
        e += 0.5 * E(idx2(i, i), idx2(j, j));
        e -= 0.5 * E(idx2(i, j), idx2(j, i));
      }
    a.esame[I] = e;
  }
}

__global__ void to_float_kernel(const double *src, float *dst, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (; i < n; i += stride) dst[i] = (float)src[i];
}

// Diagonal: same-spin string energies plus the opposite-spin Coulomb sum
// sum_{i in occ(alpha), j in occ(beta)} (ii|jj)_ab.  One block per (alpha
// string, chunk of beta strings); the alpha row of the Coulomb sum is staged in
// shared memory.
__global__ void __launch_bounds__(256) diag_kernel(int64_t nblk_b, const int64_t *rowoff, const int32_t *rowlen,
                                                   const uint64_t *ma, const uint64_t *ma_hi, const uint64_t *mb,
                                                   const uint64_t *mb_hi, const double *ea, const double *eb,
                                                   const double *eab, int npair, int n_orb, double *diag) {
  __shared__ double u[128];
  int64_t Ia = blockIdx.x / nblk_b;
  int64_t Ib = (blockIdx.x % nblk_b) * blockDim.x + threadIdx.x;
  const uint64_t al = ma[Ia], ah = hiword(ma_hi, Ia);
  for (int j = threadIdx.x; j < n_orb; j += blockDim.x) {
    double s = 0.0;
    for_occ(al, ah, [&](int i) { s += eab[(int64_t)idx2(i, i) * npair + idx2(j, j)]; });
    u[j] = s;
  }
  __syncthreads();
  if (Ib >= rowlen[Ia]) return;
  double e = ea[Ia] + eb[Ib];
  for_occ(mb[Ib], hiword(mb_hi, Ib), [&](int j) { e += u[j]; });
  diag[rowoff[Ia] + Ib] = e;
}

// ---------------------------------------------------------------------------
pq_status build_spin_tables(pq_ci_handle *h, int s, int sp, const double *h1_host, const double *eri_host) {
  cudaStream_t st = h->stream;
  SpinTablesDev &T = h->tab[s][sp];
  const std::vector<uint64_t> &masks = h->str[s][sp];
  const std::vector<uint64_t> &mhi = h->str_hi[s][sp];
  const bool two = h->wide;
  int64_t n = (int64_t)masks.size();
  T.n_str = n;
  int no = h->n_orb[s], npair = h->npair[s];
  std::vector<int32_t> perm(n);
  std::iota(perm.begin(), perm.end(), 0);
  auto hw = [&](int64_t i) { return two ? mhi[i] : 0ULL; };
  std::sort(perm.begin(), perm.end(), [&](int32_t x, int32_t y) {
    return hw(x) < hw(y) || (hw(x) == hw(y) && masks[x] < masks[y]);
  });
  std::vector<uint64_t> sorted(n), sorted_hi(two ? n : 0);
  for (int64_t i = 0; i < n; i++) {
    sorted[i] = masks[perm[i]];
    if (two) sorted_hi[i] = mhi[perm[i]];
  }
  DevBuf d_sorted, d_sorted_hi, d_perm, d_h1, d_eri, d_cnt1, d_cnt2;
  PQ_TRY(upload(T.str, masks, st));
  if (two) {
    PQ_TRY(upload(T.str_hi, mhi, st));
    PQ_TRY(upload(d_sorted_hi, sorted_hi, st));
  }
  PQ_TRY(upload(d_sorted, sorted, st));
  PQ_TRY(upload(d_perm, perm, st));
  PQ_TRY(d_h1.alloc(sizeof(double) * no * no));
  PQ_CUDA_TRY(cudaMemcpyAsync(d_h1.ptr, h1_host, sizeof(double) * no * no, cudaMemcpyHostToDevice, st));
  PQ_TRY(d_eri.alloc(sizeof(double) * npair * npair));
  PQ_CUDA_TRY(cudaMemcpyAsync(d_eri.ptr, eri_host, sizeof(double) * npair * npair, cudaMemcpyHostToDevice, st));
  PQ_TRY(d_cnt1.alloc(sizeof(int32_t) * n));
  PQ_TRY(d_cnt2.alloc(sizeof(int32_t) * n));
  PQ_TRY(T.e_same64.alloc(sizeof(double) * n));
  TableArgs a{};
  a.n_str = n;
  a.masks = T.str.as<uint64_t>();
  a.masks_hi = two ? T.str_hi.as<uint64_t>() : nullptr;
  a.sorted = d_sorted.as<uint64_t>();
  a.sorted_hi = two ? d_sorted_hi.as<uint64_t>() : nullptr;
  a.perm = d_perm.as<int32_t>();
  a.n_orb = no;
  a.npair = npair;
  a.h1 = d_h1.as<double>();
  a.eri = d_eri.as<double>();
  a.cnt1 = d_cnt1.as<int32_t>();
  a.cnt2 = d_cnt2.as<int32_t>();
  a.esame = T.e_same64.as<double>();
  int grid = (int)((n + 127) / 128);
  spin_tables_kernel<true><<<grid, 128, 0, st>>>(a);
  PQ_CUDA_TRY(cudaGetLastError());
  std::vector<int32_t> c1(n), c2(n);
  PQ_CUDA_TRY(cudaMemcpyAsync(c1.data(), a.cnt1, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st));
  PQ_CUDA_TRY(cudaMemcpyAsync(c2.data(), a.cnt2, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st));
  PQ_CUDA_TRY(cudaStreamSynchronize(st));
  std::vector<int64_t> o1(n + 1, 0), o2(n + 1, 0);
  T.max1 = T.max2 = 0;
  for (int64_t i = 0; i < n; i++) {
    o1[i + 1] = o1[i] + c1[i];
    o2[i + 1] = o2[i] + c2[i];
    T.max1 = std::max(T.max1, c1[i]);
    T.max2 = std::max(T.max2, c2[i]);
  }
  T.n1 = o1[n];
  T.n2 = o2[n];
  PQ_TRY(upload(T.s1_off, o1, st));
  PQ_TRY(upload(T.s2_off, o2, st));
  PQ_TRY(T.s1_J.alloc(sizeof(int32_t) * (T.n1 + 1)));
  PQ_TRY(T.s1_info.alloc(sizeof(int32_t) * (T.n1 + 1)));
  PQ_TRY(T.s1_F64.alloc(sizeof(double) * (T.n1 + 1)));
  PQ_TRY(T.s1_F32.alloc(sizeof(float) * (T.n1 + 1)));
  PQ_TRY(T.s2_J.alloc(sizeof(int32_t) * (T.n2 + 1)));
  PQ_TRY(T.s2_D64.alloc(sizeof(double) * (T.n2 + 1)));
  PQ_TRY(T.s2_D32.alloc(sizeof(float) * (T.n2 + 1)));
  a.off1 = T.s1_off.as<int64_t>();
  a.off2 = T.s2_off.as<int64_t>();
  a.J1 = T.s1_J.as<int32_t>();
  a.info1 = T.s1_info.as<int32_t>();
  a.F1 = T.s1_F64.as<double>();
  a.J2 = T.s2_J.as<int32_t>();
  a.D2 = T.s2_D64.as<double>();
  spin_tables_kernel<false><<<grid, 128, 0, st>>>(a);
  PQ_CUDA_TRY(cudaGetLastError());
  if (T.n1) to_float_kernel<<<1024, 256, 0, st>>>(a.F1, T.s1_F32.as<float>(), T.n1);
  if (T.n2) to_float_kernel<<<1024, 256, 0, st>>>(a.D2, T.s2_D32.as<float>(), T.n2);
  PQ_CUDA_TRY(cudaGetLastError());
  PQ_CUDA_TRY(cudaStreamSynchronize(st));
  return PQ_OK;
}

pq_status ci_build(pq_ci_handle *h) {
  const pq_ci_desc &d = h->desc;
  cudaStream_t st = h->stream;
  h->n_species = d.n_species;
  if (d.n_species == 2) return ci_build2(h);
  if (d.n_species != 1) {
    set_error("n_species=%d: one or two species are supported", d.n_species);
    return PQ_ERR_ARG;
  }
  int maxorb = 0;
  for (int s = 0; s < d.n_species; s++) {
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
  // the reference's word count: n_words = (max_orb >> 6) + 1 (determinant_creation.cpp:13); internally a
  // second word is kept only when some species has more than 64 orbitals
  h->n_words = (maxorb >> 6) + 1;
  h->wide = maxorb > 64;
  if (h->selected && h->wide) {
    set_error("selected string lists hold at most 64 orbitals per species");
    return PQ_ERR_ARG;
  }
  for (int s = 0; s < d.n_species && !h->selected; s++) {
    int ne[2] = {d.n_alpha[s], d.n_beta[s]};
    for (int sp = 0; sp < 2; sp++)
      PQ_TRY(make_strings(d.n_orb[s], ne[sp], d.ex_level[s][sp], h->str[s][sp], h->lvl[s][sp],
                          h->wide ? &h->str_hi[s][sp] : nullptr));
  }
  // integral blocks: alpha index 0, beta index 1 % n_blocks (slater_condon_singleparticle.cpp:11)
  const int A = 0, B = 1 % h->n_blocks[0];
  const double *h1a = d.h1[0][A], *h1b = d.h1[0][B];
  const double *eaa = d.eri[0][A][0][A], *ebb = d.eri[0][B][0][B], *eab = d.eri[0][A][0][B];
  if (!h1a || !h1b || !eaa || !ebb || !eab) {
    set_error("missing integral block (h1 or eri pointer is NULL)");
    return PQ_ERR_ARG;
  }
  // addressing: row Ia keeps the prefix of beta strings with level <= limit
  const std::vector<int32_t> &la = h->lvl[0][0], &lb = h->lvl[0][1];
  int64_t na = (int64_t)la.size(), nb = (int64_t)lb.size();
  int tot = d.ex_level[0][2], mc = d.max_collective;
  h->rowoff.assign(na, 0);
  h->rowlen.assign(na, 0);
  int64_t acc = 0;
  bool full = true;
  for (int64_t i = 0; i < na; i++) {
    int lim = std::min(tot, mc) - la[i];
    int32_t c = 0;
    while (lim >= 0 && c < nb && lb[c] <= lim) c++;
    h->rowoff[i] = acc;
    h->rowlen[i] = c;
    acc += c;
    if (c != nb) full = false;
  }
  h->n_dets = acc;
  h->full = full;
  PQ_TRY(upload(h->d_rowoff, h->rowoff, st));
  PQ_TRY(upload(h->d_rowlen, h->rowlen, st));
  PQ_TRY(build_spin_tables(h, 0, 0, h1a, eaa));
  PQ_TRY(build_spin_tables(h, 0, 1, h1b, ebb));
  // cross block, row-major [pair_alpha][pair_beta]
  int npair = h->npair[0];
  std::vector<double> eab_rm((size_t)npair * npair);
  for (int r = 0; r < npair; r++)
    for (int c = 0; c < npair; c++) eab_rm[(size_t)r * npair + c] = eab[(size_t)r + (size_t)c * npair];
  PQ_TRY(upload(h->d_eab64, eab_rm, st));
  std::vector<float> eab32(eab_rm.begin(), eab_rm.end());
  PQ_TRY(upload(h->d_eab32, eab32, st));
  std::vector<float> eba32((size_t)npair * npair);
  for (int r = 0; r < npair; r++)
    for (int c = 0; c < npair; c++) eba32[(size_t)c * npair + r] = eab32[(size_t)r * npair + c];
  PQ_TRY(upload(h->d_eba32, eba32, st));
  // diagonal
  PQ_TRY(h->d_diag.alloc(sizeof(double) * (h->n_dets + 1)));
  int64_t nblk_b = (nb + 255) / 256;
  if (h->n_dets > 0) {
    diag_kernel<<<(unsigned)(na * nblk_b), 256, 0, st>>>(nblk_b, h->d_rowoff.as<int64_t>(), h->d_rowlen.as<int32_t>(),
                                                         h->tab[0][0].str.as<uint64_t>(), h->tab[0][0].str_hi.as<uint64_t>(),
                                                         h->tab[0][1].str.as<uint64_t>(), h->tab[0][1].str_hi.as<uint64_t>(),
                                                         h->tab[0][0].e_same64.as<double>(),
                                                         h->tab[0][1].e_same64.as<double>(), h->d_eab64.as<double>(),
                                                         npair, h->n_orb[0], h->d_diag.as<double>());
    PQ_CUDA_TRY(cudaGetLastError());
  }
  PQ_CUDA_TRY(cudaStreamSynchronize(st));
  h->fp32_v2 = sigma32_v2_applicable(h) && getenv("PQ_SIGMA32_GATHER") == nullptr;
  h->fp32_tc = h->fp32_v2 && sigma32_tc_applicable(h) && getenv("PQ_SIGMA32_NO_TC") == nullptr;
  h->fp32_ss = h->fp32_tc && sigma32_ss_applicable(h) && getenv("PQ_SIGMA32_NO_SS") == nullptr;
  return PQ_OK;
}

}  // namespace pq
