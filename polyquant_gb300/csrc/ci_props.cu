// Properties of CI vectors on the device: <S^2> of each state and species and
// the one-particle reduced density matrix of one state, species and spin.
//
// <S^2> follows POLYQUANT_DETSET::evaluate_s2 (src/ci/detset/s2.cpp:4-123):
// diagonal n_a + s_z (s_z - 1) from the open shells of each determinant
// (n_a open-shell alpha electrons, s_z = n_a - n_open / 2), and for every
// alpha single h_a -> p_a paired with the beta single p_a -> h_a (a spin
// flip) the term -phase_a phase_b C_I C_J.
// The 1-RDM follows create_1rdm (src/ci/detset/rdm1.cpp:4-72): C_I^2 on the
// occupied orbitals of the chosen spin, and phase C_I C_J on (k, l) and
// (l, k) for each single of that spin between I and an earlier J (hole k in
// I, particle l).
// Thread <-> determinant (one species: grid of alpha strings x beta blocks;
// two species: CTA per species-0 pair, threads over its species-1 block),
// per-block reduction in shared memory, then one atomic per block and entry.
// With two species each property is evaluated for the chosen species with
// the other species' strings held fixed, as in the reference's per-species
// loops.
#include <algorithm>

#include "ci_conn.cuh"
#include "pq_bits.cuh"
#include "pq_internal.h"

namespace pq {

constexpr int PROP_THREADS = 128;
constexpr int S2_MAXV = 8;

__global__ void __launch_bounds__(PROP_THREADS) s2_kernel(ConnArgs a, int na, const double *C, int64_t ldc, int nvec,
                                                          double *out) {
  __shared__ double red[S2_MAXV][PROP_THREADS / 32];
  const int ia = blockIdx.x;
  double acc[S2_MAXV];
#pragma unroll
  for (int v = 0; v < S2_MAXV; v++) acc[v] = 0.0;
  for (int ib = blockIdx.y * blockDim.x + threadIdx.x; ia < na && ib < a.rowlen[ia]; ib += gridDim.y * blockDim.x) {
    const ConnRow r = conn_row(a, ia, ib);
    double cI[S2_MAXV];
#pragma unroll
    for (int v = 0; v < S2_MAXV; v++) cI[v] = v < nvec ? C[r.I + v * ldc] : 0.0;
    const uint64_t open = r.am ^ r.bm, openh = r.amh ^ r.bmh;
    const int n_open = popc2(open, openh), n_a = popc2(open & r.am, openh & r.amh);
    const double sz = n_a - 0.5 * n_open;
    const double d = n_a + sz * (sz - 1.0);
#pragma unroll
    for (int v = 0; v < S2_MAXV; v++) acc[v] += cI[v] * cI[v] * d;
    for (int s = 0; s < r.n1a; s++) {
      const int Ja = a.a1_J[r.a1b + s], infa = a.a1_info[r.a1b + s];
      const uint64_t jam = a.astr[Ja], jamh = hiword(a.astr_hi, Ja);
      const int ha = first_set(r.am & ~jam, r.amh & ~jamh), pa = first_set(jam & ~r.am, jamh & ~r.amh);
      if (!occupied(r.bm, r.bmh, pa) || occupied(r.bm, r.bmh, ha)) continue;
      uint64_t jbm = r.bm, jbmh = r.bmh;
      flip_orb(jbm, jbmh, pa);
      flip_orb(jbm, jbmh, ha);
      for (int q = 0; q < r.n1b; q++) {
        const int Jb = a.b1_J[r.b1b + q];
        if (a.bstr[Jb] != jbm || hiword(a.bstr_hi, Jb) != jbmh) continue;
        if (Jb < a.rowlen[Ja]) {
          const int64_t J = a.rowoff[Ja] + Jb;
          const double ph = ((infa ^ a.b1_info[r.b1b + q]) & 1) ? -1.0 : 1.0;
#pragma unroll
          for (int v = 0; v < S2_MAXV; v++)
            if (v < nvec) acc[v] -= ph * cI[v] * C[J + v * ldc];
        }
        break;
      }
    }
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int v = 0; v < S2_MAXV; v++) {
    double x = acc[v];
    for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) red[v][w] = x;
  }
  __syncthreads();
  if (threadIdx.x < nvec) {
    double x = 0.0;
    for (int i = 0; i < PROP_THREADS / 32; i++) x += red[threadIdx.x][i];
    atomicAdd(out + threadIdx.x, x);
  }
}

// rdm[k + l * n] (column-major n x n), spin 0 = alpha, 1 = beta
__global__ void __launch_bounds__(PROP_THREADS) rdm1_kernel(ConnArgs a, int na, int n, int spin, const double *C,
                                                            double *rdm) {
  extern __shared__ double acc[];  // n x n
  for (int i = threadIdx.x; i < n * n; i += blockDim.x) acc[i] = 0.0;
  __syncthreads();
  const int ia = blockIdx.x;
  for (int ib = blockIdx.y * blockDim.x + threadIdx.x; ia < na && ib < a.rowlen[ia]; ib += gridDim.y * blockDim.x) {
    const ConnRow r = conn_row(a, ia, ib);
    const double cI = C[r.I];
    const uint64_t mine = spin == 0 ? r.am : r.bm, mineh = spin == 0 ? r.amh : r.bmh;
    const double c2 = cI * cI;
    if (fabs(c2) > 1e-16) for_occ(mine, mineh, [&](int o) { atomicAdd(acc + o * (n + 1), c2); });
    const int ns = spin == 0 ? r.n1a : r.n1b;
    for (int s = 0; s < ns; s++) {
      int64_t J = -1;
      int info;
      uint64_t jm, jmh;
      if (spin == 0) {
        const int Ja = a.a1_J[r.a1b + s];
        info = a.a1_info[r.a1b + s];
        jm = a.astr[Ja];
        jmh = hiword(a.astr_hi, Ja);
        if (r.ib < a.rowlen[Ja]) J = a.rowoff[Ja] + r.ib;
      } else {
        const int Jb = a.b1_J[r.b1b + s];
        info = a.b1_info[r.b1b + s];
        jm = a.bstr[Jb];
        jmh = hiword(a.bstr_hi, Jb);
        if (Jb < a.rowlen[r.ia]) J = a.rowoff[r.ia] + Jb;
      }
      if (J < 0 || J > r.I) continue;  // each pair once, from the later determinant
      const double c = ((info & 1) ? -cI : cI) * C[J];
      if (fabs(c) <= 1e-16) continue;
      const int k = first_set(mine & ~jm, mineh & ~jmh), l = first_set(jm & ~mine, jmh & ~mineh);
      atomicAdd(acc + k + l * n, c);
      atomicAdd(acc + l + k * n, c);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n * n; i += blockDim.x)
    if (acc[i] != 0.0) atomicAdd(rdm + i, acc[i]);
}

// ---- two species: determinant (a0, b0, a1, b1) of the product space built
// by ci_two.cu (species-0 prefix rows x per-level species-1 blocks)
struct TwoAddr {
  const int32_t *e_a, *e_b, *elev, *rowoff0, *rowlen0, *prowoff, *prowlen, *pdet_a, *pdet_b;
  const int64_t *ebase, *pfirst, *psize;
  int npa1;
  const uint64_t *str[2][2], *str_hi[2][2];  // str_hi: orbitals 64..127 (NULL for one-word strings)
  const int64_t *s1_off[2][2];
  const int32_t *s1_J[2][2], *s1_info[2][2];
};

__device__ __forceinline__ int64_t two_lookup(const TwoAddr &t, int a0, int b0, int a1, int b1) {
  if (b0 >= t.rowlen0[a0]) return -1;
  const int ie = t.rowoff0[a0] + b0;
  const int L = t.elev[ie];
  if (L < 0) return -1;
  const int64_t r = (int64_t)L * t.npa1 + a1;
  if (b1 >= t.prowlen[r]) return -1;
  return t.ebase[ie] + t.prowoff[r] + b1;
}

// CTA per species-0 pair ie, threads over its species-1 block
__global__ void __launch_bounds__(PROP_THREADS) s2_two_kernel(TwoAddr t, int sp, const double *C, int64_t ldc,
                                                              int nvec, double *out) {
  __shared__ double red[S2_MAXV][PROP_THREADS / 32];
  const int ie = blockIdx.x;
  double acc[S2_MAXV];
#pragma unroll
  for (int v = 0; v < S2_MAXV; v++) acc[v] = 0.0;
  const int L = t.elev[ie];
  const int64_t nq = L < 0 ? 0 : t.psize[L];
  for (int64_t q = threadIdx.x; q < nq; q += blockDim.x) {
    int d[4] = {t.e_a[ie], t.e_b[ie], t.pdet_a[t.pfirst[L] + q], t.pdet_b[t.pfirst[L] + q]};
    const int64_t I = t.ebase[ie] + q;
    const int ia = d[2 * sp], ib = d[2 * sp + 1];
    const uint64_t am = t.str[sp][0][ia], bm = t.str[sp][1][ib];
    const uint64_t amh = hiword(t.str_hi[sp][0], ia), bmh = hiword(t.str_hi[sp][1], ib);
    double cI[S2_MAXV];
#pragma unroll
    for (int v = 0; v < S2_MAXV; v++) cI[v] = v < nvec ? C[I + v * ldc] : 0.0;
    const uint64_t open = am ^ bm, openh = amh ^ bmh;
    const int n_open = popc2(open, openh), n_a = popc2(open & am, openh & amh);
    const double sz = n_a - 0.5 * n_open;
    const double dg = n_a + sz * (sz - 1.0);
#pragma unroll
    for (int v = 0; v < S2_MAXV; v++) acc[v] += cI[v] * cI[v] * dg;
    const int64_t a1b = t.s1_off[sp][0][ia], b1b = t.s1_off[sp][1][ib];
    const int n1a = (int)(t.s1_off[sp][0][ia + 1] - a1b), n1b = (int)(t.s1_off[sp][1][ib + 1] - b1b);
    for (int s = 0; s < n1a; s++) {
      const int Ja = t.s1_J[sp][0][a1b + s], infa = t.s1_info[sp][0][a1b + s];
      const uint64_t jam = t.str[sp][0][Ja], jamh = hiword(t.str_hi[sp][0], Ja);
      const int ha = first_set(am & ~jam, amh & ~jamh), pa = first_set(jam & ~am, jamh & ~amh);
      if (!occupied(bm, bmh, pa) || occupied(bm, bmh, ha)) continue;
      uint64_t jbm = bm, jbmh = bmh;
      flip_orb(jbm, jbmh, pa);
      flip_orb(jbm, jbmh, ha);
      for (int q2 = 0; q2 < n1b; q2++) {
        const int Jb = t.s1_J[sp][1][b1b + q2];
        if (t.str[sp][1][Jb] != jbm || hiword(t.str_hi[sp][1], Jb) != jbmh) continue;
        int e[4] = {d[0], d[1], d[2], d[3]};
        e[2 * sp] = Ja;
        e[2 * sp + 1] = Jb;
        const int64_t J = two_lookup(t, e[0], e[1], e[2], e[3]);
        if (J >= 0) {
          const double ph = ((infa ^ t.s1_info[sp][1][b1b + q2]) & 1) ? -1.0 : 1.0;
#pragma unroll
          for (int v = 0; v < S2_MAXV; v++)
            if (v < nvec) acc[v] -= ph * cI[v] * C[J + v * ldc];
        }
        break;
      }
    }
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int v = 0; v < S2_MAXV; v++) {
    double x = acc[v];
    for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) red[v][w] = x;
  }
  __syncthreads();
  if (threadIdx.x < nvec) {
    double x = 0.0;
    for (int i = 0; i < PROP_THREADS / 32; i++) x += red[threadIdx.x][i];
    atomicAdd(out + threadIdx.x, x);
  }
}

__global__ void __launch_bounds__(PROP_THREADS) rdm1_two_kernel(TwoAddr t, int sp, int spin, int n, const double *C,
                                                                double *rdm) {
  extern __shared__ double acc[];  // n x n
  for (int i = threadIdx.x; i < n * n; i += blockDim.x) acc[i] = 0.0;
  __syncthreads();
  const int ie = blockIdx.x;
  const int L = t.elev[ie];
  const int64_t nq = L < 0 ? 0 : t.psize[L];
  for (int64_t q = threadIdx.x; q < nq; q += blockDim.x) {
    int d[4] = {t.e_a[ie], t.e_b[ie], t.pdet_a[t.pfirst[L] + q], t.pdet_b[t.pfirst[L] + q]};
    const int64_t I = t.ebase[ie] + q;
    const double cI = C[I];
    const int si = d[2 * sp + spin];
    const uint64_t mine = t.str[sp][spin][si], mineh = hiword(t.str_hi[sp][spin], si);
    const double c2 = cI * cI;
    if (fabs(c2) > 1e-16) for_occ(mine, mineh, [&](int o) { atomicAdd(acc + o * (n + 1), c2); });
    const int64_t b = t.s1_off[sp][spin][si];
    const int ns = (int)(t.s1_off[sp][spin][si + 1] - b);
    for (int s = 0; s < ns; s++) {
      const int Js = t.s1_J[sp][spin][b + s], info = t.s1_info[sp][spin][b + s];
      int e[4] = {d[0], d[1], d[2], d[3]};
      e[2 * sp + spin] = Js;
      const int64_t J = two_lookup(t, e[0], e[1], e[2], e[3]);
      if (J < 0 || J > I) continue;  // each pair once, from the later determinant
      const double c = ((info & 1) ? -cI : cI) * C[J];
      if (fabs(c) <= 1e-16) continue;
      const uint64_t jm = t.str[sp][spin][Js], jmh = hiword(t.str_hi[sp][spin], Js);
      const int k = first_set(mine & ~jm, mineh & ~jmh), l = first_set(jm & ~mine, jmh & ~mineh);
      atomicAdd(acc + k + l * n, c);
      atomicAdd(acc + l + k * n, c);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n * n; i += blockDim.x)
    if (acc[i] != 0.0) atomicAdd(rdm + i, acc[i]);
}

static TwoAddr make_two(const pq_ci_handle *h) {
  TwoAddr t{};
  t.e_a = h->d_e_a.as<int32_t>();
  t.e_b = h->d_e_b.as<int32_t>();
  t.elev = h->d_elev.as<int32_t>();
  t.rowoff0 = h->d_rowoff.as<int32_t>();
  t.rowlen0 = h->d_rowlen.as<int32_t>();
  t.prowoff = h->d_prowoff.as<int32_t>();
  t.prowlen = h->d_prowlen.as<int32_t>();
  t.pdet_a = h->d_pdet_a.as<int32_t>();
  t.pdet_b = h->d_pdet_b.as<int32_t>();
  t.ebase = h->d_ebase.as<int64_t>();
  t.pfirst = h->d_pfirst.as<int64_t>();
  t.psize = h->d_psize.as<int64_t>();
  t.npa1 = (int)h->str[1][0].size();
  for (int s = 0; s < 2; s++)
    for (int sp = 0; sp < 2; sp++) {
      t.str[s][sp] = h->tab[s][sp].str.as<uint64_t>();
      t.str_hi[s][sp] = h->tab[s][sp].str_hi.as<uint64_t>();
      t.s1_off[s][sp] = h->tab[s][sp].s1_off.as<int64_t>();
      t.s1_J[s][sp] = h->tab[s][sp].s1_J.as<int32_t>();
      t.s1_info[s][sp] = h->tab[s][sp].s1_info.as<int32_t>();
    }
  return t;
}


}  // namespace pq

using namespace pq;

extern "C" {

pq_status pq_ci_s2(pq_ci_handle *h, const double *C, int64_t ldc, int32_t nvec, double *s2) {
  clear_error();
  if (!h || !C || !s2 || nvec < 1 || ldc < (h ? h->n_dets : 0)) {
    set_error("pq_ci_s2: bad arguments");
    return PQ_ERR_ARG;
  }
  const int ns = h->n_species;
  DevBuf out;
  PQ_TRY(out.alloc(sizeof(double) * S2_MAXV));
  std::vector<double> part(S2_MAXV);
  for (int sp = 0; sp < ns; sp++)
    for (int v0 = 0; v0 < nvec; v0 += S2_MAXV) {
      const int c = std::min(S2_MAXV, nvec - v0);
      PQ_CUDA_TRY(cudaMemsetAsync(out.ptr, 0, sizeof(double) * S2_MAXV, h->stream));
      if (ns == 1) {
        const ConnArgs a = make_conn_args(h);
        const int na = (int)h->rowlen.size();
        const int maxlen = *std::max_element(h->rowlen.begin(), h->rowlen.end());
        const dim3 grid((unsigned)na, (unsigned)std::min((maxlen + PROP_THREADS - 1) / PROP_THREADS, 65535));
        s2_kernel<<<grid, PROP_THREADS, 0, h->stream>>>(a, na, C + (size_t)v0 * ldc, ldc, c, out.as<double>());
      } else {
        s2_two_kernel<<<(unsigned)h->e_a.size(), PROP_THREADS, 0, h->stream>>>(make_two(h), sp, C + (size_t)v0 * ldc,
                                                                               ldc, c, out.as<double>());
      }
      PQ_CUDA_TRY(cudaGetLastError());
      PQ_CUDA_TRY(cudaMemcpyAsync(part.data(), out.ptr, sizeof(double) * c, cudaMemcpyDeviceToHost, h->stream));
      PQ_CUDA_TRY(cudaStreamSynchronize(h->stream));
      for (int v = 0; v < c; v++) s2[(size_t)(v0 + v) * ns + sp] = part[v];
    }
  return PQ_OK;
}

pq_status pq_ci_rdm1(pq_ci_handle *h, const double *C, int32_t species, int32_t spin, double *rdm) {
  clear_error();
  if (!h || !C || !rdm || spin < 0 || spin > 1 || species < 0 || species >= h->n_species) {
    set_error("pq_ci_rdm1: bad arguments");
    return PQ_ERR_ARG;
  }
  const int n = h->n_orb[species];
  DevBuf out;
  PQ_TRY(out.alloc(sizeof(double) * n * n));
  PQ_CUDA_TRY(cudaMemsetAsync(out.ptr, 0, sizeof(double) * n * n, h->stream));
  const size_t smem = sizeof(double) * n * n;
  if (h->n_species == 1) {
    const ConnArgs a = make_conn_args(h);
    const int na = (int)h->rowlen.size();
    const int maxlen = *std::max_element(h->rowlen.begin(), h->rowlen.end());
    const dim3 grid((unsigned)na, (unsigned)std::min((maxlen + PROP_THREADS - 1) / PROP_THREADS, 65535));
    if (smem > 48 * 1024) PQ_CUDA_TRY(cudaFuncSetAttribute(rdm1_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    rdm1_kernel<<<grid, PROP_THREADS, smem, h->stream>>>(a, na, n, spin, C, out.as<double>());
  } else {
    if (smem > 48 * 1024)
      PQ_CUDA_TRY(cudaFuncSetAttribute(rdm1_two_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    rdm1_two_kernel<<<(unsigned)h->e_a.size(), PROP_THREADS, smem, h->stream>>>(make_two(h), species, spin, n, C,
                                                                               out.as<double>());
  }
  PQ_CUDA_TRY(cudaGetLastError());
  PQ_CUDA_TRY(cudaMemcpyAsync(rdm, out.ptr, sizeof(double) * n * n, cudaMemcpyDeviceToHost, h->stream));
  PQ_CUDA_TRY(cudaStreamSynchronize(h->stream));
  return PQ_OK;
}

}  // extern "C"
