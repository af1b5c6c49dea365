// FP32 sigma for full-CI spaces, restructured so that every large gather is
// coalesced or reused (used by the mixed-precision Davidson; the FP64 kernel in
// ci_sigma.cu is bound by the FP64 pipe, this one by memory requests).
//
// Same matrix elements as ci_sigma.cu (reference: src/ci/detset/
// direct_singleparticle.cpp:238-372, slater_condon_singleparticle.cpp), split
// into three kinds of work on the det-interleaved vectors X[a][b][v]:
//   1. alpha-side terms (diagonal, alpha singles, alpha-alpha doubles): CTA per
//      alpha string, thread per beta string; the partner determinants
//      (Ja, Ib) of a warp are consecutive in memory.
//   2. beta-side terms (beta singles, beta-beta doubles): the same kernel on the
//      transposed copy XT[b][a], result transposed back and added.
//   For four vectors of a full-CI space whose doubles fill at least 3 % of a
//   row, the same-spin doubles of both sides are instead dense GEMMs on the
//   tcgen05 tensor cores (ci_sigma32_ss.cu) and passes 1-2 keep the diagonal
//   and the singles, whose opposite-spin Coulomb sums then come from a
//   precomputed [pair][column string] table.
//   3. alpha-beta doubles: for blocks of four vectors, up to 16 orbitals and
//      64 alpha singles per string, a GEMM per alpha string on the tcgen05
//      tensor cores (ci_sigma32_tc.cu).  Otherwise input-stationary on the CUDA cores: CTA
//      per alpha string Ja, lane per alpha single (Ja -> Ia_i).  For each beta
//      string Ib the warp loads the vectors C(Ja, Jb) of Ib's beta singles once
//      (one broadcast load each) and every lane applies its own coefficient
//      sign_i sign_j (pair_i | pair_j) from a shared-memory table, then adds its
//      partial sum into sigma(Ia_i, Ib) with one vector atomic.  Each loaded
//      vector is used by all alpha neighbours of Ja instead of once.
// The atomics make the summation order, and so the last bits of the FP32
// result, vary between runs.
#include <algorithm>

#include "pq_internal.h"

namespace pq {

__device__ __forceinline__ int idx2s(int i, int j) { return i > j ? i * (i + 1) / 2 + j : j * (j + 1) / 2 + i; }

template <int NV> struct FVec;
template <> struct FVec<1> {
  using V = float;
  static __device__ __forceinline__ float ld(const float *p) { return __ldg(p); }
};
template <> struct FVec<2> {
  using V = float2;
  static __device__ __forceinline__ float2 ld(const float *p) { return __ldg(reinterpret_cast<const float2 *>(p)); }
};
template <> struct FVec<4> {
  using V = float4;
  static __device__ __forceinline__ float4 ld(const float *p) { return __ldg(reinterpret_cast<const float4 *>(p)); }
};

__device__ __forceinline__ void vfma(float &acc, float c, float x) { acc = fmaf(c, x, acc); }
__device__ __forceinline__ void vfma(float2 &acc, float c, float2 x) {
  acc.x = fmaf(c, x.x, acc.x);
  acc.y = fmaf(c, x.y, acc.y);
}
__device__ __forceinline__ void vfma(float4 &acc, float c, float4 x) {
  acc.x = fmaf(c, x.x, acc.x);
  acc.y = fmaf(c, x.y, acc.y);
  acc.z = fmaf(c, x.z, acc.z);
  acc.w = fmaf(c, x.w, acc.w);
}
template <typename V> __device__ __forceinline__ V vzero();
template <> __device__ __forceinline__ float vzero<float>() { return 0.f; }
template <> __device__ __forceinline__ float2 vzero<float2>() { return make_float2(0.f, 0.f); }
template <> __device__ __forceinline__ float4 vzero<float4>() { return make_float4(0.f, 0.f, 0.f, 0.f); }

__device__ __forceinline__ float fflip(float v, uint32_t neg) { return __int_as_float(__float_as_int(v) ^ (int)(neg << 31)); }

struct RowSideArgs {
  const int64_t *s1_off;
  const int32_t *s1_J, *s1_info;
  const float *s1_F;
  const int64_t *s2_off;
  const int32_t *s2_J;
  const float *s2_D;
  const uint64_t *col_str;  // occupations of the column strings
  const float *erc;         // row-major [pair_row][pair_col]
  int n_orb, npair, max1;
  int64_t nrow, ncol, nblk;
  const double *diag;       // diagonal in [row][col] order (used with DIAG)
  double shift;
  const float *X;
  float *Y;
  const float *coul;        // without DOUBLES: [pair_row][col] = sum_{k in occ(col)} (pair_row | kk)
};

// Row-side terms: CTA per row string, thread per column string.
// DOUBLES = false leaves the same-spin doubles to the tensor-core GEMMs (ci_sigma32_ss.cu) and takes the
// singles' opposite-spin Coulomb sums from the precomputed table p.coul (one coalesced load per single
// instead of a sum over the column string's occupied orbitals).
template <int NV, bool DIAG, bool DOUBLES>
__global__ void __launch_bounds__(256) rowside_kernel(RowSideArgs p) {
  extern __shared__ float jrow[];  // [e][k] = (pair_e | kk) for the row string's singles e
  using V = typename FVec<NV>::V;
  // rows vary fastest: concurrently resident CTAs share one block of columns,
  // so the partner rows they read stay in L2
  const int64_t r = blockIdx.x % p.nrow;
  const int64_t c = (blockIdx.x / p.nrow) * 256 + threadIdx.x;
  const int64_t e0 = p.s1_off[r];
  const int n1 = (int)(p.s1_off[r + 1] - e0);
  if (DOUBLES) {
    for (int t = threadIdx.x; t < n1 * p.n_orb; t += 256) {
      int e = t / p.n_orb, k = t - e * p.n_orb;
      jrow[t] = p.erc[(int64_t)(p.s1_info[e0 + e] >> 1) * p.npair + idx2s(k, k)];
    }
    __syncthreads();
  }
  if (c >= p.ncol) return;
  const uint64_t mc = p.col_str[c];
  V acc = vzero<V>();
  if (DIAG) {
    const int64_t I = r * p.ncol + c;
    vfma(acc, (float)(p.diag[I] - p.shift), FVec<NV>::ld(p.X + I * NV));
  }
  for (int e = 0; e < n1; e++) {
    const int J = __ldg(p.s1_J + e0 + e);
    const int info = __ldg(p.s1_info + e0 + e);
    float h = __ldg(p.s1_F + e0 + e);
    if (DOUBLES) {
      const float *jr = jrow + e * p.n_orb;
      uint64_t m = mc;
      while (m) {
        int k = __ffsll((long long)m) - 1;
        h += jr[k];
        m &= m - 1;
      }
    } else {
      h += __ldg(p.coul + (int64_t)(info >> 1) * p.ncol + c);
    }
    vfma(acc, fflip(h, (uint32_t)(info & 1)), FVec<NV>::ld(p.X + ((int64_t)J * p.ncol + c) * NV));
  }
  if (DOUBLES) {
    const int64_t d0 = p.s2_off[r], d1 = p.s2_off[r + 1];
    for (int64_t e = d0; e < d1; e++) {
      const int J = __ldg(p.s2_J + e);
      vfma(acc, __ldg(p.s2_D + e), FVec<NV>::ld(p.X + ((int64_t)J * p.ncol + c) * NV));
    }
  }
  *reinterpret_cast<V *>(p.Y + (r * p.ncol + c) * NV) = acc;
}

// out[c][r] (=, or += with ADD) in[r][c] for NV-float elements
template <int NV, bool ADD>
__global__ void vtranspose_kernel(const float *in, int64_t R, int64_t C, float *out) {
  using V = typename FVec<NV>::V;
  __shared__ V tile[32][33];
  const int64_t r0 = (int64_t)blockIdx.y * 32, c0 = (int64_t)blockIdx.x * 32;
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int64_t r = r0 + y, c = c0 + threadIdx.x;
    if (r < R && c < C) tile[y][threadIdx.x] = *reinterpret_cast<const V *>(in + (r * C + c) * NV);
  }
  __syncthreads();
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int64_t c = c0 + y, r = r0 + threadIdx.x;
    if (r < R && c < C) {
      V *o = reinterpret_cast<V *>(out + (c * R + r) * NV);
      V v = tile[threadIdx.x][y];
      if (ADD) {
        V w = *o;
        const float *a = reinterpret_cast<const float *>(&v);
        float *b = reinterpret_cast<float *>(&w);
#pragma unroll
        for (int i = 0; i < NV; i++) b[i] += a[i];
        *o = w;
      } else {
        *o = v;
      }
    }
  }
}

struct ABArgs {
  const int64_t *a_off;
  const int32_t *a_J, *a_info;
  const int64_t *b_off;
  const int32_t *b_J, *b_info;
  const float *eab;  // row-major [pair_alpha][pair_beta]
  int npair;
  int64_t na, nb;
  int chunk, nchunks;
  const float *X;
  float *Y;
};

constexpr int AB_MAXI = 64;  // alpha singles per string handled by one CTA (two per lane)

template <int NV>
__global__ void __launch_bounds__(128) ab_scatter_kernel(ABArgs p) {
  // W2[pair_b][lane] = (coefficient of alpha single lane, of alpha single lane + 32):
  // one 8-byte load per lane and partner, consecutive across the warp
  extern __shared__ float2 W2[];
  using V = typename FVec<NV>::V;
  const int64_t Ja = blockIdx.x / p.nchunks;
  const int ch = (int)(blockIdx.x % p.nchunks);
  const int64_t a0 = p.a_off[Ja];
  const int n1 = (int)(p.a_off[Ja + 1] - a0);
  for (int t = threadIdx.x; t < 32 * p.npair; t += 128) {
    const int q = t >> 5, l = t & 31;
    float2 w = make_float2(0.f, 0.f);
    if (l < n1) {
      const int info = p.a_info[a0 + l];
      w.x = fflip(p.eab[(int64_t)(info >> 1) * p.npair + q], (uint32_t)(info & 1));
    }
    if (l + 32 < n1) {
      const int info = p.a_info[a0 + l + 32];
      w.y = fflip(p.eab[(int64_t)(info >> 1) * p.npair + q], (uint32_t)(info & 1));
    }
    W2[q * 32 + l] = w;
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool v0 = lane < n1, v1 = lane + 32 < n1;
  const int64_t row0 = v0 ? (int64_t)__ldg(p.a_J + a0 + lane) * p.nb : 0;
  const int64_t row1 = v1 ? (int64_t)__ldg(p.a_J + a0 + lane + 32) * p.nb : 0;
  const float2 *wl = W2 + lane;
  const float *xrow = p.X + Ja * p.nb * NV;
  // per-warp staging of one beta string's signed partner vectors and pair codes
  V *xs = reinterpret_cast<V *>(W2 + 32 * p.npair) + warp * AB_MAXI;
  int *ps = reinterpret_cast<int *>(reinterpret_cast<V *>(W2 + 32 * p.npair) + 4 * AB_MAXI) + warp * AB_MAXI;
  const int64_t b_lo = (int64_t)ch * p.chunk, b_hi = (b_lo + p.chunk < p.nb) ? b_lo + p.chunk : p.nb;
  // lane l fetches partners l and l + 32 of a beta string (coalesced table reads, one gather each);
  // the partner's phase is applied to its vector here, once
  auto fetch = [&](int64_t Ib, V &xa, V &xb, int &ia, int &ib, int &n) {
    n = 0;
    ia = ib = 0;
    xa = xb = vzero<V>();
    if (Ib >= b_hi) return;
    const int64_t e0 = p.b_off[Ib];
    n = (int)(p.b_off[Ib + 1] - e0);
    if (lane < n) {
      const int info = __ldg(p.b_info + e0 + lane);
      ia = info >> 1;
      xa = FVec<NV>::ld(xrow + (int64_t)__ldg(p.b_J + e0 + lane) * NV);
      float *f = reinterpret_cast<float *>(&xa);
#pragma unroll
      for (int v = 0; v < NV; v++) f[v] = fflip(f[v], (uint32_t)(info & 1));
    }
    if (lane + 32 < n) {
      const int info = __ldg(p.b_info + e0 + lane + 32);
      ib = info >> 1;
      xb = FVec<NV>::ld(xrow + (int64_t)__ldg(p.b_J + e0 + lane + 32) * NV);
      float *f = reinterpret_cast<float *>(&xb);
#pragma unroll
      for (int v = 0; v < NV; v++) f[v] = fflip(f[v], (uint32_t)(info & 1));
    }
  };
  V xa, xb;
  int ia, ib, n;
  int64_t Ib = b_lo + warp;
  fetch(Ib, xa, xb, ia, ib, n);
  for (; Ib < b_hi; Ib += 4) {
    const int ncur = n;
    xs[lane] = xa;
    xs[lane + 32] = xb;
    ps[lane] = ia;
    ps[lane + 32] = ib;
    __syncwarp();
    fetch(Ib + 4, xa, xb, ia, ib, n);  // next string's loads overlap this string's arithmetic
    V acc0 = vzero<V>(), acc1 = vzero<V>();
#pragma unroll 4
    for (int j = 0; j < ncur; j++) {
      const V x = xs[j];
      const float2 w = wl[ps[j] * 32];
      vfma(acc0, w.x, x);
      vfma(acc1, w.y, x);
    }
    __syncwarp();
    if (v0) atomicAdd(reinterpret_cast<V *>(p.Y + (row0 + Ib) * NV), acc0);
    if (v1) atomicAdd(reinterpret_cast<V *>(p.Y + (row1 + Ib) * NV), acc1);
  }
}

// ---------------------------------------------------------------------------
bool sigma32_v2_applicable(const pq_ci_handle *h) {
  if (h->n_species != 1 || !h->full || h->wide) return false;
  const int npair = h->npair[0];
  if (h->tab[0][0].max1 > AB_MAXI || h->tab[0][1].max1 > AB_MAXI) return false;
  const size_t wbytes = sizeof(float) * (size_t)AB_MAXI * npair;
  return wbytes <= 100 * 1024;
}

template <int NV>
static pq_status sigma32_v2_impl(pq_ci_handle *h, const float *X, float *Y, double shift) {
  cudaStream_t st = h->stream;
  const int64_t na = h->tab[0][0].n_str, nb = h->tab[0][1].n_str, n = h->n_dets;
  const int npair = h->npair[0], n_orb = h->n_orb[0];
  PQ_TRY(h->x_t.ensure(sizeof(float) * NV * (size_t)(n + 1)));
  PQ_TRY(h->z_t.ensure(sizeof(float) * NV * (size_t)(n + 1)));
  float *XT = h->x_t.as<float>(), *ZT = h->z_t.as<float>();
  const dim3 tb(32, 8);
  // 1. XT[b][a] = X[a][b]
  vtranspose_kernel<NV, false><<<dim3((unsigned)((nb + 31) / 32), (unsigned)((na + 31) / 32)), tb, 0, st>>>(X, na, nb, XT);
  PQ_CUDA_TRY(cudaGetLastError());
  // 2. alpha side (with the diagonal) -> Y
  // same-spin doubles on the tensor cores (4 roots, full CI) or in the row-side gathers
  const bool ss = NV == 4 && h->fp32_ss;
  const bool doubles = !ss;
  if (ss) PQ_TRY(ci_sigma32_ss_prepare(h));
  auto rowside = [&](int spin_row, const float *src, float *dst, const float *erc, bool diag) -> pq_status {
    const SpinTablesDev &tr = h->tab[0][spin_row];
    const SpinTablesDev &tc = h->tab[0][1 - spin_row];
    RowSideArgs a{};
    a.s1_off = tr.s1_off.as<int64_t>();
    a.s1_J = tr.s1_J.as<int32_t>();
    a.s1_info = tr.s1_info.as<int32_t>();
    a.s1_F = tr.s1_F32.as<float>();
    a.s2_off = tr.s2_off.as<int64_t>();
    a.s2_J = tr.s2_J.as<int32_t>();
    a.s2_D = tr.s2_D32.as<float>();
    a.col_str = tc.str.as<uint64_t>();
    a.erc = erc;
    a.n_orb = n_orb;
    a.npair = npair;
    a.max1 = tr.max1;
    a.nrow = tr.n_str;
    a.ncol = tc.n_str;
    a.nblk = (a.ncol + 255) / 256;
    a.diag = h->d_diag.as<double>();
    a.shift = shift;
    a.X = src;
    a.Y = dst;
    a.coul = ss ? ci_sigma32_ss_coulomb(h, spin_row) : nullptr;
    const size_t smem = doubles ? sizeof(float) * (size_t)std::max(tr.max1, 1) * n_orb : 0;
    const int64_t grid = a.nrow * a.nblk;
    if (diag && doubles)
      rowside_kernel<NV, true, true><<<(unsigned)grid, 256, smem, st>>>(a);
    else if (diag)
      rowside_kernel<NV, true, false><<<(unsigned)grid, 256, smem, st>>>(a);
    else if (doubles)
      rowside_kernel<NV, false, true><<<(unsigned)grid, 256, smem, st>>>(a);
    else
      rowside_kernel<NV, false, false><<<(unsigned)grid, 256, smem, st>>>(a);
    PQ_CUDA_TRY(cudaGetLastError());
    return PQ_OK;
  };
  PQ_TRY(rowside(0, X, Y, h->d_eab32.as<float>(), true));
  // 3. beta side on the transposed copy -> ZT[b][a]
  PQ_TRY(rowside(1, XT, ZT, h->d_eba32.as<float>(), false));
  // 4. Y[a][b] += ZT[b][a]
  vtranspose_kernel<NV, true><<<dim3((unsigned)((na + 31) / 32), (unsigned)((nb + 31) / 32)), tb, 0, st>>>(ZT, nb, na, Y);
  PQ_CUDA_TRY(cudaGetLastError());
  if (ss) PQ_TRY(ci_sigma32_same_spin_tc(h, X, Y));
  // 5. alpha-beta doubles: on the tensor cores where the shape allows (ci_sigma32_tc.cu), else
  // scattered with vector atomics
  if (h->fp32_tc && NV == 4) return ci_sigma32_ab_tc(h, X, Y, NV);
  ABArgs b{};
  const SpinTablesDev &ta = h->tab[0][0], &tbb = h->tab[0][1];
  b.a_off = ta.s1_off.as<int64_t>();
  b.a_J = ta.s1_J.as<int32_t>();
  b.a_info = ta.s1_info.as<int32_t>();
  b.b_off = tbb.s1_off.as<int64_t>();
  b.b_J = tbb.s1_J.as<int32_t>();
  b.b_info = tbb.s1_info.as<int32_t>();
  b.eab = h->d_eab32.as<float>();
  b.npair = npair;
  b.na = na;
  b.nb = nb;
  b.chunk = 512;
  b.nchunks = (int)((nb + b.chunk - 1) / b.chunk);
  b.X = X;
  b.Y = Y;
  const size_t smem = sizeof(float2) * 32 * (size_t)npair + (sizeof(float) * NV + sizeof(int)) * 4 * AB_MAXI;
  if (smem > 48 * 1024) PQ_CUDA_TRY(cudaFuncSetAttribute(ab_scatter_kernel<NV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int64_t grid = na * b.nchunks;
  if (grid > 0x7fffffffLL) {
    set_error("sigma32: grid too large");
    return PQ_ERR_ARG;
  }
  ab_scatter_kernel<NV><<<(unsigned)grid, 128, smem, st>>>(b);
  PQ_CUDA_TRY(cudaGetLastError());
  return PQ_OK;
}

pq_status ci_sigma32_v2(pq_ci_handle *h, const void *X, void *Y, int nvp, double shift) {
  if (nvp == 1) return sigma32_v2_impl<1>(h, (const float *)X, (float *)Y, shift);
  if (nvp == 2) return sigma32_v2_impl<2>(h, (const float *)X, (float *)Y, shift);
  if (nvp == 4) return sigma32_v2_impl<4>(h, (const float *)X, (float *)Y, shift);
  set_error("sigma32: unsupported width %d", nvp);
  return PQ_ERR_ARG;
}

}  // namespace pq
