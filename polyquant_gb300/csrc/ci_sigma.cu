// sigma = H C for one species, matrix-free, on the GPU.
//
// Reference: src/ci/detset/direct_singleparticle.cpp:238-372
// (sigma_one_species_class_singleshot).  The reference visits every unordered
// connected pair (I, J) once and updates both sigma_I and sigma_J from
// per-thread private copies.  Here each output determinant I is owned by one
// thread that gathers H_IJ C_J over all connected J, so no atomics or private
// copies are needed; the element formulas are the reference's
// (slater_condon_singleparticle.cpp:53-175), evaluated from tables built in
// ci_setup.cu.
//
// Work decomposition: one CTA per (alpha string Ia, block of beta strings);
// thread <-> determinant (Ia, Ib).  Everything that depends only on Ia is
// staged once per CTA in shared memory:
//   Wa[pair]        = sum_{k in occ(Ia)} (kk|pair)_ab  (opposite-spin Coulomb of beta singles)
//   Jrow[e][k]      = (pair_e|kk)_ab for the CTA's alpha singles e (read from
//                     the integrals in global memory when it does not fit)
//   Tab[e][pair_b]  = sign_e (pair_e|pair_b)_ab        (alpha-beta doubles)
// C/sigma are interleaved by determinant (X[det*NV + v]) so one vector load
// fetches all roots of a determinant.
#include <algorithm>

#include "ci_conn.cuh"
#include "pq_bits.cuh"
#include "pq_internal.h"

namespace pq {

__device__ __forceinline__ int idx2d(int i, int j) { return i > j ? i * (i + 1) / 2 + j : j * (j + 1) / 2 + i; }

template <typename T> struct SpinView {
  const uint64_t *str, *str_hi;  // str_hi: orbitals 64..127 (NULL for one-word strings)
  const int64_t *s1_off;
  const int32_t *s1_J;
  const int32_t *s1_info;
  const T *s1_F;
  const int64_t *s2_off;
  const int32_t *s2_J;
  const T *s2_D;
};

template <typename T> struct SigmaArgs {
  SpinView<T> a, b;
  const int64_t *rowoff;
  const int32_t *rowlen;
  const T *eab;  // row-major [pair_alpha][pair_beta]
  const double *diag;
  double shift;
  int n_orb, npair, max1a;
  int jrow_global;  // the alpha singles' Coulomb rows are read from eab instead of shared memory
  int64_t nblk_b;
  const T *X;
  T *Y;
};

// vector loads/stores of NV consecutive values
template <typename T, int NV> struct VecIO;
template <> struct VecIO<float, 1> {
  static __device__ __forceinline__ void ld(const float *p, float (&r)[1]) { r[0] = __ldg(p); }
  static __device__ __forceinline__ void st(float *p, const float (&r)[1]) { p[0] = r[0]; }
};
template <> struct VecIO<float, 2> {
  static __device__ __forceinline__ void ld(const float *p, float (&r)[2]) {
    float2 v = __ldg(reinterpret_cast<const float2 *>(p));
    r[0] = v.x, r[1] = v.y;
  }
  static __device__ __forceinline__ void st(float *p, const float (&r)[2]) {
    *reinterpret_cast<float2 *>(p) = make_float2(r[0], r[1]);
  }
};
template <> struct VecIO<float, 4> {
  static __device__ __forceinline__ void ld(const float *p, float (&r)[4]) {
    float4 v = __ldg(reinterpret_cast<const float4 *>(p));
    r[0] = v.x, r[1] = v.y, r[2] = v.z, r[3] = v.w;
  }
  static __device__ __forceinline__ void st(float *p, const float (&r)[4]) {
    *reinterpret_cast<float4 *>(p) = make_float4(r[0], r[1], r[2], r[3]);
  }
};
template <> struct VecIO<double, 1> {
  static __device__ __forceinline__ void ld(const double *p, double (&r)[1]) { r[0] = __ldg(p); }
  static __device__ __forceinline__ void st(double *p, const double (&r)[1]) { p[0] = r[0]; }
};
template <> struct VecIO<double, 2> {
  static __device__ __forceinline__ void ld(const double *p, double (&r)[2]) {
    double2 v = __ldg(reinterpret_cast<const double2 *>(p));
    r[0] = v.x, r[1] = v.y;
  }
  static __device__ __forceinline__ void st(double *p, const double (&r)[2]) {
    *reinterpret_cast<double2 *>(p) = make_double2(r[0], r[1]);
  }
};
template <> struct VecIO<double, 4> {
  static __device__ __forceinline__ void ld(const double *p, double (&r)[4]) {
    double2 v0 = __ldg(reinterpret_cast<const double2 *>(p));
    double2 v1 = __ldg(reinterpret_cast<const double2 *>(p) + 1);
    r[0] = v0.x, r[1] = v0.y, r[2] = v1.x, r[3] = v1.y;
  }
  static __device__ __forceinline__ void st(double *p, const double (&r)[4]) {
    reinterpret_cast<double2 *>(p)[0] = make_double2(r[0], r[1]);
    reinterpret_cast<double2 *>(p)[1] = make_double2(r[2], r[3]);
  }
};

template <typename T, int NV> __device__ __forceinline__ void fma_vec(T (&acc)[NV], T c, const T *src) {
  T x[NV];
  VecIO<T, NV>::ld(src, x);
#pragma unroll
  for (int v = 0; v < NV; v++) acc[v] = fma(c, x[v], acc[v]);
}

// v or -v selected by the low bit of `neg`, on the integer pipe
__device__ __forceinline__ float flip_sign(float v, uint32_t neg) { return __int_as_float(__float_as_int(v) ^ (int)(neg << 31)); }
__device__ __forceinline__ double flip_sign(double v, uint32_t neg) {
  return __hiloint2double(__double2hiint(v) ^ (int)(neg << 31), __double2loint(v));
}

constexpr int SIGMA_THREADS = 256;
constexpr int SIGMA_CHUNK = 8;

// PK > 0: the thread's beta singles (J << 10 | pair << 1 | phase bit) are held
// in PK registers and the alpha-beta loop runs alpha-neighbour-outer, so all
// CTAs of one alpha string sweep the same rows of C at the same time (the L2
// working set stays small).  Needs TAB, J < 2^22, pair < 512, <= PK singles.
template <typename T, int NV, bool FULL, bool TAB, int PK>
__global__ void __launch_bounds__(SIGMA_THREADS, (PK > 0 ? 2 : 1)) sigma_one_species_kernel(SigmaArgs<T> p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *Wa = reinterpret_cast<T *>(smem_raw);
  T *Jrow = Wa + p.npair;
  T *Tab = Jrow + (p.jrow_global ? 0 : p.max1a * p.n_orb);

  const int64_t Ia = blockIdx.x / p.nblk_b;
  const int Ib = (int)(blockIdx.x % p.nblk_b) * SIGMA_THREADS + threadIdx.x;
  const uint64_t ma = p.a.str[Ia], mah = hiword(p.a.str_hi, Ia);
  const int64_t a1_0 = p.a.s1_off[Ia];
  const int na1 = (int)(p.a.s1_off[Ia + 1] - a1_0);
  const int npair = p.npair, n_orb = p.n_orb;

  for (int q = threadIdx.x; q < npair; q += SIGMA_THREADS) {
    T s = 0;
    for_occ(ma, mah, [&](int k) { s += p.eab[(int64_t)idx2d(k, k) * npair + q]; });
    Wa[q] = s;
  }
  for (int t = threadIdx.x; t < (p.jrow_global ? 0 : na1 * n_orb); t += SIGMA_THREADS) {
    int e = t / n_orb, k = t - e * n_orb;
    int pa = p.a.s1_info[a1_0 + e] >> 1;
    Jrow[t] = p.eab[(int64_t)pa * npair + idx2d(k, k)];
  }
  if (TAB) {
    for (int t = threadIdx.x; t < na1 * npair; t += SIGMA_THREADS) {
      int e = t / npair, q = t - e * npair;
      int info = p.a.s1_info[a1_0 + e];
      T v = p.eab[(int64_t)(info >> 1) * npair + q];
      Tab[t] = (info & 1) ? -v : v;
    }
  }
  __syncthreads();

  const int lenI = p.rowlen[Ia];
  if (Ib >= lenI) return;
  const int64_t rowI = p.rowoff[Ia];
  const int64_t I = rowI + Ib;
  const uint64_t mb = p.b.str[Ib], mbh = hiword(p.b.str_hi, Ib);

  T acc[NV];
  {
    T x[NV];
    VecIO<T, NV>::ld(p.X + I * NV, x);
    const T dI = (T)(p.diag[I] - p.shift);
#pragma unroll
    for (int v = 0; v < NV; v++) acc[v] = dI * x[v];
  }
  const int64_t b1_0 = p.b.s1_off[Ib], b1_1 = p.b.s1_off[Ib + 1];
  // beta singles: sign * (F + opposite-spin Coulomb from alpha occupations)
  for (int64_t e = b1_0; e < b1_1; e++) {
    const int Jb = __ldg(p.b.s1_J + e);
    if (!FULL && Jb >= lenI) continue;
    const int info = __ldg(p.b.s1_info + e);
    T hv = __ldg(p.b.s1_F + e) + Wa[info >> 1];
    if (info & 1) hv = -hv;
    fma_vec<T, NV>(acc, hv, p.X + (rowI + Jb) * NV);
  }
  // beta-beta doubles
  {
    const int64_t e0 = p.b.s2_off[Ib], e1 = p.b.s2_off[Ib + 1];
    for (int64_t e = e0; e < e1; e++) {
      const int Jb = __ldg(p.b.s2_J + e);
      if (!FULL && Jb >= lenI) continue;
      fma_vec<T, NV>(acc, __ldg(p.b.s2_D + e), p.X + (rowI + Jb) * NV);
    }
  }
  // alpha singles: sign * (F + opposite-spin Coulomb from beta occupations)
  for (int e = 0; e < na1; e++) {
    const int Ja = __ldg(p.a.s1_J + a1_0 + e);
    if (!FULL && Ib >= __ldg(p.rowlen + Ja)) continue;
    const int info = __ldg(p.a.s1_info + a1_0 + e);
    T hv = __ldg(p.a.s1_F + a1_0 + e);
    if (p.jrow_global) {
      const T *er = p.eab + (int64_t)(info >> 1) * npair;
      for_occ(mb, mbh, [&](int k) { hv += __ldg(er + idx2d(k, k)); });
    } else {
      const T *jr = Jrow + e * n_orb;
      for_occ(mb, mbh, [&](int k) { hv += jr[k]; });
    }
    if (info & 1) hv = -hv;
    fma_vec<T, NV>(acc, hv, p.X + (__ldg(p.rowoff + Ja) + Ib) * NV);
  }
  // alpha-alpha doubles
  {
    const int64_t e0 = p.a.s2_off[Ia], e1 = p.a.s2_off[Ia + 1];
    for (int64_t e = e0; e < e1; e++) {
      const int Ja = __ldg(p.a.s2_J + e);
      if (!FULL && Ib >= __ldg(p.rowlen + Ja)) continue;
      fma_vec<T, NV>(acc, __ldg(p.a.s2_D + e), p.X + (__ldg(p.rowoff + Ja) + Ib) * NV);
    }
  }
  // alpha-beta doubles: sign_a sign_b (pair_a | pair_b)_ab
  if constexpr (PK > 0) {
    uint32_t bpk[PK];
    const int nb1 = (int)(b1_1 - b1_0);
#pragma unroll
    for (int c = 0; c < PK; c++)
      bpk[c] = c < nb1 ? (((uint32_t)__ldg(p.b.s1_J + b1_0 + c) << 10) | (uint32_t)__ldg(p.b.s1_info + b1_0 + c))
                       : 0xffffffffu;
    for (int e = 0; e < na1; e++) {
      const int Ja = __ldg(p.a.s1_J + a1_0 + e);
      const int64_t ro = __ldg(p.rowoff + Ja);
      const int la = FULL ? 0x7fffffff : __ldg(p.rowlen + Ja);
      const T *row = Tab + e * npair;
#pragma unroll
      for (int c = 0; c < PK; c++) {
        const uint32_t w = bpk[c];
        const int Jb = (int)(w >> 10);
        if (c < nb1 && (FULL || Jb < la)) {
          const T coef = flip_sign(row[(w >> 1) & 511u], w & 1u);
          fma_vec<T, NV>(acc, coef, p.X + (ro + Jb) * NV);
        }
      }
    }
  } else {
    for (int64_t j0 = b1_0; j0 < b1_1; j0 += SIGMA_CHUNK) {
      int Jb[SIGMA_CHUNK], pb[SIGMA_CHUNK];
      uint32_t sb[SIGMA_CHUNK];
#pragma unroll
      for (int c = 0; c < SIGMA_CHUNK; c++) {
        if (j0 + c < b1_1) {
          Jb[c] = __ldg(p.b.s1_J + j0 + c);
          int info = __ldg(p.b.s1_info + j0 + c);
          pb[c] = info >> 1;
          sb[c] = (uint32_t)(info & 1);
        } else {
          Jb[c] = 0x7fffffff;  // never below any row length
          pb[c] = 0;
          sb[c] = 0;
        }
      }
      for (int e = 0; e < na1; e++) {
        const int Ja = __ldg(p.a.s1_J + a1_0 + e);
        const int64_t ro = __ldg(p.rowoff + Ja);
        const int la = FULL ? 0x7fffffff : __ldg(p.rowlen + Ja);
        const T *row;
        uint32_t sa = 0;
        if (TAB) {
          row = Tab + e * npair;
        } else {
          const int info = __ldg(p.a.s1_info + a1_0 + e);
          row = p.eab + (int64_t)(info >> 1) * npair;
          sa = (uint32_t)(info & 1);
        }
#pragma unroll
        for (int c = 0; c < SIGMA_CHUNK; c++) {
          if (Jb[c] < la) {
            const T coef = flip_sign(TAB ? row[pb[c]] : __ldg(row + pb[c]), sa ^ sb[c]);
            fma_vec<T, NV>(acc, coef, p.X + (ro + Jb[c]) * NV);
          }
        }
      }
    }
  }
  VecIO<T, NV>::st(p.Y + I * NV, acc);
}

template <typename T>
static SpinView<T> make_view(const SpinTablesDev &t);
template <> SpinView<double> make_view<double>(const SpinTablesDev &t) {
  return {t.str.as<uint64_t>(), t.str_hi.as<uint64_t>(), t.s1_off.as<int64_t>(), t.s1_J.as<int32_t>(),
          t.s1_info.as<int32_t>(), t.s1_F64.as<double>(), t.s2_off.as<int64_t>(), t.s2_J.as<int32_t>(), t.s2_D64.as<double>()};
}
template <> SpinView<float> make_view<float>(const SpinTablesDev &t) {
  return {t.str.as<uint64_t>(), t.str_hi.as<uint64_t>(), t.s1_off.as<int64_t>(), t.s1_J.as<int32_t>(),
          t.s1_info.as<int32_t>(), t.s1_F32.as<float>(), t.s2_off.as<int64_t>(), t.s2_J.as<int32_t>(), t.s2_D32.as<float>()};
}

template <typename T, int NV, bool FULL, bool TAB, int PK>
static pq_status launch_sigma(const SigmaArgs<T> &a, int64_t na, size_t smem, cudaStream_t st) {
  auto kern = sigma_one_species_kernel<T, NV, FULL, TAB, PK>;
  if (smem > 48 * 1024) PQ_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int64_t grid = na * a.nblk_b;
  if (grid > 0x7fffffffLL) {
    set_error("grid too large");
    return PQ_ERR_ARG;
  }
  if (grid > 0) kern<<<(unsigned)grid, SIGMA_THREADS, smem, st>>>(a);
  PQ_CUDA_TRY(cudaGetLastError());
  return PQ_OK;
}

template <typename T, int NV>
static pq_status sigma_dispatch(pq_ci_handle *h, const T *X, T *Y, double shift) {
  SigmaArgs<T> a{};
  a.a = make_view<T>(h->tab[0][0]);
  a.b = make_view<T>(h->tab[0][1]);
  a.rowoff = h->d_rowoff.as<int64_t>();
  a.rowlen = h->d_rowlen.as<int32_t>();
  a.eab = std::is_same<T, double>::value ? (const T *)h->d_eab64.ptr : (const T *)h->d_eab32.ptr;
  a.diag = h->d_diag.as<double>();
  a.shift = shift;
  a.n_orb = h->n_orb[0];
  a.npair = h->npair[0];
  a.max1a = h->tab[0][0].max1;
  int64_t nb = h->tab[0][1].n_str, na = h->tab[0][0].n_str;
  a.nblk_b = (nb + SIGMA_THREADS - 1) / SIGMA_THREADS;
  a.X = X;
  a.Y = Y;
  size_t base = sizeof(T) * ((size_t)a.npair + (size_t)a.max1a * a.n_orb);
  size_t tab = sizeof(T) * (size_t)a.max1a * a.npair;
  const bool use_tab = base + tab <= 100 * 1024;
  // large orbital spaces: the Coulomb rows of the alpha singles stay in global memory (L2)
  a.jrow_global = base > 160 * 1024;
  if (a.jrow_global) base = sizeof(T) * (size_t)a.npair;
  size_t smem = base + (use_tab ? tab : 0);
  if (smem > 200 * 1024) {
    set_error("sigma shared-memory staging %zu bytes too large", smem);
    return PQ_ERR_ARG;
  }
  cudaStream_t st = h->stream;
  // packed-register alpha-beta path when the beta singles fit the encoding
  const int max1b = h->tab[0][1].max1;
  const bool pack_ok = use_tab && nb < (1 << 22) && a.npair <= 511;
  const int pk = !pack_ok ? 0 : (max1b <= 32 ? 32 : (max1b <= 64 ? 64 : 0));
  if (h->full) {
    if (pk == 32) return launch_sigma<T, NV, true, true, 32>(a, na, smem, st);
    if (pk == 64) return launch_sigma<T, NV, true, true, 64>(a, na, smem, st);
    return use_tab ? launch_sigma<T, NV, true, true, 0>(a, na, smem, st) : launch_sigma<T, NV, true, false, 0>(a, na, smem, st);
  }
  if (pk == 32) return launch_sigma<T, NV, false, true, 32>(a, na, smem, st);
  if (pk == 64) return launch_sigma<T, NV, false, true, 64>(a, na, smem, st);
  return use_tab ? launch_sigma<T, NV, false, true, 0>(a, na, smem, st) : launch_sigma<T, NV, false, false, 0>(a, na, smem, st);
}

pq_status ci_sigma_il(pq_ci_handle *h, const void *X, void *Y, int nvp, int precision, double shift,
                      bool allow_scratch) {
  if (h->use_explicit && precision == PQ_FP64 && shift == 0.0) return ci_ham_spmv(h, X, Y, nvp);
  if (h->n_species == 2) return ci_sigma2_il(h, X, Y, nvp, precision, shift);
  if (precision == PQ_FP32 && allow_scratch && h->fp32_v2) return ci_sigma32_v2(h, X, Y, nvp, shift);
  if (precision == PQ_FP64) {
    if (nvp == 1) return sigma_dispatch<double, 1>(h, (const double *)X, (double *)Y, shift);
    if (nvp == 2) return sigma_dispatch<double, 2>(h, (const double *)X, (double *)Y, shift);
    if (nvp == 4) return sigma_dispatch<double, 4>(h, (const double *)X, (double *)Y, shift);
  } else if (precision == PQ_FP32) {
    if (nvp == 1) return sigma_dispatch<float, 1>(h, (const float *)X, (float *)Y, shift);
    if (nvp == 2) return sigma_dispatch<float, 2>(h, (const float *)X, (float *)Y, shift);
    if (nvp == 4) return sigma_dispatch<float, 4>(h, (const float *)X, (float *)Y, shift);
  }
  set_error("unsupported interleave width %d / precision %d (widths 1, 2, 4)", nvp, precision);
  return PQ_ERR_ARG;
}

// ---------------------------------------------------------------------------
// column-major (n x nvec, ld) <-> interleaved (n x nvp) conversions
template <typename T>
__global__ void to_il_kernel(const double *C, int64_t ldc, int64_t n, int v0, int nv, int nvp, T *X) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (; i < n; i += stride)
    for (int v = 0; v < nvp; v++) X[i * nvp + v] = v < nv ? (T)C[i + (int64_t)(v0 + v) * ldc] : T(0);
}
template <typename T>
__global__ void from_il_kernel(const T *Y, int64_t n, int v0, int nv, int nvp, double *S, int64_t lds) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (; i < n; i += stride)
    for (int v = 0; v < nv; v++) S[i + (int64_t)(v0 + v) * lds] = (double)Y[i * nvp + v];
}

pq_status ci_to_il(pq_ci_handle *h, const double *C, int64_t ldc, int v0, int nv, int nvp, int precision, void *X) {
  int64_t n = h->n_dets;
  unsigned grid = (unsigned)std::min<int64_t>((n + 255) / 256, 152 * 16);
  if (grid == 0) return PQ_OK;
  if (precision == PQ_FP64)
    to_il_kernel<double><<<grid, 256, 0, h->stream>>>(C, ldc, n, v0, nv, nvp, (double *)X);
  else
    to_il_kernel<float><<<grid, 256, 0, h->stream>>>(C, ldc, n, v0, nv, nvp, (float *)X);
  PQ_CUDA_TRY(cudaGetLastError());
  return PQ_OK;
}

pq_status ci_from_il(pq_ci_handle *h, const void *Y, int v0, int nv, int nvp, int precision, double *S, int64_t lds) {
  int64_t n = h->n_dets;
  unsigned grid = (unsigned)std::min<int64_t>((n + 255) / 256, 152 * 16);
  if (grid == 0) return PQ_OK;
  if (precision == PQ_FP64)
    from_il_kernel<double><<<grid, 256, 0, h->stream>>>((const double *)Y, n, v0, nv, nvp, S, lds);
  else
    from_il_kernel<float><<<grid, 256, 0, h->stream>>>((const float *)Y, n, v0, nv, nvp, S, lds);
  PQ_CUDA_TRY(cudaGetLastError());
  return PQ_OK;
}

}  // namespace pq

namespace pq {

// Columns H[:, I_c] of the Hamiltonian for a list of determinants I_c (one
// species), written into column-major W (zeroed by the caller): the exact
// FP64 sigma of the unit vectors e_{I_c} from the connections of I_c alone.
// Block c handles column c; its threads walk the connection list of I_c.
__global__ void unit_columns_kernel(ConnArgs a, const int32_t *cia, const int32_t *cib, int64_t n, double *W) {
  const int c = blockIdx.x;
  double *w = W + (int64_t)c * n;
  const ConnRow r = conn_row(a, cia[c], cib[c]);
  const int64_t tot = r.total();
  for (int64_t t = threadIdx.x; t < tot; t += blockDim.x) {
    double v;
    const int64_t J = conn_elem(a, r, t, &v);
    if (J >= 0) w[J] = v;
  }
}

pq_status ci_unit_columns(pq_ci_handle *h, const std::vector<int64_t> &dets, double *W) {
  if (h->n_species != 1) {
    set_error("ci_unit_columns: one species only");
    return PQ_ERR_STATE;
  }
  const int m = (int)dets.size();
  std::vector<int32_t> ia(m), ib(m);
  for (int c = 0; c < m; c++) {
    const int64_t I = dets[c];
    const int64_t r = (int64_t)(std::upper_bound(h->rowoff.begin(), h->rowoff.end(), I) - h->rowoff.begin()) - 1;
    ia[c] = (int32_t)r;
    ib[c] = (int32_t)(I - h->rowoff[r]);
  }
  DevBuf dia, dib;
  PQ_TRY(upload(dia, ia, h->stream));
  PQ_TRY(upload(dib, ib, h->stream));
  PQ_CUDA_TRY(cudaMemsetAsync(W, 0, sizeof(double) * (size_t)h->n_dets * m, h->stream));
  const ConnArgs a = make_conn_args(h);
  unit_columns_kernel<<<m, 256, 0, h->stream>>>(a, dia.as<int32_t>(), dib.as<int32_t>(), h->n_dets, W);
  PQ_CUDA_TRY(cudaGetLastError());
  PQ_CUDA_TRY(cudaStreamSynchronize(h->stream));  // the index lists are freed on return
  return PQ_OK;
}

}  // namespace pq
