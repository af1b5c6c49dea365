// Batched sigma and lockstep block Davidson over many independent CI problems.
//
// Each problem is a full-product determinant space: species 0 (electrons) is
// the complete alpha x beta string product, optionally times a complete
// species-1 (positron) product of P determinants, so that determinant
// (Ia, Ib, Jp) sits at ((Ia * Nb + Ib) * P + Jp).  Viewing the interleaved
// work vector of one problem as rows Ie = Ia * Nb + Ib of L = P * w values
// (w = padded vector count), the positron determinant rides along as extra
// columns: every electron connection Ie <- Je moves one contiguous row of L
// values, and the positron and electron-positron terms act inside the row.
// This restates, for the product layout, the terms of
// sigma_one_species_class_singleshot (src/ci/direct_singleparticle.cpp:238-372)
// and sigma_two_species_class_singleshot
// (src/ci/direct_mixedparticle.cpp:269-611) with the Slater-Condon elements of
// slater_condon_singleparticle.cpp and slater_condon_mixedparticle.cpp.
//
// One persistent kernel evaluates sigma for every active problem of a group
// per Davidson iteration: warps pull work units (problem, alpha string, block
// of beta strings) from one atomic counter in descending cost order, and a
// per-problem call record selects FP64 or FP32, the vector width and the
// buffers.  The per-iteration launch sequence (call records host->device,
// batched layout conversion, counter reset, sigma, batched conversion back) is
// captured once as a CUDA graph and replayed.  The launch shape (warps per
// CTA, rows per work unit) is chosen by timing candidates on a sample of the
// group's work units.
#include <cublas_v2.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <memory>
#include <numeric>
#include <vector>

#include "pq_internal.h"

namespace pq {
namespace batch {

constexpr int JMAX = 5;             // columns per lane: rows of at most 160 values
constexpr int MAXROW = 32 * JMAX;   // staging values per warp (group path)
constexpr int LANE_MAXL = 16;       // widest row of the one-lane-per-row path
constexpr int STAGE = 32 * LANE_MAXL > MAXROW ? 32 * LANE_MAXL : MAXROW;  // staging values per warp
constexpr int MAX_P = 40;           // positron determinants (rows of 40 * 4 values)

template <typename T> struct ProbT {
  const T *a1F, *b1F, *a2D, *b2D;  // singles (same-spin part, unsigned) and signed same-spin doubles
  const T *eab;                    // (pair_alpha | pair_beta) of species 0, row-major
  const T *ep[2][2];               // [electron spin][positron spin] (pair_e | pair_p), row-major
  const T *ps_h, *pd_h;            // positron single / double elements (signed, complete)
  const T *dpt;                    // [x][pair_e][Jp]: sum over occupied positron orbitals r of (pq|rr)
  const T *dea, *deb;              // [I][y][pair_p]: sum over occupied electron orbitals p of (pp|rs)
  const T *mtab;                   // [x][pair_e][e]: sign_p(e) (pair_e | rs(e)) for positron single entry e
};

struct Prob {
  const uint64_t *astr, *bstr;
  const int64_t *a1_off, *b1_off, *a2_off, *b2_off;
  const int32_t *a1_J, *a1_info, *b1_J, *b1_info, *a2_J, *b2_J;
  const int32_t *ps_off, *ps_code, *pd_off, *pd_I;  // CSR over Jp
  const double *diag;
  int64_t n_dets;
  int na, nb, npe, npp, P, nps;  // nps: positron single entries over all Jp
  double cf;
  ProbT<float> f;
  ProbT<double> d;
};

// Per-problem arguments of one batched sigma launch.
struct Call {
  int active, precision, lw, cnt;  // lw = log2 of the padded width w; cnt <= w real columns
  int lane_rows;                   // 1: one lane per row (rows of <= 16 values), 0: lane groups per row
  double shift;                    // FP32: sigma of (H - shift), added back in FP64
  void *X, *Y;                     // interleaved work vectors [det][w]
  const double *src;               // column-major FP64 input (leading dimension n_dets)
  double *dst;                     // column-major FP64 output
};

struct Unit {
  int prob, ia, b0, nrows;
};

struct Chunk {
  int prob;
  int64_t d0, d1;
};

template <typename T> __device__ __forceinline__ const ProbT<T> &pt(const Prob &p);
template <> __device__ __forceinline__ const ProbT<float> &pt<float>(const Prob &p) { return p.f; }
template <> __device__ __forceinline__ const ProbT<double> &pt<double>(const Prob &p) { return p.d; }

__device__ __forceinline__ int pairdiag(int k) { return k * (k + 3) / 2; }  // idx2(k, k)

// One work unit: rows (ia, b0 .. b0+nrows-1) of one problem, one warp.
// Lanes form R = 32 / G groups of G lanes; a group owns one row and lane gl of
// the group owns the row's columns gl + j * G (j < J, < L).  Matrix elements
// are computed G at a time (one per lane) and broadcast with shuffles; rows
// are addressed by 32-bit row indices and one 64-bit base per connection.
template <typename T, int J>
__device__ void do_rows(const Prob &p, const Call &cl, const Unit &U, T *stg, int lane, int G) {
  const ProbT<T> &q = pt<T>(p);
  const int P = p.P, lw = cl.lw, L = P << lw;
  const int R = 32 / G, g = lane / G, gl = lane - g * G;
  const T *__restrict__ X = (const T *)cl.X;
  T *__restrict__ Y = (T *)cl.Y;
  const int ia = U.ia, nb = p.nb, npe = p.npe, npp = p.npp;
  const int64_t a1b = p.a1_off[ia];
  const int a1n = (int)(p.a1_off[ia + 1] - a1b);
  const int64_t a2b = p.a2_off[ia];
  const int a2n = (int)(p.a2_off[ia + 1] - a2b);
  const uint64_t amask = p.astr[ia];
  const T cf = (T)p.cf;
  const int rowa = ia * nb;
  T *srow = stg + g * G;  // staging of one row (L <= G when R > 1)
  for (int r0 = 0; r0 < U.nrows; r0 += R) {
    const bool rok = r0 + g < U.nrows;
    const int ib = rok ? U.b0 + r0 + g : 0;
    const int Ie = rowa + ib;
    const int64_t b1b = p.b1_off[ib];
    const int b1n = rok ? (int)(p.b1_off[ib + 1] - b1b) : 0;
    const int64_t b2b = p.b2_off[ib];
    const int b2n = rok ? (int)(p.b2_off[ib + 1] - b2b) : 0;
    const uint64_t bmask = p.bstr[ib];
    const int b1max = __reduce_max_sync(0xffffffffu, b1n);
    const int b2max = __reduce_max_sync(0xffffffffu, b2n);
    T acc[J];
    {
      const T *xr = X + (int64_t)Ie * L;
      const double *dg = p.diag + (int64_t)Ie * P;
#pragma unroll
      for (int j = 0; j < J; j++) {
        const int c = gl + j * G;
        acc[j] = T(0);
        if (rok && c < L) {
          const T x = xr[c];
          acc[j] = (T)(dg[c >> lw] - cl.shift) * x;
          if (P > 1) srow[c] = x;
        }
      }
    }
    // positron terms inside the row: positron singles and doubles, and the
    // electron-diagonal x positron-single cross term
    if (P > 1) {
      __syncwarp();
      const T *dea = q.dea + (int64_t)ia * 2 * npp, *deb = q.deb + (int64_t)ib * 2 * npp;
#pragma unroll
      for (int j = 0; j < J; j++) {
        const int c = gl + j * G;
        if (!rok || c >= L) continue;
        const int Jp = c >> lw, v = c & ((1 << lw) - 1);
        T s = T(0);
        for (int e = p.ps_off[Jp]; e < p.ps_off[Jp + 1]; e++) {
          const int code = p.ps_code[e];
          const int Ip = code & 255, y = (code >> 8) & 1, prs = code >> 10;
          const T de = dea[y * npp + prs] + deb[y * npp + prs];
          const T t = q.ps_h[e] + ((code >> 9) & 1 ? -cf : cf) * de;
          s += t * srow[(Ip << lw) + v];
        }
        for (int e = p.pd_off[Jp]; e < p.pd_off[Jp + 1]; e++) s += q.pd_h[e] * srow[(p.pd_I[e] << lw) + v];
        acc[j] += s;
      }
      __syncwarp();
    }
    // electron singles (spin x): same-species element, electron-single x
    // positron-diagonal and electron-single x positron-single cross terms
#pragma unroll 1
    for (int x = 0; x < 2; x++) {
      const int nmax = x == 0 ? a1n : b1max;
      for (int t0 = 0; t0 < nmax; t0 += G) {
        const int t = t0 + gl;
        int Jr = -1;
        T val = T(0);
        int ph = 0, ng = 0;
        if (x == 0 && t < a1n && rok) {
          const int64_t e = a1b + t;
          const int info = p.a1_info[e];
          ph = info >> 1;
          ng = info & 1;
          T f = q.a1F[e];
          const T *er = q.eab + (int64_t)ph * npe;
          for (uint64_t m = bmask; m; m &= m - 1) f += er[pairdiag(__ffsll((long long)m) - 1)];
          val = ng ? -f : f;
          Jr = p.a1_J[e] * nb + ib;
        } else if (x == 1 && t < b1n) {
          const int64_t e = b1b + t;
          const int info = p.b1_info[e];
          ph = info >> 1;
          ng = info & 1;
          T f = q.b1F[e];
          for (uint64_t m = amask; m; m &= m - 1) f += q.eab[(int64_t)pairdiag(__ffsll((long long)m) - 1) * npe + ph];
          val = ng ? -f : f;
          Jr = rowa + p.b1_J[e];
        }
        const int cnt = min(G, nmax - t0);
        if (P == 1) {
#pragma unroll 4
          for (int i = 0; i < cnt; i++) {
            const int Ji = __shfl_sync(0xffffffffu, Jr, i, G);
            const T vi = __shfl_sync(0xffffffffu, val, i, G);
            if (Ji >= 0) {
              const T *xr = X + (int64_t)Ji * L;
#pragma unroll
              for (int j = 0; j < J; j++) {
                const int c = gl + j * G;
                if (c < L) acc[j] += vi * xr[c];
              }
            }
          }
        } else {
          for (int i = 0; i < cnt; i++) {
            const int Ji = __shfl_sync(0xffffffffu, Jr, i, G);
            const T vi = __shfl_sync(0xffffffffu, val, i, G);
            const int phi = __shfl_sync(0xffffffffu, ph, i, G);
            const int ngi = __shfl_sync(0xffffffffu, ng, i, G);
            const T *xr = X + (int64_t)(Ji >= 0 ? Ji : 0) * L;
            T xv[J];
#pragma unroll
            for (int j = 0; j < J; j++) {
              const int c = gl + j * G;
              xv[j] = (Ji >= 0 && c < L) ? xr[c] : T(0);
              if (c < L) srow[c] = xv[j];
            }
            __syncwarp();
            if (Ji >= 0) {
              const T sc = ngi ? -cf : cf;
              const T *dpt = q.dpt + ((int64_t)x * npe + phi) * P;
              const T *mt = q.mtab + ((int64_t)x * npe + phi) * p.nps;
#pragma unroll
              for (int j = 0; j < J; j++) {
                const int c = gl + j * G;
                if (c >= L) continue;
                const int Jp = c >> lw, v = c & ((1 << lw) - 1);
                T s = vi * xv[j];
                T t = dpt[Jp] * xv[j];
                for (int e = p.ps_off[Jp]; e < p.ps_off[Jp + 1]; e++) t += mt[e] * srow[((p.ps_code[e] & 255) << lw) + v];
                acc[j] += s + sc * t;
              }
            }
            __syncwarp();
          }
        }
      }
    }
    // same-spin doubles
#pragma unroll 1
    for (int x = 0; x < 2; x++) {
      const int nmax = x == 0 ? a2n : b2max;
      for (int t0 = 0; t0 < nmax; t0 += G) {
        const int t = t0 + gl;
        int Jr = -1;
        T val = T(0);
        if (x == 0 && t < a2n && rok) {
          val = q.a2D[a2b + t];
          Jr = p.a2_J[a2b + t] * nb + ib;
        } else if (x == 1 && t < b2n) {
          val = q.b2D[b2b + t];
          Jr = rowa + p.b2_J[b2b + t];
        }
        const int cnt = min(G, nmax - t0);
#pragma unroll 4
        for (int i = 0; i < cnt; i++) {
          const int Ji = __shfl_sync(0xffffffffu, Jr, i, G);
          const T vi = __shfl_sync(0xffffffffu, val, i, G);
          if (Ji >= 0) {
            const T *xr = X + (int64_t)Ji * L;
#pragma unroll
            for (int j = 0; j < J; j++) {
              const int c = gl + j * G;
              if (c < L) acc[j] += vi * xr[c];
            }
          }
        }
      }
    }
    // opposite-spin doubles: alpha single x beta single
#pragma unroll 1
    for (int s = 0; s < a1n; s++) {
      const int64_t ea = a1b + s;
      const int infa = p.a1_info[ea];
      const int rowj = p.a1_J[ea] * nb;
      const T *erow = q.eab + (int64_t)(infa >> 1) * npe;
      for (int t0 = 0; t0 < b1max; t0 += G) {
        const int t = t0 + gl;
        int Jr = -1;
        T val = T(0);
        if (t < b1n) {
          const int infb = p.b1_info[b1b + t];
          const T v = erow[infb >> 1];
          val = ((infa ^ infb) & 1) ? -v : v;
          Jr = rowj + p.b1_J[b1b + t];
        }
        const int cnt = min(G, b1max - t0);
#pragma unroll 4
        for (int i = 0; i < cnt; i++) {
          const int Ji = __shfl_sync(0xffffffffu, Jr, i, G);
          const T vi = __shfl_sync(0xffffffffu, val, i, G);
          if (Ji >= 0) {
            const T *xr = X + (int64_t)Ji * L;
#pragma unroll
            for (int j = 0; j < J; j++) {
              const int c = gl + j * G;
              if (c < L) acc[j] += vi * xr[c];
            }
          }
        }
      }
    }
    {
      T *yr = Y + (int64_t)Ie * L;
#pragma unroll
      for (int j = 0; j < J; j++) {
        const int c = gl + j * G;
        if (rok && c < L) yr[c] = acc[j];
      }
    }
    __syncwarp();
  }
}

// Narrow rows (L = P * w <= 16 values): one lane per row, so 32 rows of the
// unit advance together.  The alpha-side connections are warp-uniform (same
// alpha string) and their partner rows (Ja, Ib..Ib+31) are consecutive in
// memory; the beta-side and alpha-beta connections are per lane.  Positron and
// cross terms use the lane's own staging slot (no cross-lane traffic).
template <typename T, int LV>
__device__ void do_rows_lane(const Prob &p, const Call &cl, const Unit &U, T *stg, int lane) {
  const ProbT<T> &q = pt<T>(p);
  const int P = p.P, lw = cl.lw, L = P << lw;
  const T *__restrict__ X = (const T *)cl.X;
  T *__restrict__ Y = (T *)cl.Y;
  const int ia = U.ia, nb = p.nb, npe = p.npe, npp = p.npp;
  const int64_t a1b = p.a1_off[ia];
  const int a1n = (int)(p.a1_off[ia + 1] - a1b);
  const int64_t a2b = p.a2_off[ia];
  const int a2n = (int)(p.a2_off[ia + 1] - a2b);
  const uint64_t amask = p.astr[ia];
  const T cf = (T)p.cf;
  const int rowa = ia * nb;
  T *slot = stg + lane * LV;  // this lane's staging slot
  for (int r0 = 0; r0 < U.nrows; r0 += 32) {
    const bool rok = r0 + lane < U.nrows;
    const int ib = rok ? U.b0 + r0 + lane : U.b0;
    const int Ie = rowa + ib;
    const int64_t b1b = p.b1_off[ib];
    const int b1n = rok ? (int)(p.b1_off[ib + 1] - b1b) : 0;
    const int64_t b2b = p.b2_off[ib];
    const int b2n = rok ? (int)(p.b2_off[ib + 1] - b2b) : 0;
    const uint64_t bmask = p.bstr[ib];
    T acc[LV];
    {
      const T *xr = X + (int64_t)Ie * L;
      const double *dg = p.diag + (int64_t)Ie * P;
#pragma unroll
      for (int c = 0; c < LV; c++) {
        acc[c] = T(0);
        if (c < L) {
          const T x = xr[c];
          acc[c] = (T)(dg[c >> lw] - cl.shift) * x;
          if (P > 1) slot[c] = x;
        }
      }
    }
    if (P > 1) {
      const T *dea = q.dea + (int64_t)ia * 2 * npp, *deb = q.deb + (int64_t)ib * 2 * npp;
#pragma unroll
      for (int c = 0; c < LV; c++) {
        if (c >= L) continue;
        const int Jp = c >> lw, v = c & ((1 << lw) - 1);
        T s = T(0);
        for (int e = p.ps_off[Jp]; e < p.ps_off[Jp + 1]; e++) {
          const int code = p.ps_code[e];
          const int Ip = code & 255, y = (code >> 8) & 1, prs = code >> 10;
          const T de = dea[y * npp + prs] + deb[y * npp + prs];
          const T t = q.ps_h[e] + ((code >> 9) & 1 ? -cf : cf) * de;
          s += t * slot[(Ip << lw) + v];
        }
        for (int e = p.pd_off[Jp]; e < p.pd_off[Jp + 1]; e++) s += q.pd_h[e] * slot[(p.pd_I[e] << lw) + v];
        acc[c] += s;
      }
    }
    // electron singles
#pragma unroll 1
    for (int x = 0; x < 2; x++) {
      const int n1 = x == 0 ? a1n : b1n;
      for (int t = 0; t < n1; t++) {
        int info, Jr;
        T f;
        if (x == 0) {
          const int64_t e = a1b + t;
          info = p.a1_info[e];
          f = q.a1F[e];
          const T *er = q.eab + (int64_t)(info >> 1) * npe;
          for (uint64_t m = bmask; m; m &= m - 1) f += er[pairdiag(__ffsll((long long)m) - 1)];
          Jr = p.a1_J[e] * nb + ib;
        } else {
          const int64_t e = b1b + t;
          info = p.b1_info[e];
          f = q.b1F[e];
          for (uint64_t m = amask; m; m &= m - 1)
            f += q.eab[(int64_t)pairdiag(__ffsll((long long)m) - 1) * npe + (info >> 1)];
          Jr = rowa + p.b1_J[e];
        }
        const T val = (info & 1) ? -f : f;
        const T *xr = X + (int64_t)Jr * L;
        if (P == 1) {
#pragma unroll
          for (int c = 0; c < LV; c++)
            if (c < L) acc[c] += val * xr[c];
        } else {
          const int ph = info >> 1;
          const T sc = (info & 1) ? -cf : cf;
          T xv[LV];
#pragma unroll
          for (int c = 0; c < LV; c++) {
            xv[c] = c < L ? xr[c] : T(0);
            if (c < L) slot[c] = xv[c];
          }
          const T *dpt = q.dpt + ((int64_t)x * npe + ph) * P;
          const T *mt = q.mtab + ((int64_t)x * npe + ph) * p.nps;
#pragma unroll
          for (int c = 0; c < LV; c++) {
            if (c >= L) continue;
            const int Jp = c >> lw, v = c & ((1 << lw) - 1);
            T t = dpt[Jp] * xv[c];
            for (int e = p.ps_off[Jp]; e < p.ps_off[Jp + 1]; e++) t += mt[e] * slot[((p.ps_code[e] & 255) << lw) + v];
            acc[c] += val * xv[c] + sc * t;
          }
        }
      }
    }
    // same-spin doubles
#pragma unroll 1
    for (int x = 0; x < 2; x++) {
      const int n2 = x == 0 ? a2n : b2n;
#pragma unroll 2
      for (int t = 0; t < n2; t++) {
        T val;
        int Jr;
        if (x == 0) {
          val = q.a2D[a2b + t];
          Jr = p.a2_J[a2b + t] * nb + ib;
        } else {
          val = q.b2D[b2b + t];
          Jr = rowa + p.b2_J[b2b + t];
        }
        const T *xr = X + (int64_t)Jr * L;
#pragma unroll
        for (int c = 0; c < LV; c++)
          if (c < L) acc[c] += val * xr[c];
      }
    }
    // opposite-spin doubles
#pragma unroll 1
    for (int s = 0; s < a1n; s++) {
      const int64_t ea = a1b + s;
      const int infa = p.a1_info[ea];
      const int rowj = p.a1_J[ea] * nb;
      const T *erow = q.eab + (int64_t)(infa >> 1) * npe;
#pragma unroll 2
      for (int t = 0; t < b1n; t++) {
        const int infb = p.b1_info[b1b + t];
        const T v = erow[infb >> 1];
        const T val = ((infa ^ infb) & 1) ? -v : v;
        const T *xr = X + (int64_t)(rowj + p.b1_J[b1b + t]) * L;
#pragma unroll
        for (int c = 0; c < LV; c++)
          if (c < L) acc[c] += val * xr[c];
      }
    }
    if (rok) {
      T *yr = Y + (int64_t)Ie * L;
#pragma unroll
      for (int c = 0; c < LV; c++)
        if (c < L) yr[c] = acc[c];
    }
  }
}

template <typename T>
__device__ __forceinline__ void do_unit(const Prob &p, const Call &cl, const Unit &U, T *stg, int lane) {
  const int L = p.P << cl.lw;
  if (cl.lane_rows) {
    if (L <= 4)
      do_rows_lane<T, 4>(p, cl, U, stg, lane);
    else if (L <= 8)
      do_rows_lane<T, 8>(p, cl, U, stg, lane);
    else
      do_rows_lane<T, 16>(p, cl, U, stg, lane);
    return;
  }
  const int G = L >= 32 ? 32 : (L <= 1 ? 1 : 1 << (32 - __clz(L - 1)));
  switch ((L + G - 1) / G) {
    case 1: do_rows<T, 1>(p, cl, U, stg, lane, G); break;
    case 2: do_rows<T, 2>(p, cl, U, stg, lane, G); break;
    case 3: do_rows<T, 3>(p, cl, U, stg, lane, G); break;
    case 4: do_rows<T, 4>(p, cl, U, stg, lane, G); break;
    default: do_rows<T, JMAX>(p, cl, U, stg, lane, G); break;
  }
}

__global__ void __launch_bounds__(256, 3) batch_sigma_kernel(const Prob *__restrict__ probs,
                                                          const Call *__restrict__ calls,
                                                          const Unit *__restrict__ units, int n_units,
                                                          unsigned *counter) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned char *stg = smem + (size_t)warp * STAGE * sizeof(double);
  for (;;) {
    unsigned u = 0;
    if (lane == 0) u = atomicAdd(counter, 1u);
    u = __shfl_sync(0xffffffffu, u, 0);
    if (u >= (unsigned)n_units) break;
    const Unit U = units[u];
    const Call cl = calls[U.prob];
    if (!cl.active) continue;
    if (cl.precision == PQ_FP64)
      do_unit<double>(probs[U.prob], cl, U, (double *)stg, lane);
    else
      do_unit<float>(probs[U.prob], cl, U, (float *)stg, lane);
  }
}

// column-major FP64 -> interleaved work vector of each active problem
__global__ void batch_to_il_kernel(const Chunk *__restrict__ chunks, const Call *__restrict__ calls,
                                   const Prob *__restrict__ probs) {
  const Chunk ck = chunks[blockIdx.x];
  const Call cl = calls[ck.prob];
  if (!cl.active) return;
  const int64_t n = probs[ck.prob].n_dets;
  const int w = 1 << cl.lw;
  for (int64_t d = ck.d0 + threadIdx.x; d < ck.d1; d += blockDim.x)
    for (int v = 0; v < w; v++) {
      const double x = v < cl.cnt ? cl.src[v * n + d] : 0.0;
      if (cl.precision == PQ_FP64)
        ((double *)cl.X)[d * w + v] = x;
      else
        ((float *)cl.X)[d * w + v] = (float)x;
    }
}

// interleaved result -> column-major FP64 (FP32 results get shift * src added)
__global__ void batch_from_il_kernel(const Chunk *__restrict__ chunks, const Call *__restrict__ calls,
                                     const Prob *__restrict__ probs) {
  const Chunk ck = chunks[blockIdx.x];
  const Call cl = calls[ck.prob];
  if (!cl.active) return;
  const int64_t n = probs[ck.prob].n_dets;
  const int w = 1 << cl.lw;
  for (int64_t d = ck.d0 + threadIdx.x; d < ck.d1; d += blockDim.x)
    for (int v = 0; v < cl.cnt; v++) {
      if (cl.precision == PQ_FP64)
        cl.dst[v * n + d] = ((const double *)cl.Y)[d * w + v];
      else
        cl.dst[v * n + d] = (double)((const float *)cl.Y)[d * w + v] + cl.shift * cl.src[v * n + d];
    }
}

constexpr int64_t CHUNK_DETS = 1 << 16;

}  // namespace batch
}  // namespace pq

using namespace pq;
using namespace pq::batch;

// Device copies of the per-problem tables that the batched kernel needs beyond
// the problem's own handle.
struct BatchTables {
  DevBuf ps_off, ps_code, pd_off, pd_I;
  DevBuf ps_h64, ps_h32, pd_h64, pd_h32, dpt64, dpt32, dea64, dea32, deb64, deb32, mt64, mt32;
};

struct BatchPlan {
  std::vector<int> members;
  DevBuf units, chunks;
  int n_units = 0, n_chunks = 0;
  int warps = 8, blocks = 0;
  cudaGraphExec_t graph = nullptr;
  ~BatchPlan() {
    if (graph) cudaGraphExecDestroy(graph);
  }
};

struct pq_ci_batch {
  cudaStream_t stream = nullptr;
  bool own_stream = false;  // created here because the caller passed the legacy default stream
  std::vector<pq_ci_handle *> h;
  std::vector<std::unique_ptr<BatchTables>> tabs;
  std::vector<Prob> prob;
  DevBuf d_prob, d_calls, d_counter;
  Call *h_calls = nullptr;  // pinned
  int wmax = 4;             // widest interleaved block per problem and launch
  // launch shape picked by the autotuner (0: not tuned yet)
  int tuned_warps = 0, tuned_rows = 0;
  std::unique_ptr<BatchPlan> all;  // plan over every problem (pq_ci_batch_sigma)
  ~pq_ci_batch() {
    if (stream) cudaStreamSynchronize(stream);
    all.reset();
    for (auto *x : h) delete x;
    if (h_calls) cudaFreeHost(h_calls);
    if (own_stream) cudaStreamDestroy(stream);
  }
};

namespace pq {
namespace {

int idx2h(int i, int j) { return i > j ? i * (i + 1) / 2 + j : j * (j + 1) / 2 + i; }
int between(uint64_t m, int lo, int hi) {
  int c = 0;
  for (int o = lo + 1; o < hi; o++) c += (int)((m >> o) & 1ULL);
  return c;
}

template <typename T> const T *dptr(const DevBuf &b) { return b.ptr ? b.as<T>() : nullptr; }

// True when the handle's determinant list is the full product described at
// the top of this file; P receives the species-1 block size (1 for one species).
bool full_product(const pq_ci_handle *h, int *P) {
  const int64_t na = (int64_t)h->str[0][0].size(), nb = (int64_t)h->str[0][1].size();
  if (h->n_species == 1) {
    *P = 1;
    return h->full && h->n_dets == na * nb;
  }
  const int64_t pa = (int64_t)h->str[1][0].size(), pb = (int64_t)h->str[1][1].size();
  *P = (int)(pa * pb);
  if (h->n_dets != na * nb * pa * pb) return false;
  if ((int64_t)h->e_a.size() != na * nb) return false;
  for (size_t ie = 0; ie < h->ebase.size(); ie++)
    if (h->ebase[ie] != (int64_t)ie * pa * pb) return false;
  return true;
}

template <typename T> pq_status upload_pair(DevBuf &b64, DevBuf &b32, const std::vector<T> &v, cudaStream_t st) {
  std::vector<float> f(v.begin(), v.end());
  PQ_TRY(upload(b64, v, st));
  PQ_TRY(upload(b32, f, st));
  return PQ_OK;
}

// Species-1 operator tables of a two-species full-product problem, on the host
// in FP64 from the caller's integrals (valid only while the batch is created).
pq_status build_positron_tables(pq_ci_handle *h, BatchTables &bt, Prob &pr, cudaStream_t st) {
  const pq_ci_desc &d = h->desc;
  const int n = d.n_orb[1], npp = h->npair[1], npe = h->npair[0], ne = d.n_orb[0];
  const int nb1 = h->n_blocks[1], nb0 = h->n_blocks[0];
  const std::vector<uint64_t> &SA = h->str[1][0], &SB = h->str[1][1];
  const int na1 = (int)SA.size(), nbb1 = (int)SB.size(), P = na1 * nbb1;
  auto h1 = [&](int y, int i, int j) { return d.h1[1][y % nb1][i + (int64_t)j * n]; };
  auto E = [&](int y0, int y1, int P0, int P1) {
    const int b0 = y0 % nb1, b1 = y1 % nb1;
    if (b0 <= b1) return d.eri[1][b0][1][b1][P0 + (int64_t)P1 * npp];
    return d.eri[1][b1][1][b0][P1 + (int64_t)P0 * npp];
  };
  auto EP = [&](int x, int y, int Pe, int Pp) { return d.eri[0][x % nb0][1][y % nb1][Pe + (int64_t)Pp * npe]; };
  auto find = [](const std::vector<uint64_t> &S, uint64_t m) {
    for (size_t i = 0; i < S.size(); i++)
      if (S[i] == m) return (int)i;
    return -1;
  };
  std::vector<int32_t> ps_off(P + 1, 0), pd_off(P + 1, 0), ps_code, pd_I;
  std::vector<double> ps_h, pd_h;
  for (int Jp = 0; Jp < P; Jp++) {
    const int ja = Jp / nbb1, jb = Jp % nbb1;
    const uint64_t m[2] = {SA[ja], SB[jb]};
    // singles of spin y: hole hh occupied in the string of Jp, particle pp empty
    for (int y = 0; y < 2; y++) {
      for (int hh = 0; hh < n; hh++) {
        if (!((m[y] >> hh) & 1ULL)) continue;
        for (int pp = 0; pp < n; pp++) {
          if ((m[y] >> pp) & 1ULL) continue;
          const uint64_t km = m[y] ^ (1ULL << hh) ^ (1ULL << pp);
          const int k = find(y == 0 ? SA : SB, km);
          if (k < 0) continue;
          const int Ip = y == 0 ? k * nbb1 + jb : ja * nbb1 + k;
          const int lo = std::min(hh, pp), hi = std::max(hh, pp);
          const int neg = between(m[y], lo, hi) & 1;
          const int php = idx2h(hh, pp);
          double f = h1(y, hh, pp);
          for (int kk = 0; kk < n; kk++) {
            if ((m[y] >> kk) & 1ULL) f += E(y, y, php, idx2h(kk, kk)) - E(y, y, idx2h(hh, kk), idx2h(kk, pp));
            if ((m[1 - y] >> kk) & 1ULL) f += E(y, 1 - y, php, idx2h(kk, kk));
          }
          ps_code.push_back(Ip | (y << 8) | (neg << 9) | (php << 10));
          ps_h.push_back(neg ? -f : f);
        }
      }
    }
    ps_off[Jp + 1] = (int32_t)ps_code.size();
    // same-spin doubles
    for (int y = 0; y < 2; y++) {
      for (int h0 = 0; h0 < n; h0++)
        for (int h1_ = h0 + 1; h1_ < n; h1_++) {
          if (!((m[y] >> h0) & 1ULL) || !((m[y] >> h1_) & 1ULL)) continue;
          for (int p0 = 0; p0 < n; p0++)
            for (int p1 = p0 + 1; p1 < n; p1++) {
              if (((m[y] >> p0) & 1ULL) || ((m[y] >> p1) & 1ULL)) continue;
              const uint64_t km = m[y] ^ (1ULL << h0) ^ (1ULL << h1_) ^ (1ULL << p0) ^ (1ULL << p1);
              const int k = find(y == 0 ? SA : SB, km);
              if (k < 0) continue;
              const int Ip = y == 0 ? k * nbb1 + jb : ja * nbb1 + k;
              const int a0 = std::min(h0, p0), b0 = std::max(h0, p0), a1 = std::min(h1_, p1), b1 = std::max(h1_, p1);
              int nperm = between(m[y], a0, b0) + between(m[y], a1, b1);
              if (a0 < a1 && a1 < b0 && b0 < b1) nperm++;
              const double v = E(y, y, idx2h(h0, p0), idx2h(h1_, p1)) - E(y, y, idx2h(h0, p1), idx2h(h1_, p0));
              pd_I.push_back(Ip);
              pd_h.push_back((nperm & 1) ? -v : v);
            }
        }
    }
    // opposite-spin doubles
    for (int ha = 0; ha < n; ha++) {
      if (!((m[0] >> ha) & 1ULL)) continue;
      for (int pa = 0; pa < n; pa++) {
        if ((m[0] >> pa) & 1ULL) continue;
        const int ka = find(SA, m[0] ^ (1ULL << ha) ^ (1ULL << pa));
        if (ka < 0) continue;
        const int sa = between(m[0], std::min(ha, pa), std::max(ha, pa)) & 1;
        for (int hb = 0; hb < n; hb++) {
          if (!((m[1] >> hb) & 1ULL)) continue;
          for (int pb = 0; pb < n; pb++) {
            if ((m[1] >> pb) & 1ULL) continue;
            const int kb = find(SB, m[1] ^ (1ULL << hb) ^ (1ULL << pb));
            if (kb < 0) continue;
            const int sb = between(m[1], std::min(hb, pb), std::max(hb, pb)) & 1;
            const double v = E(0, 1, idx2h(ha, pa), idx2h(hb, pb));
            pd_I.push_back(ka * nbb1 + kb);
            pd_h.push_back(((sa ^ sb) & 1) ? -v : v);
          }
        }
      }
    }
    pd_off[Jp + 1] = (int32_t)pd_I.size();
  }
  // electron-single x positron-diagonal: dpt[x][pair_e][Jp]
  std::vector<double> dpt((size_t)2 * npe * P, 0.0);
  for (int x = 0; x < 2; x++)
    for (int pe = 0; pe < npe; pe++)
      for (int Jp = 0; Jp < P; Jp++) {
        const uint64_t m[2] = {SA[Jp / nbb1], SB[Jp % nbb1]};
        double s = 0.0;
        for (int y = 0; y < 2; y++)
          for (int r = 0; r < n; r++)
            if ((m[y] >> r) & 1ULL) s += EP(x, y, pe, idx2h(r, r));
        dpt[((size_t)x * npe + pe) * P + Jp] = s;
      }
  // electron-diagonal x positron-single: de[I][y][pair_p] per electron string
  auto de_table = [&](const std::vector<uint64_t> &S, int x) {
    std::vector<double> t(S.size() * 2 * npp, 0.0);
    for (size_t I = 0; I < S.size(); I++)
      for (int y = 0; y < 2; y++)
        for (int pq = 0; pq < npp; pq++) {
          double s = 0.0;
          for (int o = 0; o < ne; o++)
            if ((S[I] >> o) & 1ULL) s += EP(x, y, idx2h(o, o), pq);
          t[(I * 2 + y) * npp + pq] = s;
        }
    return t;
  };
  std::vector<double> dea = de_table(h->str[0][0], 0), deb = de_table(h->str[0][1], 1);
  // electron-single x positron-single coefficients per (electron spin, electron pair, positron entry)
  const int nps = (int)ps_code.size();
  std::vector<double> mtab((size_t)2 * npe * std::max(nps, 1), 0.0);
  for (int x = 0; x < 2; x++)
    for (int pe = 0; pe < npe; pe++)
      for (int e = 0; e < nps; e++) {
        const int code = ps_code[e];
        const double v = EP(x, (code >> 8) & 1, pe, code >> 10);
        mtab[((size_t)x * npe + pe) * nps + e] = ((code >> 9) & 1) ? -v : v;
      }
  if (ps_code.empty()) ps_code.push_back(0), ps_h.push_back(0.0);
  if (pd_I.empty()) pd_I.push_back(0), pd_h.push_back(0.0);
  PQ_TRY(upload(bt.ps_off, ps_off, st));
  PQ_TRY(upload(bt.pd_off, pd_off, st));
  PQ_TRY(upload(bt.ps_code, ps_code, st));
  PQ_TRY(upload(bt.pd_I, pd_I, st));
  PQ_TRY(upload_pair(bt.ps_h64, bt.ps_h32, ps_h, st));
  PQ_TRY(upload_pair(bt.pd_h64, bt.pd_h32, pd_h, st));
  PQ_TRY(upload_pair(bt.dpt64, bt.dpt32, dpt, st));
  PQ_TRY(upload_pair(bt.dea64, bt.dea32, dea, st));
  PQ_TRY(upload_pair(bt.deb64, bt.deb32, deb, st));
  PQ_TRY(upload_pair(bt.mt64, bt.mt32, mtab, st));
  PQ_CUDA_TRY(cudaStreamSynchronize(st));  // host vectors go out of scope
  pr.ps_off = bt.ps_off.as<int32_t>();
  pr.ps_code = bt.ps_code.as<int32_t>();
  pr.pd_off = bt.pd_off.as<int32_t>();
  pr.pd_I = bt.pd_I.as<int32_t>();
  pr.d.ps_h = bt.ps_h64.as<double>();
  pr.f.ps_h = bt.ps_h32.as<float>();
  pr.d.pd_h = bt.pd_h64.as<double>();
  pr.f.pd_h = bt.pd_h32.as<float>();
  pr.d.dpt = bt.dpt64.as<double>();
  pr.f.dpt = bt.dpt32.as<float>();
  pr.d.dea = bt.dea64.as<double>();
  pr.f.dea = bt.dea32.as<float>();
  pr.d.deb = bt.deb64.as<double>();
  pr.f.deb = bt.deb32.as<float>();
  pr.d.mtab = bt.mt64.as<double>();
  pr.f.mtab = bt.mt32.as<float>();
  pr.nps = nps;
  for (int x = 0; x < 2; x++)
    for (int y = 0; y < 2; y++) {
      pr.d.ep[x][y] = h->d_ep64[x][y].as<double>();
      pr.f.ep[x][y] = h->d_ep32[x][y].as<float>();
    }
  pr.npp = npp;
  pr.cf = d.charge[0] * d.charge[1];
  return PQ_OK;
}

pq_status make_prob(pq_ci_handle *h, BatchTables &bt, Prob &pr, cudaStream_t st) {
  int P = 1;
  if (!full_product(h, &P)) {
    set_error("pq_ci_batch: every problem must be a full product of complete string spaces (full CI per species)");
    return PQ_ERR_ARG;
  }
  if (P > MAX_P) {
    set_error("pq_ci_batch: %d species-1 determinants exceed the batched kernel's limit of %d", P, MAX_P);
    return PQ_ERR_ARG;
  }
  if (h->wide) {
    set_error("pq_ci_batch: batched problems hold at most 64 orbitals per species (one-word strings)");
    return PQ_ERR_ARG;
  }
  pr = Prob{};
  const SpinTablesDev &A = h->tab[0][0], &B = h->tab[0][1];
  pr.astr = A.str.as<uint64_t>();
  pr.bstr = B.str.as<uint64_t>();
  pr.a1_off = A.s1_off.as<int64_t>();
  pr.b1_off = B.s1_off.as<int64_t>();
  pr.a2_off = A.s2_off.as<int64_t>();
  pr.b2_off = B.s2_off.as<int64_t>();
  pr.a1_J = A.s1_J.as<int32_t>();
  pr.a1_info = A.s1_info.as<int32_t>();
  pr.b1_J = B.s1_J.as<int32_t>();
  pr.b1_info = B.s1_info.as<int32_t>();
  pr.a2_J = A.s2_J.as<int32_t>();
  pr.b2_J = B.s2_J.as<int32_t>();
  pr.d.a1F = A.s1_F64.as<double>();
  pr.f.a1F = A.s1_F32.as<float>();
  pr.d.b1F = B.s1_F64.as<double>();
  pr.f.b1F = B.s1_F32.as<float>();
  pr.d.a2D = A.s2_D64.as<double>();
  pr.f.a2D = A.s2_D32.as<float>();
  pr.d.b2D = B.s2_D64.as<double>();
  pr.f.b2D = B.s2_D32.as<float>();
  if (h->n_species == 1) {
    pr.d.eab = h->d_eab64.as<double>();
    pr.f.eab = h->d_eab32.as<float>();
  } else {
    pr.d.eab = h->d_eabs64[0].as<double>();
    pr.f.eab = h->d_eabs32[0].as<float>();
  }
  pr.diag = h->d_diag.as<double>();
  pr.n_dets = h->n_dets;
  pr.na = (int)h->str[0][0].size();
  pr.nb = (int)h->str[0][1].size();
  pr.npe = h->npair[0];
  pr.P = P;
  pr.cf = 0.0;
  if (h->n_species == 2 && P > 1) PQ_TRY(build_positron_tables(h, bt, pr, st));
  return PQ_OK;
}

// estimated cost of one determinant row of a problem (connections x row width)
double row_cost(const pq_ci_handle *h, const Prob &pr, int w) {
  const SpinTablesDev &A = h->tab[0][0], &B = h->tab[0][1];
  const double na = (double)std::max<int64_t>(1, A.n_str), nb = (double)std::max<int64_t>(1, B.n_str);
  const double s1a = A.n1 / na, s1b = B.n1 / nb, s2a = A.n2 / na, s2b = B.n2 / nb;
  const double conn = 1.0 + s1a + s1b + s2a + s2b + s1a * s1b;
  const double L = (double)pr.P * w;
  return conn * std::max(L, 8.0) + (pr.P > 1 ? (s1a + s1b) * L * 10.0 : 0.0);
}

// one lane per determinant row when the widest row of the problem is narrow
int lane_rows(const pq_ci_batch *B, int pi) { return B->prob[pi].P * B->wmax <= LANE_MAXL ? 1 : 0; }

// Work units of a group: rows (ia, b0 .. b0 + nrows) in descending cost order.
pq_status make_plan(pq_ci_batch *B, const std::vector<int> &members, int warps, int rows_mult, BatchPlan &pl) {
  struct U {
    double cost;
    Unit u;
  };
  std::vector<U> us;
  std::vector<Chunk> ch;
  for (int pi : members) {
    const Prob &pr = B->prob[pi];
    const int L = pr.P * B->wmax;
    const int G = L >= 32 ? 32 : (L <= 1 ? 1 : 1 << (32 - __builtin_clz((unsigned)(L - 1))));
    const int nrows = (lane_rows(B, pi) ? 32 : 32 / G) * rows_mult;
    const double rc = row_cost(B->h[pi], pr, B->wmax);
    for (int ia = 0; ia < pr.na; ia++)
      for (int b0 = 0; b0 < pr.nb; b0 += nrows) {
        const int nr = std::min(nrows, pr.nb - b0);
        us.push_back({rc * nr, Unit{pi, ia, b0, nr}});
      }
    for (int64_t d0 = 0; d0 < pr.n_dets; d0 += CHUNK_DETS) ch.push_back(Chunk{pi, d0, std::min(pr.n_dets, d0 + CHUNK_DETS)});
  }
  std::stable_sort(us.begin(), us.end(), [](const U &a, const U &b) { return a.cost > b.cost; });
  std::vector<Unit> uv(us.size());
  for (size_t i = 0; i < us.size(); i++) uv[i] = us[i].u;
  if (uv.size() > 0x7fffffff || ch.size() > 0x7fffffff) {
    set_error("pq_ci_batch: too many work units");
    return PQ_ERR_ARG;
  }
  pl.members = members;
  pl.n_units = (int)uv.size();
  pl.n_chunks = (int)ch.size();
  PQ_TRY(upload(pl.units, uv, B->stream));
  PQ_TRY(upload(pl.chunks, ch, B->stream));
  pl.warps = warps;
  const size_t smem = (size_t)warps * STAGE * sizeof(double);
  int per_sm = 0;
  PQ_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_sigma_kernel, warps * 32, smem));
  int dev = 0, sms = 0;
  PQ_CUDA_TRY(cudaGetDevice(&dev));
  PQ_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  pl.blocks = std::max(1, per_sm) * sms;
  PQ_CUDA_TRY(cudaStreamSynchronize(B->stream));
  return PQ_OK;
}

pq_status launch_sigma(pq_ci_batch *B, const BatchPlan &pl, const Unit *units, int n_units) {
  PQ_CUDA_TRY(cudaMemsetAsync(B->d_counter.ptr, 0, sizeof(unsigned), B->stream));
  if (n_units > 0) {
    const size_t smem = (size_t)pl.warps * STAGE * sizeof(double);
    batch_sigma_kernel<<<pl.blocks, pl.warps * 32, smem, B->stream>>>(B->d_prob.as<Prob>(), B->d_calls.as<Call>(),
                                                                       units, n_units, B->d_counter.as<unsigned>());
    PQ_CUDA_TRY(cudaGetLastError());
  }
  return PQ_OK;
}

// the per-iteration sequence: call records, conversion in, sigma, conversion out
pq_status enqueue_step(pq_ci_batch *B, const BatchPlan &pl) {
  PQ_CUDA_TRY(cudaMemcpyAsync(B->d_calls.ptr, B->h_calls, sizeof(Call) * B->h.size(), cudaMemcpyHostToDevice,
                              B->stream));
  if (pl.n_chunks > 0) {
    batch_to_il_kernel<<<pl.n_chunks, 256, 0, B->stream>>>(pl.chunks.as<Chunk>(), B->d_calls.as<Call>(),
                                                            B->d_prob.as<Prob>());
    PQ_CUDA_TRY(cudaGetLastError());
  }
  PQ_TRY(launch_sigma(B, pl, pl.units.as<Unit>(), pl.n_units));
  if (pl.n_chunks > 0) {
    batch_from_il_kernel<<<pl.n_chunks, 256, 0, B->stream>>>(pl.chunks.as<Chunk>(), B->d_calls.as<Call>(),
                                                              B->d_prob.as<Prob>());
    PQ_CUDA_TRY(cudaGetLastError());
  }
  return PQ_OK;
}

// Run one step through the plan's CUDA graph (captured on first use).
pq_status run_step(pq_ci_batch *B, BatchPlan &pl) {
  if (!pl.graph) {
    cudaGraph_t g = nullptr;
    PQ_CUDA_TRY(cudaStreamBeginCapture(B->stream, cudaStreamCaptureModeThreadLocal));
    pq_status s = enqueue_step(B, pl);
    cudaError_t e = cudaStreamEndCapture(B->stream, &g);
    if (s != PQ_OK) {
      if (g) cudaGraphDestroy(g);
      return s;
    }
    PQ_CUDA_TRY(e);
    e = cudaGraphInstantiate(&pl.graph, g, 0);
    cudaGraphDestroy(g);
    PQ_CUDA_TRY(e);
  }
  PQ_CUDA_TRY(cudaGraphLaunch(pl.graph, B->stream));
  return PQ_OK;
}

// Ensure every member's work vectors hold n_dets x wmax values of the widest type.
pq_status ensure_work(pq_ci_batch *B, const std::vector<int> &members) {
  for (int pi : members) {
    pq_ci_handle *h = B->h[pi];
    const size_t bytes = sizeof(double) * (size_t)B->wmax * (size_t)(h->n_dets + 1);
    PQ_TRY(h->x_il.ensure(bytes));
    PQ_TRY(h->y_il.ensure(bytes));
  }
  return PQ_OK;
}

// Autotuner: time the sigma kernel for each launch shape on a strided sample of
// the group's work units (FP32, full width), keep the fastest.
pq_status autotune(pq_ci_batch *B, const std::vector<int> &members) {
  static const int cand[][2] = {{4, 1}, {8, 1}, {4, 2}, {8, 2}, {4, 4}, {8, 4}};
  PQ_TRY(ensure_work(B, members));
  for (size_t i = 0; i < B->h.size(); i++) B->h_calls[i] = Call{};
  for (int pi : members) {
    pq_ci_handle *h = B->h[pi];
    Call &c = B->h_calls[pi];
    c.active = 1;
    c.lane_rows = lane_rows(B, pi);
    c.precision = PQ_FP32;
    c.lw = B->wmax == 4 ? 2 : (B->wmax == 2 ? 1 : 0);
    c.cnt = B->wmax;
    c.X = h->x_il.ptr;
    c.Y = h->y_il.ptr;
    PQ_CUDA_TRY(cudaMemsetAsync(h->x_il.ptr, 0, sizeof(float) * (size_t)B->wmax * h->n_dets, B->stream));
  }
  PQ_CUDA_TRY(cudaMemcpyAsync(B->d_calls.ptr, B->h_calls, sizeof(Call) * B->h.size(), cudaMemcpyHostToDevice, B->stream));
  cudaEvent_t e0, e1;
  PQ_CUDA_TRY(cudaEventCreate(&e0));
  PQ_CUDA_TRY(cudaEventCreate(&e1));
  float best = 1e30f;
  int bw = 8, br = 1;
  for (auto &c : cand) {
    BatchPlan pl;
    pq_status s = make_plan(B, members, c[0], c[1], pl);
    if (s != PQ_OK) break;
    // strided sample of about 1/16 of the units (all of them when few)
    std::vector<Unit> all(pl.n_units), smp;
    PQ_CUDA_TRY(cudaMemcpy(all.data(), pl.units.ptr, sizeof(Unit) * pl.n_units, cudaMemcpyDeviceToHost));
    const int stride = pl.n_units > 65536 ? 16 : 1;
    for (int i = 0; i < pl.n_units; i += stride) smp.push_back(all[i]);
    DevBuf du;
    PQ_TRY(upload(du, smp, B->stream));
    PQ_TRY(launch_sigma(B, pl, du.as<Unit>(), (int)smp.size()));
    PQ_CUDA_TRY(cudaEventRecord(e0, B->stream));
    PQ_TRY(launch_sigma(B, pl, du.as<Unit>(), (int)smp.size()));
    PQ_CUDA_TRY(cudaEventRecord(e1, B->stream));
    PQ_CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0.f;
    PQ_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
    if (ms < best) best = ms, bw = c[0], br = c[1];
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  B->tuned_warps = bw;
  B->tuned_rows = br;
  return PQ_OK;
}

pq_status get_plan(pq_ci_batch *B, const std::vector<int> &members, std::unique_ptr<BatchPlan> &pl) {
  if (!B->tuned_warps) PQ_TRY(autotune(B, members));
  pl.reset(new BatchPlan());
  return make_plan(B, members, B->tuned_warps, B->tuned_rows, *pl);
}

int log2w(int c) { return c <= 1 ? 0 : (c <= 2 ? 1 : 2); }

}  // namespace
}  // namespace pq

extern "C" {

pq_status pq_ci_batch_create(const pq_ci_desc *descs, int32_t n, void *stream, pq_ci_batch **out) {
  clear_error();
  if (!descs || !out || n < 1) {
    set_error("pq_ci_batch_create: bad arguments (n=%d)", n);
    return PQ_ERR_ARG;
  }
  *out = nullptr;
  std::unique_ptr<pq_ci_batch> B(new (std::nothrow) pq_ci_batch());
  if (!B) {
    set_error("host allocation failed");
    return PQ_ERR_OOM;
  }
  // stream capture needs a stream other than the legacy default stream
  if (stream) {
    B->stream = (cudaStream_t)stream;
  } else {
    PQ_CUDA_TRY(cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking));
    B->own_stream = true;
  }
  for (int i = 0; i < n; i++) B->tabs.emplace_back(new BatchTables());
  B->prob.resize(n);
  for (int i = 0; i < n; i++) {
    pq_ci_handle *h = nullptr;
    pq_status s = pq_ci_create(&descs[i], B->stream, &h);
    if (s != PQ_OK) return s;
    B->h.push_back(h);
    s = make_prob(h, *B->tabs[i], B->prob[i], B->stream);
    if (s != PQ_OK) {
      set_error("problem %d: %s", i, pq_last_error());
      return s;
    }
  }
  PQ_TRY(upload(B->d_prob, B->prob, B->stream));
  PQ_TRY(B->d_calls.alloc(sizeof(Call) * n));
  PQ_TRY(B->d_counter.alloc(sizeof(unsigned) * 4));
  PQ_CUDA_TRY(cudaMallocHost(&B->h_calls, sizeof(Call) * n));
  for (int i = 0; i < n; i++) B->h_calls[i] = Call{};
  PQ_CUDA_TRY(cudaStreamSynchronize(B->stream));
  *out = B.release();
  return PQ_OK;
}

pq_status pq_ci_batch_destroy(pq_ci_batch *b) {
  delete b;
  return PQ_OK;
}

pq_status pq_ci_batch_num_dets(const pq_ci_batch *b, int32_t i, int64_t *n) {
  if (!b || !n || i < 0 || i >= (int32_t)b->h.size()) {
    set_error("pq_ci_batch_num_dets: bad arguments");
    return PQ_ERR_ARG;
  }
  *n = b->h[i]->n_dets;
  return PQ_OK;
}

pq_status pq_ci_batch_tuning(const pq_ci_batch *b, int32_t *warps_per_cta, int32_t *rows_per_unit) {
  if (!b) {
    set_error("pq_ci_batch_tuning: NULL batch");
    return PQ_ERR_ARG;
  }
  if (warps_per_cta) *warps_per_cta = b->tuned_warps;
  if (rows_per_unit) *rows_per_unit = b->tuned_rows;
  return PQ_OK;
}

pq_status pq_ci_batch_sigma(pq_ci_batch *b, const double *const *C, const int64_t *ldc, int32_t nvec,
                            double *const *S, const int64_t *lds, int32_t precision) {
  clear_error();
  if (!b || !C || !S || nvec < 1) {
    set_error("pq_ci_batch_sigma: bad arguments");
    return PQ_ERR_ARG;
  }
  if (precision != PQ_FP64 && precision != PQ_FP32) {
    set_error("pq_ci_batch_sigma: precision must be PQ_FP64 or PQ_FP32");
    return PQ_ERR_ARG;
  }
  const int n = (int)b->h.size();
  for (int i = 0; i < n; i++) {
    const int64_t nd = b->h[i]->n_dets;
    if (!C[i] || !S[i] || (ldc && ldc[i] != nd) || (lds && lds[i] != nd)) {
      set_error("pq_ci_batch_sigma: problem %d: vectors must be dense column-major with leading dimension n_dets", i);
      return PQ_ERR_ARG;
    }
  }
  if (b->own_stream) PQ_CUDA_TRY(cudaDeviceSynchronize());  // order after the caller's work
  std::vector<int> members(n);
  std::iota(members.begin(), members.end(), 0);
  const int want = nvec >= 3 ? 4 : nvec;  // widest block of this call
  if (!b->all || b->wmax != want) {
    b->wmax = want;
    PQ_TRY(ensure_work(b, members));
    PQ_TRY(get_plan(b, members, b->all));
  }
  for (int v0 = 0; v0 < nvec; v0 += b->wmax) {
    PQ_CUDA_TRY(cudaStreamSynchronize(b->stream));  // the previous step has read the call records
    const int c = std::min(b->wmax, nvec - v0);
    for (int i = 0; i < n; i++) {
      pq_ci_handle *h = b->h[i];
      Call &cl = b->h_calls[i];
      cl.active = 1;
      cl.lane_rows = lane_rows(b, i);
      cl.precision = precision;
      cl.lw = log2w(c);
      cl.cnt = c;
      cl.shift = 0.0;
      cl.X = h->x_il.ptr;
      cl.Y = h->y_il.ptr;
      cl.src = C[i] + (size_t)v0 * h->n_dets;
      cl.dst = S[i] + (size_t)v0 * h->n_dets;
    }
    PQ_TRY(run_step(b, *b->all));
  }
  PQ_CUDA_TRY(cudaStreamSynchronize(b->stream));
  return PQ_OK;
}

// Lockstep block Davidson over all problems.  Problems are grouped so that a
// group's Davidson buffers fit workspace_bytes (0: 80% of the free memory);
// each group runs to completion with one batched sigma step (one graph
// launch) per requested width block per iteration.
pq_status pq_ci_batch_davidson(pq_ci_batch *b, const pq_davidson_params *p, size_t workspace_bytes,
                               double *energies, pq_davidson_report *reports) {
  clear_error();
  if (!b || !p || !energies) {
    set_error("pq_ci_batch_davidson: NULL argument");
    return PQ_ERR_ARG;
  }
  const int n = (int)b->h.size(), k = p->num_states;
  if (k < 1) {
    set_error("pq_ci_batch_davidson: num_states=%d", k);
    return PQ_ERR_ARG;
  }
  const int m0 = std::max(p->num_subspace_vec, k);
  int mmax = p->max_subspace > 0 ? p->max_subspace : std::max(2 * p->num_subspace_vec, 10 * k);
  mmax = std::max(mmax, m0 + k);
  b->wmax = k <= 1 ? 1 : (k <= 2 ? 2 : 4);
  // device bytes per determinant: V, W (mmax), X, R (k), T (max(k, m0)), work vectors, diagonal
  const double per_det = 8.0 * (2.0 * mmax + 2.0 * k + std::max(k, m0) + 2.0 * b->wmax) + 16.0;
  if (workspace_bytes == 0) {
    size_t fr = 0, tot = 0;
    PQ_CUDA_TRY(cudaMemGetInfo(&fr, &tot));
    workspace_bytes = (size_t)(0.8 * (double)fr);
  }
  if (b->own_stream) PQ_CUDA_TRY(cudaDeviceSynchronize());
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return b->h[x]->n_dets > b->h[y]->n_dets; });
  std::vector<std::vector<int>> groups;
  double used = 0.0;
  for (int pi : order) {
    const double need = per_det * (double)b->h[pi]->n_dets;
    if (groups.empty() || used + need > (double)workspace_bytes) {
      groups.emplace_back();
      used = 0.0;
    }
    groups.back().push_back(pi);
    used += need;
  }
  cublasHandle_t cb = nullptr;
  if (cublasCreate(&cb) != CUBLAS_STATUS_SUCCESS) {
    set_error("cublasCreate failed");
    return PQ_ERR_CUDA;
  }
  cublasSetStream(cb, b->stream);
  struct CbGuard {
    cublasHandle_t c;
    ~CbGuard() { cublasDestroy(c); }
  } guard{cb};
  pq_status overall = PQ_OK;
  b->all.reset();  // the sigma-call plan may assume another width
  for (const auto &grp : groups) {
    std::vector<std::unique_ptr<DavidsonRun>> runs;
    for (int pi : grp) {
      runs.emplace_back(new DavidsonRun());
      pq_status s = runs.back()->init(b->h[pi], *p, cb);
      if (s != PQ_OK) {
        set_error("problem %d: %s", pi, pq_last_error());
        return s;
      }
    }
    for (auto &r : runs)
      if (!r->pending) PQ_TRY(r->advance());  // started without a sigma request
    PQ_TRY(ensure_work(b, grp));
    std::unique_ptr<BatchPlan> pl;
    PQ_TRY(get_plan(b, grp, pl));
    for (;;) {
      int widest = 0;
      for (auto &r : runs)
        if (!r->done && r->pending) widest = std::max(widest, r->req.cnt);
      if (widest == 0) break;
      const auto t0 = std::chrono::steady_clock::now();
      for (int v0 = 0; v0 < widest; v0 += b->wmax) {
        PQ_CUDA_TRY(cudaStreamSynchronize(b->stream));
        for (int i = 0; i < n; i++) b->h_calls[i].active = 0;
        for (size_t g = 0; g < grp.size(); g++) {
          DavidsonRun &r = *runs[g];
          if (r.done || !r.pending || r.req.cnt <= v0) continue;
          pq_ci_handle *h = b->h[grp[g]];
          Call &cl = b->h_calls[grp[g]];
          const int c = std::min(b->wmax, r.req.cnt - v0);
          cl.active = 1;
          cl.lane_rows = lane_rows(b, grp[g]);
          cl.precision = r.req.precision;
          cl.lw = log2w(c);
          cl.cnt = c;
          cl.shift = r.req.precision == PQ_FP32 ? r.req.shift : 0.0;
          cl.X = h->x_il.ptr;
          cl.Y = h->y_il.ptr;
          cl.src = r.req.src + (size_t)v0 * h->n_dets;
          cl.dst = r.req.dst + (size_t)v0 * h->n_dets;
        }
        PQ_TRY(run_step(b, *pl));
      }
      PQ_CUDA_TRY(cudaStreamSynchronize(b->stream));
      const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      for (auto &r : runs)
        if (!r->done && r->pending) {
          r->rep.sigma_seconds += dt;
          PQ_TRY(r->advance());
        }
    }
    for (size_t g = 0; g < grp.size(); g++) {
      const int pi = grp[g];
      PQ_TRY(runs[g]->outputs(energies + (size_t)pi * k, nullptr));
      if (reports) reports[pi] = runs[g]->rep;
      if (runs[g]->result != PQ_OK) overall = PQ_NOT_CONVERGED;
    }
  }
  for (int i = 0; i < n; i++) b->h_calls[i] = Call{};
  if (overall != PQ_OK) set_error("pq_ci_batch_davidson: at least one problem did not converge");
  return overall;
}

}  // extern "C"
