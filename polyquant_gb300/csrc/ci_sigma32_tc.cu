// Alpha-beta doubles of the FP32 full-CI sigma on the tcgen05 tensor cores.
//
// Reference: the alpha x beta double loop of sigma_one_species_class_singleshot
// (src/ci/detset/direct_singleparticle.cpp:292-306) with the opposite-spin
// element of same_part_ham_double (slater_condon_singleparticle.cpp:107-175):
//   sigma(Ia, Ib) += sum_{a in singles(Ia)} sum_{b in singles(Ib)}
//                    s_a s_b (pair_a | pair_b) C(Ja(a), Jb(b)).
// Written as a GEMM per alpha string Ia over the interleaved vectors
// X[Ja][Jb][v] of four roots (the roots ride along the M dimension):
//   D[(Jb, v)][q] = sum_a X[Ja(a)][Jb][v] * s_a (pair_a | q)      (q: off-diagonal beta pairs)
//   sigma(Ia, Ib, v) += s_b D[(Jb(b), v)][q(b)]  for every beta single b of Ib,
// i.e. for every column Jb, each off-diagonal pair q that moves Jb to a string
// Ib adds D[(Jb, .)][q] with the single's phase into sigma(Ia, Ib, .).
//
// Kernel: persistent, one CTA per SM, alpha strings assigned round-robin.  Warp roles:
//   warp 0      TMEM owner and MMA issuer (M = 128 rows (Jb, v), N = 128
//               pairs, K = 64 singles; hi*hi + hi*lo + lo*hi in FP16 with FP32
//               accumulation; two accumulators so the epilogue overlaps);
//   warps 1-4   converters: thread (c, kq) owns beta string c of a 32-string tile
//               (operand rows 4c .. 4c + 3) and alpha singles 16 kq .. 16 kq + 15;
//               it copies the 16-byte vectors X[Ja][Jb][0..3] of its singles into a
//               shared stage with asynchronous copies, one tile ahead, then scales
//               them, splits them into FP16 hi/lo and writes its part of the K-major
//               128-byte-swizzled operand tile (two stages); they also build B per
//               alpha string from the cross-spin integrals (one buffer);
//   warps 5-8   epilogue: tcgen05.ld of the accumulator into a shared staging copy
//               of the whole tile ([Jb][q][v]), which frees the accumulator at once;
//   warps 5-11  then each thread takes targets from the tile's precomputed scatter
//               list (the distinct Ib reached from the tile's 32 beta strings, each
//               with its (Jb, q, phase) contributions: 2.1 per target at 16
//               orbitals), sums them and adds the sum into sigma(Ia, Ib) with one
//               vector reduction (red.global.add.v4.f32).  Staging full / empty are
//               mbarriers, so every wait in the kernel is bounded.
// A CTA is the only writer of its sigma rows, so the reductions never contend
// between CTAs.  On this GPU a shared-memory float atomic adds fewer values
// per clock than a global vector reduction, which carries all four roots.
// Scaling: X and the integrals are multiplied by powers of two that bring
// their largest magnitudes to [2^14, 2^15) (FP16 range, exact in FP32), and
// the result by the inverses.  The split x = hi + lo with hi, lo in FP16 keeps
// 22 significant bits; the three products are exact in FP32.
// Every mbarrier wait is bounded; a wait that runs out records an error code,
// sets an abort flag that every role polls, and the kernel winds down (the
// MMA thread waits, bounded, for its own MMAs, TMEM is freed); the host
// reports PQ_TIMEOUT.
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <utility>
#include <vector>

#include "pq_internal.h"

namespace pq {
namespace abtc {

constexpr int BM = 128;       // (Jb, v) rows per tile (TMEM lanes)
constexpr int BN = 128;       // off-diagonal beta pairs (TMEM columns per accumulator)
constexpr int BK = 64;        // alpha singles (K), one 128-byte swizzle span of FP16
constexpr int NV = 4;         // roots per determinant (interleaved); other widths use the CUDA-core path
constexpr int ASTAGES = 2;    // A operand stages
constexpr int TJB = BM / NV;  // beta strings per tile (32)
constexpr int OP_TILE = BM * BK * 2;          // 16 KB: one FP16 operand tile (A or B)
constexpr int RAW_TILE = BK * BM * 4;         // 32 KB: the gathered FP32 rows of one tile
constexpr int STG_BYTES = TJB * BN * NV * 4;  // 64 KB: the whole accumulator tile, [Jb][q][v]
constexpr int KQ = BK / 4;                    // alpha singles per converter thread (16)
constexpr int NPRE = 6;                       // scatter-list entries per processing thread loaded ahead of a tile
constexpr int NTHREADS = 384;                    // 12 warps
constexpr int CONV0 = 1, EPI0 = 5, PROC0 = 9;    // first converter / epilogue (staging) / list-only warp
constexpr int NPROC = (NTHREADS / 32 - EPI0) * 32;  // threads that process the scatter lists (224)
constexpr long long WAIT_CYCLES = 4000000000LL;  // ~2 s at 2 GHz
// shared memory: A hi/lo x ASTAGES, B hi/lo (one buffer), raw rows x 2, accumulator staging, per-warp alpha
// partner lists, barriers
constexpr int SMEM_OPS = ASTAGES * 2 * OP_TILE + 2 * OP_TILE + 2 * RAW_TILE + STG_BYTES;
constexpr int NBARS = 2 * ASTAGES + 9;  // a_full, a_empty, acc_full[2], acc_empty[2], b_full, b_empty, drain,
                                        // stg_full, stg_empty
constexpr int SMEM_BYTES = SMEM_OPS + 4 * BK * 2 + 1024 + NBARS * 8 + 16;
static_assert(SMEM_OPS % 16 == 0 && (2 * RAW_TILE) % 16 == 0, "16-byte alignment of the copy and staging areas");
static_assert(SMEM_BYTES <= 232448, "shared memory per CTA");

enum { ERR_AEMPTY = 2, ERR_AFULL = 3, ERR_ACC = 4, ERR_B = 5, ERR_STG = 6 };

struct Args {
  const float *X;          // [na][nb][NV] interleaved input (FP32)
  float *Y;                // [na][nb][NV] interleaved output, added to
  const float *xmax;       // max |X| over the input (device scalar, written by the reduction pass)
  int64_t na, nb;
  int m_tiles;             // ceil(nb * NV / BM)
  const int64_t *a_off;
  const int32_t *a_J, *a_info;
  const float *eab;        // (pair_alpha | pair_beta) row-major FP32
  int npair, n_off;        // beta pairs: all, off-diagonal (<= BN)
  float sw;                // power-of-two scale of the integrals
  // scatter lists per tile of 32 beta strings: entries t_off[t] .. t_off[t + 1] of tile t, each
  // {Ib | n << 16, up to six contributions as uint16 pairs}; a contribution is (phase << 12 | jb_local << 7 | q)
  // (a target with more than six contributions takes several entries)
  const int32_t *t_off;
  const int4 *tent;
  long long wait_cycles;
  int *err;
  long long *prof;         // per-CTA role timers (PQ_ABTC_PROFILE builds only)
};

// Role timers (only in builds with PQ_ABTC_PROFILE defined): cycles per slot, summed over a CTA's work and
// written by one thread of each role at the end.
#ifdef PQ_ABTC_PROFILE
#define PT(v) const long long v = clock64()
#define PACC(slot, v) prof_[slot] += clock64() - (v)
#else
#define PT(v)
#define PACC(slot, v)
#endif

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait: true when the phase completed, false when the budget (SM clock cycles) ran out
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, long long budget) {
  const long long t0 = clock64();
  while (!mbar_try(bar, parity)) {
    if (clock64() - t0 > budget) return false;
  }
  return true;
}
// warp-uniform bounded wait: every lane polls; the warp agrees on success only if every lane saw the phase
__device__ __forceinline__ bool warp_wait(uint32_t bar, uint32_t parity, long long budget) {
  const bool ok = mbar_wait(bar, parity, budget);
  return __all_sync(0xffffffffu, ok);
}
__device__ __forceinline__ bool warp_aborted(volatile int *flag) { return __any_sync(0xffffffffu, *flag != 0); }

// 4-byte / 16-byte asynchronous copies global -> shared (each thread waits for its own groups)
__device__ __forceinline__ void cp_async4(uint32_t dst, const void *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// UMMA shared-memory descriptor: K-major, 128-byte swizzle, 8-row groups 1024 B apart
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFF) >> 4);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

// instruction descriptor: D = F32, A = B = F16 (format 0 of kind::f16), both K-major, N = BN, M = BM
constexpr uint32_t IDESC = (1u << 4) | (0u << 7) | (0u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accum) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(IDESC), "r"(accum)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// K values of row r of an operand tile (scaled FP32) -> FP16 hi/lo tiles in the 128-byte-swizzled K-major
// layout (16-byte chunk c of row r at chunk position c ^ (r & 7)); pairs convert with one packed instruction
__device__ __forceinline__ void store_row(unsigned char *th, unsigned char *tl, int r, const float (&x)[BK]) {
#pragma unroll
  for (int c = 0; c < BK / 8; c++) {
    __half2 h[4], l[4];
#pragma unroll
    for (int e = 0; e < 4; e++) {
      const float a = x[c * 8 + 2 * e], b = x[c * 8 + 2 * e + 1];
      h[e] = __floats2half2_rn(a, b);
      const float2 f = __half22float2(h[e]);
      l[e] = __floats2half2_rn(a - f.x, b - f.y);
    }
    *reinterpret_cast<uint4 *>(th + r * 128 + ((c ^ (r & 7)) << 4)) = *reinterpret_cast<const uint4 *>(h);
    *reinterpret_cast<uint4 *>(tl + r * 128 + ((c ^ (r & 7)) << 4)) = *reinterpret_cast<const uint4 *>(l);
  }
}

// 16 K values (alpha singles 16 kq .. 16 kq + 15) of row r -> the two 16-byte chunks 2 kq, 2 kq + 1 of the
// FP16 hi/lo tiles (same swizzled layout as store_row)
__device__ __forceinline__ void store_quarter(unsigned char *th, unsigned char *tl, int r, int kq, const float (&x)[KQ]) {
#pragma unroll
  for (int hh = 0; hh < 2; hh++) {
    const int ch = 2 * kq + hh;
    __half2 h[4], l[4];
#pragma unroll
    for (int e = 0; e < 4; e++) {
      const float a = x[hh * 8 + 2 * e], b = x[hh * 8 + 2 * e + 1];
      h[e] = __floats2half2_rn(a, b);
      const float2 f = __half22float2(h[e]);
      l[e] = __floats2half2_rn(a - f.x, b - f.y);
    }
    *reinterpret_cast<uint4 *>(th + r * 128 + ((ch ^ (r & 7)) << 4)) = *reinterpret_cast<const uint4 *>(h);
    *reinterpret_cast<uint4 *>(tl + r * 128 + ((ch ^ (r & 7)) << 4)) = *reinterpret_cast<const uint4 *>(l);
  }
}

// power of two 2^e with x * 2^e in [2^14, 2^15) (1 for x == 0)
__device__ __forceinline__ float fp16_scale(float x) {
  if (!(x > 0.0f) || !isfinite(x)) return 1.0f;
  int e;
  frexpf(x, &e);  // x = f * 2^e, f in [0.5, 1)
  return ldexpf(1.0f, 15 - e);
}

__global__ void __launch_bounds__(NTHREADS, 1) ab_tc_kernel(Args g) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char *smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  unsigned char *a_hi = smem;                                  // [ASTAGES] x 16 KB
  unsigned char *a_lo = a_hi + ASTAGES * OP_TILE;              // [ASTAGES] x 16 KB
  unsigned char *b_hi = a_lo + ASTAGES * OP_TILE;              // 16 KB
  unsigned char *b_lo = b_hi + OP_TILE;                        // 16 KB
  float *raw = reinterpret_cast<float *>(b_lo + OP_TILE);      // [2][BK][BM]
  float *stg = raw + 2 * BK * BM;                              // [TJB][BN][NV], column swizzled by the row
  uint16_t *ja_all = reinterpret_cast<uint16_t *>(reinterpret_cast<unsigned char *>(stg) + STG_BYTES);  // [4][BK]
  uint64_t *bars = reinterpret_cast<uint64_t *>(ja_all + 4 * BK);
  uint64_t *a_full = bars, *a_empty = bars + ASTAGES, *acc_full = bars + 2 * ASTAGES;
  uint64_t *acc_empty = acc_full + 2, *b_full = acc_full + 4, *b_empty = acc_full + 5, *drain = acc_full + 6;
  uint64_t *stg_full = acc_full + 7, *stg_empty = acc_full + 8;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(stg_empty + 1);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#ifdef PQ_ABTC_PROFILE
  long long prof_[16] = {0};
  const long long prof_start = clock64();
#endif
  if (threadIdx.x == 0) {
    for (int s = 0; s < ASTAGES; s++) {
      mbar_init(smem_u32(a_full + s), 4);
      mbar_init(smem_u32(a_empty + s), 1);
    }
    for (int s = 0; s < 2; s++) {
      mbar_init(smem_u32(acc_full + s), 1);
      mbar_init(smem_u32(acc_empty + s), 4);
    }
    mbar_init(smem_u32(b_full), 4);
    mbar_init(smem_u32(b_empty), 1);
    mbar_init(smem_u32(drain), 1);
    mbar_init(smem_u32(stg_full), 4);
    mbar_init(smem_u32(stg_empty), NPROC / 32);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(2 * BN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const int mt = g.m_tiles;
  const int64_t row_len = g.nb * NV;  // floats in one alpha row of X and Y

  if (warp == 0) {
    // ---- MMA issuer
    if (lane == 0) {
      int seq = 0, grp = 0;
      bool ok = true;
      for (int64_t ia = blockIdx.x; ia < g.na && ok && !*abort_flag; ia += gridDim.x, grp++) {
        PT(tb0);
        if (!mbar_wait(smem_u32(b_full), (uint32_t)(grp & 1), g.wait_cycles)) {
          atomicCAS(g.err, 0, ERR_B);
          ok = false;
          break;
        }
        PACC(3, tb0);
        const uint32_t bh = smem_u32(b_hi), bl = smem_u32(b_lo);
        for (int t = 0; t < mt; t++, seq++) {
          const int s = seq % ASTAGES, a = seq & 1;
          const uint32_t ps = (uint32_t)((seq / ASTAGES) & 1), pa = (uint32_t)((seq >> 1) & 1);
          PT(tw0);
          if (!mbar_wait(smem_u32(acc_empty + a), pa ^ 1u, g.wait_cycles)) {
            atomicCAS(g.err, 0, ERR_ACC);
            ok = false;
            break;
          }
          PACC(1, tw0);
          PT(tw1);
          if (!mbar_wait(smem_u32(a_full + s), ps, g.wait_cycles)) {
            atomicCAS(g.err, 0, ERR_AFULL);
            ok = false;
            break;
          }
          PACC(2, tw1);
          if (*abort_flag) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t d = tmem + (uint32_t)(a * BN);
          const uint32_t ah = smem_u32(a_hi + s * OP_TILE), al = smem_u32(a_lo + s * OP_TILE);
#pragma unroll
          for (int kk = 0; kk < BK / 16; kk++) {
            const uint32_t off = kk * 32;  // 16 FP16 values along K
            mma_f16(d, smem_desc(ah + off), smem_desc(bh + off), kk > 0 ? 1u : 0u);
            mma_f16(d, smem_desc(ah + off), smem_desc(bl + off), 1u);
            mma_f16(d, smem_desc(al + off), smem_desc(bh + off), 1u);
          }
          mma_commit(smem_u32(a_empty + s));
          mma_commit(smem_u32(acc_full + a));
        }
        if (!ok) break;
        mma_commit(smem_u32(b_empty));  // B of this alpha string is free once its MMAs completed
      }
      if (!ok) *abort_flag = 1;
      // every MMA issued here has completed before TMEM is freed
      mma_commit(smem_u32(drain));
      mbar_wait(smem_u32(drain), 0, WAIT_CYCLES);
    }
    __syncwarp();
  } else if (warp < EPI0) {
    // ---- converters.  A: thread (c = lane, kq = warp - CONV0) owns beta string c of the tile (its four
    // operand rows 4c .. 4c + 3) and alpha singles 16 kq .. 16 kq + 15: it copies the 16-byte vectors
    // X[Ja(k)][Jb][0..3] of its singles into the raw stage, one tile ahead, and converts only what it copied
    // (no cross-thread wait).  B: thread r = 32 kq + c owns the off-diagonal beta pair q = r.
    const int kq = warp - CONV0, c = lane;
    const int r = threadIdx.x - 32 * CONV0;       // 0..127
    uint16_t *ja = ja_all + kq * BK;              // this warp's copy of the alpha partner list
    const float sx = fp16_scale(*g.xmax);
    int seq = 0, grp = 0;
    bool stop = false;
    int i = 1;
    while ((i + 1) * i / 2 <= r) i++;  // off-diagonal pair r = i(i-1)/2 + j, j < i
    const int qfull = r + i;           // its idx2(i, j) = i(i+1)/2 + j
    const bool qv = r < g.n_off;
    for (int64_t ia = blockIdx.x; ia < g.na && !stop; ia += gridDim.x, grp++) {
      const int64_t base = g.a_off[ia];
      const int n1 = (int)(g.a_off[ia + 1] - base);
      ja[lane] = (uint16_t)(lane < n1 ? g.a_J[base + lane] : 0);
      ja[lane + 32] = (uint16_t)(lane + 32 < n1 ? g.a_J[base + lane + 32] : 0);
      __syncwarp();
      PT(cb0);
      if (!warp_wait(smem_u32(b_empty), (uint32_t)(grp & 1) ^ 1u, g.wait_cycles)) {
        if (lane == 0) atomicCAS(g.err, 0, ERR_B);
        *abort_flag = 1;
        break;
      }
      if (warp_aborted(abort_flag)) break;
      PACC(5, cb0);
      PT(cb1);
      {
        // B[q][k] = s_k (pair_k | q) * sw for the off-diagonal beta pair q = r
        float w[BK];
#pragma unroll
        for (int k = 0; k < BK; k++) {
          w[k] = 0.0f;
          if (qv && k < n1) {
            const int info = __ldg(g.a_info + base + k);
            const float x = __ldg(g.eab + (int64_t)(info >> 1) * g.npair + qfull) * g.sw;
            w[k] = (info & 1) ? -x : x;
          }
        }
        store_row(b_hi, b_lo, r, w);
      }
      PACC(6, cb1);
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_u32(b_full));
      auto issue = [&](int t, int stage) {
        const int64_t e = (int64_t)t * BM + 4 * c;  // first float of beta string c of tile t in an alpha row
        if (e < row_len) {
          const float *col = g.X + e;
          const uint32_t dst = smem_u32(raw + stage * BK * BM + 4 * c);
#pragma unroll 4
          for (int j = 0; j < KQ; j++) {
            const int k = kq * KQ + j;
            if (k < n1) cp_async16(dst + k * BM * 4, col + (int64_t)ja[k] * row_len);
          }
        }
        cp_commit();
      };
      issue(0, seq & 1);
      for (int t = 0; t < mt; t++) {
        PT(cl0);
        if (t + 1 < mt)
          issue(t + 1, (seq + 1) & 1);
        else
          cp_commit();  // an empty group keeps one group per tile
        PACC(10, cl0);
        const int s = seq % ASTAGES;
        const uint32_t ps = (uint32_t)((seq / ASTAGES) & 1);
        PT(ca0);
        if (!warp_wait(smem_u32(a_empty + s), ps ^ 1u, g.wait_cycles)) {
          if (lane == 0) atomicCAS(g.err, 0, ERR_AEMPTY);
          *abort_flag = 1;
          stop = true;
          break;
        }
        if (warp_aborted(abort_flag)) {
          stop = true;
          break;
        }
        PACC(7, ca0);
        PT(cc0);
        cp_wait<1>();  // this tile's copies have landed (the next tile's may still be in flight)
        PACC(9, cc0);
        PT(cs0);
        {
          const bool in = (int64_t)t * BM + 4 * c < row_len;
          const float *src = raw + (seq & 1) * BK * BM + 4 * c;
          float x[NV][KQ];
#pragma unroll
          for (int j = 0; j < KQ; j++) {
            const int k = kq * KQ + j;
            float4 v4 = make_float4(0.f, 0.f, 0.f, 0.f);
            if (in && k < n1) v4 = *reinterpret_cast<const float4 *>(src + k * BM);
            x[0][j] = v4.x * sx;
            x[1][j] = v4.y * sx;
            x[2][j] = v4.z * sx;
            x[3][j] = v4.w * sx;
          }
#pragma unroll
          for (int v = 0; v < NV; v++) store_quarter(a_hi + s * OP_TILE, a_lo + s * OP_TILE, 4 * c + v, kq, x[v]);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_u32(a_full + s));
        PACC(8, cs0);
        seq++;
      }
      cp_wait<0>();
      __syncwarp();
    }
  } else {
    // ---- epilogue.  Per tile: warps EPI0 .. EPI0 + 3 copy the accumulator into the staging area ([Jb][q][v],
    // the column swizzled by the row) and release the accumulator; then they and the list-only warps
    // PROC0 .. take targets of the tile's scatter list, sum their contributions from the staging area and
    // add each sum into sigma(Ia, target) with one vector reduction.  Staging full / empty are mbarriers
    // with bounded waits.
    const bool stager = warp < PROC0;
    const int q4 = warp & 3;                 // TMEM lane quadrant of a staging warp
    const int te = threadIdx.x - 32 * EPI0;  // 0 .. NPROC - 1
    int seq = 0;
    bool dead = false;
    // the two inverse scales are powers of two inside the FP32 range, and so is their product
    const float unscale = (1.0f / g.sw) * (1.0f / fp16_scale(*g.xmax));
    const int jl = 8 * q4 + (lane >> 2), vv = lane & 3;  // a staging lane's accumulator row (beta string, root)
    for (int64_t ia = blockIdx.x; ia < g.na; ia += gridDim.x) {
      float *yrow = g.Y + ia * row_len;
      for (int t = 0; t < mt; t++, seq++) {
        if (dead) continue;
        // this tile's first NPRE list entries per thread: the loads do not depend on the accumulator, so
        // their latency overlaps the wait for it and the staging
        const int k0 = g.t_off[t], k1 = g.t_off[t + 1];
        int4 pre[NPRE];
#pragma unroll
        for (int i = 0; i < NPRE; i++) {
          const int k = k0 + te + NPROC * i;
          pre[i] = k < k1 ? __ldg(g.tent + k) : make_int4(0, 0, 0, 0);
        }
        PT(ew0);
        if (stager) {
          const int a = seq & 1;
          const uint32_t pa = (uint32_t)((seq >> 1) & 1);
          bool ok = warp_wait(smem_u32(acc_full + a), pa, g.wait_cycles);
          ok = ok && warp_wait(smem_u32(stg_empty), (uint32_t)(seq & 1) ^ 1u, g.wait_cycles);
          if (!ok || warp_aborted(abort_flag)) {
            if (!ok && lane == 0) atomicCAS(g.err, 0, ERR_STG);
            *abort_flag = 1;
            dead = true;
            continue;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const uint32_t taddr = tmem + ((uint32_t)(q4 * 32) << 16) + (uint32_t)(a * BN);
          float *srow = stg + (int64_t)jl * BN * NV + vv;
#pragma unroll 1
          for (int c0 = 0; c0 < BN; c0 += 32) {
            float d[32];
            tmem_ld32(taddr + c0, d);
#pragma unroll
            for (int j = 0; j < 32; j++) srow[((c0 + j) ^ (jl & 7)) * NV] = d[j];
          }
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
          __syncwarp();
          if (lane == 0) {
            mbar_arrive(smem_u32(acc_empty + a));  // the MMAs may refill this accumulator
            mbar_arrive(smem_u32(stg_full));
          }
        }
        PACC(11, ew0);
        PT(es0);
        if (!warp_wait(smem_u32(stg_full), (uint32_t)(seq & 1), g.wait_cycles) || warp_aborted(abort_flag)) {
          if (lane == 0) atomicCAS(g.err, 0, ERR_STG);
          *abort_flag = 1;
          dead = true;
          continue;
        }
        // one entry: sum its contributions from the staging area, one vector reduction into sigma
        auto apply = [&](const int4 &ent) {
          const int n = ent.x >> 16;
          if (n == 0) return;
          const uint32_t w3[3] = {(uint32_t)ent.y, (uint32_t)ent.z, (uint32_t)ent.w};
          float4 sm = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
          for (int u = 0; u < 6; u++) {
            if (u < n) {
              const uint32_t en = (w3[u >> 1] >> (16 * (u & 1))) & 0xFFFFu;
              const int rl = (int)((en >> 7) & 31), qq = (int)(en & 127);
              const float4 x = *reinterpret_cast<const float4 *>(stg + ((int64_t)rl * BN + (qq ^ (rl & 7))) * NV);
              const float f = (en & 4096u) ? -1.0f : 1.0f;
              sm.x = fmaf(f, x.x, sm.x);
              sm.y = fmaf(f, x.y, sm.y);
              sm.z = fmaf(f, x.z, sm.z);
              sm.w = fmaf(f, x.w, sm.w);
            }
          }
          asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(yrow + (int64_t)(ent.x & 0xFFFF) * NV),
                       "f"(sm.x * unscale), "f"(sm.y * unscale), "f"(sm.z * unscale), "f"(sm.w * unscale)
                       : "memory");
        };
#pragma unroll
        for (int i = 0; i < NPRE; i++) apply(pre[i]);
        // the rest of the tile's entries (tiles with more than NPRE x NPROC), four loads at a time
        for (int kb = k0 + te + NPROC * NPRE; kb < k1; kb += 4 * NPROC) {
          int4 ent[4];
#pragma unroll
          for (int i = 0; i < 4; i++) ent[i] = kb + NPROC * i < k1 ? __ldg(g.tent + kb + NPROC * i) : make_int4(0, 0, 0, 0);
#pragma unroll
          for (int i = 0; i < 4; i++) apply(ent[i]);
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_u32(stg_empty));
        PACC(12, es0);
      }
    }
  }
#ifdef PQ_ABTC_PROFILE
  {
    const long long tot = clock64() - prof_start;
    long long *o = g.prof + blockIdx.x * 16;
    if (threadIdx.x == 0) {
      o[0] = tot;
      for (int i = 1; i <= 3; i++) o[i] = prof_[i];
    }
    if (threadIdx.x == 32 * CONV0) {
      o[4] = tot;
      for (int i = 5; i <= 10; i++) o[i] = prof_[i];
    }
    if (threadIdx.x == 32 * EPI0)
      for (int i = 11; i <= 12; i++) o[i] = prof_[i];
  }
#endif
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * BN) : "memory");
}

// btab[Jb][q] for every beta single of Jb: q = off-diagonal index of its pair (row length BN), entry
// (Ib << 1 | phase); every other entry stays 0xFFFF
__global__ void btab_kernel(const int64_t *off, const int32_t *J, const int32_t *info, int64_t nb, uint16_t *btab) {
  const int64_t jb = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (jb >= nb) return;
  for (int64_t e = off[jb]; e < off[jb + 1]; e++) {
    const int pr = info[e] >> 1;  // idx2(i, j) with i > j for a single
    int i = 1;
    while ((i + 1) * (i + 2) / 2 <= pr) i++;  // largest i with i(i+1)/2 <= pr
    const int q = pr - i;                     // i(i-1)/2 + j
    btab[jb * BN + q] = (uint16_t)(((uint32_t)J[e] << 1) | (uint32_t)(info[e] & 1));
  }
}

// xmax = max |X| (as the bit pattern of a non-negative float, so integer max orders it)
__global__ void absmax_kernel(const float *X, int64_t n, unsigned *xmax) {
  float m = 0.0f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    m = fmaxf(m, fabsf(X[i]));
  for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(xmax, __float_as_uint(m));
}

}  // namespace abtc

// The tensor-core alpha-beta path applies to one-species full CI with at most
// 16 orbitals (the 120 off-diagonal beta pairs fit N = 128), at most 64 alpha
// singles per string (K = 64), fewer than 32768 beta strings (16-bit targets
// in the scatter table) and fewer than 65536 alpha strings (16-bit partner
// lists).
bool sigma32_tc_applicable(const pq_ci_handle *h) {
  if (h->n_species != 1 || !h->full) return false;
  const int n = h->n_orb[0];
  if (n > 16 || n * (n - 1) / 2 > abtc::BN) return false;
  if (h->tab[0][0].max1 > abtc::BK) return false;
  return h->tab[0][1].n_str < 32768 && h->tab[0][0].n_str < 65536;
}

static pq_status ab_tc_impl(pq_ci_handle *h, const float *X, float *Y) {
  using namespace abtc;
  cudaStream_t st = h->stream;
  const int64_t na = h->tab[0][0].n_str, nb = h->tab[0][1].n_str;
  const int n = h->n_orb[0], npair = h->npair[0];
  if (!h->tc_ready) {
    // one-off: the beta scatter table, the integral scale, the kernel's shared-memory limit
    PQ_TRY(h->tc_btab.alloc(sizeof(uint16_t) * (size_t)BN * nb + 16));
    PQ_CUDA_TRY(cudaMemsetAsync(h->tc_btab.ptr, 0xFF, sizeof(uint16_t) * (size_t)BN * nb, st));
    const SpinTablesDev &tb = h->tab[0][1];
    btab_kernel<<<(unsigned)((nb + 255) / 256), 256, 0, st>>>(tb.s1_off.as<int64_t>(), tb.s1_J.as<int32_t>(),
                                                            tb.s1_info.as<int32_t>(), nb, h->tc_btab.as<uint16_t>());
    PQ_CUDA_TRY(cudaGetLastError());
    // scatter lists per tile of TJB beta strings: the distinct targets of the tile's (Jb, q) entries, each
    // with its contributions, so the epilogue issues one reduction per target instead of one per entry
    {
      std::vector<uint16_t> bt((size_t)BN * nb);
      PQ_CUDA_TRY(cudaMemcpyAsync(bt.data(), h->tc_btab.ptr, sizeof(uint16_t) * bt.size(), cudaMemcpyDeviceToHost, st));
      PQ_CUDA_TRY(cudaStreamSynchronize(st));
      const int tiles = (int)((nb + TJB - 1) / TJB);
      std::vector<int32_t> toff(tiles + 1, 0);
      std::vector<int4> tent;
      std::vector<std::pair<int32_t, uint16_t>> items;
      for (int t = 0; t < tiles; t++) {
        items.clear();
        for (int jl = 0; jl < TJB && (int64_t)t * TJB + jl < nb; jl++) {
          const uint16_t *row = bt.data() + ((int64_t)t * TJB + jl) * BN;
          for (int q = 0; q < BN; q++)
            if (row[q] != 0xFFFFu)
              items.push_back({(int32_t)(row[q] >> 1), (uint16_t)(((row[q] & 1u) << 12) | ((unsigned)jl << 7) | (unsigned)q)});
        }
        std::sort(items.begin(), items.end());
        for (size_t u = 0; u < items.size();) {
          size_t w = u;
          while (w < items.size() && items[w].first == items[u].first) w++;
          // one entry per six contributions of a target
          for (size_t x0 = u; x0 < w; x0 += 6) {
            const size_t x1 = std::min(w, x0 + 6);
            uint32_t c6[6] = {0, 0, 0, 0, 0, 0};
            for (size_t x = x0; x < x1; x++) c6[x - x0] = items[x].second;
            tent.push_back(make_int4(items[u].first | (int)((x1 - x0) << 16), (int)(c6[0] | (c6[1] << 16)),
                                     (int)(c6[2] | (c6[3] << 16)), (int)(c6[4] | (c6[5] << 16))));
          }
          u = w;
        }
        if (tent.size() > (size_t)INT32_MAX / 2) {
          set_error("sigma32 tensor-core path: scatter lists too large");
          return PQ_ERR_ARG;
        }
        toff[t + 1] = (int32_t)tent.size();
      }
      if (tent.empty()) tent.push_back(make_int4(0, 0, 0, 0));
      PQ_TRY(upload(h->tc_toff, toff, st));
      PQ_TRY(upload(h->tc_tinfo, tent, st));
      h->tc_btab.release();  // the table itself is no longer needed
      PQ_CUDA_TRY(cudaStreamSynchronize(st));
    }
    std::vector<float> e((size_t)npair * npair);
    PQ_CUDA_TRY(cudaMemcpyAsync(e.data(), h->d_eab32.ptr, sizeof(float) * e.size(), cudaMemcpyDeviceToHost, st));
    PQ_CUDA_TRY(cudaStreamSynchronize(st));
    float wmax = 0.0f;
    for (float x : e) wmax = std::max(wmax, std::fabs(x));
    int ex = 0;
    std::frexp(wmax, &ex);
    h->tc_sw = wmax > 0.0f ? std::ldexp(1.0f, 15 - ex) : 1.0f;
    PQ_CUDA_TRY(cudaFuncSetAttribute(ab_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
    PQ_TRY(h->tc_aux.alloc(64));
    int dev = 0;
    PQ_CUDA_TRY(cudaGetDevice(&dev));
    PQ_CUDA_TRY(cudaDeviceGetAttribute(&h->tc_sms, cudaDevAttrMultiProcessorCount, dev));
    h->tc_ready = true;
  }
  unsigned *xmax = h->tc_aux.as<unsigned>();
  int *err = reinterpret_cast<int *>(xmax + 1);
  PQ_CUDA_TRY(cudaMemsetAsync(h->tc_aux.ptr, 0, 8, st));
  const int64_t len = na * nb * NV;
  absmax_kernel<<<(unsigned)std::min<int64_t>((len + 255) / 256, 152 * 8), 256, 0, st>>>(X, len, xmax);
  PQ_CUDA_TRY(cudaGetLastError());
  Args a{};
  a.X = X;
  a.Y = Y;
  a.xmax = reinterpret_cast<const float *>(xmax);
  a.na = na;
  a.nb = nb;
  a.m_tiles = (int)((nb * NV + BM - 1) / BM);
  const SpinTablesDev &ta = h->tab[0][0];
  a.a_off = ta.s1_off.as<int64_t>();
  a.a_J = ta.s1_J.as<int32_t>();
  a.a_info = ta.s1_info.as<int32_t>();
  a.eab = h->d_eab32.as<float>();
  a.npair = npair;
  a.n_off = n * (n - 1) / 2;
  a.sw = h->tc_sw;
  a.t_off = h->tc_toff.as<int32_t>();
  a.tent = h->tc_tinfo.as<int4>();
  a.wait_cycles = WAIT_CYCLES;
  a.err = err;
#ifdef PQ_ABTC_PROFILE
  DevBuf prof;
  PQ_TRY(prof.alloc(sizeof(long long) * 16 * 1024));
  PQ_CUDA_TRY(cudaMemsetAsync(prof.ptr, 0, sizeof(long long) * 16 * 1024, st));
  a.prof = prof.as<long long>();
#endif
  const unsigned grid = (unsigned)std::min<int64_t>(na, h->tc_sms > 0 ? h->tc_sms : 148);
  ab_tc_kernel<<<grid, NTHREADS, SMEM_BYTES, st>>>(a);
  PQ_CUDA_TRY(cudaGetLastError());
  int herr = 0;
  PQ_CUDA_TRY(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  PQ_CUDA_TRY(cudaStreamSynchronize(st));
  if (herr != 0) {
    set_error("sigma32 alpha-beta tensor-core kernel: a pipeline wait ran out (code %d)", herr);
    return PQ_TIMEOUT;
  }
#ifdef PQ_ABTC_PROFILE
  {
    std::vector<long long> pr((size_t)16 * grid);
    PQ_CUDA_TRY(cudaMemcpy(pr.data(), prof.ptr, sizeof(long long) * pr.size(), cudaMemcpyDeviceToHost));
    const char *names[13] = {"total", "mma:wait_acc_empty", "mma:wait_a_full", "mma:wait_b_full", "conv:total",
                             "conv:wait_b_empty", "conv:b_build", "conv:wait_a_empty", "conv:convert_store",
                             "conv:wait_copies", "conv:issue_copies", "epi:wait_acc_full", "epi:scatter"};
    for (int i = 0; i < 13; i++) {
      double m = 0;
      for (unsigned b = 0; b < grid; b++) m += (double)pr[16 * b + i];
      fprintf(stderr, "abtc-prof %-22s %14.0f cycles/CTA\n", names[i], m / grid);
    }
  }
#endif
  return PQ_OK;
}

pq_status ci_sigma32_ab_tc(pq_ci_handle *h, const void *X, void *Y, int nvp) {
  if (nvp == abtc::NV) return ab_tc_impl(h, (const float *)X, (float *)Y);
  set_error("sigma32 tensor-core path: width %d (the path takes %d vectors)", nvp, abtc::NV);
  return PQ_ERR_ARG;
}

}  // namespace pq
