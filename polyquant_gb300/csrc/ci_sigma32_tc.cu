// Alpha-beta doubles of the FP32 full-CI sigma on the tcgen05 tensor cores.
//
// Reference: the alpha x beta double loop of sigma_one_species_class_singleshot
// (src/ci/detset/direct_singleparticle.cpp:292-306) with the opposite-spin
// element of same_part_ham_double (slater_condon_singleparticle.cpp:107-175):
//   sigma(Ia, Ib) += sum_{a in singles(Ia)} sum_{b in singles(Ib)}
//                    s_a s_b (pair_a | pair_b) C(Ja(a), Jb(b)).
// Written as a GEMM per (alpha string Ia, root v):
//   D[Jb][q] = sum_a X_v[Ja(a)][Jb] * s_a (pair_a | q)      (q: off-diagonal beta pairs)
//   sigma(Ia, Ib) += s_b D[Jb(b)][q(b)]  for every beta single b of Ib,
// i.e. for every column Jb, each off-diagonal pair q that moves Jb to a string
// Ib scatters D[Jb][q] with the single's phase into the sigma row of Ia.
//
// Kernel: persistent, one CTA per SM, alpha strings assigned round-robin; the
// roots of one alpha string share its B operand.  Warp roles:
//   warp 0      TMA producer: one 512-byte bulk copy per alpha single per
//               128-column tile of the planar vector X_v (rows Ja(a));
//   warp 1      TMEM owner and MMA issuer (M = 128 columns Jb, N = 128 pairs,
//               K = 64 singles; hi*hi + hi*lo + lo*hi in FP16 with FP32
//               accumulation; two accumulators so the epilogue overlaps);
//   warps 2-5   converters: scaled FP32 rows -> FP16 hi/lo in the K-major
//               128-byte-swizzled operand layout; they also build B per alpha
//               string from the cross-spin integrals;
//   warps 6-9   epilogue: tcgen05.ld of the accumulator, scatter through the
//               [pair][Jb] table into the sigma row in shared memory; at the
//               end of an item the row is written (scaled back) to Z_v[Ia].
// Scaling: X and the integrals are multiplied by powers of two that bring
// their largest magnitudes to [2^14, 2^15) (FP16 range, exact in FP32), and
// the result by the inverse.  The split x = hi + lo with hi, lo in FP16 keeps
// 22 significant bits; the three products are exact in FP32.
// Every mbarrier wait is bounded; a wait that runs out records an error code,
// sets an abort flag that every role polls, and the kernel winds down (the
// producer waits, bounded, for its own copies, the MMA thread for its own
// MMAs, TMEM is freed); the host reports PQ_TIMEOUT.
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>

#include "pq_internal.h"

namespace pq {
namespace abtc {

constexpr int BM = 128;       // beta columns per tile (TMEM lanes)
constexpr int BN = 128;       // off-diagonal beta pairs (TMEM columns per accumulator)
constexpr int BK = 64;        // alpha singles (K), one 128-byte swizzle span of FP16
constexpr int STAGES = 2;
constexpr int OP_TILE = BM * BK * 2;          // 16 KB: one FP16 operand tile (A or B)
constexpr int RAW_TILE = BK * BM * 4;         // 32 KB: the FP32 rows of one tile
constexpr int NTHREADS = 320;                 // 10 warps
constexpr int CONV0 = 2, EPI0 = 6;            // first converter / epilogue warp
constexpr long long WAIT_CYCLES = 4000000000LL;  // ~2 s at 2 GHz
constexpr int MAX_ROW = 12928;                // sigma row floats held in shared memory (n_beta <= this)
// shared memory: A hi/lo x STAGES, B hi/lo, raw x STAGES, sigma row, barriers
constexpr int SMEM_OPS = STAGES * 2 * OP_TILE + 2 * OP_TILE + STAGES * RAW_TILE;
constexpr int SMEM_BYTES = SMEM_OPS + MAX_ROW * 4 + 1024 + 256;

enum { ERR_RAW = 1, ERR_AEMPTY = 2, ERR_AFULL = 3, ERR_ACC = 4, ERR_B = 5 };

struct Args {
  const float *Xp;         // [v][na][nbp] planar input (FP32)
  float *Zp;               // [v][na][nbp] planar output
  const float *xmax;       // max |X| over the input (device scalar, written by the layout pass)
  int64_t na, nb, nbp;
  int nvp;
  int m_tiles;             // nbp / BM
  const int64_t *a_off;
  const int32_t *a_J, *a_info;
  const float *eab;        // (pair_alpha | pair_beta) row-major FP32
  int npair, n_off;        // beta pairs: all, off-diagonal (<= BN)
  float sw;                // power-of-two scale of the integrals
  const uint16_t *btab;    // [q][nb]: (Ib << 1 | phase) of the single of Jb through pair q, or 0xFFFF
  long long wait_cycles;
  int *err;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
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

// one-dimensional bulk copy global -> shared, completion counted on `bar` (16-byte aligned, size % 16 == 0)
__device__ __forceinline__ void bulk_load(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

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

// x = hi + lo with hi, lo in FP16 (x already scaled into FP16 range)
__device__ __forceinline__ void split_h(float x, __half &h, __half &l) {
  h = __float2half_rn(x);
  l = __float2half_rn(x - __half2float(h));
}

// 8 consecutive K values of row r -> one 16-byte chunk c of the 128-byte-swizzled K-major tile
__device__ __forceinline__ void store_chunk(unsigned char *tile, int r, int c, const __half (&v)[8]) {
  *reinterpret_cast<uint4 *>(tile + r * 128 + ((c ^ (r & 7)) << 4)) = *reinterpret_cast<const uint4 *>(v);
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
  unsigned char *a_hi = smem;                                   // [STAGES] x 16 KB
  unsigned char *a_lo = a_hi + STAGES * OP_TILE;                // [STAGES] x 16 KB
  unsigned char *b_hi = a_lo + STAGES * OP_TILE;                // 16 KB
  unsigned char *b_lo = b_hi + OP_TILE;                         // 16 KB
  float *raw = reinterpret_cast<float *>(b_lo + OP_TILE);       // [STAGES][BK][BM]
  float *srow = raw + STAGES * BK * BM;                         // [MAX_ROW]
  uint64_t *bars = reinterpret_cast<uint64_t *>(srow + MAX_ROW);
  uint64_t *raw_full = bars, *raw_empty = bars + 2, *a_full = bars + 4, *a_empty = bars + 6;
  uint64_t *acc_full = bars + 8, *acc_empty = bars + 10, *b_full = bars + 12, *b_empty = bars + 13, *drain = bars + 14;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 15);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; s++) {
      mbar_init(smem_u32(raw_full + s), 1);
      mbar_init(smem_u32(raw_empty + s), 4);
      mbar_init(smem_u32(a_full + s), 4);
      mbar_init(smem_u32(a_empty + s), 1);
      mbar_init(smem_u32(acc_full + s), 1);
      mbar_init(smem_u32(acc_empty + s), 4);
    }
    mbar_init(smem_u32(b_full), 4);
    mbar_init(smem_u32(b_empty), 1);
    mbar_init(smem_u32(drain), 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(2 * BN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const int mt = g.m_tiles;

  if (warp == 0) {
    // ---- producer: 512-byte rows of X_v, one per alpha single, per tile
    int seq = 0;
    bool stop = false;
    for (int64_t ia = blockIdx.x; ia < g.na && !stop; ia += gridDim.x) {
      const int64_t base = g.a_off[ia];
      const int n1 = (int)(g.a_off[ia + 1] - base);
      const int ja0 = lane < n1 ? g.a_J[base + lane] : 0;
      const int ja1 = lane + 32 < n1 ? g.a_J[base + lane + 32] : 0;
      for (int v = 0; v < g.nvp && !stop; v++) {
        const float *xv = g.Xp + (int64_t)v * g.na * g.nbp;
        for (int t = 0; t < mt; t++) {
          const int s = seq & 1;
          const uint32_t ph = (uint32_t)((seq >> 1) & 1);
          if (!warp_wait(smem_u32(raw_empty + s), ph ^ 1u, g.wait_cycles)) {
            if (lane == 0) atomicCAS(g.err, 0, ERR_RAW);
            *abort_flag = 1;
            stop = true;
            break;
          }
          if (warp_aborted(abort_flag)) {
            stop = true;
            break;
          }
          const uint32_t bar = smem_u32(raw_full + s);
          if (lane == 0) mbar_expect_tx(bar, (uint32_t)(n1 * BM * 4));
          __syncwarp();
          float *dst = raw + s * BK * BM;
          const int64_t col = (int64_t)t * BM;
          if (lane < n1) bulk_load(smem_u32(dst + lane * BM), xv + ja0 * g.nbp + col, BM * 4, bar);
          if (lane + 32 < n1) bulk_load(smem_u32(dst + (lane + 32) * BM), xv + ja1 * g.nbp + col, BM * 4, bar);
          seq++;
        }
      }
    }
    // the copies of the last stages must have landed before the CTA exits
    if (lane == 0)
      for (int j = seq > STAGES ? seq - STAGES : 0; j < seq; j++)
        mbar_wait(smem_u32(raw_full + (j & 1)), (uint32_t)((j >> 1) & 1), WAIT_CYCLES);
    __syncwarp();
  } else if (warp == 1) {
    // ---- MMA issuer
    if (lane == 0) {
      int seq = 0, grp = 0;
      bool ok = true;
      for (int64_t ia = blockIdx.x; ia < g.na && ok && !*abort_flag; ia += gridDim.x, grp++) {
        if (!mbar_wait(smem_u32(b_full), (uint32_t)(grp & 1), g.wait_cycles)) {
          atomicCAS(g.err, 0, ERR_B);
          *abort_flag = 1;
          break;
        }
        for (int v = 0; v < g.nvp && ok; v++) {
          for (int t = 0; t < mt; t++, seq++) {
            const int s = seq & 1, a = seq & 1;
            const uint32_t ph = (uint32_t)((seq >> 1) & 1);
            if (!mbar_wait(smem_u32(acc_empty + a), ph ^ 1u, g.wait_cycles)) {
              atomicCAS(g.err, 0, ERR_ACC);
              ok = false;
              break;
            }
            if (!mbar_wait(smem_u32(a_full + s), ph, g.wait_cycles)) {
              atomicCAS(g.err, 0, ERR_AFULL);
              ok = false;
              break;
            }
            if (*abort_flag) {
              ok = false;
              break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t d = tmem + (uint32_t)(a * BN);
            const uint32_t ah = smem_u32(a_hi + s * OP_TILE), al = smem_u32(a_lo + s * OP_TILE);
            const uint32_t bh = smem_u32(b_hi), bl = smem_u32(b_lo);
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
        }
        if (!ok) {
          *abort_flag = 1;
          break;
        }
        mma_commit(smem_u32(b_empty));  // B of this alpha string is free once its MMAs completed
      }
      // every MMA issued here has completed before TMEM is freed
      mma_commit(smem_u32(drain));
      mbar_wait(smem_u32(drain), 0, WAIT_CYCLES);
    }
    __syncwarp();
  } else if (warp < EPI0) {
    // ---- converters: B per alpha string, A per tile; thread <-> operand row
    const int r = threadIdx.x - 32 * CONV0;  // 0..127
    int seq = 0, grp = 0;
    bool stop = false;
    for (int64_t ia = blockIdx.x; ia < g.na && !stop; ia += gridDim.x, grp++) {
      const int64_t base = g.a_off[ia];
      const int n1 = (int)(g.a_off[ia + 1] - base);
      if (!warp_wait(smem_u32(b_empty), (uint32_t)(grp & 1) ^ 1u, g.wait_cycles)) {
        if (lane == 0) atomicCAS(g.err, 0, ERR_B);
        *abort_flag = 1;
        break;
      }
      if (warp_aborted(abort_flag)) break;
      {
        // B[q][k] = s_k (pair_k | q) * sw for the off-diagonal beta pair q = r
        int i = 1;
        while ((i + 1) * i / 2 <= r) i++;  // r = i(i-1)/2 + j with j < i
        const int qfull = r + i;           // idx2(i, j) = i(i+1)/2 + j
        const bool qv = r < g.n_off;
        for (int c = 0; c < BK / 8; c++) {
          __half h[8], l[8];
#pragma unroll
          for (int e = 0; e < 8; e++) {
            const int k = c * 8 + e;
            float w = 0.0f;
            if (qv && k < n1) {
              const int info = __ldg(g.a_info + base + k);
              w = __ldg(g.eab + (int64_t)(info >> 1) * g.npair + qfull) * g.sw;
              if (info & 1) w = -w;
            }
            split_h(w, h[e], l[e]);
          }
          store_chunk(b_hi, r, c, h);
          store_chunk(b_lo, r, c, l);
        }
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_u32(b_full));
      const float sx = fp16_scale(*g.xmax);
      for (int v = 0; v < g.nvp && !stop; v++) {
        for (int t = 0; t < mt; t++) {
          const int s = seq & 1;
          const uint32_t ph = (uint32_t)((seq >> 1) & 1);
          bool ok = warp_wait(smem_u32(raw_full + s), ph, g.wait_cycles);
          if (ok) ok = warp_wait(smem_u32(a_empty + s), ph ^ 1u, g.wait_cycles);
          if (!ok) {
            if (lane == 0) atomicCAS(g.err, 0, ERR_AEMPTY);
            *abort_flag = 1;
            stop = true;
            break;
          }
          if (warp_aborted(abort_flag)) {
            stop = true;
            break;
          }
          const float *src = raw + s * BK * BM;
          unsigned char *th = a_hi + s * OP_TILE, *tl = a_lo + s * OP_TILE;
          for (int c = 0; c < BK / 8; c++) {
            __half h[8], l[8];
#pragma unroll
            for (int e = 0; e < 8; e++) {
              const int k = c * 8 + e;
              const float x = k < n1 ? src[k * BM + r] * sx : 0.0f;
              split_h(x, h[e], l[e]);
            }
            store_chunk(th, r, c, h);
            store_chunk(tl, r, c, l);
          }
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          __syncwarp();
          if (lane == 0) {
            mbar_arrive(smem_u32(a_full + s));
            mbar_arrive(smem_u32(raw_empty + s));
          }
          seq++;
        }
      }
    }
  } else {
    // ---- epilogue: accumulator -> scatter into the sigma row -> Z_v[ia].  The four epilogue warps meet at
    // named barriers, so none of them leaves the loop early: after an abort they skip the work but keep
    // the same sequence of barriers.
    const int q = warp & 3;                  // TMEM lane quadrant of this warp
    const int et = threadIdx.x - 32 * EPI0;  // 0..127
    int seq = 0;
    bool dead = false;
    for (int i = et; i < MAX_ROW; i += 128) srow[i] = 0.0f;
    asm volatile("bar.sync 1, 128;" ::: "memory");
    const float inv = 1.0f / (fp16_scale(*g.xmax) * g.sw);
    for (int64_t ia = blockIdx.x; ia < g.na; ia += gridDim.x) {
      for (int v = 0; v < g.nvp; v++) {
        for (int t = 0; t < mt; t++, seq++) {
          if (dead) continue;
          const int a = seq & 1;
          const uint32_t ph = (uint32_t)((seq >> 1) & 1);
          if (!warp_wait(smem_u32(acc_full + a), ph, g.wait_cycles)) {
            if (lane == 0) atomicCAS(g.err, 0, ERR_ACC);
            *abort_flag = 1;
            dead = true;
            continue;
          }
          if (warp_aborted(abort_flag)) {
            dead = true;
            continue;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const int64_t jb = (int64_t)t * BM + q * 32 + lane;
          const bool live = jb < g.nb;
          const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(a * BN);
#pragma unroll 1
          for (int c0 = 0; c0 < BN; c0 += 32) {
            float d[32];
            tmem_ld32(taddr + c0, d);
            if (live && c0 < g.n_off) {
              const uint16_t *tb = g.btab + (int64_t)c0 * g.nb + jb;
#pragma unroll
              for (int j = 0; j < 32; j++) {
                const uint16_t e = __ldg(tb + (int64_t)j * g.nb);
                if (e != 0xFFFFu) atomicAdd(srow + (e >> 1), (e & 1) ? -d[j] : d[j]);
              }
            }
          }
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
          __syncwarp();
          if (lane == 0) mbar_arrive(smem_u32(acc_empty + a));
        }
        asm volatile("bar.sync 1, 128;" ::: "memory");
        float *z = g.Zp + ((int64_t)v * g.na + ia) * g.nbp;
        for (int i = et; i < g.nbp; i += 128) {
          if (!dead) z[i] = srow[i] * inv;
          srow[i] = 0.0f;
        }
        asm volatile("bar.sync 1, 128;" ::: "memory");
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * BN) : "memory");
}

}  // namespace abtc
}  // namespace pq

namespace pq {
namespace abtc {

// btab[q][Jb] for every beta single of Jb: q = off-diagonal index of its pair, entry (Ib << 1 | phase)
__global__ void btab_kernel(const int64_t *off, const int32_t *J, const int32_t *info, int64_t nb, uint16_t *btab) {
  const int64_t jb = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (jb >= nb) return;
  for (int64_t e = off[jb]; e < off[jb + 1]; e++) {
    const int pr = info[e] >> 1;  // idx2(i, j) with i > j for a single
    int i = 1;
    while ((i + 1) * (i + 2) / 2 <= pr) i++;  // largest i with i(i+1)/2 <= pr
    const int q = pr - i;                     // i(i-1)/2 + j
    btab[(int64_t)q * nb + jb] = (uint16_t)(((uint32_t)J[e] << 1) | (uint32_t)(info[e] & 1));
  }
}

// Xp[v][a][b] = X[(a * nb + b) * NV + v] (rows padded to nbp; the padding is left as it is), and
// xmax = max |X| (as the bit pattern of a non-negative float, so integer max orders it)
template <int NV>
__global__ void to_planar_kernel(const float *X, int64_t na, int64_t nb, int64_t nbp, float *Xp, unsigned *xmax) {
  float m = 0.0f;
  const int64_t n = na * nb;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = i / nb, b = i - a * nb;
#pragma unroll
    for (int v = 0; v < NV; v++) {
      const float x = X[i * NV + v];
      Xp[((int64_t)v * na + a) * nbp + b] = x;
      m = fmaxf(m, fabsf(x));
    }
  }
  for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(xmax, __float_as_uint(m));
}

// Y[(a * nb + b) * NV + v] += Zp[v][a][b]
template <int NV>
__global__ void planar_add_kernel(const float *Zp, int64_t na, int64_t nb, int64_t nbp, float *Y) {
  const int64_t n = na * nb;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = i / nb, b = i - a * nb;
#pragma unroll
    for (int v = 0; v < NV; v++) Y[i * NV + v] += Zp[((int64_t)v * na + a) * nbp + b];
  }
}

}  // namespace abtc

// The tensor-core alpha-beta path applies to one-species full CI with at most
// 16 orbitals (the 120 off-diagonal beta pairs fit N = 128), at most 64 alpha
// singles per string (K = 64) and a beta row that fits shared memory.
bool sigma32_tc_applicable(const pq_ci_handle *h) {
  if (h->n_species != 1 || !h->full) return false;
  const int n = h->n_orb[0];
  if (n > 16 || n * (n - 1) / 2 > abtc::BN) return false;
  if (h->tab[0][0].max1 > abtc::BK) return false;
  const int64_t nb = h->tab[0][1].n_str;
  return nb <= abtc::MAX_ROW && nb < 32768;
}

template <int NV>
static pq_status ab_tc_impl(pq_ci_handle *h, const float *X, float *Y) {
  using namespace abtc;
  cudaStream_t st = h->stream;
  const int64_t na = h->tab[0][0].n_str, nb = h->tab[0][1].n_str;
  const int64_t nbp = (nb + BM - 1) / BM * BM;
  const int n = h->n_orb[0], npair = h->npair[0];
  if (!h->tc_ready) {
    // one-off: the beta scatter table, the integral scale, the kernel's shared-memory limit
    PQ_TRY(h->tc_btab.alloc(sizeof(uint16_t) * (size_t)BN * nb + 16));
    PQ_CUDA_TRY(cudaMemsetAsync(h->tc_btab.ptr, 0xFF, sizeof(uint16_t) * (size_t)BN * nb, st));
    const SpinTablesDev &tb = h->tab[0][1];
    btab_kernel<<<(unsigned)((nb + 255) / 256), 256, 0, st>>>(tb.s1_off.as<int64_t>(), tb.s1_J.as<int32_t>(),
                                                            tb.s1_info.as<int32_t>(), nb, h->tc_btab.as<uint16_t>());
    PQ_CUDA_TRY(cudaGetLastError());
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
  const size_t planar = sizeof(float) * (size_t)NV * na * nbp;
  if (h->tc_xp.bytes < planar) {
    PQ_TRY(h->tc_xp.alloc(planar));
    PQ_CUDA_TRY(cudaMemsetAsync(h->tc_xp.ptr, 0, planar, st));  // the row padding stays zero
  }
  PQ_TRY(h->tc_zp.ensure(planar));
  unsigned *xmax = h->tc_aux.as<unsigned>();
  int *err = reinterpret_cast<int *>(xmax + 1);
  PQ_CUDA_TRY(cudaMemsetAsync(h->tc_aux.ptr, 0, 8, st));
  const unsigned g = (unsigned)std::min<int64_t>((na * nb + 255) / 256, 152 * 16);
  to_planar_kernel<NV><<<g, 256, 0, st>>>(X, na, nb, nbp, h->tc_xp.as<float>(), xmax);
  PQ_CUDA_TRY(cudaGetLastError());
  Args a{};
  a.Xp = h->tc_xp.as<float>();
  a.Zp = h->tc_zp.as<float>();
  a.xmax = reinterpret_cast<const float *>(xmax);
  a.na = na;
  a.nb = nb;
  a.nbp = nbp;
  a.nvp = NV;
  a.m_tiles = (int)(nbp / BM);
  const SpinTablesDev &ta = h->tab[0][0];
  a.a_off = ta.s1_off.as<int64_t>();
  a.a_J = ta.s1_J.as<int32_t>();
  a.a_info = ta.s1_info.as<int32_t>();
  a.eab = h->d_eab32.as<float>();
  a.npair = npair;
  a.n_off = n * (n - 1) / 2;
  a.sw = h->tc_sw;
  a.btab = h->tc_btab.as<uint16_t>();
  a.wait_cycles = WAIT_CYCLES;
  a.err = err;
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
  planar_add_kernel<NV><<<g, 256, 0, st>>>(h->tc_zp.as<float>(), na, nb, nbp, Y);
  PQ_CUDA_TRY(cudaGetLastError());
  return PQ_OK;
}

pq_status ci_sigma32_ab_tc(pq_ci_handle *h, const void *X, void *Y, int nvp) {
  if (nvp == 1) return ab_tc_impl<1>(h, (const float *)X, (float *)Y);
  if (nvp == 2) return ab_tc_impl<2>(h, (const float *)X, (float *)Y);
  if (nvp == 4) return ab_tc_impl<4>(h, (const float *)X, (float *)Y);
  set_error("sigma32 tensor-core path: unsupported width %d", nvp);
  return PQ_ERR_ARG;
}

}  // namespace pq
