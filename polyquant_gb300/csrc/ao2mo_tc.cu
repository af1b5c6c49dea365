// Split-precision AO->MO transform on the tcgen05 tensor cores.
//
// Same two pair-symmetric half transforms as the FP64 path (ao2mo.cu): for
// each slice S (a symmetric n x n matrix: one ket AO pair in half 1, one bra MO
// pair in half 2), T = C^T S C, written packed (i >= j).  Each slice costs two
// GEMMs, both in the "A (M x K, K-major) times B (N x K, K-major)^T" form:
//   GEMM 1:  U^T[m][nu] = sum_mu Ct[m][mu] S[nu][mu]    (A = C^T shared, B = S per slice)
//   GEMM 2:  T[m][n]   = sum_nu U^T[m][nu] Ct[n][nu]    (A = U^T per slice, B = C^T shared)
// Operands are split into a high and a low part (x = x_hi + x_lo) in BF16 or
// TF32 and each product is formed as hi*hi + hi*lo + lo*hi with FP32
// accumulation in tensor memory (three MMAs per K step).  BF16 and TF32 keep
// FP32's 8-bit exponent, so no per-block scaling is needed for range.
//
// GEMM kernel: persistent, one CTA per SM looping over 128 x 256 output
// tiles, warp-specialised: one thread issues TMA tile loads (128-byte
// swizzle, a ring of two stages of K = 128 bytes of each of A_hi, A_lo, B_hi,
// B_lo), one thread issues the tcgen05.mma instructions into one of two TMEM
// accumulators (128 lanes x 256 FP32 columns each), and four warps drain the
// other accumulator with tcgen05.ld for the epilogue (BF16/TF32 split of the
// result for the next GEMM, or the packed lower triangle).  Every mbarrier
// wait is bounded; a wait that runs out records an error code and the kernel
// winds down (waits, bounded again, for its own loads and MMAs, frees TMEM).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "pq_internal.h"

namespace pq {

namespace tc {

constexpr int BM = 128;          // output rows per CTA (TMEM lanes)
constexpr int BN = 256;          // output columns per CTA (TMEM columns, UMMA N)
constexpr int ROW_BYTES = 128;   // K extent of one stage, in bytes (one swizzle span)
// Persistent warp-specialised GEMM: one CTA per SM, a ring of two 96 KB
// operand stages, and two TMEM accumulators (2 x 256 columns) so the epilogue
// of one tile overlaps the loads and MMAs of the next.
constexpr int STAGES = 2;
constexpr int A_TILE = BM * ROW_BYTES;  // 16 KB
constexpr int B_TILE = BN * ROW_BYTES;  // 32 KB
constexpr int STAGE_BYTES = 2 * A_TILE + 2 * B_TILE;
constexpr int EPI_WARPS = 4;
constexpr int EPI_LD = 33;                                  // per-warp 32 x 32 staging, odd stride
constexpr int EPI_BYTES = EPI_WARPS * 32 * EPI_LD * 4;      // 16.5 KB
constexpr int NBARS = 2 * STAGES + 4 + 1;                   // full, empty, acc_full[2], acc_empty[2], drain
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + EPI_BYTES + 1024 /*align*/ + 256 /*barriers, slots*/;
constexpr int GEMM_THREADS = 64 + 32 * EPI_WARPS;           // producer warp, MMA warp, epilogue warps
constexpr long long WAIT_CYCLES = 4000000000LL;  // ~2 s at 2 GHz

enum { EPI_SPLIT = 0, EPI_PACK = 1 };
enum { ERR_TIMEOUT_FULL = 1, ERR_TIMEOUT_MMA = 2, ERR_TIMEOUT_ACC = 3 };

struct GemmArgs {
  int M, N, K;                 // logical sizes
  int m_tiles;                 // ceil(M / BM)
  int nbatch;                  // batch entries (tiles = nbatch * m_tiles)
  int a_batched, b_batched;    // operand varies with the batch index
  int a_rows, b_rows;          // rows per batch in the operand tensors
  int ld_out;                  // EPI_SPLIT: row length of the split output
  void *out_hi, *out_lo;       // EPI_SPLIT outputs [b][M][ld_out]
  float *out_pack;             // EPI_PACK output [b][M(M+1)/2]
  int64_t pack_stride;         // elements per batch of out_pack
  long long wait_cycles;       // budget of the pipeline waits (the wind-down waits keep WAIT_CYCLES)
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
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, long long budget = WAIT_CYCLES) {
  const long long t0 = clock64();
  while (!mbar_try(bar, parity)) {
    if (clock64() - t0 > budget) return false;
  }
  return true;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

// UMMA shared-memory descriptor: K-major, 128-byte swizzle, 8-row groups 1024 B apart
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFF) >> 4);        // start address
  d |= (uint64_t)1 << 16;                         // leading byte offset (unused for this layout)
  d |= (uint64_t)(1024 >> 4) << 32;               // stride byte offset: 8 rows x 128 B
  d |= (uint64_t)1 << 46;                         // descriptor version for tcgen05
  d |= (uint64_t)2 << 61;                         // 128-byte swizzle
  return d;
}

// instruction descriptor: D = F32, A/B format (1 = BF16 for kind::f16, 2 = TF32), K-major A and B
__host__ __device__ constexpr uint32_t instr_desc(uint32_t ab_format) {
  return (1u << 4) | (ab_format << 7) | (ab_format << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
}

template <bool TF32>
__device__ __forceinline__ void mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accum) {
  if constexpr (TF32) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accum)
        : "memory");
  } else {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accum)
        : "memory");
  }
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

__device__ __forceinline__ float tf32_round(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// TF32 = operands stored as FP32 (tf32-rounded); otherwise BF16.
// Roles: warp 0 lane 0 issues TMA loads into the stage ring, warp 1 lane 0
// issues the MMAs (tile i into accumulator i & 1), warps 2..5 drain the
// accumulators (warp w reads TMEM lanes 32 (w & 3) .. + 31) through a
// per-warp shared-memory staging block into coalesced row stores.  Barriers:
// full[s] (loads landed), empty[s] (MMAs reading stage s done), acc_full[a]
// (tile's MMAs done), acc_empty[a] (epilogue done with accumulator a).  Every
// wait is bounded; a wait that runs out sets the error word and an abort flag
// that every role polls, the producer then waits (bounded) for its own loads
// in flight, the MMA thread for its own MMAs, and the CTA frees TMEM.
template <bool TF32, int EPI>
__global__ void __launch_bounds__(GEMM_THREADS, 1)
    tc_gemm_kernel(const __grid_constant__ CUtensorMap tmA_hi, const __grid_constant__ CUtensorMap tmA_lo,
                   const __grid_constant__ CUtensorMap tmB_hi, const __grid_constant__ CUtensorMap tmB_lo, GemmArgs g) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // 1024-byte alignment of the shared-window address (128-byte swizzle atoms)
  unsigned char *smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  float *epi = reinterpret_cast<float *>(smem + STAGES * STAGE_BYTES);
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + STAGES * STAGE_BYTES + EPI_BYTES);
  uint64_t *full = bars, *empty = bars + STAGES, *accf = bars + 2 * STAGES, *acce = bars + 2 * STAGES + 2;
  uint64_t *drain = bars + 2 * STAGES + 4;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + NBARS);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int ESZ = TF32 ? 4 : 2;
  constexpr int BK = ROW_BYTES / ESZ;  // K elements per stage
  constexpr int UK = TF32 ? 8 : 16;    // K per MMA instruction
  const int nst = (g.K + BK - 1) / BK;
  const int n_tiles = g.nbatch * g.m_tiles;

  if (threadIdx.x == 0) {
    for (int i = 0; i < STAGES; i++) {
      mbar_init(smem_u32(full + i), 1);
      mbar_init(smem_u32(empty + i), 1);
    }
    for (int a = 0; a < 2; a++) {
      mbar_init(smem_u32(accf + a), 1);
      mbar_init(smem_u32(acce + a), EPI_WARPS);
    }
    mbar_init(smem_u32(drain), 1);
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

  if (warp == 0 && lane == 0) {
    // ---- producer
    int gs = 0;
    for (int t = blockIdx.x; t < n_tiles && !*abort_flag; t += gridDim.x) {
      const int b = t / g.m_tiles, mt = t - b * g.m_tiles;
      const int ya = (g.a_batched ? b * g.a_rows : 0) + mt * BM;
      const int yb = g.b_batched ? b * g.b_rows : 0;
      for (int s = 0; s < nst; s++, gs++) {
        const int slot = gs % STAGES;
        const uint32_t ph = (uint32_t)((gs / STAGES) & 1);
        if (!mbar_wait(smem_u32(empty + slot), ph ^ 1u, g.wait_cycles)) {
          atomicCAS(g.err, 0, ERR_TIMEOUT_MMA);
          *abort_flag = 1;
          break;
        }
        if (*abort_flag) break;
        unsigned char *st = smem + slot * STAGE_BYTES;
        const uint32_t bar = smem_u32(full + slot);
        mbar_expect_tx(bar, STAGE_BYTES);
        const int x = s * BK;
        tma_load_2d(smem_u32(st), &tmA_hi, x, ya, bar);
        tma_load_2d(smem_u32(st + A_TILE), &tmA_lo, x, ya, bar);
        tma_load_2d(smem_u32(st + 2 * A_TILE), &tmB_hi, x, yb, bar);
        tma_load_2d(smem_u32(st + 2 * A_TILE + B_TILE), &tmB_lo, x, yb, bar);
      }
    }
    // the loads of the last stages must have landed before the CTA exits
    for (int j = gs > STAGES ? gs - STAGES : 0; j < gs; j++)
      mbar_wait(smem_u32(full + (j % STAGES)), (uint32_t)((j / STAGES) & 1));
  } else if (warp == 1 && lane == 0) {
    // ---- MMA issuer
    const uint32_t idesc = instr_desc(TF32 ? 2u : 1u);
    int gs = 0, i = 0;
    for (int t = blockIdx.x; t < n_tiles && !*abort_flag; t += gridDim.x, i++) {
      const int a = i & 1;
      const uint32_t aph = (uint32_t)((i >> 1) & 1);
      if (!mbar_wait(smem_u32(acce + a), aph ^ 1u, g.wait_cycles)) {
        atomicCAS(g.err, 0, ERR_TIMEOUT_ACC);
        *abort_flag = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t d = tmem + (uint32_t)(a * BN);
      bool ok = true;
      for (int s = 0; s < nst; s++, gs++) {
        const int slot = gs % STAGES;
        const uint32_t ph = (uint32_t)((gs / STAGES) & 1);
        if (!mbar_wait(smem_u32(full + slot), ph, g.wait_cycles)) {
          atomicCAS(g.err, 0, ERR_TIMEOUT_FULL);
          *abort_flag = 1;
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        unsigned char *st = smem + slot * STAGE_BYTES;
        const uint32_t a_hi = smem_u32(st), a_lo = smem_u32(st + A_TILE);
        const uint32_t b_hi = smem_u32(st + 2 * A_TILE), b_lo = smem_u32(st + 2 * A_TILE + B_TILE);
#pragma unroll
        for (int kk = 0; kk < BK / UK; kk++) {
          const uint32_t off = kk * UK * ESZ;  // bytes along K inside the swizzle span
          const uint32_t acc0 = (s > 0 || kk > 0) ? 1u : 0u;
          mma<TF32>(d, smem_desc(a_hi + off), smem_desc(b_hi + off), idesc, acc0);
          mma<TF32>(d, smem_desc(a_hi + off), smem_desc(b_lo + off), idesc, 1u);
          mma<TF32>(d, smem_desc(a_lo + off), smem_desc(b_hi + off), idesc, 1u);
        }
        mma_commit(smem_u32(empty + slot));  // frees the stage once these MMAs completed
      }
      if (!ok) break;
      mma_commit(smem_u32(accf + a));
    }
    // every MMA issued by this thread has completed before TMEM is freed
    mma_commit(smem_u32(drain));
    mbar_wait(smem_u32(drain), 0);
  } else if (warp >= 2) {
    // ---- epilogue
    const int q = warp & 3;  // TMEM lane quadrant of this warp
    float *stg = epi + (warp - 2) * 32 * EPI_LD;
    int i = 0;
    for (int t = blockIdx.x; t < n_tiles; t += gridDim.x, i++) {
      const int a = i & 1;
      const uint32_t aph = (uint32_t)((i >> 1) & 1);
      const bool ok = mbar_wait(smem_u32(accf + a), aph, g.wait_cycles);
      if (!ok || *abort_flag) {
        if (!ok && lane == 0) atomicCAS(g.err, 0, ERR_TIMEOUT_ACC);
        *abort_flag = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int b = t / g.m_tiles, mt = t - b * g.m_tiles;
      const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(a * BN);
      const int row0 = mt * BM + q * 32;
      for (int c0 = 0; c0 < BN; c0 += 32) {
        float v[32];
        tmem_ld32(taddr + c0, v);  // v[j] = D[row0 + lane][c0 + j]
#pragma unroll
        for (int j = 0; j < 32; j++) stg[lane * EPI_LD + j] = v[j];
        __syncwarp();
        if constexpr (EPI == EPI_SPLIT) {
          // four lanes per row, eight consecutive columns per lane: 16-byte stores
          // (rows of ld_out = a multiple of 8 elements, so n0 keeps them aligned)
          const int cq = (lane & 3) * 8, n0 = c0 + cq;
#pragma unroll
          for (int it = 0; it < 4; it++) {
            const int rr = it * 8 + (lane >> 2), m = row0 + rr;
            if (m >= g.M || n0 >= g.N) continue;
            float x[8];
#pragma unroll
            for (int k = 0; k < 8; k++) x[k] = stg[rr * EPI_LD + cq + k];
            const int64_t o = ((int64_t)b * g.M + m) * g.ld_out + n0;
            if constexpr (TF32) {
              float h[8], l[8];
#pragma unroll
              for (int k = 0; k < 8; k++) {
                h[k] = tf32_round(x[k]);
                l[k] = tf32_round(x[k] - h[k]);
              }
              float *oh = static_cast<float *>(g.out_hi) + o, *ol = static_cast<float *>(g.out_lo) + o;
              if (n0 + 8 <= g.N) {
                reinterpret_cast<float4 *>(oh)[0] = make_float4(h[0], h[1], h[2], h[3]);
                reinterpret_cast<float4 *>(oh)[1] = make_float4(h[4], h[5], h[6], h[7]);
                reinterpret_cast<float4 *>(ol)[0] = make_float4(l[0], l[1], l[2], l[3]);
                reinterpret_cast<float4 *>(ol)[1] = make_float4(l[4], l[5], l[6], l[7]);
              } else {
                for (int k = 0; k < g.N - n0; k++) oh[k] = h[k], ol[k] = l[k];
              }
            } else {
              __nv_bfloat162 h2[4], l2[4];
#pragma unroll
              for (int k = 0; k < 4; k++) {
                h2[k] = __floats2bfloat162_rn(x[2 * k], x[2 * k + 1]);
                l2[k] = __floats2bfloat162_rn(x[2 * k] - __low2float(h2[k]), x[2 * k + 1] - __high2float(h2[k]));
              }
              __nv_bfloat16 *oh = static_cast<__nv_bfloat16 *>(g.out_hi) + o;
              __nv_bfloat16 *ol = static_cast<__nv_bfloat16 *>(g.out_lo) + o;
              if (n0 + 8 <= g.N) {
                *reinterpret_cast<uint4 *>(oh) = *reinterpret_cast<const uint4 *>(h2);
                *reinterpret_cast<uint4 *>(ol) = *reinterpret_cast<const uint4 *>(l2);
              } else {
                const __nv_bfloat16 *hs = reinterpret_cast<const __nv_bfloat16 *>(h2);
                const __nv_bfloat16 *ls = reinterpret_cast<const __nv_bfloat16 *>(l2);
                for (int k = 0; k < g.N - n0; k++) oh[k] = hs[k], ol[k] = ls[k];
              }
            }
          }
        } else {
          const int n = c0 + lane;
          for (int rr = 0; rr < 32; rr++) {
            const int m = row0 + rr;
            if (m >= g.M) break;
            if (n <= m && n < g.N)
              g.out_pack[(int64_t)b * g.pack_stride + (int64_t)m * (m + 1) / 2 + n] = stg[rr * EPI_LD + lane];
          }
        }
        __syncwarp();
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_u32(acce + a));
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * BN) : "memory");
}

// ---------------------------------------------------------------------------
// operand preparation
template <bool TF32> struct Split;
// The split works in FP32: hi + lo carry at most 2 x 8 (BF16) or 2 x 11
// (TF32) significant bits, fewer than FP32's 24, and GB300 runs FP64
// arithmetic at a small fraction of the FP32 rate (one FP64 -> FP32
// conversion per element remains for FP64 sources).
template <> struct Split<false> {
  using T = __nv_bfloat16;
  static __device__ __forceinline__ void run(float x, T &h, T &l) {
    h = __float2bfloat16_rn(x);
    l = __float2bfloat16_rn(x - __bfloat162float(h));
  }
};
template <> struct Split<true> {
  using T = float;
  static __device__ __forceinline__ void run(float x, T &h, T &l) {
    h = tf32_round(x);
    l = tf32_round(x - h);
  }
};

// Ct[m][mu] = C[mu + m*ldc], split, row length ld (>= n_ao)
template <bool TF32>
__global__ void split_ct_kernel(const double *C, int64_t ldc, int n_ao, int n_mo, int ld, typename Split<TF32>::T *hi,
                                typename Split<TF32>::T *lo) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)n_mo * ld) return;
  int m = (int)(i / ld), mu = (int)(i - (int64_t)m * ld);
  float x = mu < n_ao ? (float)C[mu + (int64_t)m * ldc] : 0.0f;
  Split<TF32>::run(x, hi[i], lo[i]);
}

__device__ __forceinline__ int64_t tri64(int64_t i, int64_t j) { return i > j ? i * (i + 1) / 2 + j : j * (j + 1) / 2 + i; }

// slice b of a pair-matrix source, split: S[b][nu][mu] = src(tri(mu,nu), b0 + b)
// src64: column-major (ld x ncols) FP64 pair matrix (element (r, c) at r + c*ld)
// src32: row-major FP32 pair rows (element (r, c) at c*ld + r), i.e. row c holds the slice
// Split two consecutive row elements (a at o, b at o + 1; o even, so the pair
// is 4-byte (BF16) or 8-byte (TF32) aligned) into hi/lo with one vector store
// each when both are wanted.
template <bool TF32>
__device__ __forceinline__ void split_store2(typename Split<TF32>::T *H, typename Split<TF32>::T *L, int64_t o, float a,
                                             float b, bool va, bool vb) {
  if (va && vb) {
    if constexpr (TF32) {
      const float ha = tf32_round(a), hb = tf32_round(b);
      *reinterpret_cast<float2 *>(H + o) = make_float2(ha, hb);
      *reinterpret_cast<float2 *>(L + o) = make_float2(tf32_round(a - ha), tf32_round(b - hb));
    } else {
      const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
      *reinterpret_cast<__nv_bfloat162 *>(H + o) = h;
      *reinterpret_cast<__nv_bfloat162 *>(L + o) = __floats2bfloat162_rn(a - __low2float(h), b - __high2float(h));
    }
  } else {
    if (va) Split<TF32>::run(a, H[o], L[o]);
    if (vb) Split<TF32>::run(b, H[o + 1], L[o + 1]);
  }
}

// One block per (slice, 32x32 tile of the lower triangle): the tile is read
// with consecutive pair indices (mu <= nu) and written to both triangles, the
// upper one through a shared-memory transpose, so loads and stores are
// coalesced and every slice spreads over many SMs.  Each thread handles two
// consecutive columns (16 column pairs x 16 rows per pass).
template <bool TF32>
__global__ void __launch_bounds__(256) split_slices_kernel(const double *src64, const float *src32, int64_t ld, int n,
                                                           int ld_row, int64_t b0, typename Split<TF32>::T *hi,
                                                           typename Split<TF32>::T *lo) {
  __shared__ float tile[32][33];
  const int nt = (n + 31) / 32;
  const int tv = blockIdx.y / nt, tm = blockIdx.y - tv * nt;
  if (tm > tv) return;
  const int64_t b = blockIdx.x, c = b0 + b;
  typename Split<TF32>::T *H = hi + b * (int64_t)n * ld_row, *L = lo + b * (int64_t)n * ld_row;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  for (int y = ty; y < 32; y += 16) {
    const int nu = tv * 32 + y, mu = tm * 32 + 2 * tx;
    const bool va = nu < n && mu <= nu, vb = nu < n && mu + 1 <= nu;
    float xa = 0.0f, xb = 0.0f;
    const int64_t pr = (int64_t)nu * (nu + 1) / 2 + mu;
    if (va) xa = src64 ? (float)src64[pr + c * ld] : src32[c * ld + pr];
    if (vb) xb = src64 ? (float)src64[pr + 1 + c * ld] : src32[c * ld + pr + 1];
    split_store2<TF32>(H, L, (int64_t)nu * ld_row + mu, xa, xb, va, vb);
    tile[y][2 * tx] = xa;
    tile[y][2 * tx + 1] = xb;
  }
  __syncthreads();
  for (int y = ty; y < 32; y += 16) {
    const int row = tm * 32 + y, nu = tv * 32 + 2 * tx;
    const bool va = nu < n && row < nu, vb = nu + 1 < n && row < nu + 1;
    split_store2<TF32>(H, L, (int64_t)row * ld_row + nu, tile[2 * tx][y], tile[2 * tx + 1][y], va, vb);
  }
}

// full column-major pair matrix from the 8-fold packed vector: one block per
// 32x32 tile of the lower triangle (row tile >= column tile), read along
// packed rows, written to both triangles through a shared-memory transpose
__global__ void __launch_bounds__(256) expand_packed8_kernel(const double *packed, int64_t np, double *full) {
  __shared__ double tile[32][33];
  const int64_t tr = blockIdx.y, tcol = blockIdx.x;
  if (tcol > tr) return;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int y = ty; y < 32; y += 8) {
    const int64_t r = tr * 32 + y, c = tcol * 32 + tx;
    double x = 0.0;
    if (r < np && c <= r) {
      x = packed[r * (r + 1) / 2 + c];
      full[r * np + c] = x;  // element (c, r): column r, contiguous in c
    }
    tile[y][tx] = x;
  }
  __syncthreads();
  for (int y = ty; y < 32; y += 8) {
    const int64_t c = tcol * 32 + y, r = tr * 32 + tx;
    if (r < np && c < r) full[c * np + r] = tile[tx][y];  // element (r, c): column c, contiguous in r
  }
}

// out[c*rows + r] = in[r*cols + c] (FP32 tiles), optionally widened to FP64
template <typename TO>
__global__ void transpose32_kernel(const float *in, int64_t rows, int64_t cols, TO *out) {
  __shared__ float tile[32][33];
  int64_t r0 = (int64_t)blockIdx.y * 32, c0 = (int64_t)blockIdx.x * 32;
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    int64_t r = r0 + y, c = c0 + threadIdx.x;
    if (r < rows && c < cols) tile[y][threadIdx.x] = in[r * cols + c];
  }
  __syncthreads();
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    int64_t c = c0 + y, r = r0 + threadIdx.x;
    if (r < rows && c < cols) out[c * rows + r] = (TO)tile[threadIdx.x][y];
  }
}

}  // namespace tc

// ---------------------------------------------------------------------------
// budget of the GEMM pipeline waits; pq_debug_set_wait_budget changes it for tests of the timeout path
static long long g_gemm_wait_cycles = tc::WAIT_CYCLES;

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  }
  return fn;
}

// 2-D tensor map over a row-major (rows x kdim) operand, box (BK x box_rows), 128-byte swizzle
static pq_status make_map(CUtensorMap *m, const void *base, bool tf32, int64_t rows, int64_t kdim, int64_t ld,
                          int box_rows) {
  auto fn = encode_fn();
  if (!fn) {
    set_error("cuTensorMapEncodeTiled is not available from the driver");
    return PQ_ERR_CUDA;
  }
  const int esz = tf32 ? 4 : 2;
  cuuint64_t dims[2] = {(cuuint64_t)kdim, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)(ld * esz)};
  cuuint32_t box[2] = {(cuuint32_t)(tc::ROW_BYTES / esz), (cuuint32_t)box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = fn(m, tf32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base),
                  dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d): rows=%lld k=%lld ld=%lld", (int)r, (long long)rows, (long long)kdim,
              (long long)ld);
    return PQ_ERR_CUDA;
  }
  return PQ_OK;
}

struct Operand {
  const void *hi, *lo;
  int64_t rows;  // total rows in memory
  int64_t ld;    // row length in elements
};

template <bool TF32, int EPI>
static pq_status run_gemm(const Operand &A, const Operand &B, bool a_batched, bool b_batched, int M, int N, int K,
                          int nbatch, const tc::GemmArgs &gin, cudaStream_t st) {
  CUtensorMap ma_hi, ma_lo, mb_hi, mb_lo;
  PQ_TRY(make_map(&ma_hi, A.hi, TF32, A.rows, K, A.ld, tc::BM));
  PQ_TRY(make_map(&ma_lo, A.lo, TF32, A.rows, K, A.ld, tc::BM));
  PQ_TRY(make_map(&mb_hi, B.hi, TF32, B.rows, K, B.ld, tc::BN));
  PQ_TRY(make_map(&mb_lo, B.lo, TF32, B.rows, K, B.ld, tc::BN));
  tc::GemmArgs g = gin;
  g.M = M;
  g.N = N;
  g.K = K;
  g.m_tiles = (M + tc::BM - 1) / tc::BM;
  g.a_batched = a_batched;
  g.b_batched = b_batched;
  g.a_rows = M;
  g.b_rows = N;
  g.nbatch = nbatch;
  g.wait_cycles = g_gemm_wait_cycles;
  auto kern = tc::tc_gemm_kernel<TF32, EPI>;
  PQ_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::SMEM_BYTES));
  int dev = 0, sms = 0;
  PQ_CUDA_TRY(cudaGetDevice(&dev));
  PQ_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int64_t tiles = (int64_t)nbatch * g.m_tiles;
  const int grid = (int)std::min<int64_t>(tiles, sms);  // persistent: one CTA per SM
  kern<<<grid, tc::GEMM_THREADS, tc::SMEM_BYTES, st>>>(ma_hi, ma_lo, mb_hi, mb_lo, g);
  PQ_CUDA_TRY(cudaGetLastError());
  return PQ_OK;
}

// Work buffers of the split-precision transform, kept per device between calls (grow-only) so that repeated
// transforms allocate nothing; calls on one device are serialised by the mutex (they share the buffers, and
// each call synchronises its stream before it returns).  pq_ao2mo_release_workspace frees them.
struct Ao2moWorkspace {
  DevBuf full, cth, ctl, sh, sl, uh, ul, H1, H1t, Erow, err;
};
static std::mutex g_ws_mu;
static Ao2moWorkspace g_ws[64];

template <bool TF32>
static pq_status ao2mo_tc_impl(const double *eri_ao, int layout, int64_t n, const double *C, int64_t ldc, int64_t nm,
                               double *eri_mo, cudaStream_t st) {
  using E = typename tc::Split<TF32>::T;
  const int64_t npa = n * (n + 1) / 2, npm = nm * (nm + 1) / 2;
  const int ld = (int)((n + 7) / 8 * 8);    // AO row length (16-byte rows for TMA)
  int dev = 0;
  PQ_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) {
    set_error("pq_ao2mo: device ordinal %d out of range", dev);
    return PQ_ERR_STATE;
  }
  std::lock_guard<std::mutex> lock(g_ws_mu);
  Ao2moWorkspace &w = g_ws[dev];
  DevBuf &full = w.full, &cth = w.cth, &ctl = w.ctl, &sh = w.sh, &sl = w.sl, &uh = w.uh, &ul = w.ul, &H1 = w.H1,
         &H1t = w.H1t, &err = w.err;
  const double *pairs = eri_ao;
  if (layout == PQ_AO_PACKED8) {
    PQ_TRY(full.ensure(sizeof(double) * npa * npa));
    const unsigned nt = (unsigned)((npa + 31) / 32);
    if (nt > 65535) {
      set_error("ao2mo: too many pairs for the expansion grid");
      return PQ_ERR_ARG;
    }
    tc::expand_packed8_kernel<<<dim3(nt, nt), 256, 0, st>>>(eri_ao, npa, full.as<double>());
    PQ_CUDA_TRY(cudaGetLastError());
    pairs = full.as<double>();
  }
  PQ_TRY(err.ensure(sizeof(int)));
  PQ_CUDA_TRY(cudaMemsetAsync(err.ptr, 0, sizeof(int), st));
  // C^T split, rows = MO, row length ld (AO)
  PQ_TRY(cth.ensure(sizeof(E) * nm * ld));
  PQ_TRY(ctl.ensure(sizeof(E) * nm * ld));
  tc::split_ct_kernel<TF32><<<(unsigned)((nm * ld + 255) / 256), 256, 0, st>>>(C, ldc, (int)n, (int)nm, ld, cth.as<E>(),
                                                                               ctl.as<E>());
  PQ_CUDA_TRY(cudaGetLastError());
  // slices per batch: S (n x ld) and U^T (nm x ld) in hi/lo
  const int64_t bt = std::max<int64_t>(1, std::min<int64_t>(std::max(npa, npm), 4096));
  PQ_TRY(sh.ensure(sizeof(E) * bt * n * ld));
  PQ_TRY(sl.ensure(sizeof(E) * bt * n * ld));
  PQ_TRY(uh.ensure(sizeof(E) * bt * nm * ld));
  PQ_TRY(ul.ensure(sizeof(E) * bt * nm * ld));
  PQ_TRY(H1.ensure(sizeof(float) * npa * npm));
  tc::GemmArgs g{};
  g.err = err.as<int>();
  Operand ct{cth.ptr, ctl.ptr, nm, ld};
  auto half = [&](const double *src64, const float *src32, int64_t ld_src, int64_t nslices, float *out) -> pq_status {
    for (int64_t b0 = 0; b0 < nslices; b0 += bt) {
      const int nb = (int)std::min(bt, nslices - b0);
      const unsigned ntile = (unsigned)((n + 31) / 32);
      tc::split_slices_kernel<TF32><<<dim3((unsigned)nb, ntile * ntile), 256, 0, st>>>(src64, src32, ld_src, (int)n, ld,
                                                                                      b0, sh.as<E>(), sl.as<E>());
      PQ_CUDA_TRY(cudaGetLastError());
      // GEMM 1: U^T[b] (nm x n) = Ct (nm x n) . S[b]^T, K = n
      Operand S{sh.ptr, sl.ptr, (int64_t)nb * n, ld};
      tc::GemmArgs g1 = g;
      g1.out_hi = uh.ptr;
      g1.out_lo = ul.ptr;
      g1.ld_out = ld;
      PQ_TRY((run_gemm<TF32, tc::EPI_SPLIT>(ct, S, false, true, (int)nm, (int)n, (int)n, nb, g1, st)));
      // GEMM 2: T[b] (nm x nm) = U^T[b] . Ct^T, K = n; packed lower triangle
      Operand U{uh.ptr, ul.ptr, (int64_t)nb * nm, ld};
      tc::GemmArgs g2 = g;
      g2.out_pack = out + b0 * npm;
      g2.pack_stride = npm;
      PQ_TRY((run_gemm<TF32, tc::EPI_PACK>(U, ct, true, false, (int)nm, (int)nm, (int)n, nb, g2, st)));
    }
    return PQ_OK;
  };
  // half 1 over AO ket pairs: H1[ket][ij]
  PQ_TRY(half(pairs, nullptr, npa, npa, H1.as<float>()));
  // H1t[ij][ket], in the expanded pair matrix's memory when there is one (it is not read again):
  // each reuse saves an allocation and a synchronising free inside the call
  float *h1t = nullptr;
  if (layout == PQ_AO_PACKED8 && full.bytes >= sizeof(float) * npa * npm) {
    h1t = full.as<float>();
  } else {
    PQ_TRY(H1t.ensure(sizeof(float) * npa * npm));
    h1t = H1t.as<float>();
  }
  {
    dim3 grid((unsigned)((npm + 31) / 32), (unsigned)((npa + 31) / 32));
    if (grid.y > 65535) {
      set_error("ao2mo: too many pairs for the transpose grid");
      return PQ_ERR_ARG;
    }
    tc::transpose32_kernel<float><<<grid, dim3(32, 8), 0, st>>>(H1.as<float>(), npa, npm, h1t);
    PQ_CUDA_TRY(cudaGetLastError());
  }
  // half 2 over MO bra pairs: Erow[ij][kl], in H1's memory when it fits (npm <= npa); slices read from rows of H1t
  float *erow = H1.as<float>();
  if (npm > npa) {
    PQ_TRY(w.Erow.ensure(sizeof(float) * npm * npm));
    erow = w.Erow.as<float>();
  }
  PQ_TRY(half(nullptr, h1t, npa, npm, erow));
  {
    dim3 grid((unsigned)((npm + 31) / 32), (unsigned)((npm + 31) / 32));
    tc::transpose32_kernel<double><<<grid, dim3(32, 8), 0, st>>>(erow, npm, npm, eri_mo);
    PQ_CUDA_TRY(cudaGetLastError());
  }
  int herr = 0;
  PQ_CUDA_TRY(cudaMemcpyAsync(&herr, err.ptr, sizeof(int), cudaMemcpyDeviceToHost, st));
  PQ_CUDA_TRY(cudaStreamSynchronize(st));
  if (herr) {
    set_error("ao2mo tensor-core GEMM: bounded wait gave up (code %d)", herr);
    return PQ_TIMEOUT;
  }
  return PQ_OK;
}

pq_status ao2mo_tc(const double *eri_ao, int layout, int64_t n_ao, const double *Ca, int64_t lda, int64_t nmo, int mode,
                   double *eri_mo, cudaStream_t st) {
  if (n_ao > tc::BN || nmo > tc::BN) {
    set_error("pq_ao2mo: split-precision modes support n_ao, n_mo <= %d", tc::BN);
    return PQ_ERR_ARG;
  }
  if (mode == PQ_XFORM_BF16X3) return ao2mo_tc_impl<false>(eri_ao, layout, n_ao, Ca, lda, nmo, eri_mo, st);
  return ao2mo_tc_impl<true>(eri_ao, layout, n_ao, Ca, lda, nmo, eri_mo, st);
}

}  // namespace pq

extern "C" pq_status pq_ao2mo_release_workspace(void) {
  std::lock_guard<std::mutex> lock(pq::g_ws_mu);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    pq::set_error("pq_ao2mo_release_workspace: no current device");
    return PQ_ERR_STATE;
  }
  pq::Ao2moWorkspace &w = pq::g_ws[dev];
  for (pq::DevBuf *b : {&w.full, &w.cth, &w.ctl, &w.sh, &w.sl, &w.uh, &w.ul, &w.H1, &w.H1t, &w.Erow, &w.err}) b->release();
  return PQ_OK;
}

extern "C" pq_status pq_debug_set_wait_budget(long long cycles) {
  pq::g_gemm_wait_cycles = cycles > 0 ? cycles : pq::tc::WAIT_CYCLES;
  return PQ_OK;
}
