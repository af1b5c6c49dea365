// Same-spin doubles of the FP32 full-CI sigma as dense GEMMs on the tcgen05 tensor cores.
//
// Reference: the alpha-alpha and beta-beta double loops of
// sigma_one_species_class_singleshot (src/ci/detset/direct_singleparticle.cpp:238-372)
// with the same-spin element of same_part_ham_double (slater_condon_singleparticle.cpp:107-175).
// In a full-CI space the same-spin doubles of one spin are a fixed matrix
// D[I][J] over the strings of that spin (784 entries per row at 16 orbitals,
// 6 % of a row), so with the interleaved vectors X[Ja][Jb][v]:
//   alpha side  Y[Ia][(Ib, v)] += sum_Ja Da[Ia][Ja] X[Ja][(Ib, v)]
//   beta side   Y[Ia][Ib][v]   += sum_Jb Db[Ib][Jb] X[Ia][Jb][v]
// Both are GEMMs C[m][n] = sum_k A[m][k] B[n][k] with K-major operands:
//   alpha: A = Da, B[(Ib, v)][Ja] = X[Ja][Ib][v]      (a transposed copy of X)
//   beta:  A = Db, B[(Ia, v)][Jb] = X[Ia][Jb][v]      (the roots split into rows)
// The dense matrix is 6 % filled but the tensor cores do the dense product
// faster than the CUDA cores gather the sparse one; (m, k) tiles of D that are
// entirely zero (23 % at 16 orbitals) are skipped through a per-m-tile list.
//
// Precision: D and X are scaled by powers of two into [2^14, 2^15) and split
// into FP16 hi + lo (22 significant bits); each product is hi*hi + hi*lo +
// lo*hi with FP32 accumulation in TMEM, as in the alpha-beta kernel
// (ci_sigma32_tc.cu).
//
// Kernel: persistent, one CTA per SM, 128 x 256 output tiles.  Warp 0 lane 0
// issues TMA loads (128-byte swizzle) of A_hi, A_lo, B_hi, B_lo into a ring of
// two 96 KB stages; warp 1 lane 0 issues the MMAs (M = 128, N = 256, K = 16,
// three per K step) into one of two TMEM accumulators (2 x 256 columns); warps
// 2-5 drain the other accumulator with tcgen05.ld and add the tile into sigma
// (the tile is owned by one CTA: plain read-modify-write, no atomics).  Every
// mbarrier wait is bounded; a wait that runs out records an error code and sets
// an abort flag that every role polls, the producer waits (bounded) for its own
// loads, the MMA thread for its own MMAs, TMEM is freed and the host reports
// PQ_TIMEOUT.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "pq_internal.h"

namespace pq {
namespace ssg {

constexpr int BM = 128;          // output rows per tile (TMEM lanes)
constexpr int BN = 256;          // output columns per tile (TMEM columns per accumulator)
constexpr int BK = 64;           // K per stage: one 128-byte swizzle span of FP16
constexpr int STAGES = 2;
constexpr int A_TILE = BM * 128;  // 16 KB
constexpr int B_TILE = BN * 128;  // 32 KB
constexpr int STAGE_BYTES = 2 * A_TILE + 2 * B_TILE;
constexpr int EPI_WARPS = 4;
constexpr int THREADS = 64 + 32 * EPI_WARPS;  // producer warp, MMA warp, epilogue warps
constexpr int NBARS = 2 * STAGES + 4 + 1;     // full, empty, acc_full[2], acc_empty[2], drain
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 /*align*/ + 256 /*barriers, slots*/;
constexpr int NGROUP = 8;                     // n tiles per scheduling group (L2 reuse of the A panels)
constexpr long long WAIT_CYCLES = 4000000000LL;  // ~2 s at 2 GHz
static_assert(SMEM_BYTES <= 232448, "shared memory per CTA");

enum { ERR_TIMEOUT_FULL = 1, ERR_TIMEOUT_MMA = 2, ERR_TIMEOUT_ACC = 3 };
enum { OUT_ALPHA = 0, OUT_BETA = 1 };

struct Args {
  int M, N;                 // output rows (strings of the doubles' spin) and columns (4 x strings of the other)
  int m_tiles, n_tiles;
  const int32_t *kt_off;    // [m_tiles + 1]: range of m tile mt in kt_list
  const int32_t *kt_list;   // k tiles (units of BK) of D with a nonzero entry
  float *Y;                 // sigma, interleaved [Ia][Ib][v]
  int64_t ldy;              // floats per alpha row of Y (4 x beta strings)
  int mode;                 // OUT_ALPHA: Y[m * ldy + n];  OUT_BETA: Y[(n >> 2) * ldy + 4 m + (n & 3)]
  const unsigned *xmax;     // max |X| (float bits)
  float inv_sd;             // 1 / scale of D
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
  d |= (uint64_t)((addr & 0x3FFFF) >> 4);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}
// instruction descriptor: D = F32, A = B = F16, both K-major, N = BN, M = BM
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

// power of two 2^e with x * 2^e in [2^14, 2^15) (1 for x == 0)
__device__ __forceinline__ float fp16_scale(float x) {
  if (!(x > 0.0f) || !isfinite(x)) return 1.0f;
  int e;
  frexpf(x, &e);
  return ldexpf(1.0f, 15 - e);
}

// tile t -> (m tile, n tile): groups of NGROUP n tiles, m tiles outer inside a group, so the CTAs running
// at one time share a few A panels (rows of D) and a few B panels (rows of the vector operand) in L2
__device__ __forceinline__ void tile_coords(const Args &g, int t, int &mt, int &nt) {
  const int per_group = g.m_tiles * NGROUP;
  const int grp = t / per_group, r = t - grp * per_group;
  const int gw = min(NGROUP, g.n_tiles - grp * NGROUP);
  mt = r / gw;
  nt = grp * NGROUP + (r - mt * gw);
}

__global__ void __launch_bounds__(THREADS, 1)
    ss_gemm_kernel(const __grid_constant__ CUtensorMap tmA_hi, const __grid_constant__ CUtensorMap tmA_lo,
                   const __grid_constant__ CUtensorMap tmB_hi, const __grid_constant__ CUtensorMap tmB_lo, Args g) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char *smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + STAGES * STAGE_BYTES);
  uint64_t *full = bars, *empty = bars + STAGES, *accf = bars + 2 * STAGES, *acce = bars + 2 * STAGES + 2;
  uint64_t *drain = bars + 2 * STAGES + 4;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + NBARS);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n_tiles_total = g.m_tiles * g.n_tiles;

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
    for (int t = blockIdx.x; t < n_tiles_total && !*abort_flag; t += gridDim.x) {
      int mt, nt;
      tile_coords(g, t, mt, nt);
      const int k0 = g.kt_off[mt], k1 = g.kt_off[mt + 1];
      for (int j = k0; j < k1; j++, gs++) {
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
        const int x = g.kt_list[j] * BK;
        tma_load_2d(smem_u32(st), &tmA_hi, x, mt * BM, bar);
        tma_load_2d(smem_u32(st + A_TILE), &tmA_lo, x, mt * BM, bar);
        tma_load_2d(smem_u32(st + 2 * A_TILE), &tmB_hi, x, nt * BN, bar);
        tma_load_2d(smem_u32(st + 2 * A_TILE + B_TILE), &tmB_lo, x, nt * BN, bar);
      }
    }
    // the loads of the last stages must have landed before the CTA exits
    for (int j = gs > STAGES ? gs - STAGES : 0; j < gs; j++)
      mbar_wait(smem_u32(full + (j % STAGES)), (uint32_t)((j / STAGES) & 1));
  } else if (warp == 1 && lane == 0) {
    // ---- MMA issuer
    int gs = 0, i = 0;
    for (int t = blockIdx.x; t < n_tiles_total && !*abort_flag; t += gridDim.x) {
      int mt, nt;
      tile_coords(g, t, mt, nt);
      const int k0 = g.kt_off[mt], k1 = g.kt_off[mt + 1];
      if (k1 == k0) continue;  // an all-zero band of D: no accumulator, no epilogue
      const int a = i & 1;
      const uint32_t aph = (uint32_t)((i >> 1) & 1);
      i++;
      if (!mbar_wait(smem_u32(acce + a), aph ^ 1u, g.wait_cycles)) {
        atomicCAS(g.err, 0, ERR_TIMEOUT_ACC);
        *abort_flag = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t d = tmem + (uint32_t)(a * BN);
      bool ok = true;
      for (int j = k0; j < k1; j++, gs++) {
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
        for (int kk = 0; kk < BK / 16; kk++) {
          const uint32_t off = kk * 32;  // bytes along K inside the swizzle span
          const uint32_t acc0 = (j > k0 || kk > 0) ? 1u : 0u;
          mma_f16(d, smem_desc(a_hi + off), smem_desc(b_hi + off), acc0);
          mma_f16(d, smem_desc(a_hi + off), smem_desc(b_lo + off), 1u);
          mma_f16(d, smem_desc(a_lo + off), smem_desc(b_hi + off), 1u);
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
    // ---- epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31
    const int q = warp & 3;
    const float unscale_x = 1.0f / fp16_scale(__uint_as_float(*g.xmax));
    int i = 0;
    for (int t = blockIdx.x; t < n_tiles_total; t += gridDim.x) {
      int mt, nt;
      tile_coords(g, t, mt, nt);
      if (g.kt_off[mt + 1] == g.kt_off[mt]) continue;
      const int a = i & 1;
      const uint32_t aph = (uint32_t)((i >> 1) & 1);
      i++;
      const bool ok = mbar_wait(smem_u32(accf + a), aph, g.wait_cycles);
      if (!ok || *abort_flag) {
        if (!ok && lane == 0) atomicCAS(g.err, 0, ERR_TIMEOUT_ACC);
        *abort_flag = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(a * BN);
      const int m = mt * BM + q * 32 + lane;  // this lane's output row
      for (int c0 = 0; c0 < BN; c0 += 32) {
        float v[32];
        tmem_ld32(taddr + c0, v);  // v[j] = C[m][nt * BN + c0 + j]; every lane of the warp takes part
        const int n0 = nt * BN + c0;
        if (m < g.M && n0 < g.N) {
#pragma unroll
          for (int j4 = 0; j4 < 8; j4++) {
            const int n = n0 + 4 * j4;
            if (n < g.N) {  // N is a multiple of 4
              float4 *p = g.mode == OUT_ALPHA
                              ? reinterpret_cast<float4 *>(g.Y + (int64_t)m * g.ldy + n)
                              : reinterpret_cast<float4 *>(g.Y + (int64_t)(n >> 2) * g.ldy + 4 * (int64_t)m);
              float4 y = *p;
              y.x += v[4 * j4] * g.inv_sd * unscale_x;
              y.y += v[4 * j4 + 1] * g.inv_sd * unscale_x;
              y.z += v[4 * j4 + 2] * g.inv_sd * unscale_x;
              y.w += v[4 * j4 + 3] * g.inv_sd * unscale_x;
              *p = y;
            }
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
// setup and operand preparation

// max |D| of the same-spin doubles (positive doubles order like their bit patterns)
__global__ void absmax64_kernel(const double *D, int64_t n, unsigned long long *out) {
  double m = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    m = fmax(m, fabs(D[i]));
  for (int o = 16; o; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

// dense D[I][J] (FP16 hi/lo of sd * element, row pitch ldk) from the CSR doubles of one spin list, and the
// flags of the (128-row, 64-column) tiles that hold an entry
__global__ void dense_doubles_kernel(const int64_t *s2_off, const int32_t *s2_J, const double *s2_D, int64_t n_str,
                                     int64_t ldk, double sd, int k_tiles, __half *hi, __half *lo, uint8_t *flags) {
  for (int64_t I = blockIdx.x; I < n_str; I += gridDim.x) {
    const int64_t e0 = s2_off[I], e1 = s2_off[I + 1];
    for (int64_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
      const int J = s2_J[e];
      const double d = s2_D[e] * sd;
      const __half h = __float2half_rn((float)d);
      hi[I * ldk + J] = h;
      lo[I * ldk + J] = __float2half_rn((float)(d - (double)__half2float(h)));
      flags[(I / BM) * k_tiles + J / BK] = 1;
    }
  }
}

// alpha operand: B[(Ib, v)][Ja] = sx * X[Ja][Ib][v] as FP16 hi/lo (a tiled transpose of the na x ncol matrix X)
__global__ void op_alpha_kernel(const float *X, int64_t na, int64_t ncol, int64_t ldk, const unsigned *xmax, __half *hi,
                                __half *lo) {
  __shared__ float tile[32][33];
  const float sx = fp16_scale(__uint_as_float(*xmax));
  const int64_t r0 = (int64_t)blockIdx.y * 32, c0 = (int64_t)blockIdx.x * 32;
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int64_t r = r0 + y, c = c0 + threadIdx.x;
    tile[y][threadIdx.x] = (r < na && c < ncol) ? X[r * ncol + c] : 0.0f;
  }
  __syncthreads();
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int64_t c = c0 + y, r = r0 + threadIdx.x;
    if (c < ncol && r < na) {
      const float x = tile[threadIdx.x][y] * sx;
      const __half h = __float2half_rn(x);
      hi[c * ldk + r] = h;
      lo[c * ldk + r] = __float2half_rn(x - __half2float(h));
    }
  }
}

// beta operand: B[(Ia, v)][Jb] = sx * X[Ia][Jb][v] as FP16 hi/lo
__global__ void op_beta_kernel(const float *X, int64_t na, int64_t nb, int64_t ldk, const unsigned *xmax, __half *hi,
                               __half *lo) {
  const float sx = fp16_scale(__uint_as_float(*xmax));
  const int64_t total = na * nb;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ia = i / nb, jb = i - ia * nb;
    const float4 x4 = reinterpret_cast<const float4 *>(X)[i];
    const float xs[4] = {x4.x * sx, x4.y * sx, x4.z * sx, x4.w * sx};
#pragma unroll
    for (int v = 0; v < 4; v++) {
      const __half h = __float2half_rn(xs[v]);
      hi[(ia * 4 + v) * ldk + jb] = h;
      lo[(ia * 4 + v) * ldk + jb] = __float2half_rn(xs[v] - __half2float(h));
    }
  }
}

// coul[pair][c] = sum_{k in occ(c)} E[pair][kk] (E row-major [pair_row][pair_col]) for the column strings c:
// the opposite-spin Coulomb sum of a row-side single with pair index `pair` and column string c
__global__ void coulomb_table_kernel(const float *E, int npair, const uint64_t *col_str, int64_t ncol, float *coul) {
  const int64_t total = (int64_t)npair * ncol;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int pr = (int)(i / ncol);
    const int64_t c = i - (int64_t)pr * ncol;
    float s = 0.0f;
    for (uint64_t m = col_str[c]; m; m &= m - 1) {
      const int k = __ffsll((long long)m) - 1;
      s += E[(int64_t)pr * npair + k * (k + 3) / 2];
    }
    coul[i] = s;
  }
}

__global__ void absmax32_kernel(const float *X, int64_t n, unsigned *xmax) {
  float m = 0.0f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    m = fmaxf(m, fabsf(X[i]));
  for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(xmax, __float_as_uint(m));
}

}  // namespace ssg

// Per-handle state of the same-spin GEMMs: dense D of each spin list (the beta list shares the alpha one
// when both lists and their integrals are the same), its nonzero k tiles per m tile, the operand buffer.
struct SameSpinGemm {
  struct Side {
    DevBuf hi, lo, kt_off, kt_list;
    int64_t n = 0, ldk = 0;
    int m_tiles = 0;
    float inv_sd = 1.0f;
  };
  Side side[2];
  bool shared_beta = false;
  DevBuf coul[2];  // opposite-spin Coulomb sums of the row-side singles: [pair_row][col string], per row spin
  DevBuf op_hi, op_lo, aux;  // vector operand (reused by both sides), aux = {xmax, err}
};

void ss_delete(SameSpinGemm *g) { delete g; }

static PFN_cuTensorMapEncodeTiled_v12000 ss_encode_fn() {
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

// 2-D tensor map over a row-major FP16 (rows x kdim) operand with row pitch ld, box (BK x box_rows),
// 128-byte swizzle; reads past kdim or rows return zeros
static pq_status ss_map(CUtensorMap *m, const void *base, int64_t rows, int64_t kdim, int64_t ld, int box_rows) {
  auto fn = ss_encode_fn();
  if (!fn) {
    set_error("cuTensorMapEncodeTiled is not available from the driver");
    return PQ_ERR_CUDA;
  }
  cuuint64_t dims[2] = {(cuuint64_t)kdim, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)(ld * 2)};
  cuuint32_t box[2] = {(cuuint32_t)ssg::BK, (cuuint32_t)box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void *>(base), dims, strides, box, es,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d): rows=%lld k=%lld ld=%lld", (int)r, (long long)rows, (long long)kdim,
              (long long)ld);
    return PQ_ERR_CUDA;
  }
  return PQ_OK;
}

// The same-spin GEMMs apply to one-species full CI with 4 interleaved roots when the doubles fill at least
// 3 % of a row (below that the dense product does more work than it saves) and the string lists are short
// enough for the dense matrices (at most 32768 strings per spin: 2 x 2 GB of FP16).
bool sigma32_ss_applicable(const pq_ci_handle *h) {
  if (h->n_species != 1 || !h->full || h->wide) return false;
  for (int sp = 0; sp < 2; sp++) {
    const SpinTablesDev &t = h->tab[0][sp];
    if (t.n_str < 256 || t.n_str > 32768) return false;
    if ((double)t.n2 < 0.03 * (double)t.n_str * (double)t.n_str) return false;
  }
  return true;
}

static pq_status ss_build_side(pq_ci_handle *h, int sp, SameSpinGemm::Side &S) {
  using namespace ssg;
  cudaStream_t st = h->stream;
  const SpinTablesDev &t = h->tab[0][sp];
  S.n = t.n_str;
  S.ldk = (S.n + BK - 1) / BK * BK;  // 16-byte row pitch for TMA; the tail reads back as zeros
  S.m_tiles = (int)((S.n + BM - 1) / BM);
  const int k_tiles = (int)(S.ldk / BK);
  DevBuf dmax, flags;
  PQ_TRY(dmax.alloc(8));
  PQ_CUDA_TRY(cudaMemsetAsync(dmax.ptr, 0, 8, st));
  if (t.n2 > 0)
    absmax64_kernel<<<(unsigned)std::min<int64_t>((t.n2 + 255) / 256, 152 * 8), 256, 0, st>>>(
        t.s2_D64.as<double>(), t.n2, dmax.as<unsigned long long>());
  PQ_CUDA_TRY(cudaGetLastError());
  unsigned long long bits = 0;
  PQ_CUDA_TRY(cudaMemcpyAsync(&bits, dmax.ptr, 8, cudaMemcpyDeviceToHost, st));
  PQ_CUDA_TRY(cudaStreamSynchronize(st));
  double dm;
  memcpy(&dm, &bits, 8);
  int ex = 0;
  std::frexp(dm, &ex);
  const double sd = dm > 0.0 ? std::ldexp(1.0, 15 - ex) : 1.0;
  S.inv_sd = (float)(1.0 / sd);
  const size_t bytes = sizeof(__half) * (size_t)S.n * S.ldk;
  PQ_TRY(S.hi.alloc(bytes));
  PQ_TRY(S.lo.alloc(bytes));
  PQ_TRY(flags.alloc((size_t)S.m_tiles * k_tiles));
  PQ_CUDA_TRY(cudaMemsetAsync(S.hi.ptr, 0, bytes, st));
  PQ_CUDA_TRY(cudaMemsetAsync(S.lo.ptr, 0, bytes, st));
  PQ_CUDA_TRY(cudaMemsetAsync(flags.ptr, 0, (size_t)S.m_tiles * k_tiles, st));
  dense_doubles_kernel<<<(unsigned)std::min<int64_t>(S.n, 152 * 16), 128, 0, st>>>(
      t.s2_off.as<int64_t>(), t.s2_J.as<int32_t>(), t.s2_D64.as<double>(), S.n, S.ldk, sd, k_tiles, S.hi.as<__half>(),
      S.lo.as<__half>(), flags.as<uint8_t>());
  PQ_CUDA_TRY(cudaGetLastError());
  std::vector<uint8_t> f((size_t)S.m_tiles * k_tiles);
  PQ_CUDA_TRY(cudaMemcpyAsync(f.data(), flags.ptr, f.size(), cudaMemcpyDeviceToHost, st));
  PQ_CUDA_TRY(cudaStreamSynchronize(st));
  std::vector<int32_t> off(S.m_tiles + 1, 0), list;
  for (int mt = 0; mt < S.m_tiles; mt++) {
    for (int kt = 0; kt < k_tiles; kt++)
      if (f[(size_t)mt * k_tiles + kt]) list.push_back(kt);
    off[mt + 1] = (int32_t)list.size();
  }
  if (list.empty()) list.push_back(0);
  PQ_TRY(upload(S.kt_off, off, st));
  PQ_TRY(upload(S.kt_list, list, st));
  PQ_CUDA_TRY(cudaStreamSynchronize(st));
  return PQ_OK;
}

static pq_status ss_prepare(pq_ci_handle *h);

static pq_status ss_build_coulomb(pq_ci_handle *h, int spin_row, DevBuf &out) {
  cudaStream_t st = h->stream;
  const SpinTablesDev &tc = h->tab[0][1 - spin_row];
  const int npair = h->npair[0];
  const int64_t ncol = tc.n_str;
  PQ_TRY(out.alloc(sizeof(float) * (size_t)npair * ncol + 16));
  // rows of the alpha side read (pair_alpha | pair_beta), of the beta side (pair_beta | pair_alpha)
  const float *E = spin_row == 0 ? h->d_eab32.as<float>() : h->d_eba32.as<float>();
  ssg::coulomb_table_kernel<<<(unsigned)std::min<int64_t>(((int64_t)npair * ncol + 255) / 256, 152 * 16), 256, 0, st>>>(
      E, npair, tc.str.as<uint64_t>(), ncol, out.as<float>());
  PQ_CUDA_TRY(cudaGetLastError());
  return PQ_OK;
}

const float *ci_sigma32_ss_coulomb(const pq_ci_handle *h, int spin_row) {
  return h->ss ? h->ss->coul[spin_row].as<float>() : nullptr;
}

pq_status ci_sigma32_ss_prepare(pq_ci_handle *h) { return ss_prepare(h); }

size_t ci_sigma32_ss_bytes(const pq_ci_handle *h) {
  if (!h->ss) return 0;
  const SameSpinGemm &g = *h->ss;
  size_t b = g.op_hi.bytes + g.op_lo.bytes + g.aux.bytes + g.coul[0].bytes + g.coul[1].bytes;
  for (const SameSpinGemm::Side &s : g.side) b += s.hi.bytes + s.lo.bytes + s.kt_off.bytes + s.kt_list.bytes;
  return b;
}

static pq_status ss_prepare(pq_ci_handle *h) {
  if (h->ss) return PQ_OK;
  SameSpinGemm *g = new (std::nothrow) SameSpinGemm();
  if (!g) {
    set_error("host allocation failed");
    return PQ_ERR_OOM;
  }
  h->ss.reset(g);
  const pq_ci_desc &d = h->desc;
  // identical spin lists with identical integrals: the beta doubles are the alpha ones
  g->shared_beta = h->n_blocks[0] == 1 && d.n_alpha[0] == d.n_beta[0] && d.ex_level[0][0] == d.ex_level[0][1];
  pq_status s = ss_build_side(h, 0, g->side[0]);
  if (s == PQ_OK && !g->shared_beta) s = ss_build_side(h, 1, g->side[1]);
  if (s == PQ_OK) s = g->aux.alloc(16);
  if (s == PQ_OK) s = ss_build_coulomb(h, 0, g->coul[0]);
  if (s == PQ_OK) s = ss_build_coulomb(h, 1, g->coul[1]);
  if (s == PQ_OK) {
    cudaError_t e = cudaFuncSetAttribute(ssg::ss_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, ssg::SMEM_BYTES);
    if (e != cudaSuccess) {
      set_error("cudaFuncSetAttribute(ss_gemm_kernel) failed: %s", cudaGetErrorString(e));
      s = PQ_ERR_CUDA;
    }
  }
  if (s != PQ_OK) h->ss.reset();
  return s;
}

static pq_status ss_run(pq_ci_handle *h, const SameSpinGemm::Side &S, int64_t n_cols, int mode, float *Y, int64_t ldy) {
  using namespace ssg;
  SameSpinGemm &g = *h->ss;
  CUtensorMap ma_hi, ma_lo, mb_hi, mb_lo;
  PQ_TRY(ss_map(&ma_hi, S.hi.ptr, S.n, S.n, S.ldk, BM));
  PQ_TRY(ss_map(&ma_lo, S.lo.ptr, S.n, S.n, S.ldk, BM));
  PQ_TRY(ss_map(&mb_hi, g.op_hi.ptr, n_cols, S.n, S.ldk, BN));
  PQ_TRY(ss_map(&mb_lo, g.op_lo.ptr, n_cols, S.n, S.ldk, BN));
  Args a{};
  a.M = (int)S.n;
  a.N = (int)n_cols;
  a.m_tiles = S.m_tiles;
  a.n_tiles = (int)((n_cols + BN - 1) / BN);
  a.kt_off = S.kt_off.as<int32_t>();
  a.kt_list = S.kt_list.as<int32_t>();
  a.Y = Y;
  a.ldy = ldy;
  a.mode = mode;
  a.xmax = g.aux.as<unsigned>();
  a.inv_sd = S.inv_sd;
  a.wait_cycles = WAIT_CYCLES;
  a.err = reinterpret_cast<int *>(g.aux.as<unsigned>() + 1);
  const int64_t tiles = (int64_t)a.m_tiles * a.n_tiles;
  const unsigned grid = (unsigned)std::min<int64_t>(tiles, h->tc_sms > 0 ? h->tc_sms : 148);
  ss_gemm_kernel<<<grid, THREADS, SMEM_BYTES, h->stream>>>(ma_hi, ma_lo, mb_hi, mb_lo, a);
  PQ_CUDA_TRY(cudaGetLastError());
  return PQ_OK;
}

// Y += the alpha-alpha and beta-beta doubles of the 4-root interleaved block X (full CI, FP32)
pq_status ci_sigma32_same_spin_tc(pq_ci_handle *h, const float *X, float *Y) {
  using namespace ssg;
  PQ_TRY(ss_prepare(h));
  SameSpinGemm &g = *h->ss;
  cudaStream_t st = h->stream;
  const int64_t na = h->tab[0][0].n_str, nb = h->tab[0][1].n_str;
  if (h->tc_sms == 0) {
    int dev = 0;
    PQ_CUDA_TRY(cudaGetDevice(&dev));
    PQ_CUDA_TRY(cudaDeviceGetAttribute(&h->tc_sms, cudaDevAttrMultiProcessorCount, dev));
  }
  const SameSpinGemm::Side &SA = g.side[0], &SB = g.shared_beta ? g.side[0] : g.side[1];
  // the vector operand of either side: (4 x strings of one spin) rows of ldk FP16 of the other
  const size_t op_bytes = sizeof(__half) * std::max((size_t)(4 * nb) * SA.ldk, (size_t)(4 * na) * SB.ldk) + 16;
  PQ_TRY(g.op_hi.ensure(op_bytes));
  PQ_TRY(g.op_lo.ensure(op_bytes));
  PQ_CUDA_TRY(cudaMemsetAsync(g.aux.ptr, 0, 8, st));
  const int64_t len = na * nb * 4;
  absmax32_kernel<<<(unsigned)std::min<int64_t>((len + 255) / 256, 152 * 8), 256, 0, st>>>(X, len, g.aux.as<unsigned>());
  PQ_CUDA_TRY(cudaGetLastError());
  // alpha side: B[(Ib, v)][Ja]
  op_alpha_kernel<<<dim3((unsigned)((4 * nb + 31) / 32), (unsigned)((na + 31) / 32)), dim3(32, 8), 0, st>>>(
      X, na, 4 * nb, SA.ldk, g.aux.as<unsigned>(), g.op_hi.as<__half>(), g.op_lo.as<__half>());
  PQ_CUDA_TRY(cudaGetLastError());
  PQ_TRY(ss_run(h, SA, 4 * nb, OUT_ALPHA, Y, 4 * nb));
  // beta side: B[(Ia, v)][Jb]
  op_beta_kernel<<<(unsigned)std::min<int64_t>((na * nb + 255) / 256, 152 * 16), 256, 0, st>>>(
      X, na, nb, SB.ldk, g.aux.as<unsigned>(), g.op_hi.as<__half>(), g.op_lo.as<__half>());
  PQ_CUDA_TRY(cudaGetLastError());
  PQ_TRY(ss_run(h, SB, 4 * na, OUT_BETA, Y, 4 * nb));
  int herr = 0;
  PQ_CUDA_TRY(cudaMemcpyAsync(&herr, g.aux.as<unsigned>() + 1, sizeof(int), cudaMemcpyDeviceToHost, st));
  PQ_CUDA_TRY(cudaStreamSynchronize(st));
  if (herr != 0) {
    set_error("sigma32 same-spin tensor-core GEMM: a pipeline wait ran out (code %d)", herr);
    return PQ_TIMEOUT;
  }
  return PQ_OK;
}

}  // namespace pq
