// Occupation strings of up to 128 orbitals as two 64-bit words: `lo` holds
// orbitals 0..63 (bit o = orbital o), `hi` orbitals 64..127.  Problems with at
// most 64 orbitals per species keep no hi words (the pointer is NULL and the
// word reads as 0), so their kernels run the one-word loops.
#pragma once
#include <stdint.h>

namespace pq {

__device__ __forceinline__ uint64_t hiword(const uint64_t *hi, int64_t i) { return hi ? hi[i] : 0ull; }

// f(k) for every occupied orbital k of the string (lo, hi), ascending
template <typename F> __device__ __forceinline__ void for_occ(uint64_t lo, uint64_t hi, F &&f) {
  for (uint64_t m = lo; m; m &= m - 1) f(__ffsll((long long)m) - 1);
  for (uint64_t m = hi; m; m &= m - 1) f(64 + __ffsll((long long)m) - 1);
}

__device__ __forceinline__ bool occupied(uint64_t lo, uint64_t hi, int o) {
  return o < 64 ? ((lo >> o) & 1ull) != 0 : ((hi >> (o - 64)) & 1ull) != 0;
}

}  // namespace pq

namespace pq {

__device__ __forceinline__ int popc2(uint64_t lo, uint64_t hi) { return __popcll(lo) + __popcll(hi); }

// lowest set orbital of (lo, hi); -1 when both words are zero
__device__ __forceinline__ int first_set(uint64_t lo, uint64_t hi) {
  return lo ? __ffsll((long long)lo) - 1 : (hi ? 64 + __ffsll((long long)hi) - 1 : -1);
}

__device__ __forceinline__ void flip_orb(uint64_t &lo, uint64_t &hi, int o) {
  if (o < 64)
    lo ^= 1ull << o;
  else
    hi ^= 1ull << (o - 64);
}

}  // namespace pq
