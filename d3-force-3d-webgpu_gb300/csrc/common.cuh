// Shared device helpers of the force-layout engine (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#define FL_WARP 32
#define FL_FULL 0xffffffffu

// Bits of the device error word (reported by fl_sync as FL_E_TIMEOUT / FL_E_OVERFLOW).
#define FL_ERR_LOOKBACK 1u   // a decoupled look-back gave up waiting for a predecessor tile
#define FL_ERR_STACK 2u      // a tree walk ran out of stack
#define FL_ERR_TREE 4u       // the bottom-up pass found a malformed tree (guard tripped)

// Bounded spin: a device wait never lasts longer than this many polls.
#define FL_SPIN_LIMIT (1u << 22)

namespace fl {

// Float <-> unsigned with the same order, for atomicMin/atomicMax on floats.
__device__ __forceinline__ uint32_t ordered(float f) {
  uint32_t b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float unordered(uint32_t u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// 32-bit integer hash ("lowbias32", C. Wellons, public domain): the jiggle's random source.
__host__ __device__ __forceinline__ uint32_t mix32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

// d3's jiggle distribution, (random() - 0.5) * 1e-6 (src/jiggle.js:1-3), drawn from a hash of
// (a, b, axis, step, seed) so that it is reproducible for a seed and identical at both ends of
// a pair: the sign makes it antisymmetric (a < b: +, a > b: -).
__device__ __forceinline__ float jiggle(uint32_t a, uint32_t b, uint32_t axis, uint32_t step,
                                        uint32_t seed) {
  uint32_t lo = a < b ? a : b, hi = a < b ? b : a;
  uint32_t h = mix32(lo ^ mix32(hi ^ mix32(seed ^ mix32(step * 4u + axis))));
  float j = ((float)h * 2.3283064365386963e-10f - 0.5f) * 1e-6f;
  return a <= b ? j : -j;
}

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FL_FULL, v, o);
  return v;
}

// Add one key's digit to a shared histogram, from a whole warp (all lanes call it; `ok` marks
// the lanes with a key). When every key of the warp has the same digit (typical of the high
// digits of spatially ordered keys) one atomic adds them all; otherwise each lane adds its own.
__device__ __forceinline__ void hist_add(uint32_t* sh, uint32_t d, bool ok) {
  const uint32_t lo = __reduce_min_sync(FL_FULL, ok ? d : 0xffffffffu);
  const uint32_t hi = __reduce_max_sync(FL_FULL, ok ? d : 0u);
  if (lo == hi) {
    const uint32_t cnt = __popc(__ballot_sync(FL_FULL, ok));
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(&sh[lo], cnt);
  } else if (ok) {
    atomicAdd(&sh[d], 1u);
  }
}

// Relaxed 32-bit load that bypasses L1 (for flags written by other SMs).
__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed(uint32_t* p, uint32_t v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

}  // namespace fl

// Reduction record shared by the bounding-box and centre passes (device memory, reset before
// each use): ordered-uint min/max of positions, and their exact sum.
//
// The sums are exact integers: every position x contributes x * 2^kSumFracBits truncated toward
// zero, as a 128-bit two's-complement integer (sum_hi:sum_lo), and integer addition does not
// depend on its order. So the centre force's mean is the same whatever the grid, the blocks'
// order or the graph's place in a batch: a layout is bit-reproducible, alone or among others.
// The range covers |x| < 2^50 at a resolution of 2^-40 (sums of up to 2^28 positions cannot
// overflow); a position outside it (or not finite) is counted in `bad`, and the mean is NaN.
constexpr int kSumFracBits = 40;
struct FlReduce {
  uint32_t lo[3];
  uint32_t hi[3];
  uint32_t bad;
  uint32_t pad;
  unsigned long long sum_lo[3];
  unsigned long long sum_hi[3];
};

namespace fl {

// x * 2^kSumFracBits, truncated toward zero, as an exact 128-bit integer, from x's bits alone
// (no floating-point rounding); counts x in `bad` when it is outside the range.
__device__ __forceinline__ __int128 fx128(float x, uint32_t& bad) {
  const uint32_t b = __float_as_uint(x);
  const int e = (int)((b >> 23) & 255u);
  if (e == 0) return 0;  // zero or subnormal: below the resolution
  if (e >= 127 + 50) {   // |x| >= 2^50, inf or NaN
    ++bad;
    return 0;
  }
  const unsigned __int128 m = (unsigned __int128)((b & 0x7fffffu) | 0x800000u);  // x = m 2^(e-150)
  const int sh = e - 150 + kSumFracBits;
  const unsigned __int128 v = sh >= 0 ? m << sh : (sh > -24 ? m >> -sh : (unsigned __int128)0);
  return (b >> 31) ? -(__int128)v : (__int128)v;
}

__device__ __forceinline__ __int128 shfl_xor128(__int128 v, int o) {
  unsigned long long lo = (unsigned long long)v;
  unsigned long long hi = (unsigned long long)((unsigned __int128)v >> 64);
  lo = __shfl_xor_sync(FL_FULL, lo, o);
  hi = __shfl_xor_sync(FL_FULL, hi, o);
  return (__int128)(((unsigned __int128)hi << 64) | lo);
}

__device__ __forceinline__ __int128 shfl_down128(__int128 v, int o) {
  unsigned long long lo = (unsigned long long)v;
  unsigned long long hi = (unsigned long long)((unsigned __int128)v >> 64);
  lo = __shfl_down_sync(FL_FULL, lo, o);
  hi = __shfl_down_sync(FL_FULL, hi, o);
  return (__int128)(((unsigned __int128)hi << 64) | lo);
}

// Adds v to the 128-bit accumulator (hi:lo) in global or shared memory. The carry out of the
// low word is taken from the value the low atomic replaced, so the total number of carries is
// that of the whole sum, in any order: the result is exact and order-independent.
__device__ __forceinline__ void atomic_add128(unsigned long long* lo, unsigned long long* hi,
                                              __int128 v) {
  const unsigned long long a = (unsigned long long)v;
  const unsigned long long b = (unsigned long long)((unsigned __int128)v >> 64);
  const unsigned long long old = atomicAdd(lo, a);
  const unsigned long long c = b + (old + a < old ? 1ull : 0ull);
  if (c) atomicAdd(hi, c);
}

// The sum of axis k of a reduction record as a double (NaN when a position was out of range).
__device__ __forceinline__ double sum_of(const FlReduce& r, int k) {
  if (r.bad) return __longlong_as_double(0x7ff8000000000000ll);
  const double v = (double)(long long)r.sum_hi[k] * 18446744073709551616.0 + (double)r.sum_lo[k];
  return v * 9.094947017729282379150390625e-13;  // 2^-40
}

}  // namespace fl
