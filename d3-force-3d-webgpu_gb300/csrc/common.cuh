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
// each use): ordered-uint min/max of positions and their FP64 sum.
struct FlReduce {
  uint32_t lo[3];
  uint32_t hi[3];
  uint32_t pad[2];
  double sum[3];
  double pad2;
};
