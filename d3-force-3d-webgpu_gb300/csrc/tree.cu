// forceManyBody on the GPU: the d3 Barnes-Hut tree, built every tick and walked per point.
//
// The tree is exactly the one d3-octree / d3-quadtree / d3-binarytree build for
// src/manyBody.js (cube = floor(min) with a power-of-two size, midpoint splits, children in the
// order bit k = coordinate k above the midpoint), cut at LEVELS levels (21 in 3D, 24 in 1D/2D):
//
//   morton     the d3 cube from the bounding box, each point's cell at the finest level (exact),
//              interleaved into a left-aligned Morton key in d3's child order; the sort's digit
//              histograms are counted in the same pass
//   sort       onesweep radix sort of (key, node) over the top 31 (3D) / 32 (2D) key bits, then
//              the run fix-up that orders keys equal in those bits by the rest (sort.cu)
//   build      Karras (2012) binary radix tree over the sorted keys; each internal node's d3
//              depth = common prefix bits / DIMS; the sorted (position, strength) of the points,
//              and each point's d3 leaf depth (from the deeper of its two neighbour prefixes)
//   heads      a binary node whose depth is deeper than its parent's heads a d3 cell (the binary
//              nodes below it at the same depth are splits inside that cell); its d3 children
//              are counted, and child slots are allocated by a scan (every cell's children are
//              contiguous, so the walk reads them in one sweep)
//   cells      each cell's value and centre of mass as manyBody.js accumulate() defines them
//              (value = sqrt(4 / 2^DIMS) times the sum of the children's values; centroid
//              weighted by the children's |value|). When the strengths share one sign this
//              recursion has a closed form, value(D) = sum_p s_p c^(leafDepth_p - D) and centroid
//              weights |s_p| c^leafDepth_p, so every cell is a range sum of exact int64
//              fixed-point prefix sums over the sorted points. With strengths of both signs the
//              recursion itself runs over the d3 cells, from the deepest up through the child
//              slots, with atomic arrival counts: d3's FP64 values bit for bit (so cells that
//              cancel are skipped as d3 skips them), FP64 centroid sums for the top levels.
//   slots      each cell writes its children (position or centroid, value at own depth, and for
//              a child cell its child range and depth) into its slots
//   walk       a group of G consecutive sorted points (G = 32: a warp, or 16) walks the union of
//              their d3 traversals: batches of up to G children are gathered from the group's
//              stack in shared memory and loaded lane-parallel, and every lane applies apply()
//              of manyBody.js for its own point, two children per round in packed FP32 pairs:
//              a cell is approximated at the first (widest) depth of its chain where
//              w^2 / theta^2 < l, points are summed exactly, distanceMin / distanceMax as d3;
//              cells that some lane must open are pushed with the mask of those lanes.
//
// Points with the same code at the finest level share the deepest cell as its children.
#include <math.h>

#include <atomic>
#include <cuda/atomic>
#include <cmath>

#include "kernels.h"

namespace {

constexpr uint32_t kLeaf = 0x80000000u;
constexpr uint32_t kIndex = 0x7fffffffu;
constexpr uint32_t kLeafMark = 0x7fffffffu;  // meta word of a point (a cell's is count | depth << 26)
constexpr uint32_t kCountMask = (1u << 26) - 1;
constexpr uint32_t kNoParent = 0xffffffffu;  // a point alone in its graph (batches)
constexpr uint8_t kGapDepth = 0xff;          // an internal index between two graphs (batches)
constexpr int kThreads = 256;

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

struct alignas(32) D4 {  // four exact fixed-point sums
  long long x, y, z, w;
};
__host__ __device__ __forceinline__ D4 mk4(long long a, long long b, long long c, long long d) {
  return {a, b, c, d};
}

__device__ __forceinline__ uint64_t spread3(uint64_t x) {  // 21 bits -> every third bit
  x &= 0x1fffffull;
  x = (x | x << 32) & 0x1f00000000ffffull;
  x = (x | x << 16) & 0x1f0000ff0000ffull;
  x = (x | x << 8) & 0x100f00f00f00f00full;
  x = (x | x << 4) & 0x10c30c30c30c30c3ull;
  x = (x | x << 2) & 0x1249249249249249ull;
  return x;
}
__device__ __forceinline__ uint64_t spread2(uint64_t x) {  // 32 bits -> every other bit
  x &= 0xffffffffull;
  x = (x | x << 16) & 0x0000ffff0000ffffull;
  x = (x | x << 8) & 0x00ff00ff00ff00ffull;
  x = (x | x << 4) & 0x0f0f0f0f0f0f0f0full;
  x = (x | x << 2) & 0x3333333333333333ull;
  x = (x | x << 1) & 0x5555555555555555ull;
  return x;
}

__device__ __forceinline__ int levels_of(int ndim) { return ndim == 3 ? 21 : 24; }

// c^k with c = sqrt(4 / 2^DIMS) (the per-level scale of manyBody.js accumulate()): c is a power
// of sqrt(2), c^k = 2^(k (2 - DIMS) / 2), so it is an exact power of two, times sqrt(2) when the
// exponent is odd.
__device__ __forceinline__ float damp(int ndim, int k) {
  const int e2 = k * (2 - ndim);  // |e2| <= 2 * 24 (levels): the power of two is a normal float
  const float odd = (e2 & 1) ? 1.41421356237309515f : 1.f;
  return odd * __int_as_float((127 + (e2 >> 1)) << 23);
}

// Conversions between FP32 and 64-bit integers in integer arithmetic: the hardware's 64-bit
// conversions issue on the FP64 pipe, a small fraction of the FP32 rate on this part.
// f2ll_rn: round to nearest even, |v| < 2^63 (above 2^24 a float is an integer: its significand
// shifted into place; below, the 32-bit conversion rounds).
__device__ __forceinline__ long long f2ll_rn(float v) {
  const uint32_t b = __float_as_uint(v);
  const int e = (int)((b >> 23) & 255u) - 150;  // |v| = significand * 2^e
  if (e < 0) return (long long)__float2int_rn(v);
  const long long m = (long long)((b & 0x7fffffu) | 0x800000u) << e;
  return (b >> 31) ? -m : m;
}
// ll2f_rn: the nearest float (ties to even) to a 64-bit integer.
__device__ __forceinline__ float ll2f_rn(long long v) {
  const unsigned long long u = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
  float r;
  if (u < (1ull << 24)) {
    r = (float)(uint32_t)u;
  } else {
    const int lz = __clzll((long long)u);
    const unsigned long long w = u << lz;  // top bit at 63
    uint32_t m = (uint32_t)(w >> 40);      // 24 significant bits
    const unsigned long long rest = w & ((1ull << 40) - 1);
    if (rest > (1ull << 39) || (rest == (1ull << 39) && (m & 1u))) ++m;
    r = (float)m * __int_as_float((127 + 40 - lz) << 23);  // m <= 2^24, 2^(40 - lz): exact
  }
  return v < 0 ? -r : r;
}

// (x - o) * 2^F as an exact integer: x - o is rounded once in FP32 and its rounding error
// recovered exactly (Knuth's TwoSum); both parts scale exactly by the power of two 2^F.
__device__ __forceinline__ long long fx_offset(float x, float o, float scaleF) {
  const float s = x - o;
  const float bb = s - x;
  const float e = (x - (s - bb)) + (-o - bb);
  const long long d = f2ll_rn(s * scaleF) + f2ll_rn(e * scaleF);
  return d < 0 ? 0 : d;
}
// floor(W * D / 2^62) for W, D >= 0 (the 128-bit product's bits 62..125)
__device__ __forceinline__ long long mulhi62(long long W, long long D) {
  const unsigned long long hi = __umul64hi((unsigned long long)W, (unsigned long long)D);
  const unsigned long long lo = (unsigned long long)W * (unsigned long long)D;
  return (long long)((hi << 2) | (lo >> 62));
}
// 2^F of the fixed-point offsets: u = (x - origin) / size = offset / 2^62, F = 62 - log2(size)
__device__ __forceinline__ float offset_scale(const float* cube) {
  int F = 62 - (int)cube[4];
  F = F < -100 ? -100 : F > 100 ? 100 : F;
  return __int_as_float((F + 127) << 23);
}

// 4^-k as an exact float (k <= 31)
__device__ __forceinline__ float pow4neg(uint32_t k) { return __int_as_float((127 - 2 * (int)k) << 23); }

// floor((floor(x) - origin) * 2^e) for e < 0, in FP64 where every step is exact. Not inlined:
// inlined, the compiler predicates it into the common path, which then pays its FP64 work.
__device__ __noinline__ float cell_of_wide(float x, float origin, int e) {
  return (float)floor(ldexp(floor((double)x) - (double)origin, e));
}

// The cell index of x at the finest level, floor((x - origin) * 2^e), in exact arithmetic:
// e >= 0: floor(x * 2^e) and origin * 2^e are exact floats, and so is their difference, an
// integer below 2^24; e < 0 (cubes wider than 2^LEVELS): cell_of_wide.
__device__ __forceinline__ uint64_t cell_of(float x, float origin, int e, uint32_t top) {
  float c;
  if (e >= 0) {
    const float s = __int_as_float((e + 127) << 23);
    c = floorf(x * s) - origin * s;
  } else {
    c = cell_of_wide(x, origin, e);
  }
  c = fminf(fmaxf(c, 0.f), (float)top);
  return (uint64_t)(uint32_t)c;  // below 2^24: a 32-bit conversion (the 64-bit one is FP64-pipe)
}

// d3 cover() of a bounding box (d3-octree): origin = floor(min); a power-of-two size doubled
// until max < origin + size (FP64, one thread). cube5 = origin x, y, z, size, log2 size.
__device__ void d3_cover(const FlReduce* red, int ndim, float* cube5) {
  double lo0 = 0, lo1 = 0, lo2 = 0, hi0 = 0, hi1 = 0, hi2 = 0;
  lo0 = floor((double)fl::unordered(~red->lo[0])), hi0 = (double)fl::unordered(red->hi[0]);
  if (ndim > 1) lo1 = floor((double)fl::unordered(~red->lo[1])), hi1 = (double)fl::unordered(red->hi[1]);
  if (ndim > 2) lo2 = floor((double)fl::unordered(~red->lo[2])), hi2 = (double)fl::unordered(red->hi[2]);
  double size = 1;
  int lg = 0;
  while (lg < 1100 && !(hi0 < lo0 + size && (ndim < 2 || hi1 < lo1 + size) && (ndim < 3 || hi2 < lo2 + size)))
    size *= 2, ++lg;
  cube5[0] = (float)lo0, cube5[1] = (float)lo1, cube5[2] = (float)lo2;
  cube5[3] = (float)size, cube5[4] = (float)lg;
}

// The left-aligned Morton key of p in the cube with the given origin, e = LEVELS - log2(size).
__device__ __forceinline__ uint64_t morton_key(float4 p, const float* origin, int e, int ndim) {
  const int L = levels_of(ndim), bits = L * ndim;
  const uint32_t top = (1u << L) - 1;
  const uint64_t qx = cell_of(p.x, origin[0], e, top);
  uint64_t key;
  if (ndim == 3)
    key = spread3(qx) | spread3(cell_of(p.y, origin[1], e, top)) << 1 |
          spread3(cell_of(p.z, origin[2], e, top)) << 2;
  else if (ndim == 2)
    key = spread2(qx) | spread2(cell_of(p.y, origin[1], e, top)) << 1;
  else
    key = qx;
  return key << (64 - bits);
}

// Bounding box -> d3 cube -> keys; digit histograms of the sort passes in the same read.
constexpr int kMortonThreads = 1024;

__global__ void __launch_bounds__(kMortonThreads) k_morton(const float4* __restrict__ pos, int n,
                                                     int ndim, const FlReduce* red,
                                                     uint64_t* __restrict__ keys,
                                                     uint32_t* __restrict__ vals,
                                                     uint32_t* __restrict__ hist, int lo_bit,
                                                     float* cube_out) {
  __shared__ float s_cube[5];
  __shared__ uint32_t sh[8 * 256];
  const int passes = (64 - lo_bit + 7) / 8;
  if (threadIdx.x == 0) {
    d3_cover(red, ndim, s_cube);
    if (blockIdx.x == 0)
      for (int k = 0; k < 5; ++k) cube_out[k] = s_cube[k];
  }
  for (int i = threadIdx.x; i < 8 * 256; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  const int e = levels_of(ndim) - (int)s_cube[4];
  const int stride = gridDim.x * blockDim.x;
  for (int base = blockIdx.x * blockDim.x; base < n; base += stride) {
    const int i = base + threadIdx.x;
    const bool ok = i < n;
    uint64_t key = 0;
    if (ok) {
      key = morton_key(pos[i], s_cube, e, ndim);
      keys[i] = key;
      vals[i] = (uint32_t)i;
    }
    for (int p = 0; p < passes; ++p)
      fl::hist_add(sh + p * 256, (uint32_t)(key >> (lo_bit + 8 * p)) & 255u, ok);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < passes * 256; i += blockDim.x)
    if (sh[i]) atomicAdd(&hist[i], sh[i]);
}

// ---- batches of graphs: the per-graph tick values, the keys, and the sort by graph

// One thread per graph: the graph's d3 cube from its bounding box, the walk's threshold, its
// distances, this tick's alpha, its velocity multiplier and its centre force's shift.
__global__ void __launch_bounds__(kThreads) k_bgraph(int graphs, int ndim, const int32_t* __restrict__ off,
                                                     const FlReduce* __restrict__ red,
                                                     const FlBatchParams* __restrict__ prm,
                                                     const double* __restrict__ alpha,
                                                     FlGraph* __restrict__ gr) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= graphs) return;
  FlGraph o;
  const int first = off[g], count = off[g + 1] - off[g];
  if (count > 0) {
    d3_cover(red + g, ndim, o.origin);
  } else {
    o.origin[0] = o.origin[1] = o.origin[2] = 0.f, o.size = 1.f, o.lg = 0.f;
  }
  const FlBatchParams p = prm[g];
  o.T0 = (float)((double)o.size * (double)o.size / p.theta2);
  o.dmin2 = (float)p.dmin2;
  o.dmax2 = p.dmax2 > 3e38 ? INFINITY : (float)p.dmax2;
  o.alpha = (float)alpha[g];
  o.decay = (float)p.decay;
  const double c[3] = {p.cx, p.cy, p.cz};
  for (int k = 0; k < 3; ++k) {
    const double d = k < ndim && count > 0 && p.cstrength != 0 ? (fl::sum_of(red[g], k) / count - c[k]) * p.cstrength : 0.0;
    const float h = (float)d;
    o.shift[k] = make_float2(h, (float)(d - (double)h));
  }
  o.first = first, o.count = count;
  o.frozen = alpha[g] < 0.0 ? 1 : 0;
  o.fx = p.fx;
  o.tick0 = p.tick0;
  o.citer = p.citer, o.cinv = p.cinv, o.cstr = p.cstr;
  o.pad = 0u;
  gr[g] = o;
}

// Morton keys of a batch, each point in its own graph's cube; histograms as k_morton.
__global__ void __launch_bounds__(kMortonThreads) k_bmorton(const float4* __restrict__ pos, int n,
                                                      int ndim, const uint32_t* __restrict__ gid,
                                                      const FlGraph* __restrict__ gr,
                                                      uint64_t* __restrict__ keys,
                                                      uint32_t* __restrict__ vals,
                                                      uint32_t* __restrict__ hist, int lo_bit) {
  __shared__ uint32_t sh[8 * 256];
  const int passes = (64 - lo_bit + 7) / 8;
  for (int i = threadIdx.x; i < 8 * 256; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  const int stride = gridDim.x * blockDim.x;
  for (int base = blockIdx.x * blockDim.x; base < n; base += stride) {
    const int i = base + threadIdx.x;
    const bool ok = i < n;
    uint64_t key = 0;
    if (ok) {
      const FlGraph& g = gr[gid[i]];
      key = morton_key(pos[i], g.origin, levels_of(ndim) - (int)g.lg, ndim);
      keys[i] = key;
      vals[i] = (uint32_t)i;
    }
    for (int p = 0; p < passes; ++p)
      fl::hist_add(sh + p * 256, (uint32_t)(key >> (lo_bit + 8 * p)) & 255u, ok);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < passes * 256; i += blockDim.x)
    if (sh[i]) atomicAdd(&hist[i], sh[i]);
}

// The second sort's input: the graph of each point in Morton order, in key bits [48, 64), and
// the point's Morton-order position; with the histograms of those two digits.
// The graph of node `node`: the last g with off[g] <= node (graph offsets in shared memory).
__device__ __forceinline__ uint32_t graph_of(const int32_t* s_off, int graphs, uint32_t node) {
  int lo = 0, hi = graphs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if ((uint32_t)s_off[mid] <= node) lo = mid;
    else hi = mid - 1;
  }
  return (uint32_t)lo;
}
constexpr int kGidSearchMax = 8192;  // graphs whose offsets the key kernel searches in shared memory

__global__ void __launch_bounds__(kMortonThreads) k_bgidkey(int n, const uint32_t* __restrict__ mperm,
                                                      const uint32_t* __restrict__ gid,
                                                      const int32_t* __restrict__ off, int graphs,
                                                      uint64_t* __restrict__ keys,
                                                      uint32_t* __restrict__ vals,
                                                      uint32_t* __restrict__ hist) {
  __shared__ uint32_t sh[2 * 256];
  __shared__ int32_t s_off[kGidSearchMax];
  const bool search = graphs <= kGidSearchMax;
  for (int i = threadIdx.x; i < 2 * 256; i += blockDim.x) sh[i] = 0;
  if (search)
    for (int i = threadIdx.x; i < graphs; i += blockDim.x) s_off[i] = off[i];
  __syncthreads();
  const int stride = gridDim.x * blockDim.x;
  for (int base = blockIdx.x * blockDim.x; base < n; base += stride) {
    const int i = base + threadIdx.x;
    const bool ok = i < n;
    uint64_t key = 0;
    if (ok) {
      // a node's graph: from the offsets (a search in shared memory) rather than a random read
      const uint32_t node = mperm[i];
      key = (uint64_t)(search ? graph_of(s_off, graphs, node) : gid[node]) << 48;
      keys[i] = key;
      vals[i] = (uint32_t)i;
    }
    fl::hist_add(sh, (uint32_t)(key >> 48) & 255u, ok);
    fl::hist_add(sh + 256, (uint32_t)(key >> 56) & 255u, ok);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 2 * 256; i += blockDim.x)
    if (sh[i]) atomicAdd(&hist[i], sh[i]);
}

// The order by (graph, Morton code): position j takes the Morton-order point at order2[j].
__global__ void __launch_bounds__(kThreads) k_bgather(int n, const uint32_t* __restrict__ order2,
                                                      const uint64_t* __restrict__ mkeys,
                                                      const uint32_t* __restrict__ mperm,
                                                      const uint32_t* __restrict__ gid,
                                                      uint64_t* __restrict__ skeys,
                                                      uint32_t* __restrict__ perm,
                                                      uint32_t* __restrict__ gid_pos) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const uint32_t v = order2[j];
  const uint32_t node = mperm[v];
  skeys[j] = mkeys[v];
  perm[j] = node;
  // graph g's points take sorted positions [off[g], off[g + 1]), the same range its nodes have
  gid_pos[j] = gid[j];
}

// Common prefix of sorted keys i and j (index tie-break), -1 outside [lo, hi] (one graph's range)
__device__ __forceinline__ int kdelta(const uint64_t* __restrict__ k, int lo, int hi, uint64_t ki,
                                      int i, int j) {
  if (j < lo || j > hi) return -1;
  uint64_t kj = k[j];
  return ki != kj ? __clzll(ki ^ kj) : 64 + __clz(i ^ j);
}

// Modular (wrapping) 64-bit arithmetic: in a batch, the prefix over all graphs' records may pass
// 2^63 (each graph has its own scale); the difference of two prefix values within one graph is
// still its exact sum, which that graph's scale keeps below 2^62.
__device__ __forceinline__ long long wadd(long long a, long long b) {
  return (long long)((unsigned long long)a + (unsigned long long)b);
}
__device__ __forceinline__ long long wsub(long long a, long long b) {
  return (long long)((unsigned long long)a - (unsigned long long)b);
}
__device__ __forceinline__ D4 add4(D4 a, D4 b) {
  return mk4(wadd(a.x, b.x), wadd(a.y, b.y), wadd(a.z, b.z), wadd(a.w, b.w));
}
__device__ __forceinline__ D4 shfl_up4(D4 v, int o) {
  return mk4(__shfl_up_sync(FL_FULL, v.x, o), __shfl_up_sync(FL_FULL, v.y, o),
             __shfl_up_sync(FL_FULL, v.z, o), __shfl_up_sync(FL_FULL, v.w, o));
}

// Inclusive prefix of one D4 per thread over a 256-thread block: written to out[i] (i >= 0),
// the block's total to tot[blockIdx.x]. Every thread of the block must call it.
__device__ void block_prefix4(D4 v, D4* out, D4* tot, int i) {
  __shared__ D4 s_warp[kThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    D4 y = shfl_up4(v, o);
    if (lane >= o) v = add4(v, y);
  }
  if (lane == 31) s_warp[warp] = v;
  __syncthreads();
  if (warp) {
    D4 b = s_warp[0];
    for (int w = 1; w < warp; ++w) b = add4(b, s_warp[w]);
    v = add4(v, b);
  }
  if (i >= 0) out[i] = v;
  if (threadIdx.x == kThreads - 1) tot[blockIdx.x] = v;
}

// Karras (2012), "Maximizing parallelism in the construction of BVHs, octrees, and k-d trees":
// internal node i covers sorted range [first, last] and splits it where the common prefix grows.
// Thread i also gathers sorted point i and, for the closed-form cell sums, its record
// (|a|, |a| u_x, |a| u_y, |a| u_z) with a = strength * c^leafDepth and u = (p - origin) / size in
// [0, 1) the position in the d3 cube, as exact fixed point (scale 2^fx_exp, chosen so that no
// sum over all points overflows), prefix-summed within the block. Integer sums are exact, and
// cheap where FP64 is not.
// PART: 1, the points (sorted leaves, records, their block prefix); 2, the internal nodes;
// 0, both in one kernel.
template <int PART>
__global__ void __launch_bounds__(kThreads) k_build(
    const uint64_t* __restrict__ k, const uint32_t* __restrict__ perm,
    const float4* __restrict__ pos, const float* __restrict__ strength, int n, int ndim,
    uint32_t* __restrict__ left, uint32_t* __restrict__ right, uint32_t* __restrict__ parent,
    uint32_t* __restrict__ leaf_parent, uint32_t* __restrict__ range, uint8_t* __restrict__ depth,
    float4* __restrict__ leaf, D4* __restrict__ wsum, D4* __restrict__ wtot,
    const float* __restrict__ cube, int fx_exp, FlSegs seg) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int L = levels_of(ndim), bits = L * ndim;
  // the sorted range of this point's graph (a batch), and that graph's cube
  int lo = 0, hi = n - 1;
  const float* cb = cube;
  int fe = fx_exp;
  if (seg.graphs && i < n) {
    const uint32_t g = seg.gid_pos[i];
    lo = seg.off[g], hi = seg.off[g + 1] - 1;
    cb = seg.g[g].origin;
    fe = seg.g[g].fx;
  }
  const uint64_t ki = i < n ? k[i] : 0;
  const int up = i < n ? kdelta(k, lo, hi, ki, i, i + 1) : -1;
  const int dn = i < n ? kdelta(k, lo, hi, ki, i, i - 1) : -1;
  if (PART != 2 && i < n && lo == hi) leaf_parent[i] = kNoParent;  // alone in its graph: no tree
  D4 wrec = mk4(0, 0, 0, 0);
  if (PART != 2 && i < n) {
    const uint32_t node = perm[i];
    float4 p = pos[node];
    p.w = strength[node];
    leaf[i] = p;
    if (wsum) {
      const int dmx = up > dn ? up : dn;
      const int lD = (dmx >= bits ? L : dmx / ndim) + 1;  // the point's d3 leaf depth
      const float sF = offset_scale(cb);
      const long long W =
          f2ll_rn(fabsf(p.w * damp(ndim, lD)) * __int_as_float((fe + 127) << 23));
      wrec = mk4(W, mulhi62(W, fx_offset(p.x, cb[0], sF)),
                 ndim > 1 ? mulhi62(W, fx_offset(p.y, cb[1], sF)) : 0,
                 ndim > 2 ? mulhi62(W, fx_offset(p.z, cb[2], sF)) : 0);
    }
  }
  if (PART != 2 && wsum)  // block-uniform
    block_prefix4(wrec, wsum, wtot, i < n ? i : -1);
  if (PART == 1 || i >= n - 1) return;
  if (i == hi) {  // the last point of a graph: this internal index belongs to no tree
    left[i] = right[i] = kNoParent;
    range[2 * i] = range[2 * i + 1] = (uint32_t)i;
    depth[i] = kGapDepth;
    return;
  }
  if (i == lo) parent[i] = (uint32_t)i;  // a graph's root is its own parent
  const int d = up > dn ? 1 : -1;
  const int dmin = up > dn ? dn : up;
  int64_t lmax = 2;
  while (kdelta(k, lo, hi, ki, i, (int)(i + lmax * d)) > dmin) lmax *= 2;
  int64_t len = 0;
  for (int64_t t = lmax >> 1; t >= 1; t >>= 1)
    if (kdelta(k, lo, hi, ki, i, (int)(i + (len + t) * d)) > dmin) len += t;
  const int j = (int)(i + len * d);
  const int dnode = kdelta(k, lo, hi, ki, i, j);
  int64_t s = 0, t = len;
  do {
    t = (t + 1) >> 1;
    if (kdelta(k, lo, hi, ki, i, (int)(i + (s + t) * d)) > dnode) s += t;
  } while (t > 1);
  const int split = (int)(i + s * d + (d < 0 ? -1 : 0));
  const int first = i < j ? i : j, last = i < j ? j : i;
  uint32_t l = first == split ? (kLeaf | (uint32_t)split) : (uint32_t)split;
  uint32_t r = last == split + 1 ? (kLeaf | (uint32_t)(split + 1)) : (uint32_t)(split + 1);
  left[i] = l, right[i] = r;
  if (l & kLeaf) leaf_parent[l & kIndex] = (uint32_t)i;
  else parent[l] = (uint32_t)i;
  if (r & kLeaf) leaf_parent[r & kIndex] = (uint32_t)i;
  else parent[r] = (uint32_t)i;
  range[2 * i] = (uint32_t)first, range[2 * i + 1] = (uint32_t)last;
  int dep = dnode >= bits ? L : dnode / ndim;
  depth[i] = (uint8_t)(dep > L ? L : dep);
}

// Every binary node below the root that is a d3 child (a point, or an internal node deeper than
// its parent: the first node of another cell) finds the head of its parent's cell, climbing the
// binary nodes of equal depth, and marks its octant (its keys' digit at the parent's depth) in
// the head's octant mask. head_of[] keeps head | octant << 27 | 1 << 31 for the slots.
// Threads [0, n-1) take the internal nodes, [n-1, 2n-1) the points (sorted order).
__global__ void __launch_bounds__(kThreads) k_frontier(
    int n, int ndim, const uint64_t* __restrict__ skeys, const uint32_t* __restrict__ parent,
    const uint32_t* __restrict__ leaf_parent, const uint32_t* __restrict__ range,
    const uint8_t* __restrict__ depth, uint32_t* __restrict__ omask,
    uint32_t* __restrict__ head_of, uint32_t* err) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 2 * n - 1) return;
  const bool pt = t >= n - 1;
  const uint32_t x = pt ? (uint32_t)(t - (n - 1)) : (uint32_t)t;
  uint32_t rec = 0;
  // the parent cell's binary node: none for a graph's root, an index between two graphs, or a
  // point alone in its graph
  uint32_t p = kNoParent;
  if (pt) p = leaf_parent[x];
  else if (depth[x] != kGapDepth && parent[x] != x) p = parent[x];
  if (p != kNoParent) {
    const int Dp = depth[p];
    if (pt || depth[x] > Dp) {
      uint32_t h = p;
      for (int guard = 0;; ++guard) {  // equal depths: splits inside one cell
        const uint32_t up = parent[h];
        if (up == h || depth[up] < Dp) break;
        h = up;
        if (guard > 64) {
          atomicOr(err, FL_ERR_TREE);
          break;
        }
      }
      uint32_t oct = 0;
      if (Dp < levels_of(ndim)) {
        const uint64_t k = skeys[pt ? x : range[2 * x]];
        oct = (uint32_t)(k >> (64 - ndim * (Dp + 1))) & ((1u << ndim) - 1u);
        atomicOr(omask + h, (1u << oct) | (pt ? 0u : 1u << (16 + oct)));  // cells also above
      }
      rec = h | (oct << 27) | 0x80000000u;
    }
  }
  head_of[t] = rec;
}


// Exclusive prefix of the block totals, in place, by one block of kTopThreads: each thread sums
// a run of consecutive totals, a warp-shuffle scan of the threads' sums (two levels) gives each
// run its start, and the thread rewrites its run. For the child counts (u32) and the
// fixed-point point records (D4).
constexpr int kTopThreads = 1024;
__device__ __forceinline__ uint32_t top_add(uint32_t a, uint32_t b) { return a + b; }
__device__ __forceinline__ D4 top_add(D4 a, D4 b) { return add4(a, b); }
__device__ __forceinline__ uint32_t top_up(uint32_t v, int o) { return __shfl_up_sync(FL_FULL, v, o); }
__device__ __forceinline__ D4 top_up(D4 v, int o) { return shfl_up4(v, o); }

template <typename T>
__device__ __forceinline__ void top_scan(T* tot, int nb, T zero) {
  __shared__ T s_warp[kTopThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int per = (nb + kTopThreads - 1) / kTopThreads, a = threadIdx.x * per;
  const int b = a + per < nb ? a + per : nb;
  T sum = zero;
#pragma unroll 8
  for (int t = a; t < b; ++t) sum = top_add(sum, tot[t]);
  T x = sum;  // inclusive scan within the warp
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T y = top_up(x, o);
    if (lane >= o) x = top_add(x, y);
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {  // inclusive scan of the warp totals
    T w = s_warp[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const T y = top_up(w, o);
      if (lane >= o) w = top_add(w, y);
    }
    s_warp[lane] = w;
  }
  __syncthreads();
  T run = warp ? s_warp[warp - 1] : zero;
  const T y = top_up(x, 1);  // exclusive within the warp: the previous lane's inclusive sum
  if (lane) run = top_add(run, y);
#pragma unroll 8
  for (int t = a; t < b; ++t) {
    const T v = tot[t];
    tot[t] = run;
    run = top_add(run, v);
  }
}

__global__ void __launch_bounds__(kTopThreads) k_top_u32(uint32_t* tot, int nb) {
  top_scan<uint32_t>(tot, nb, 0u);
}

__global__ void __launch_bounds__(kTopThreads) k_top4(D4* tot, int nb) {
  top_scan<D4>(tot, nb, mk4(0, 0, 0, 0));
}

// first child slot of head x: slots [0, roots) hold the roots (one per graph), children follow
// in head order
__device__ __forceinline__ uint32_t first_slot(const uint32_t* first, const uint32_t* ctot,
                                               uint32_t x, uint32_t roots) {
  return roots + first[x] + ctot[x >> 8];
}

// The cell of head i from the prefix sums (strengths of one sign, `sign`): its centroid and its
// value at its own depth, in closed form.
__device__ __forceinline__ float4 closed_cell(uint32_t i, int ndim, float sign,
                                              const uint32_t* __restrict__ range,
                                              const uint8_t* __restrict__ depth,
                                              const D4* __restrict__ P, const D4* __restrict__ Ptot,
                                              const float4* __restrict__ leaf,
                                              const float* __restrict__ cube1, int fx_exp,
                                              const FlSegs& seg) {
  const uint32_t a = range[2 * i], b = range[2 * i + 1];
  const float* cube = seg.graphs ? seg.g[seg.gid_pos[a]].origin : cube1;
  const int fe = seg.graphs ? seg.g[seg.gid_pos[a]].fx : fx_exp;
  // prefix sums: within the 256-point block, plus the blocks before it; exact in fixed point
  const D4 hi = add4(P[b], Ptot[b >> 8]);
  const D4 lo = a ? add4(P[a - 1], Ptot[(a - 1) >> 8]) : mk4(0, 0, 0, 0);
  const long long W = wsub(hi.x, lo.x);
  const int D = depth[i];
  float4 out;
  if (W > 0) {
    // centroid = p0 + size * sum(w (u - u0)) / sum(w), about the range's first point p0: the
    // integer sums give the offsets exactly, so FP32 keeps the precision of the cell, not the cube
    const float4 p0 = leaf[a];
    const float fW = ll2f_rn(W);
    const float sF = offset_scale(cube), r = cube[3] / fW;
    out.x = p0.x + ll2f_rn(wsub(wsub(hi.y, lo.y), mulhi62(W, fx_offset(p0.x, cube[0], sF)))) * r;
    out.y = ndim > 1 ? p0.y + ll2f_rn(wsub(wsub(hi.z, lo.z), mulhi62(W, fx_offset(p0.y, cube[1], sF)))) * r : 0.f;
    out.z = ndim > 2 ? p0.z + ll2f_rn(wsub(wsub(hi.w, lo.w), mulhi62(W, fx_offset(p0.z, cube[2], sF)))) * r : 0.f;
    out.w = sign * fW * __int_as_float((127 - fe) << 23) * damp(ndim, -D);
  } else {
    out = leaf[a];
    out.w = 0.f;
  }
  return out;
}

// Whether internal node i heads a d3 cell, and how many d3 children that cell has (its occupied
// octants; at the deepest level, where the keys are equal, its points); the counts' exclusive
// prefix within the block (first[]) and the block's total (ctot[]), for the slots. CLOSED (strengths
// of one sign): a head's cell from the prefix sums too (closed_cell), into cell[]. Otherwise the
// heads without child cells (where the recursion starts) are listed in up_list[0, *up_count).
template <bool CLOSED>
__global__ void __launch_bounds__(kThreads) k_heads(int n, int ndim,
                                                    const uint32_t* __restrict__ parent,
                                                    const uint32_t* __restrict__ range,
                                                    const uint8_t* __restrict__ depth,
                                                    const uint32_t* __restrict__ omask,
                                                    uint32_t* __restrict__ count,
                                                    uint32_t* __restrict__ first,
                                                    uint32_t* __restrict__ ctot, float sign,
                                                    const D4* __restrict__ P,
                                                    const D4* __restrict__ Ptot,
                                                    const float4* __restrict__ leaf,
                                                    const float* __restrict__ cube, int fx_exp,
                                                    float4* __restrict__ cell, FlSegs seg,
                                                    uint32_t* __restrict__ up_list,
                                                    uint32_t* __restrict__ up_count) {
  __shared__ uint32_t s_warp[kThreads / 32];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t c = 0;
  bool start = false;
  if (i < n - 1) {
    const int D = depth[i];
    if (D != kGapDepth) {
      const uint32_t pa = parent[i];
      const bool head = pa == (uint32_t)i || depth[pa] < D;  // a graph's root, or a deeper cell
      if (head) {
        if (D >= levels_of(ndim)) {
          c = range[2 * i + 1] - range[2 * i] + 1;
          start = true;
        } else {
          const uint32_t om = omask[i];
          c = __popc(om & 0xffffu);
          start = !(om >> 16);
        }
      }
    }
    count[i] = c;
    if (CLOSED && c)
      cell[i] = closed_cell((uint32_t)i, ndim, sign, range, depth, P, Ptot, leaf, cube, fx_exp, seg);
  }
  if (!CLOSED) {  // one atomic per warp
    const uint32_t bal = __ballot_sync(FL_FULL, start);
    if (bal) {
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(up_count, (uint32_t)__popc(bal));
      base = __shfl_sync(FL_FULL, base, 0);
      if (start) up_list[base + __popc(bal & ((1u << lane) - 1u))] = (uint32_t)i;
    }
  }
  uint32_t x = c;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(FL_FULL, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  uint32_t before = 0;
  for (int w = 0; w < warp; ++w) before += s_warp[w];
  if (i < n - 1) first[i] = before + x - c;
  if (threadIdx.x == kThreads - 1) ctot[blockIdx.x] = before + x;
}

// The recursion itself (strengths of both signs), over the d3 cells from the deepest up, reading
// each head's children from its slots (k_slots has written the points and every slot's meta).
// The heads without child cells (k_heads listed them) start, one per thread. A finished cell
// writes itself into its slot among its parent's children and counts itself in at the parent;
// the last of the parent's child cells to arrive (their octants are the high half of the
// parent's octant mask) puts the parent on its block's queue in shared memory, and the block
// works through the queue a round at a time, one head per thread, until it is empty. So the
// chain of dependent steps is the d3 depth, and a round's heads sit on consecutive lanes: FP64
// runs at 2 lanes per clock per SM, and a warp instruction costs its 16 clocks however few of
// its lanes are active, so heads climbing alone on scattered lanes made this pass FP64-bound.
// A head combines its children as accumulate() does (src/manyBody.js:42-71). With
// fp64_depth > 0 every value is d3's FP64 number bit for bit: the children's values summed in
// slot order, which is d3's octant order (z << 2 | y << 1 | x), a chain of one-child cells
// scaled by c once per level, the sum scaled by c (c1, d3's Math.sqrt(4 / 2^dims), correctly
// rounded); each cell's FP64 value rides in slot64 beside its slot (a point's strength too,
// converted by k_slots on full warps). So a cell whose children cancel is skipped
// (`!quad.value`, src/manyBody.js:74) exactly when d3 skips it: a cancellation can leave d3 an
// FP64 residual, a value that d3 opens like any other. Centroids are weighted by the FP32
// values, summed in FP64 above fp64_depth and in FP32 below. fp64_depth 0 runs all of it in
// FP32 (values within 2^-20 of their children's |values| count as 0), for precision
// comparisons.
// Children whose slots are loaded together: 1 measured fastest at 1M nodes (48 registers, more
// blocks resident; 2 and 4 children, 60 and 70 registers, were 6 and 20 us slower per tick).
constexpr int kUpBatch = 1;
constexpr uint32_t kNoHead = 0xffffffffu;

// One head of the recursion: combine its children into its cell, write the cell into its slot
// and count it in at its parent. Returns the parent when this was its last child cell to
// arrive, else kNoHead (also after a graph's root, and on a malformed tree).
__device__ __forceinline__ uint32_t cells_up_one(
    uint32_t h, int n, int ndim, const uint32_t* __restrict__ head_of,
    const uint32_t* __restrict__ omask, const uint8_t* __restrict__ depth,
    const uint32_t* __restrict__ count, const uint32_t* __restrict__ first,
    const uint32_t* __restrict__ ctot, uint32_t* __restrict__ arrive, float4* cdata,
    const uint2* __restrict__ cmeta, double* slot64, int fp64_depth, double c1, uint32_t* err,
    const FlSegs& seg) {
  const uint32_t roots = seg.graphs ? (uint32_t)seg.graphs : 1u;
  const uint32_t nslots = 2u * (uint32_t)n + 1u;
  const bool exact = fp64_depth > 0;
  const int D = depth[h];
  const uint32_t cnt = count[h], fs = first_slot(first, ctot, h, roots);
  // the parent's record: its loads overlap the children's
  const uint32_t rec = head_of[h];
  const bool root = !(rec & 0x80000000u);
  const uint32_t p = rec & kCountMask, oct = (rec >> 27) & 15u;
  uint32_t pcnt = 0, pfirst = 0, ptot = 0, pmask = 0;
  if (!root) pcnt = count[p], pfirst = first[p], ptot = ctot[p >> 8], pmask = omask[p];
  if (fs + cnt > nslots) {  // a malformed tree
    atomicOr(err, FL_ERR_TREE);
    return kNoHead;
  }
  const bool wide = D < fp64_depth;
  double sv = 0, sa = 0, sx = 0, sy = 0, sz = 0;
  float fv = 0, fa = 0, fx = 0, fy = 0, fz = 0;
  float4 firstpos = make_float4(0, 0, 0, 0);
  for (uint32_t j0 = 0; j0 < cnt; j0 += kUpBatch) {
    uint2 m[kUpBatch];
    float4 q[kUpBatch];
    double v64[kUpBatch];
#pragma unroll
    for (int k = 0; k < kUpBatch; ++k) {
      if (j0 + k < cnt) {
        m[k] = cmeta[fs + j0 + k];
        q[k] = __ldcg(cdata + fs + j0 + k);
        v64[k] = exact ? __ldcg(slot64 + fs + j0 + k) : 0.0;
      }
    }
#pragma unroll
    for (int k = 0; k < kUpBatch; ++k) {
      if (j0 + k >= cnt) break;
      float v32 = q[k].w;  // the centroid weight's value
      double v = 0;
      if (m[k].y == kLeafMark) {
        v = v64[k];  // the point's strength, as k_slots wrote it
      } else {
        // the chain of one-child cells from D + 1 down to the child's depth scales by c
        const int cd = (int)(m[k].y >> 26);
        v32 *= damp(ndim, cd - D - 1);
        if (exact) {
          v = v64[k];
          for (int l = cd - D - 1; l > 0; --l) v *= c1;
        }
      }
      if (j0 + k == 0) firstpos = q[k];
      const float a = fabsf(v32);
      if (exact) {
        // d3 skips children whose value is 0 (or NaN): tested on the bits
        const unsigned long long b = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
        if (b == 0 || b > 0x7ff0000000000000ull) continue;
        sv += v;
      } else {
        if (!(a > 0.f)) continue;
        fv += v32;
      }
      fa += a;
      if (wide) sa += a, sx += (double)a * q[k].x, sy += (double)a * q[k].y, sz += (double)a * q[k].z;
      else fx += a * q[k].x, fy += a * q[k].y, fz += a * q[k].z;
    }
  }
  float4 out;
  if (wide)
    out = sa > 0 ? make_float4((float)(sx / sa), (float)(sy / sa), (float)(sz / sa), 0.f) : firstpos;
  else
    out = fa > 0.f ? make_float4(fx / fa, fy / fa, fz / fa, 0.f) : firstpos;
  double val = 0;
  if (exact) {
    val = sv * c1;
    out.w = (float)val;
    // a residual below FP32's range stays a value the walk does not skip
    if (val != 0 && out.w == 0.f) out.w = copysignf(1.17549435e-38f, (float)val);
  } else {
    out.w = fabsf(fv) <= fa * 0x1p-20f ? 0.f : (float)((double)fv * c1);
  }
  if (root) {  // a graph's root: its own slot
    cdata[seg.graphs ? seg.gid_pos[h] : 0u] = out;
    return kNoHead;
  }
  const uint32_t pfs = roots + pfirst + ptot;
  const uint32_t rank = (uint32_t)__popc(pmask & ((1u << oct) - 1u)), slot = pfs + rank;
  if (rank >= pcnt || pfs + pcnt > nslots) {  // a malformed tree
    atomicOr(err, FL_ERR_TREE);
    return kNoHead;
  }
  cdata[slot] = out;
  if (exact) slot64[slot] = val;
  // acquire-release: each arrival publishes its cell; the last sees all of them
  const uint32_t w = cuda::atomic_ref<uint32_t, cuda::thread_scope_device>(arrive[p])
                         .fetch_add(1u, cuda::memory_order_acq_rel);
  return w + 1u == (uint32_t)__popc(pmask >> 16) ? p : kNoHead;
}

__global__ void __launch_bounds__(kThreads) k_cells_up(
    int n, int ndim, const uint32_t* __restrict__ head_of, const uint32_t* __restrict__ omask,
    const uint8_t* __restrict__ depth, const uint32_t* __restrict__ count,
    const uint32_t* __restrict__ first, const uint32_t* __restrict__ ctot,
    uint32_t* __restrict__ arrive, float4* cdata, const uint2* __restrict__ cmeta,
    double* slot64, int fp64_depth, double c1, uint32_t* err, FlSegs seg,
    const uint32_t* __restrict__ up_list, const uint32_t* __restrict__ up_count) {
  __shared__ uint32_t s_queue[kThreads];
  __shared__ uint32_t s_len;
  const uint32_t starts = min(*up_count, (uint32_t)(n - 1));
  if (blockIdx.x * blockDim.x >= starts) return;  // the whole block
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t h = t < starts ? up_list[t] : kNoHead;
  for (int round = 0;; ++round) {
    if (threadIdx.x == 0) s_len = 0;
    __syncthreads();
    if (h != kNoHead) {
      if (round > 64) {  // deeper than any d3 tree: a malformed tree
        atomicOr(err, FL_ERR_TREE);
      } else {
        const uint32_t next = cells_up_one(h, n, ndim, head_of, omask, depth, count, first,
                                           ctot, arrive, cdata, cmeta, slot64, fp64_depth, c1,
                                           err, seg);
        if (next != kNoHead) s_queue[atomicAdd(&s_len, 1u)] = next;
      }
    }
    __syncthreads();
    const uint32_t len = s_len;
    h = threadIdx.x < len ? s_queue[threadIdx.x] : kNoHead;
    if (len == 0) return;  // block-uniform
    __syncthreads();  // everyone has its head before the queue is reset
  }
}

// Every d3 child writes itself into its slot of its head's cell: the head's first slot plus the
// child's rank (occupied octants before its own; at the deepest level, its place in the range);
// the root also fills slot 0. Threads as in k_frontier.
__global__ void __launch_bounds__(kThreads) k_slots(
    int n, int ndim, const uint32_t* __restrict__ head_of, const uint32_t* __restrict__ omask,
    const uint32_t* __restrict__ parent,
    const uint32_t* __restrict__ range, const uint8_t* __restrict__ depth,
    const uint32_t* __restrict__ count, const uint32_t* __restrict__ first,
    const uint32_t* __restrict__ ctot, const float4* __restrict__ cell,
    const float4* __restrict__ leaf, float4* __restrict__ cdata, uint2* __restrict__ cmeta,
    uint32_t* err, FlSegs seg, bool cells_later, double* __restrict__ slot64) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 2 * n - 1) return;
  const bool pt = t >= n - 1;
  const uint32_t x = pt ? (uint32_t)(t - (n - 1)) : (uint32_t)t;
  const uint32_t roots = seg.graphs ? (uint32_t)seg.graphs : 1u;
  if (!pt && depth[x] != kGapDepth && parent[x] == x) {  // a graph's root: its own slot
    const uint32_t rs = seg.graphs ? seg.gid_pos[x] : 0u;
    if (!cells_later) cdata[rs] = cell[x];
    cmeta[rs] = make_uint2(first_slot(first, ctot, x, roots), count[x] | ((uint32_t)depth[x] << 26));
  }
  const uint32_t rec = head_of[t];
  if (!(rec & 0x80000000u)) return;
  const uint32_t h = rec & kCountMask, oct = (rec >> 27) & 15u;
  const uint32_t rank = depth[h] >= levels_of(ndim)
                            ? (pt ? x : range[2 * x]) - range[2 * h]
                            : (uint32_t)__popc(omask[h] & ((1u << oct) - 1u));
  const uint32_t slot = first_slot(first, ctot, h, roots) + rank;
  if (rank >= count[h] || slot >= 2u * (uint32_t)n + 1u) {  // a malformed tree
    atomicOr(err, FL_ERR_TREE);
    return;
  }
  if (pt) {
    const float4 l = leaf[x];
    cdata[slot] = l;
    // the recursion's FP64 value of the point, converted here on full warps
    if (slot64) slot64[slot] = (double)l.w;
    cmeta[slot] = make_uint2(x, kLeafMark);
  } else {
    if (!cells_later) cdata[slot] = cell[x];
    cmeta[slot] = make_uint2(first_slot(first, ctot, x, roots), count[x] | ((uint32_t)depth[x] << 26));
  }
}

constexpr int kWalkThreads = 128;
constexpr int kWalkWarps = kWalkThreads / 32;
constexpr int kStack = 96;  // entries per group in shared memory; deeper entries spill to global
// A group's stack never holds more than (levels + 1) * G entries: every batch pushes at most G
// entries (the cells its lanes open), and the entries on the stack form layers, one per batch
// whose pushes are not yet consumed, holding cells of strictly increasing depth.
__host__ __device__ constexpr int kWalkStackLayers(int ndim) { return (ndim == 3 ? 21 : 24) + 1; }
constexpr int kWalkSpillPerWarp = 704;  // max over dims and group sizes of NG ((levels+1) G - kStack)
constexpr int kWalkBlocksPerSm = 10;    // blocks of the persistent walk grid per SM
// the largest layout whose walk runs one point per warp by default (FL_TUNE_WALK_GROUP 0)
constexpr int kLaneWalkMaxNodes = 32768;

// Packed FP32 pairs (the f32x2 arithmetic of sm_100 and later): two children per instruction.
__device__ __forceinline__ uint64_t pk2(float a, float b) {
  uint64_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ float2 up2(uint64_t x) {
  float2 r;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(x));
  return r;
}
__device__ __forceinline__ uint64_t sub2(uint64_t a, uint64_t b) {
  uint64_t d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ uint64_t mul2(uint64_t a, uint64_t b) {
  uint64_t d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ uint64_t fma2(uint64_t a, uint64_t b, uint64_t c) {
  uint64_t d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ float rcp_approx(float x) {  // the reciprocal __fdividef multiplies by
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

template <int NG>
struct WalkShared {
  uint4 stack[kWalkWarps][NG][kStack];  // per point group: first child slot, count, top depth, lanes
  // the batches, one entry per child: what every test reads ...
  // per pair of children (2j, 2j + 1): {x, x', y, y'} and {z, z', value, value'}, the value at
  // the chain's top depth times alpha, in the packed layout the f32x2 arithmetic reads
  float4 data[kWalkWarps][32];
  uint4 test[kWalkWarps][32];   // open threshold, uncommon-case bound, lane mask, slot / index
  // ... and what only a push or an uncommon case reads
  uint2 cold[kWalkWarps][32];   // meta word (count | depth << 26, or kLeafMark), chain top depth
  uint32_t own[kWalkWarps][32];  // the gather: which stack entry each child of the batch is from
};

// The less common cases of apply() (src/manyBody.js:73-115) for one child: a chain of cells
// whose widest cell is too close (the child is approximated at the first, widest, depth of the
// chain that passes the theta test), a zero component of the displacement (d3 replaces it with
// a jiggle) and distanceMin. `va` arrives as the value at the chain's top depth.
// The jiggle's ids of a pair are the graph's own, so that a layout draws the same jiggles alone
// or in any batch: a point's node index less its graph's first node (`first`), and for a cell
// the graph's node count `ng` plus the cell's first child slot counted from the graph's first
// (`cellbase`: the slot before it). Outside a batch: first 0, ng = n, cellbase 0.
template <int NDIM>
__device__ __forceinline__ void rare_case(uint32_t meta, uint32_t top, uint32_t idx, float T0,
                                          float dmin2, uint32_t myid, uint32_t first,
                                          uint32_t ng, uint32_t cellbase,
                                          const uint32_t* __restrict__ perm, int n, uint32_t step,
                                          uint32_t seed, float& va, float& dx, float& dy,
                                          float& dz, float& l) {
  if (meta != kLeafMark) {
    const uint32_t D = (meta >> 26) & 31u;
    if (top < D && T0 * pow4neg(top) >= l) {
      uint32_t k = top + 1;
      while (k < D && T0 * pow4neg(k) >= l) ++k;
      va *= damp(NDIM, (int)top - (int)k);  // value(k) = value(top) c^(top - k)
    }
  }
  if (dx == 0.f || (NDIM > 1 && dy == 0.f) || (NDIM > 2 && dz == 0.f)) {
    const uint32_t other =
        meta == kLeafMark
            ? perm[idx < (uint32_t)n ? idx : 0] - first
            : ng + (idx - cellbase);
    myid -= first;
    if (dx == 0.f) dx = fl::jiggle(myid, other, 0, step, seed), l += dx * dx;
    if (NDIM > 1 && dy == 0.f) dy = fl::jiggle(myid, other, 1, step, seed), l += dy * dy;
    if (NDIM > 2 && dz == 0.f) dz = fl::jiggle(myid, other, 2, step, seed), l += dz * dz;
  }
  if (l < dmin2) l = sqrtf(dmin2 * l);
}

// The walk of G consecutive sorted points (G = 32: a warp; 16: half a warp each, with its own
// stack and batches, so that fewer points share, and pay for, one union of traversals).
//
// Per child and testing lane, the common case costs one theta compare (opened?), one compare
// against the uncommon-case bound, the force and two ballots. The bound folds two tests into
// one: a chain cell whose widest depth is too close for this point (l <= threshold at the top
// depth) and distanceMin (l < dmin2, i.e. l <= the float below dmin2).
// stats (STATS): [0] child tests (G per child), [1] tests a lane's own traversal needed,
// [2] deepest stack, [3] lanes that opened a cell, [4] lanes that applied a cell or point,
// [5] pair rounds that took the uncommon-case branch.
__device__ __forceinline__ float below(float d2) {  // l < d2 <=> l <= below(d2), for l >= 0
  return d2 > 0.f ? __uint_as_float(__float_as_uint(d2) - 1u) : -1.f;
}

// BATCH: the points belong to a batch of graphs (segs): each graph has its own tree (root slot =
// its index), cube, theta, distances and alpha; a group's points may span graphs.
template <int NDIM, int G, bool STATS, bool DMAX, bool BATCH>
__global__ void __launch_bounds__(kWalkThreads) k_walk(
    const float4* __restrict__ cdata, const uint2* __restrict__ cmeta,
    const float4* __restrict__ leaf, const uint32_t* __restrict__ perm,
    const float* __restrict__ cube, float4* __restrict__ vel, int n, float alpha,
    double theta2, float dmin2, float dmax2, uint32_t step, uint32_t seed, uint32_t* err,
    unsigned long long* stats, uint4* __restrict__ spill, int nwarps, uint32_t* work,
    FlSegs segs, const FlTick* __restrict__ tk) {
  if (tk) alpha = tk->alpha, step = tk->step, seed = tk->seed;
  constexpr int NG = 32 / G;
  // the stack of a group: kStack entries in shared memory, then up to kWalkStack(NDIM, G) in
  // all, the rest in this warp slot's region of the spill buffer
  constexpr int kAll = kWalkStackLayers(NDIM) * G, kSpilled = kAll - kStack;
  static_assert(NG * kSpilled <= kWalkSpillPerWarp, "spill region too small");
  __shared__ WalkShared<NG> sh;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int grp = lane / G, gl = lane % G, gbase = grp * G;
  const uint32_t gmask = G == 32 ? FL_FULL : (((1u << G) - 1u) << gbase);
  const uint32_t lanebit = 1u << lane;
  // (size / 2^k)^2 / theta^2 = T0 * 4^-k, exactly (a power-of-two scaling); the FP64 division
  // once per block
  __shared__ float s_T0;
  if (!BATCH && threadIdx.x == 0) s_T0 = (float)((double)cube[3] * (double)cube[3] / theta2);
  __syncthreads();
  const float T0 = BATCH ? 0.f : s_T0;
  // l < dmin2  <=>  l <= the largest float below dmin2 (l >= 0)
  const float dmin_le = below(dmin2);
  const uint32_t slot_cap = 2u * (uint32_t)n + 1u;
  unsigned long long st_tests = 0, st_useful = 0, st_open = 0, st_apply = 0, st_rare = 0;
  int maxsp = 0;
  const int wslot = blockIdx.x * kWalkWarps + warp;  // this warp's slot of a persistent grid
  uint4* stk = sh.stack[warp][grp];
  uint4* spl = spill + (size_t)wslot * kWalkSpillPerWarp + grp * kSpilled;
  auto sget = [&](int i) { return i < kStack ? stk[i] : spl[i - kStack]; };
  auto sset = [&](int i, uint4 v) {
    if (i < kStack) stk[i] = v;
    else spl[i - kStack] = v;
  };
  float4* spair = sh.data[warp] + gbase;
  uint4* stest = sh.test[warp] + gbase;
  uint2* scold = sh.cold[warp] + gbase;
  // groups of 32 points are handed out one at a time (the walk's cost varies a lot between
  // groups, so a fixed share per warp would leave some warps working long after the rest)
  int wi = lane == 0 ? (int)atomicAdd(work, 1u) : 0;
  wi = __shfl_sync(FL_FULL, wi, 0);
  while (wi < nwarps) {
  // a group: 32 consecutive sorted points, or in a batch one graph's points [x, y), at most 32
  const uint2 grp_range = BATCH ? segs.groups[wi] : make_uint2((uint32_t)wi * 32u, (uint32_t)n);
  const int base = (int)grp_range.x;
  const int t = base + lane;
  const bool live = t < (int)grp_range.y;
  const uint32_t act = __ballot_sync(FL_FULL, live) & gmask;
  const float4 me = live ? leaf[t] : make_float4(0, 0, 0, 0);
  const uint32_t myid = live ? perm[t] : 0;
  uint64_t AX = 0, AY = 0, AZ = 0;  // force sums, one per child of a round's pair
  const uint64_t MX = pk2(me.x, me.x), MY = pk2(me.y, me.y), MZ = pk2(me.z, me.z);
  // the lane's own graph: what its uncommon cases and distanceMax use
  float myT0 = T0, mydmin2 = dmin2, mydmax2 = dmax2;
  uint32_t myfirst = 0, mystep = step, myng = (uint32_t)n, mycb = 0;
  int sp;
  if (!BATCH) {
    if (gl == 0 && act) sset(0, make_uint4(0u, 1u, 0u, act));  // the root: slot 0, top depth 0
    sp = act ? 1 : 0;
  } else {
    // one root entry per graph among the group's points (a graph of one point has no tree);
    // a stack entry's third word is its top depth | graph << 8
    const uint32_t g = live ? segs.gid_pos[t] : 0xffffffffu;
    bool tree = false;
    if (live) {
      const FlGraph& gr = segs.g[g];
      myT0 = gr.T0, mydmin2 = gr.dmin2, mydmax2 = gr.dmax2;
      myfirst = (uint32_t)gr.first, mystep = step + gr.tick0, myng = (uint32_t)gr.count;
      // the graph's root sits in slot g; its first child slot less one is where the graph's
      // slots are counted from (a lone simulation's root has its children from slot 1)
      if (gr.count > 1) mycb = __ldg(&cmeta[g].x) - 1u;
      tree = gr.count > 1 && !gr.frozen;
    }
    const uint32_t peers = __match_any_sync(FL_FULL, tree ? g : 0xffffffffu) & gmask;
    const bool leader = tree && (peers & (lanebit - 1u)) == 0;
    const uint32_t leaders = __ballot_sync(FL_FULL, leader) & gmask;
    if (leader) sset(__popc(leaders & (lanebit - 1u)), make_uint4(g, 1u, g << 8, peers));
    sp = __popc(leaders);
  }
  if (sp > maxsp) maxsp = sp;
  __syncwarp();
  uint32_t guard = 0;
  const uint32_t guard_max = 4u * (uint32_t)n + 64u;
  while (__any_sync(FL_FULL, sp > 0)) {
    // each group gathers the first G children from the top of its stack, in parallel: lane gl
    // reads the gl-th entry from the top, a prefix sum of the entries' child counts places each
    // entry's children in the batch, and lane gl then finds the entry of the batch's gl-th child
    const bool has = gl < sp;
    uint4 e = has ? sget(sp - 1 - gl) : make_uint4(0u, 0u, 0u, 0u);
    if (has && (e.x >= slot_cap || e.y > slot_cap - e.x)) {  // a malformed tree: never read past it
      atomicOr(err, FL_ERR_TREE);
      e.y = e.x >= slot_cap ? 0u : slot_cap - e.x;
    }
    uint32_t inc = e.y;
#pragma unroll
    for (int o = 1; o < G; o <<= 1) {
      const uint32_t u = __shfl_up_sync(FL_FULL, inc, o, G);
      if (gl >= o) inc += u;
    }
    const uint32_t exc = inc - e.y;
    const uint32_t avail = __shfl_sync(FL_FULL, inc, G - 1, G);
    const int total = avail < (uint32_t)G ? (int)avail : G;
    // entries taken whole leave the stack; one taken in part keeps the rest (the new top)
    const uint32_t taken = __ballot_sync(FL_FULL, has && inc <= (uint32_t)total) & gmask;
    if (has && exc < (uint32_t)total && inc > (uint32_t)total)
      sset(sp - 1 - gl, make_uint4(e.x + ((uint32_t)total - exc), inc - (uint32_t)total, e.z, e.w));
    sp -= __popc(taken);
    // each entry marks where its children start; a running max carries the mark to the rest
    uint32_t* sown = sh.own[warp] + gbase;
    sown[gl] = 0u;
    __syncwarp();
    if (e.y && exc < (uint32_t)total) sown[exc] = (uint32_t)gl;
    __syncwarp();
    uint32_t own = sown[gl];
#pragma unroll
    for (int o = 1; o < G; o <<= 1) {
      const uint32_t u = __shfl_up_sync(FL_FULL, own, o, G);
      if (gl >= o && u > own) own = u;
    }
    const uint32_t own_first = __shfl_sync(FL_FULL, e.x, (int)own, G);
    const uint32_t own_exc = __shfl_sync(FL_FULL, exc, (int)own, G);
    const uint32_t my_mask = __shfl_sync(FL_FULL, e.w, (int)own, G);
    const uint32_t my_z = __shfl_sync(FL_FULL, e.z, (int)own, G);
    const uint32_t my_top = my_z & 0xffu, my_g = my_z >> 8;
    const uint32_t my_slot = own_first + ((uint32_t)gl - own_exc);
    __syncwarp();
    const int jmax = G == 32 ? total : (int)__reduce_max_sync(FL_FULL, (unsigned)total);
    if (gl < total) {
      // what does not depend on the testing point, once per child
      const float4 q = __ldg(cdata + my_slot);
      const uint2 m = __ldg(cmeta + my_slot);
      const bool lf = m.y == kLeafMark;
      const uint32_t D = (m.y >> 26) & 31u;
      uint32_t mask = q.w != 0.f ? my_mask : 0u;  // d3 skips a zero value and all it holds
      if (lf && m.x - (uint32_t)base < 32u) mask &= ~(1u << (m.x - (uint32_t)base));  // itself
      const bool chain = !lf && my_top < D;
      float T0c = T0, alc = alpha, dminc = dmin_le;
      if (BATCH) {  // the child's graph: that of the lanes that test it
        const FlGraph& gr = segs.g[my_g];
        T0c = gr.T0, alc = gr.alpha, dminc = below(gr.dmin2);
      }
      // a point is never approximated (its sum is the same either way); a cell is opened when
      // even its deepest depth fails the theta test
      const float topen = lf ? -INFINITY : T0c * pow4neg(D);
      const float ttop = chain ? T0c * pow4neg(my_top) : topen;
      const float va = chain ? q.w * alc * damp(NDIM, (int)(D - my_top)) : q.w * alc;
      float* pa = reinterpret_cast<float*>(spair + (gl & ~1));
      pa[gl & 1] = q.x, pa[2 + (gl & 1)] = q.y, pa[4 + (gl & 1)] = q.z, pa[6 + (gl & 1)] = va;
      stest[gl] = make_uint4(__float_as_uint(topen), __float_as_uint(fmaxf(ttop, dminc)), mask, m.x);
      scold[gl] = make_uint2(m.y, my_top | my_g << 8);
    } else if (gl < ((jmax + 1) & ~1)) {  // pad the group's batch: a child no lane tests
      float* pa = reinterpret_cast<float*>(spair + (gl & ~1));
      pa[gl & 1] = 0.f, pa[2 + (gl & 1)] = 0.f, pa[4 + (gl & 1)] = 0.f, pa[6 + (gl & 1)] = 0.f;
      stest[gl] = make_uint4(0u, 0u, 0u, 0u);
    }
    __syncwarp();
#pragma unroll 4
    for (int j = 0; j < jmax; j += 2) {  // two children per round: independent work to overlap
      const float4 pa = spair[j], pb = spair[j + 1];
      const uint4 r0 = stest[j], r1 = stest[j + 1];
      uint64_t DX = sub2(pk2(pa.x, pa.y), MX);
      uint64_t DY = NDIM > 1 ? sub2(pk2(pa.z, pa.w), MY) : 0ull;
      uint64_t DZ = NDIM > 2 ? sub2(pk2(pb.x, pb.y), MZ) : 0ull;
      uint64_t L = mul2(DX, DX);
      if (NDIM > 1) L = fma2(DY, DY, L);
      if (NDIM > 2) L = fma2(DZ, DZ, L);
      const float2 zp = up2(NDIM == 3 ? mul2(mul2(DX, DY), DZ) : NDIM == 2 ? mul2(DX, DY) : DX);
      float2 l = up2(L);
      const bool m0 = r0.z & lanebit, m1 = r1.z & lanebit;
      const bool o0 = m0 && __uint_as_float(r0.x) >= l.x, o1 = m1 && __uint_as_float(r1.x) >= l.y;
      const bool a0 = m0 && !o0 && (!DMAX || l.x < mydmax2), a1 = m1 && !o1 && (!DMAX || l.y < mydmax2);
      float v0 = pb.z, v1 = pb.w;
      const bool c0 = a0 && (l.x <= __uint_as_float(r0.y) || zp.x == 0.f);
      const bool c1 = a1 && (l.y <= __uint_as_float(r1.y) || zp.y == 0.f);
      // one warp-uniform branch for everything but the common case (no lane opens either child,
      // no uncommon case): the common path runs one vote, and never the code inside, even
      // predicated
      uint32_t om0 = 0, om1 = 0;
      if (__any_sync(FL_FULL, c0 || c1 || o0 || o1)) {
        if (__any_sync(FL_FULL, c0 || c1)) {
          if (STATS && lane == 0) ++st_rare;
          float2 dx = up2(DX), dy = up2(DY), dz = up2(DZ);
          if (c0) {
            const uint2 k0 = scold[j];
            rare_case<NDIM>(k0.x, k0.y & 0xffu, r0.w, myT0, mydmin2, myid, myfirst, myng, mycb,
                            perm, n, mystep, seed, v0, dx.x, dy.x, dz.x, l.x);
          }
          if (c1) {
            const uint2 k1 = scold[j + 1];
            rare_case<NDIM>(k1.x, k1.y & 0xffu, r1.w, myT0, mydmin2, myid, myfirst, myng, mycb,
                            perm, n, mystep, seed, v1, dx.y, dy.y, dz.y, l.y);
          }
          DX = pk2(dx.x, dx.y), DY = pk2(dy.x, dy.y), DZ = pk2(dz.x, dz.y);
        }
        om0 = __ballot_sync(FL_FULL, o0) & gmask;
        om1 = __ballot_sync(FL_FULL, o1) & gmask;
        // push the children some lanes of this group must open
        if (om0) {
          const uint2 k0 = scold[j];
          if (sp < kAll && gl == 0)
            sset(sp, make_uint4(r0.w, k0.x & kCountMask, (((k0.x >> 26) & 31u) + 1u) | (k0.y & ~0xffu), om0));
          ++sp;
        }
        if (om1) {
          const uint2 k1 = scold[j + 1];
          if (sp < kAll && gl == 0)
            sset(sp, make_uint4(r1.w, k1.x & kCountMask, (((k1.x >> 26) & 31u) + 1u) | (k1.y & ~0xffu), om1));
          ++sp;
        }
        if (sp > kAll) {  // beyond the bound on the stack's depth: a malformed tree
          if (gl == 0) atomicOr(err, FL_ERR_STACK);
          sp = kAll;
        }
        if (STATS && sp > maxsp) maxsp = sp;
      }
      const float2 w = up2(mul2(pk2(v0, v1), pk2(rcp_approx(l.x), rcp_approx(l.y))));
      const uint64_t W = pk2(a0 ? w.x : 0.f, a1 ? w.y : 0.f);
      AX = fma2(DX, W, AX);
      if (NDIM > 1) AY = fma2(DY, W, AY);
      if (NDIM > 2) AZ = fma2(DZ, W, AZ);
      if (STATS) {
        const uint32_t ap = __ballot_sync(FL_FULL, a0) & gmask, aq = __ballot_sync(FL_FULL, a1) & gmask;
        if (gl == 0) {
          if (j < total) st_tests += G, st_useful += __popc(r0.z & gmask);
          if (j + 1 < total) st_tests += G, st_useful += __popc(r1.z & gmask);
          st_open += __popc(om0) + __popc(om1);
          st_apply += __popc(ap) + __popc(aq);
        }
      }
    }
    __syncwarp();
    if (++guard > guard_max) {
      if (lane == 0) atomicOr(err, FL_ERR_STACK);
      break;
    }
  }
  if (live) {
    const float2 ax2 = up2(AX), ay2 = up2(AY), az2 = up2(AZ);
    float4 v = vel[myid];
    v.x += ax2.x + ax2.y;
    if (NDIM > 1) v.y += ay2.x + ay2.y;
    if (NDIM > 2) v.z += az2.x + az2.y;
    vel[myid] = v;
  }
  __syncwarp();
  wi = lane == 0 ? (int)atomicAdd(work, 1u) : 0;
  wi = __shfl_sync(FL_FULL, wi, 0);
  }
  // every warp ends on one claim past the last group; the last of those claims puts the counter
  // back to 0 for the next launch (no other warp touches it after its own last claim)
  if (lane == 0 && wi == nwarps + (int)(gridDim.x * kWalkWarps) - 1) *work = 0u;
  if (STATS) {
    if (gl == 0) {
      atomicAdd(stats, st_tests);
      atomicAdd(stats + 1, st_useful);
      atomicMax(stats + 2, (unsigned long long)maxsp);
      atomicAdd(stats + 3, st_open);
      atomicAdd(stats + 4, st_apply);
    }
    if (lane == 0) atomicAdd(stats + 5, st_rare);
  }
}

// The walk of one point per warp, for small layouts: where the union walk above has too few
// groups of 32 points to fill the device (a 1,000-node layout is 32 warps, each a long serial
// chain of rounds), each warp walks one point's own d3 traversal and its lanes test up to 32
// children of it at once. The children are gathered from the top of the point's stack as in the
// union walk; a lane tests its child against the point, applies it, takes the uncommon case or
// pushes the child's children. Each lane sums what it applied, and the warp adds the lanes'
// sums in a fixed shuffle tree, so a layout is the same run after run. The stack holds the
// bound on its depth in shared memory, 8 bytes an entry (first child slot; count | top depth
// << 26), so nothing spills and the grid is not limited by spill regions.
// stats (STATS): [0] children tested, [1] of those, the ones the point's d3 traversal needs
// (not a zero value, not the point itself; the union walk's [1], [3] and [4] count the same
// (point, child) pairs), [2] deepest stack, [3] cells opened, [4] cells or points applied,
// [5] rounds in which a lane took the uncommon case.
template <int NDIM, bool STATS, bool DMAX>
__global__ void __launch_bounds__(kWalkThreads) k_walk_lanes(
    const float4* __restrict__ cdata, const uint2* __restrict__ cmeta,
    const float4* __restrict__ leaf, const uint32_t* __restrict__ perm,
    const float* __restrict__ cube, float4* __restrict__ vel, int n, float alpha,
    double theta2, float dmin2, float dmax2, uint32_t step, uint32_t seed, uint32_t* err,
    unsigned long long* stats, uint32_t* work, const FlTick* __restrict__ tk) {
  if (tk) alpha = tk->alpha, step = tk->step, seed = tk->seed;
  // at most 32 children per round and one push per child: the union walk's bound with G = 32
  constexpr int kAll = kWalkStackLayers(NDIM) * 32;
  __shared__ uint2 s_stack[kWalkWarps][kAll];
  __shared__ uint32_t s_own[kWalkWarps][32];
  __shared__ float s_T0;
  if (threadIdx.x == 0) s_T0 = (float)((double)cube[3] * (double)cube[3] / theta2);
  __syncthreads();
  const float T0 = s_T0;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t below_me = (1u << lane) - 1u;
  const float dmin_le = below(dmin2);
  const uint32_t slot_cap = 2u * (uint32_t)n + 1u;
  unsigned long long st_tests = 0, st_useful = 0, st_open = 0, st_apply = 0, st_rare = 0;
  int maxsp = 0;
  uint2* stk = s_stack[warp];
  uint32_t* sown = s_own[warp];
  int t = lane == 0 ? (int)atomicAdd(work, 1u) : 0;
  t = __shfl_sync(FL_FULL, t, 0);
  while (t < n) {
    const float4 me = leaf[t];  // the same address in every lane: one load
    const uint32_t myid = perm[t];
    float ax = 0.f, ay = 0.f, az = 0.f;
    if (lane == 0) stk[0] = make_uint2(0u, 1u);  // the root: slot 0, one child, top depth 0
    int sp = 1;
    uint32_t guard = 0;
    const uint32_t guard_max = 4u * (uint32_t)n + 64u;
    __syncwarp();
    while (sp > 0) {
      // lane i reads the i-th entry from the top; a prefix sum of the entries' child counts
      // places each entry's children in the round, and lane j finds the entry of child j
      const bool has = lane < sp;
      const uint2 se = has ? stk[sp - 1 - lane] : make_uint2(0u, 0u);
      uint4 e = make_uint4(se.x, se.y & kCountMask, se.y >> 26, 0u);
      if (has && (e.x >= slot_cap || e.y > slot_cap - e.x)) {  // a malformed tree: never read past it
        atomicOr(err, FL_ERR_TREE);
        e.y = e.x >= slot_cap ? 0u : slot_cap - e.x;
      }
      uint32_t inc = e.y;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(FL_FULL, inc, o);
        if (lane >= o) inc += u;
      }
      const uint32_t exc = inc - e.y;
      const uint32_t avail = __shfl_sync(FL_FULL, inc, 31);
      const uint32_t total = avail < 32u ? avail : 32u;
      // entries taken whole leave the stack; one taken in part keeps the rest (the new top)
      const uint32_t taken = __ballot_sync(FL_FULL, has && inc <= total);
      if (has && exc < total && inc > total)
        stk[sp - 1 - lane] = make_uint2(e.x + (total - exc), (inc - total) | e.z << 26);
      sp -= __popc(taken);
      sown[lane] = 0u;
      __syncwarp();
      if (e.y && exc < total) sown[exc] = (uint32_t)lane;
      __syncwarp();
      uint32_t own = sown[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(FL_FULL, own, o);
        if (lane >= o && u > own) own = u;
      }
      const uint32_t own_first = __shfl_sync(FL_FULL, e.x, (int)own);
      const uint32_t own_exc = __shfl_sync(FL_FULL, exc, (int)own);
      const uint32_t my_top = __shfl_sync(FL_FULL, e.z, (int)own);
      __syncwarp();
      bool o = false, a = false, rare = false, need = false;
      uint2 m = make_uint2(0u, 0u);
      uint32_t D = 0;
      if ((uint32_t)lane < total) {
        const uint32_t slot = own_first + ((uint32_t)lane - own_exc);
        const float4 q = __ldg(cdata + slot);
        m = __ldg(cmeta + slot);
        const bool lf = m.y == kLeafMark;
        D = (m.y >> 26) & 31u;
        // d3 skips a zero value and all it holds, and the point itself
        const bool mask = q.w != 0.f && !(lf && m.x == (uint32_t)t);
        need = mask;
        const bool chain = !lf && my_top < D;
        const float topen = lf ? -INFINITY : T0 * pow4neg(D);
        const float ttop = chain ? T0 * pow4neg(my_top) : topen;
        float va = chain ? q.w * alpha * damp(NDIM, (int)(D - my_top)) : q.w * alpha;
        float dx = q.x - me.x;
        float dy = NDIM > 1 ? q.y - me.y : 0.f;
        float dz = NDIM > 2 ? q.z - me.z : 0.f;
        float l = dx * dx;
        if (NDIM > 1) l = fmaf(dy, dy, l);
        if (NDIM > 2) l = fmaf(dz, dz, l);
        const float zp = NDIM == 3 ? (dx * dy) * dz : NDIM == 2 ? dx * dy : dx;
        o = mask && topen >= l;
        a = mask && !o && (!DMAX || l < dmax2);
        rare = a && (l <= fmaxf(ttop, dmin_le) || zp == 0.f);
        if (rare)
          rare_case<NDIM>(m.y, my_top, m.x, T0, dmin2, myid, 0u, (uint32_t)n, 0u, perm, n, step,
                          seed, va, dx, dy, dz, l);
        if (a) {
          const float w = va * rcp_approx(l);
          ax = fmaf(dx, w, ax);
          if (NDIM > 1) ay = fmaf(dy, w, ay);
          if (NDIM > 2) az = fmaf(dz, w, az);
        }
      }
      // the children to open go on the stack in child order, the last on top
      const uint32_t opened = __ballot_sync(FL_FULL, o);
      if (o) {
        const int at = sp + __popc(opened & below_me);
        if (at < kAll) stk[at] = make_uint2(m.x, (m.y & kCountMask) | (D + 1u) << 26);
      }
      sp += __popc(opened);
      if (sp > kAll) {  // beyond the bound on the stack's depth: a malformed tree
        if (lane == 0) atomicOr(err, FL_ERR_STACK);
        sp = kAll;
      }
      if (STATS) {
        const uint32_t ap = __ballot_sync(FL_FULL, a), nd = __ballot_sync(FL_FULL, need);
        const bool rr = __any_sync(FL_FULL, rare);
        if (lane == 0) {
          st_tests += total, st_useful += __popc(nd), st_open += __popc(opened);
          st_apply += __popc(ap), st_rare += rr;
          if (sp > maxsp) maxsp = sp;
        }
      }
      __syncwarp();
      if (++guard > guard_max) {
        if (lane == 0) atomicOr(err, FL_ERR_STACK);
        break;
      }
    }
#pragma unroll
    for (int k = 16; k > 0; k >>= 1) {
      ax += __shfl_xor_sync(FL_FULL, ax, k);
      if (NDIM > 1) ay += __shfl_xor_sync(FL_FULL, ay, k);
      if (NDIM > 2) az += __shfl_xor_sync(FL_FULL, az, k);
    }
    if (lane == 0) {
      float4 v = vel[myid];
      v.x += ax;
      if (NDIM > 1) v.y += ay;
      if (NDIM > 2) v.z += az;
      vel[myid] = v;
    }
    __syncwarp();
    t = lane == 0 ? (int)atomicAdd(work, 1u) : 0;
    t = __shfl_sync(FL_FULL, t, 0);
  }
  // as in k_walk: the last claim past the end puts the counter back to 0
  if (lane == 0 && t == n + (int)(gridDim.x * kWalkWarps) - 1) *work = 0u;
  if (STATS && lane == 0) {
    atomicAdd(stats, st_tests);
    atomicAdd(stats + 1, st_useful);
    atomicMax(stats + 2, (unsigned long long)maxsp);
    atomicAdd(stats + 3, st_open);
    atomicAdd(stats + 4, st_apply);
    atomicAdd(stats + 5, st_rare);
  }
}

// Exact all-pairs sum (theta ~ 0; src/gpu/passes/manyBody.js:5-16 semantics): each block
// streams the points through shared memory in tiles.
constexpr int kPairThreads = 256;
__global__ void __launch_bounds__(kPairThreads) k_allpairs(const float4* __restrict__ pos,
                                                           const float* __restrict__ strength,
                                                           float4* __restrict__ vel, int n,
                                                           int ndim, float alpha, float dmin2,
                                                           float dmax2, uint32_t step,
                                                           uint32_t seed, int split,
                                                           const FlTick* __restrict__ tk) {
  if (tk) alpha = tk->alpha, step = tk->step, seed = tk->seed;
  __shared__ float4 tile[kPairThreads];
  __shared__ float3 part[kPairThreads];
  const int per = kPairThreads / split;
  const int lane = threadIdx.x % split;
  const int i = blockIdx.x * per + threadIdx.x / split;
  const bool live = i < n;
  float4 me = live ? pos[i] : make_float4(0, 0, 0, 0);
  float ax = 0.f, ay = 0.f, az = 0.f;
  for (int base = 0; base < n; base += kPairThreads) {
    const int j = base + threadIdx.x;
    float4 q = make_float4(0, 0, 0, 0);
    if (j < n) q = pos[j], q.w = strength[j];
    tile[threadIdx.x] = q;
    __syncthreads();
    const int cnt = n - base < kPairThreads ? n - base : kPairThreads;
    if (live) {
      for (int k = lane; k < cnt; k += split) {
        const float4 o = tile[k];
        if (base + k == i || o.w == 0.f) continue;
        float dx = o.x - me.x, dy = ndim > 1 ? o.y - me.y : 0.f, dz = ndim > 2 ? o.z - me.z : 0.f;
        float l = dx * dx + dy * dy + dz * dz;
        if (l >= dmax2) continue;
        if (dx == 0.f || (ndim > 1 && dy == 0.f) || (ndim > 2 && dz == 0.f)) {
          const uint32_t other = (uint32_t)(base + k);
          if (dx == 0.f) dx = fl::jiggle(i, other, 0, step, seed), l += dx * dx;
          if (ndim > 1 && dy == 0.f) dy = fl::jiggle(i, other, 1, step, seed), l += dy * dy;
          if (ndim > 2 && dz == 0.f) dz = fl::jiggle(i, other, 2, step, seed), l += dz * dz;
        }
        if (l < dmin2) l = sqrtf(dmin2 * l);
        const float w = __fdividef(o.w * alpha, l);
        ax += dx * w, ay += dy * w, az += dz * w;
      }
    }
    __syncthreads();
  }
  part[threadIdx.x] = make_float3(ax, ay, az);
  __syncthreads();
  if (!live || lane != 0) return;
  for (int s = 1; s < split; ++s) {
    float3 p = part[threadIdx.x + s];
    ax += p.x, ay += p.y, az += p.z;
  }
  float4 v = vel[i];
  v.x += ax;
  if (ndim > 1) v.y += ay;
  if (ndim > 2) v.z += az;
  vel[i] = v;
}

}  // namespace

size_t fl_tree_bytes(int64_t n) {
  const size_t m = (size_t)(n > 1 ? n - 1 : 1), N = (size_t)(n > 0 ? n : 1);
  const size_t blocks = (N + kThreads - 1) / kThreads;
  return align256(4 * m) * 3 + align256(4 * N) + align256(8 * m) + align256(m) +
         align256(4 * m) * 3 + align256(4 * (m + 1)) + align256(16 * m) + align256(16 * N) +
         align256(16 * (2 * N + 1)) +
         align256(8 * (2 * N + 1)) * 2 + align256(4 * blocks) + align256(32 * N) +
         align256(32 * blocks) + align256(4 * m) + align256(4 * (2 * N)) +
         align256((size_t)fl_walk_slots(n) * kWalkSpillPerWarp * 16) + align256(4) + 256;
}

int fl_walk_slots(int64_t n) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1)
    sms = 1;
  const int64_t warps = (n > 0 ? n : 1) + 31 >> 5;
  const int64_t want = (warps + kWalkWarps - 1) / kWalkWarps * kWalkWarps;
  const int64_t cap = (int64_t)sms * kWalkBlocksPerSm * kWalkWarps;
  return (int)(want < cap ? want : cap);
}

void fl_tree_carve(FlTreeBufs* t, void* base, int64_t n, int ndim) {
  const size_t m = (size_t)(n > 1 ? n - 1 : 1), N = (size_t)(n > 0 ? n : 1);
  const size_t blocks = (N + kThreads - 1) / kThreads;
  char* p = static_cast<char*>(base);
  auto take = [&](size_t bytes) {
    void* r = p;
    p += align256(bytes);
    return r;
  };
  t->n = (int)n, t->ndim = ndim;
  t->levels = ndim == 3 ? 21 : 24;
  t->bits = t->levels * ndim;
  t->left = (uint32_t*)take(4 * m);
  t->right = (uint32_t*)take(4 * m);
  t->parent = (uint32_t*)take(4 * m);
  t->leaf_parent = (uint32_t*)take(4 * N);
  t->range = (uint32_t*)take(8 * m);
  t->depth = (uint8_t*)take(m);
  t->count = (uint32_t*)take(4 * m);
  t->first = (uint32_t*)take(4 * m);
  t->flag = (uint32_t*)take(4 * (m + 1));
  t->up_list = (uint32_t*)take(4 * m);
  t->slot64 = (double*)take(8 * (2 * N + 1));
  t->cell = (float4*)take(16 * m);
  t->leaf = (float4*)take(16 * N);
  t->child_data = (float4*)take(16 * (2 * N + 1));
  t->child_meta = (uint2*)take(8 * (2 * N + 1));
  t->scan_scratch = take(4 * blocks);  // per-block totals of the child counts
  t->wsum = (double*)take(32 * N);
  t->wtiles = (double*)take(32 * blocks);  // per-block totals of the point records
  t->omask = (uint32_t*)take(4 * m);
  t->head_of = (uint32_t*)take(4 * (2 * N));
  t->walk_slots = fl_walk_slots(n);
  t->walk_blocks = 0;
  int dev = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&t->sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || t->sms < 1)
    t->sms = 1;
  t->spill = (uint4*)take((size_t)t->walk_slots * kWalkSpillPerWarp * 16);
  t->work = (uint32_t*)take(4);
}

void fl_launch_morton(const float4* pos, int n, int ndim, const FlReduce* red, uint64_t* keys,
                      uint32_t* vals, uint32_t* hist, int lo_bit, float* cube_out,
                      cudaStream_t st) {
  // one full wave of large blocks (2 of 1024 threads per SM, so that enough loads are in
  // flight): each block flushes its digit histograms with up to 1024 global atomics (4
  // passes), so fewer blocks contend less for the same counters (8 blocks of 256 per SM took
  // 9.5 us more per 1M keys; 1 block of 1024, 4 us more)
  int g = (n + kMortonThreads - 1) / kMortonThreads;
  if (g > 2 * fl_sms()) g = 2 * fl_sms();
  if (g < 1) g = 1;
  k_morton<<<g, kMortonThreads, 0, st>>>(pos, n, ndim, red, keys, vals, hist, lo_bit, cube_out);
}

int fl_fixed_exponent(int64_t n, double wmax) {
  if (!(wmax > 0)) return 32;
  const int e = 62 - (int)std::ceil(std::log2((double)(n > 1 ? n : 1) * wmax));
  return e < 0 ? 0 : e > 100 ? 100 : e;
}

void fl_launch_build_points(const FlTreeBufs* t, const uint64_t* skeys, const uint32_t* perm,
                            const float4* pos, const float* strength, bool closed,
                            const float* cube, int fx_exp, cudaStream_t st, int64_t* launches,
                            FlSegs segs) {
  const int n = t->n;
  const int nb = (n + kThreads - 1) / kThreads;
  k_build<1><<<nb, kThreads, 0, st>>>(skeys, perm, pos, strength, n, t->ndim, t->left, t->right,
                                      t->parent, t->leaf_parent, t->range, t->depth, t->leaf,
                                      closed ? reinterpret_cast<D4*>(t->wsum) : nullptr,
                                      reinterpret_cast<D4*>(t->wtiles), cube, fx_exp, segs);
  ++*launches;
  if (closed) {
    k_top4<<<1, kTopThreads, 0, st>>>(reinterpret_cast<D4*>(t->wtiles), nb);
    ++*launches;
  }
}

void fl_launch_build_nodes(const FlTreeBufs* t, const uint64_t* skeys, const uint32_t* perm,
                           const float4* pos, const float* strength, const float* cube,
                           int fx_exp, cudaStream_t st, int64_t* launches, FlSegs segs) {
  const int n = t->n;
  const int nb = (n + kThreads - 1) / kThreads;
  k_build<2><<<nb, kThreads, 0, st>>>(skeys, perm, pos, strength, n, t->ndim, t->left, t->right,
                                      t->parent, t->leaf_parent, t->range, t->depth, t->leaf,
                                      nullptr, nullptr, cube, fx_exp, segs);
  ++*launches;
}

void fl_launch_build(const FlTreeBufs* t, const uint64_t* skeys, const uint32_t* perm,
                     const float4* pos, const float* strength, bool closed, const float* cube,
                     int fx_exp, cudaStream_t st, int64_t* launches, FlSegs segs) {
  // two kernels: the internal nodes' searches are latency chains that want every warp an SM
  // can hold, which the points' fixed-point records and prefix (more registers) would limit
  fl_launch_build_points(t, skeys, perm, pos, strength, closed, cube, fx_exp, st, launches, segs);
  fl_launch_build_nodes(t, skeys, perm, pos, strength, cube, fx_exp, st, launches, segs);
}

void fl_launch_frontier(const FlTreeBufs* t, const uint64_t* skeys, uint32_t* err,
                        cudaStream_t st, int64_t* launches) {
  const int n = t->n, m = n - 1;
  const int g2 = (2 * n - 1 + kThreads - 1) / kThreads;
  cudaMemsetAsync(t->omask, 0, 4 * (size_t)m, st);
  k_frontier<<<g2, kThreads, 0, st>>>(n, t->ndim, skeys, t->parent, t->leaf_parent, t->range,
                                      t->depth, t->omask, t->head_of, err);
  ++*launches;
}

void fl_launch_cells(const FlTreeBufs* t, bool closed, float sign, const float* cube, int fx_exp,
                     int fp64_depth, uint32_t* err, cudaStream_t st, int64_t* launches,
                     FlSegs segs) {
  const int n = t->n, m = n - 1;
  const int g = (m + kThreads - 1) / kThreads, g2 = (2 * n - 1 + kThreads - 1) / kThreads;
  uint32_t* ctot = static_cast<uint32_t*>(t->scan_scratch);
  const D4* P = reinterpret_cast<const D4*>(t->wsum);
  const D4* Ptot = reinterpret_cast<const D4*>(t->wtiles);
  // the recursion's start list and its count, and the arrival counts (zeroed)
  uint32_t* up_count = t->flag + m;
  if (!closed) cudaMemsetAsync(t->flag, 0, 4 * (size_t)(m + 1), st);
  if (closed)
    k_heads<true><<<g, kThreads, 0, st>>>(n, t->ndim, t->parent, t->range, t->depth, t->omask,
                                          t->count, t->first, ctot, sign, P, Ptot, t->leaf, cube,
                                          fx_exp, t->cell, segs, t->up_list, up_count);
  else
    k_heads<false><<<g, kThreads, 0, st>>>(n, t->ndim, t->parent, t->range, t->depth, t->omask,
                                           t->count, t->first, ctot, sign, P, Ptot, t->leaf, cube,
                                           fx_exp, t->cell, segs, t->up_list, up_count);
  k_top_u32<<<1, kTopThreads, 0, st>>>(ctot, g);
  *launches += 2;
  k_slots<<<g2, kThreads, 0, st>>>(n, t->ndim, t->head_of, t->omask, t->parent, t->range,
                                   t->depth, t->count, t->first, ctot, t->cell, t->leaf,
                                   t->child_data, t->child_meta, err, segs, !closed,
                                   closed || fp64_depth == 0 ? nullptr : t->slot64);
  ++*launches;
  if (!closed) {
    // d3's c = Math.sqrt(4 / 2^dims), correctly rounded as IEEE sqrt is on host and device
    const double c1 = std::sqrt(4.0 / (double)(1 << t->ndim));
    k_cells_up<<<g, kThreads, 0, st>>>(n, t->ndim, t->head_of, t->omask, t->depth, t->count,
                                       t->first, ctot, t->flag, t->child_data, t->child_meta,
                                       t->slot64, fp64_depth, c1, err, segs, t->up_list, up_count);
    ++*launches;
  }
}

void fl_launch_aggregate(const FlTreeBufs* t, const uint64_t* skeys, bool closed, float sign,
                         const float* cube, int fx_exp, int fp64_depth, uint32_t* err,
                         cudaStream_t st, int64_t* launches, FlSegs segs) {
  fl_launch_frontier(t, skeys, err, st, launches);
  fl_launch_cells(t, closed, sign, cube, fx_exp, fp64_depth, err, st, launches, segs);
}

// Blocks of this walk variant resident on one SM (queried once), at most kWalkBlocksPerSm.
template <int NDIM, int G, bool STATS, bool DMAX, bool BATCH>
int walk_blocks_per_sm() {
  // an atomic: host threads racing on the first query store the same value
  static std::atomic<int> blocks{0};
  int c = blocks.load(std::memory_order_relaxed);
  if (!c) {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_walk<NDIM, G, STATS, DMAX, BATCH>,
                                                      kWalkThreads, 0) != cudaSuccess || b < 1) {
      cudaGetLastError();
      b = 1;
    }
    c = b < kWalkBlocksPerSm ? b : kWalkBlocksPerSm;
    blocks.store(c, std::memory_order_relaxed);
  }
  return c;
}

template <int NDIM, bool STATS, bool DMAX>
int walk_lanes_blocks_per_sm() {
  static std::atomic<int> blocks{0};
  int c = blocks.load(std::memory_order_relaxed);
  if (!c) {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_walk_lanes<NDIM, STATS, DMAX>,
                                                      kWalkThreads, 0) != cudaSuccess || b < 1) {
      cudaGetLastError();
      b = 1;
    }
    c = b < kWalkBlocksPerSm ? b : kWalkBlocksPerSm;
    blocks.store(c, std::memory_order_relaxed);
  }
  return c;
}

int fl_walk_group_for(int n) { return n <= kLaneWalkMaxNodes ? 1 : 32; }

void fl_launch_walk(const FlTreeBufs* t, const uint32_t* perm, const float* cube, float4* vel,
                    float alpha, double theta2, double dmin2, double dmax2, uint32_t step,
                    uint32_t seed, uint32_t* err, unsigned long long* stats, int group,
                    cudaStream_t st, FlSegs segs, const FlTick* tk) {
  const int n = t->n;
  const int warps = segs.graphs ? segs.ngroups : (n + 31) / 32;
  // a persistent grid of the blocks that fit on the device at once (and that the spill buffer
  // has regions for), each warp walking every (grid)-th group of 32 points
  const int cap = t->walk_slots / kWalkWarps;
  // the counter is 0 before a launch: zeroed with the scratch, and each launch's last claim puts
  // it back (a batch, whose tree buffers are carved anew as it grows, zeroes it here as well)
  if (segs.graphs) cudaMemsetAsync(t->work, 0, 4, st);
  const float fmax2 = dmax2 > 3e38 ? INFINITY : (float)dmax2;
#define FL_WALK_ONE(D, G, S, M, B)                                                             \
  do {                                                                                         \
    int per = walk_blocks_per_sm<D, G, S, M, B>();                                             \
    if (t->walk_blocks > 0 && t->walk_blocks < per) per = t->walk_blocks;                      \
    int g = t->sms * per;                                                                      \
    if (g > cap) g = cap;                                                                      \
    if (g < 1) g = 1;                                                                          \
    k_walk<D, G, S, M, B><<<g, kWalkThreads, 0, st>>>(                                         \
        t->child_data, t->child_meta, t->leaf, perm, cube, vel, n, alpha, theta2,              \
        (float)dmin2, fmax2, step, seed, err, stats, t->spill, warps, t->work, segs, tk);      \
  } while (0)
#define FL_WALK(D, G)                                                                          \
  do {                                                                                         \
    if (stats) FL_WALK_ONE(D, G, true, true, false);                                           \
    else if (fmax2 < INFINITY) FL_WALK_ONE(D, G, false, true, false);                          \
    else FL_WALK_ONE(D, G, false, false, false);                                               \
  } while (0)
  // a batch: distanceMax per graph (the walk tests it when any graph has a finite one)
#define FL_WALK_BATCH(D)                                                                       \
  do {                                                                                         \
    if (fmax2 < INFINITY) FL_WALK_ONE(D, 32, false, true, true);                               \
    else FL_WALK_ONE(D, 32, false, false, true);                                               \
  } while (0)
  if (!segs.graphs && group == 0) group = fl_walk_group_for(n);
  if (!segs.graphs && group == 1) {
    // one point per warp: no more blocks than the points need (the stacks are in shared
    // memory, so the grid needs no spill regions)
#define FL_LANES_ONE(D, S, M)                                                                  \
  do {                                                                                         \
    int per = walk_lanes_blocks_per_sm<D, S, M>();                                             \
    if (t->walk_blocks > 0 && t->walk_blocks < per) per = t->walk_blocks;                      \
    int g = t->sms * per;                                                                      \
    if (g > (n + kWalkWarps - 1) / kWalkWarps) g = (n + kWalkWarps - 1) / kWalkWarps;          \
    if (g < 1) g = 1;                                                                          \
    k_walk_lanes<D, S, M><<<g, kWalkThreads, 0, st>>>(                                         \
        t->child_data, t->child_meta, t->leaf, perm, cube, vel, n, alpha, theta2,              \
        (float)dmin2, fmax2, step, seed, err, stats, t->work, tk);                             \
  } while (0)
#define FL_LANES(D)                                                                            \
  do {                                                                                         \
    if (stats) FL_LANES_ONE(D, true, true);                                                    \
    else if (fmax2 < INFINITY) FL_LANES_ONE(D, false, true);                                   \
    else FL_LANES_ONE(D, false, false);                                                        \
  } while (0)
    if (t->ndim == 3) FL_LANES(3);
    else if (t->ndim == 2) FL_LANES(2);
    else FL_LANES(1);
#undef FL_LANES
#undef FL_LANES_ONE
  } else if (segs.graphs) {
    if (t->ndim == 3) FL_WALK_BATCH(3);
    else if (t->ndim == 2) FL_WALK_BATCH(2);
    else FL_WALK_BATCH(1);
  } else if (group == 32) {
    if (t->ndim == 3) FL_WALK(3, 32);
    else if (t->ndim == 2) FL_WALK(2, 32);
    else FL_WALK(1, 32);
  } else {
    if (t->ndim == 3) FL_WALK(3, 16);
    else if (t->ndim == 2) FL_WALK(2, 16);
    else FL_WALK(1, 16);
  }
#undef FL_WALK
#undef FL_WALK_BATCH
#undef FL_WALK_ONE
}

void fl_launch_allpairs(const float4* pos, const float* strength, float4* vel, int n, int ndim,
                        float alpha, float dmin2, float dmax2, uint32_t step, uint32_t seed,
                        cudaStream_t st, const FlTick* tk) {
  // threads per point: enough threads in flight for small graphs (2^18 in all), at most 16
  int split = 1;
  while (split < 16 && (int64_t)n * split < (1 << 18)) split *= 2;
  const int per = kPairThreads / split;
  const int g = (n + per - 1) / per;
  k_allpairs<<<g < 1 ? 1 : g, kPairThreads, 0, st>>>(pos, strength, vel, n, ndim, alpha, dmin2,
                                                     dmax2, step, seed, split, tk);
}

void fl_launch_bgraph(int graphs, int ndim, const int32_t* off, const FlReduce* red,
                      const FlBatchParams* prm, const double* alpha, FlGraph* gr, cudaStream_t st) {
  k_bgraph<<<(graphs + kThreads - 1) / kThreads, kThreads, 0, st>>>(graphs, ndim, off, red, prm,
                                                                    alpha, gr);
}

void fl_launch_bmorton(const float4* pos, int n, int ndim, const uint32_t* gid, const FlGraph* gr,
                       uint64_t* keys, uint32_t* vals, uint32_t* hist, int lo_bit, cudaStream_t st) {
  int g = (n + kMortonThreads - 1) / kMortonThreads;  // as fl_launch_morton
  if (g > 2 * fl_sms()) g = 2 * fl_sms();
  if (g < 1) g = 1;
  k_bmorton<<<g, kMortonThreads, 0, st>>>(pos, n, ndim, gid, gr, keys, vals, hist, lo_bit);
}

void fl_launch_bgidkey(int n, const uint32_t* mperm, const uint32_t* gid, const int32_t* off,
                       int graphs, uint64_t* keys, uint32_t* vals, uint32_t* hist, cudaStream_t st) {
  // as fl_launch_morton: few, large blocks (each flushes its histograms with global atomics
  // and loads the graph offsets once)
  int g = (n + kMortonThreads - 1) / kMortonThreads;
  if (g > 2 * fl_sms()) g = 2 * fl_sms();
  if (g < 1) g = 1;
  k_bgidkey<<<g, kMortonThreads, 0, st>>>(n, mperm, gid, off, graphs, keys, vals, hist);
}

void fl_launch_bgather(int n, const uint32_t* order2, const uint64_t* mkeys, const uint32_t* mperm,
                       const uint32_t* gid, uint64_t* skeys, uint32_t* perm, uint32_t* gid_pos,
                       cudaStream_t st) {
  k_bgather<<<(n + kThreads - 1) / kThreads, kThreads, 0, st>>>(n, order2, mkeys, mperm, gid,
                                                                 skeys, perm, gid_pos);
}
