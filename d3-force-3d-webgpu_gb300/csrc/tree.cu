// forceManyBody on the GPU: the d3 Barnes-Hut tree, built every tick and walked per point.
//
// The tree is exactly the one d3-octree / d3-quadtree / d3-binarytree build for
// src/manyBody.js (cube = floor(min) with a power-of-two size, midpoint splits, children in the
// order bit k = coordinate k above the midpoint), cut at LEVELS levels (21 in 3D, 24 in 1D/2D):
//
//   morton     the d3 cube from the bounding box, each point's cell at the finest level (exact),
//              interleaved into a left-aligned Morton key in d3's child order; the sort's digit
//              histograms are counted in the same pass
//   sort       onesweep radix sort of (key, node) (sort.cu)
//   build      Karras (2012) binary radix tree over the sorted keys; each internal node's d3
//              depth = common prefix bits / DIMS; the sorted (position, strength) of the points
//   heads      a binary node whose depth is deeper than its parent's heads a d3 cell (the binary
//              nodes below it at the same depth are splits inside that cell); its d3 children
//              are counted, and child slots are allocated by a scan (every cell's children are
//              contiguous, so the walk reads them in one sweep)
//   aggregate  bottom-up with atomic arrival flags: each cell's value and centre of mass from its
//              children exactly as manyBody.js accumulate() does (value = sqrt(4 / 2^DIMS) * sum
//              of the children's values; centroid weighted by |value|), through chains of
//              one-child cells by powers of the same factor; FP64 sums for the top levels
//   walk       one warp per 32 consecutive sorted points walks the union of their d3 traversals
//              with a stack in shared memory; every point applies apply() of manyBody.js for
//              itself: a cell is approximated at the first (widest) depth of its chain where
//              w^2 / theta^2 < l, points are summed exactly, distanceMin / distanceMax as d3.
//
// Points with the same code at the finest level share the deepest cell as its children.
#include <math.h>

#include "kernels.h"

namespace {

constexpr uint32_t kLeaf = 0x80000000u;
constexpr uint32_t kIndex = 0x7fffffffu;
constexpr uint32_t kLeafMark = 0xffffffffu;
constexpr uint32_t kCountMask = (1u << 26) - 1;
constexpr int kFp64Depth = 6;  // cells at depths < 6 sum their children in FP64
constexpr int kThreads = 256;

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

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
  const int e2 = k * (2 - ndim);
  const float odd = (e2 & 1) ? 1.41421356237309515f : 1.f;
  return ldexpf(odd, e2 >> 1);
}

// The cell index of x at the finest level, floor((x - origin) * 2^e), in exact arithmetic:
// e >= 0: floor(x * 2^e) and origin * 2^e are exact floats, and so is their difference, an
// integer below 2^24; e < 0 (cubes wider than 2^LEVELS): in FP64, where every step is exact.
__device__ __forceinline__ uint64_t cell_of(float x, float origin, int e, uint32_t top) {
  float c;
  if (e >= 0) {
    const float s = __int_as_float((e + 127) << 23);
    c = floorf(x * s) - origin * s;
  } else {
    c = (float)floor(ldexp(floor((double)x) - (double)origin, e));
  }
  c = fminf(fmaxf(c, 0.f), (float)top);
  return (uint64_t)c;
}

// Bounding box -> d3 cube -> keys; digit histograms of the sort passes in the same read.
__global__ void __launch_bounds__(kThreads) k_morton(const float4* __restrict__ pos, int n,
                                                     int ndim, const FlReduce* red,
                                                     uint64_t* __restrict__ keys,
                                                     uint32_t* __restrict__ vals,
                                                     uint32_t* __restrict__ hist, int lo_bit,
                                                     float* cube_out) {
  __shared__ float s_origin[3];
  __shared__ int s_lg;
  __shared__ uint32_t sh[8 * 256];
  const int L = levels_of(ndim), bits = L * ndim, passes = (64 - lo_bit + 7) / 8;
  if (threadIdx.x == 0) {
    // d3 cover(): x0 = floor(min); double a power-of-two size until max < x0 + size (FP64)
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    for (int k = 0; k < ndim; ++k) {
      lo[k] = floor((double)fl::unordered(~red->lo[k]));
      hi[k] = (double)fl::unordered(red->hi[k]);
    }
    double size = 1;
    int lg = 0;
    for (;;) {
      bool inside = true;
      for (int k = 0; k < ndim; ++k)
        if (!(hi[k] < lo[k] + size)) inside = false;
      if (inside || lg >= 1100) break;
      size *= 2, ++lg;
    }
    for (int k = 0; k < 3; ++k) s_origin[k] = (float)lo[k];
    s_lg = lg;
    if (blockIdx.x == 0) {
      cube_out[0] = (float)lo[0], cube_out[1] = (float)lo[1], cube_out[2] = (float)lo[2];
      cube_out[3] = (float)size;
      cube_out[4] = (float)lg;
    }
  }
  for (int i = threadIdx.x; i < 8 * 256; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  const int e = L - s_lg;
  const uint32_t top = (1u << L) - 1;
  const int stride = gridDim.x * blockDim.x;
  for (int base = blockIdx.x * blockDim.x; base < n; base += stride) {
    const int i = base + threadIdx.x;
    const bool ok = i < n;
    uint64_t key = 0;
    if (ok) {
      float4 p = pos[i];
      uint64_t qx = cell_of(p.x, s_origin[0], e, top);
      if (ndim == 3)
        key = spread3(qx) | spread3(cell_of(p.y, s_origin[1], e, top)) << 1 |
              spread3(cell_of(p.z, s_origin[2], e, top)) << 2;
      else if (ndim == 2)
        key = spread2(qx) | spread2(cell_of(p.y, s_origin[1], e, top)) << 1;
      else
        key = qx;
      key <<= (64 - bits);
      keys[i] = key;
      vals[i] = (uint32_t)i;
    }
    for (int p = 0; p < passes; ++p) {
      uint32_t d = ok ? (uint32_t)(key >> (lo_bit + 8 * p)) & 255u : 256u + (threadIdx.x & 31);
      uint32_t peers = __match_any_sync(FL_FULL, d);
      if (ok && (int)(threadIdx.x & 31) == 31 - __clz(peers)) atomicAdd(&sh[p * 256 + d], __popc(peers));
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < passes * 256; i += blockDim.x)
    if (sh[i]) atomicAdd(&hist[i], sh[i]);
}

__device__ __forceinline__ int kdelta(const uint64_t* __restrict__ k, int n, uint64_t ki, int i,
                                      int j) {
  if (j < 0 || j >= n) return -1;
  uint64_t kj = k[j];
  return ki != kj ? __clzll(ki ^ kj) : 64 + __clz(i ^ j);
}

// Karras (2012), "Maximizing parallelism in the construction of BVHs, octrees, and k-d trees":
// internal node i covers sorted range [first, last] and splits it where the common prefix grows.
__global__ void __launch_bounds__(kThreads) k_build(
    const uint64_t* __restrict__ k, const uint32_t* __restrict__ perm,
    const float4* __restrict__ pos, const float* __restrict__ strength, int n, int ndim,
    uint32_t* __restrict__ left, uint32_t* __restrict__ right, uint32_t* __restrict__ parent,
    uint32_t* __restrict__ leaf_parent, uint32_t* __restrict__ range, uint8_t* __restrict__ depth,
    float4* __restrict__ leaf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const uint32_t node = perm[i];
    float4 p = pos[node];
    p.w = strength[node];
    leaf[i] = p;
  }
  if (i >= n - 1) return;
  const int L = levels_of(ndim), bits = L * ndim;
  const uint64_t ki = k[i];
  const int up = kdelta(k, n, ki, i, i + 1), dn = kdelta(k, n, ki, i, i - 1);
  const int d = up > dn ? 1 : -1;
  const int dmin = up > dn ? dn : up;
  int64_t lmax = 2;
  while (kdelta(k, n, ki, i, (int)(i + lmax * d)) > dmin) lmax *= 2;
  int64_t len = 0;
  for (int64_t t = lmax >> 1; t >= 1; t >>= 1)
    if (kdelta(k, n, ki, i, (int)(i + (len + t) * d)) > dmin) len += t;
  const int j = (int)(i + len * d);
  const int dnode = kdelta(k, n, ki, i, j);
  int64_t s = 0, t = len;
  do {
    t = (t + 1) >> 1;
    if (kdelta(k, n, ki, i, (int)(i + (s + t) * d)) > dnode) s += t;
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

// Whether internal node i heads a d3 cell, and how many d3 children that cell has.
__global__ void __launch_bounds__(kThreads) k_heads(int n, int ndim,
                                                    const uint32_t* __restrict__ left,
                                                    const uint32_t* __restrict__ right,
                                                    const uint32_t* __restrict__ parent,
                                                    const uint32_t* __restrict__ range,
                                                    const uint8_t* __restrict__ depth,
                                                    uint32_t* __restrict__ count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  const int D = depth[i];
  const bool head = i == 0 || depth[parent[i]] < D;
  uint32_t c = 0;
  if (head) {
    if (D == levels_of(ndim)) {
      c = range[2 * i + 1] - range[2 * i] + 1;
    } else {
      uint32_t stack[16];
      int sp = 0;
      stack[sp++] = right[i];
      stack[sp++] = left[i];
      while (sp > 0) {
        uint32_t x = stack[--sp];
        if (!(x & kLeaf) && depth[x] == D && sp < 15) {
          stack[sp++] = right[x];
          stack[sp++] = left[x];
        } else {
          ++c;
        }
      }
    }
  }
  count[i] = c;
}

// Bottom-up aggregation with arrival flags (the second thread to reach a node proceeds).
__global__ void __launch_bounds__(kThreads) k_aggregate(
    int n, int ndim, const uint32_t* __restrict__ left, const uint32_t* __restrict__ right,
    const uint32_t* __restrict__ parent, const uint32_t* __restrict__ leaf_parent,
    const uint32_t* __restrict__ range, const uint8_t* __restrict__ depth,
    const uint32_t* __restrict__ count, const uint32_t* __restrict__ first,
    uint32_t* __restrict__ flag, float4* cell, const float4* __restrict__ leaf,
    float4* __restrict__ cdata, uint2* __restrict__ cmeta, uint32_t* err) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int L = levels_of(ndim);
  const double c1 = sqrt(4.0 / (double)(1 << ndim));  // sqrt(4 / numChildren)
  uint32_t node = leaf_parent[s];
  for (int guard = 0;; ++guard) {
    if (guard > 256) {
      atomicOr(err, FL_ERR_TREE);
      return;
    }
    __threadfence();
    if (atomicAdd(&flag[node], 1u) == 0) return;  // the sibling subtree is still working
    __threadfence();
    const uint32_t cnt = count[node];
    if (cnt) {
      const int D = depth[node];
      const uint32_t slot0 = first[node];
      if ((uint64_t)slot0 + cnt > 2ull * (uint64_t)n + 1ull || D > L) {  // a malformed tree
        atomicOr(err, FL_ERR_TREE);
        return;
      }
      const bool wide = D < kFp64Depth;
      double sv = 0, sa = 0, sx = 0, sy = 0, sz = 0;
      float fv = 0, fa = 0, fx = 0, fy = 0, fz = 0;
      float4 firstpos = make_float4(0, 0, 0, 0);
      uint32_t j = 0;
      auto take = [&](float4 q, float v, uint2 meta) {
        // q: position (or centroid) and own value; v: value seen at depth D + 1
        if (j == 0) firstpos = q;
        if (j < cnt) {
          cdata[slot0 + j] = q;
          cmeta[slot0 + j] = meta;
        }
        ++j;
        const float a = fabsf(v);
        if (!(a > 0.f)) return;  // d3 skips children whose value is 0
        if (wide) {
          sv += v, sa += a, sx += (double)a * q.x, sy += (double)a * q.y, sz += (double)a * q.z;
        } else {
          fv += v, fa += a, fx += a * q.x, fy += a * q.y, fz += a * q.z;
        }
      };
      auto child = [&](uint32_t x) {
        if (x & kLeaf) {
          const uint32_t li = x & kIndex;
          const float4 q = leaf[li];
          take(q, q.w, make_uint2(li, kLeafMark));
        } else {
          const float4 q = __ldcg(cell + x);
          const int Dh = depth[x];
          // the chain of one-child cells from D + 1 down to Dh scales the value by c per level
          const float v = q.w * damp(ndim, Dh - D - 1);
          take(q, v, make_uint2(first[x], count[x] | ((uint32_t)Dh << 26)));
        }
      };
      if (D == L) {
        const uint32_t a = range[2 * node], b = range[2 * node + 1];
        for (uint32_t li = a; li <= b; ++li) child(kLeaf | li);
      } else {
        uint32_t stack[16];
        int sp = 0;
        stack[sp++] = right[node];
        stack[sp++] = left[node];
        while (sp > 0) {
          uint32_t x = stack[--sp];
          if (!(x & kLeaf) && depth[x] == D && sp < 15) {
            stack[sp++] = right[x];
            stack[sp++] = left[x];
          } else {
            child(x);
          }
        }
      }
      float4 out;
      double tv, ta;
      if (wide) {
        tv = sv, ta = sa;
        if (sa > 0) out = make_float4((float)(sx / sa), (float)(sy / sa), (float)(sz / sa), 0.f);
        else out = firstpos;
      } else {
        tv = fv, ta = fa;
        if (fa > 0.f) out = make_float4(fx / fa, fy / fa, fz / fa, 0.f);
        else out = firstpos;
      }
      // d3 skips a cell whose children's values add up to 0 exactly; the sum here carries
      // rounding, so a cancellation to within 2^-20 of the magnitudes counts as 0
      out.w = fabs(tv) <= ta * 0x1p-20 ? 0.f : (float)(tv * c1);
      cell[node] = out;
      if (node == 0) {
        cdata[0] = out;
        cmeta[0] = make_uint2(slot0, cnt | ((uint32_t)D << 26));
      }
    }
    if (node == 0) return;
    node = parent[node];
  }
}

constexpr int kWalkThreads = 128;
constexpr int kWalkWarps = kWalkThreads / 32;
constexpr int kStack = 160;

__global__ void __launch_bounds__(kWalkThreads) k_walk(
    const float4* __restrict__ cdata, const uint2* __restrict__ cmeta,
    const float4* __restrict__ leaf, const uint32_t* __restrict__ perm,
    const float* __restrict__ cube, float4* __restrict__ vel, int n, int ndim, float alpha,
    double theta2, float dmin2, float dmax2, uint32_t step, uint32_t seed, uint32_t* err) {
  __shared__ float s_T[32], s_damp[32];
  __shared__ uint4 s_stack[kWalkWarps][kStack];
  if (threadIdx.x < 32) {
    const int k = threadIdx.x;
    const double w = ldexp((double)cube[3], -k);
    s_T[k] = (float)(w * w / theta2);
    s_damp[k] = damp(ndim, k);
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int t = (blockIdx.x * kWalkWarps + warp) * 32 + lane;
  const bool live = t < n;
  const uint32_t act = __ballot_sync(FL_FULL, live);
  if (!act) return;
  const float4 me = live ? leaf[t] : make_float4(0, 0, 0, 0);
  const uint32_t myid = live ? perm[t] : 0;
  float ax = 0.f, ay = 0.f, az = 0.f;
  uint4* stk = s_stack[warp];
  if (lane == 0) stk[0] = make_uint4(0u, 1u, 0u, act);  // the root: slot 0, top depth 0
  int sp = 1;
  __syncwarp();
  uint32_t guard = 0;
  const uint32_t guard_max = 4u * (uint32_t)n + 64u;
  const uint32_t slot_cap = 2u * (uint32_t)n + 1u;
  while (sp > 0) {
    const uint4 e = stk[--sp];
    __syncwarp();
    const bool mine = (e.w >> lane) & 1u;
    const uint32_t top = e.z;
    uint32_t end = e.x + e.y;
    if (end > slot_cap || e.x > end) {  // a malformed tree: report, never read out of bounds
      if (lane == 0) atomicOr(err, FL_ERR_TREE);
      end = e.x < slot_cap ? slot_cap : e.x;
    }
    for (uint32_t c0 = e.x; c0 < end; c0 += 8) {
      float4 cd[8];
      uint2 cm[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        if (c0 + j < end) {
          cd[j] = __ldg(cdata + c0 + j);
          cm[j] = __ldg(cmeta + c0 + j);
        }
      }
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        if (c0 + j >= end) break;
        const float4 q = cd[j];
        const uint2 m = cm[j];
        bool open = false;
        if (mine && q.w != 0.f && !(m.y == kLeafMark && m.x == (uint32_t)t)) {
          float dx = q.x - me.x, dy = q.y - me.y, dz = q.z - me.z;
          float l = dx * dx + dy * dy + dz * dz;
          float v = q.w;
          bool apply = true;
          if (m.y != kLeafMark) {
            const uint32_t D = (m.y >> 26) & 31u;
            if (s_T[D] >= l) {
              open = true;  // not far enough even at the deepest cell of the chain
              apply = false;
            } else {
              uint32_t k = top < D ? top : D;
              while (k < D && s_T[k] >= l) ++k;  // the widest cell of the chain that passes
              v *= s_damp[D - k];
            }
          }
          if (apply && l < dmax2) {
            if (dx == 0.f || (ndim > 1 && dy == 0.f) || (ndim > 2 && dz == 0.f)) {
              const uint32_t other =
                  m.y == kLeafMark ? perm[m.x < (uint32_t)n ? m.x : 0] : (uint32_t)n + c0 + j;
              if (dx == 0.f) dx = fl::jiggle(myid, other, 0, step, seed), l += dx * dx;
              if (ndim > 1 && dy == 0.f) dy = fl::jiggle(myid, other, 1, step, seed), l += dy * dy;
              if (ndim > 2 && dz == 0.f) dz = fl::jiggle(myid, other, 2, step, seed), l += dz * dz;
            }
            if (l < dmin2) l = sqrtf(dmin2 * l);
            const float w = __fdividef(v * alpha, l);
            ax += dx * w, ay += dy * w, az += dz * w;
          }
        }
        const uint32_t om = __ballot_sync(FL_FULL, open);
        if (om) {
          if (sp < kStack) {
            if (lane == 0) stk[sp] = make_uint4(m.x, m.y & kCountMask, (m.y >> 26) + 1u, om);
            ++sp;
          } else if (lane == 0) {
            atomicOr(err, FL_ERR_STACK);
          }
        }
        __syncwarp();
      }
    }
    if (++guard > guard_max) {
      if (lane == 0) atomicOr(err, FL_ERR_STACK);
      break;
    }
  }
  if (!live) return;
  float4 v = vel[myid];
  v.x += ax;
  if (ndim > 1) v.y += ay;
  if (ndim > 2) v.z += az;
  vel[myid] = v;
}

// Exact all-pairs sum (theta ~ 0; src/gpu/passes/manyBody.js:5-16 semantics): each block
// streams the points through shared memory in tiles.
constexpr int kPairThreads = 256;
__global__ void __launch_bounds__(kPairThreads) k_allpairs(const float4* __restrict__ pos,
                                                           const float* __restrict__ strength,
                                                           float4* __restrict__ vel, int n,
                                                           int ndim, float alpha, float dmin2,
                                                           float dmax2, uint32_t step,
                                                           uint32_t seed, int split) {
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
  return align256(4 * m) * 3 + align256(4 * N) + align256(8 * m) + align256(m) +
         align256(4 * m) * 3 + align256(16 * m) + align256(16 * N) + align256(16 * (2 * N + 1)) +
         align256(8 * (2 * N + 1)) + fl_scan_bytes((int64_t)m) + 256;
}

void fl_tree_carve(FlTreeBufs* t, void* base, int64_t n, int ndim) {
  const size_t m = (size_t)(n > 1 ? n - 1 : 1), N = (size_t)(n > 0 ? n : 1);
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
  t->flag = (uint32_t*)take(4 * m);
  t->cell = (float4*)take(16 * m);
  t->leaf = (float4*)take(16 * N);
  t->child_data = (float4*)take(16 * (2 * N + 1));
  t->child_meta = (uint2*)take(8 * (2 * N + 1));
  t->scan_scratch = take(fl_scan_bytes((int64_t)m));
}

void fl_launch_morton(const float4* pos, int n, int ndim, const FlReduce* red, uint64_t* keys,
                      uint32_t* vals, uint32_t* hist, int lo_bit, float* cube_out,
                      cudaStream_t st) {
  int g = (n + kThreads - 1) / kThreads;
  if (g > 8 * 152) g = 8 * 152;
  if (g < 1) g = 1;
  k_morton<<<g, kThreads, 0, st>>>(pos, n, ndim, red, keys, vals, hist, lo_bit, cube_out);
}

void fl_launch_build(const FlTreeBufs* t, const uint64_t* skeys, const uint32_t* perm,
                     const float4* pos, const float* strength, cudaStream_t st, int64_t* launches) {
  const int n = t->n;
  k_build<<<(n + kThreads - 1) / kThreads, kThreads, 0, st>>>(skeys, perm, pos, strength, n, t->ndim,
                                                              t->left, t->right, t->parent,
                                                              t->leaf_parent, t->range, t->depth,
                                                              t->leaf);
  ++*launches;
}

void fl_launch_aggregate(const FlTreeBufs* t, uint32_t* err, cudaStream_t st, int64_t* launches) {
  const int n = t->n, m = n - 1;
  const int g = (m + kThreads - 1) / kThreads;
  k_heads<<<g, kThreads, 0, st>>>(n, t->ndim, t->left, t->right, t->parent, t->range, t->depth,
                                  t->count);
  ++*launches;
  fl_scan_exclusive(t->count, t->first, m, 1u, t->scan_scratch, err, st, launches);
  cudaMemsetAsync(t->flag, 0, 4 * (size_t)m, st);
  k_aggregate<<<(n + kThreads - 1) / kThreads, kThreads, 0, st>>>(
      n, t->ndim, t->left, t->right, t->parent, t->leaf_parent, t->range, t->depth, t->count,
      t->first, t->flag, t->cell, t->leaf, t->child_data, t->child_meta, err);
  ++*launches;
}

void fl_launch_walk(const FlTreeBufs* t, const uint32_t* perm, const float* cube, float4* vel,
                    float alpha, double theta2, double dmin2, double dmax2, uint32_t step,
                    uint32_t seed, uint32_t* err, cudaStream_t st) {
  const int n = t->n;
  const int warps = (n + 31) / 32;
  const int g = (warps + kWalkWarps - 1) / kWalkWarps;
  const float fmax2 = dmax2 > 3e38 ? INFINITY : (float)dmax2;
  k_walk<<<g, kWalkThreads, 0, st>>>(t->child_data, t->child_meta, t->leaf, perm, cube, vel, n,
                                     t->ndim, alpha, theta2, (float)dmin2, fmax2, step, seed, err);
}

void fl_launch_allpairs(const float4* pos, const float* strength, float4* vel, int n, int ndim,
                        float alpha, float dmin2, float dmax2, uint32_t step, uint32_t seed,
                        cudaStream_t st) {
  // threads per point: enough threads in flight for small graphs (2^18 in all), at most 16
  int split = 1;
  while (split < 16 && (int64_t)n * split < (1 << 18)) split *= 2;
  const int per = kPairThreads / split;
  const int g = (n + per - 1) / per;
  k_allpairs<<<g < 1 ? 1 : g, kPairThreads, 0, st>>>(pos, strength, vel, n, ndim, alpha, dmin2,
                                                     dmax2, step, seed, split);
}
