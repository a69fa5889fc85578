// forceCollide (src/collide.js:30-95) in the all-at-once form of the reference's GPU pass
// (src/gpu/passes/collide.js:5-17): every node takes its own share of every overlapping pair,
// against one snapshot of p + v (read as p and v_in; v_out is written, so nothing is copied):
//     d = s_i - s_j,  r = r_i + r_j;  |d| < r:  v_i += d (r - |d|) / |d| * strength * r_j^2 / (r_i^2 + r_j^2)
// A zero component of d is replaced by the pair's antisymmetric jiggle.
//
// Small graphs test every pair (tiled through shared memory). Large graphs find the pairs with
// a uniform grid over cell-sorted nodes: cells 2 * max radius wide, so overlapping nodes sit in
// the same or adjacent cells. Each cell maps to a slot of a table of 2^bits >= 2n slots: cells
// are grouped in blocks (4^3, 8^2 or 64 cells) whose cells take consecutive slots in Morton
// order from a hashed block offset, so the sort by slot keeps nearby cells nearby. Two cells
// sharing a slot only cost extra distance tests; a node looks through each distinct slot of its
// 3^d neighbour cells once. Run starts are never cleared: a start is trusted only if the sorted
// keys confirm it.
#include "kernels.h"

namespace {

constexpr int kThreads = 256;

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

__device__ __forceinline__ void pair_push(float3 me, float ri2, float ri, float4 o, uint32_t idi,
                                          uint32_t idj, int ndim, float strength, uint32_t step,
                                          uint32_t seed, float3& acc) {
  const float rj = o.w, r = ri + rj;
  float dx = me.x - o.x, dy = ndim > 1 ? me.y - o.y : 0.f, dz = ndim > 2 ? me.z - o.z : 0.f;
  float l = dx * dx + dy * dy + dz * dz;
  if (!(l < r * r)) return;
  if (dx == 0.f || (ndim > 1 && dy == 0.f) || (ndim > 2 && dz == 0.f)) {
    if (dx == 0.f) dx = fl::jiggle(idi, idj, 0, step, seed), l += dx * dx;
    if (ndim > 1 && dy == 0.f) dy = fl::jiggle(idi, idj, 1, step, seed), l += dy * dy;
    if (ndim > 2 && dz == 0.f) dz = fl::jiggle(idi, idj, 2, step, seed), l += dz * dz;
  }
  const float len = sqrtf(l);
  const float k = (r - len) / len * strength;
  const float rj2 = rj * rj, w = rj2 / (ri2 + rj2);
  acc.x += dx * k * w;
  acc.y += dy * k * w;
  acc.z += dz * k * w;
}

__global__ void __launch_bounds__(kThreads) k_collide_allpairs(
    const float4* __restrict__ pos, const float4* __restrict__ vel_in, float4* __restrict__ vel_out,
    const float* __restrict__ radius, int n, int ndim, float strength, uint32_t step,
    uint32_t seed, int split, const FlTick* __restrict__ tk) {
  if (tk) step = tk->step, seed = tk->seed;
  __shared__ float4 tile[kThreads];
  __shared__ float3 part[kThreads];
  const int per = kThreads / split;
  const int lane = threadIdx.x % split;
  const int i = blockIdx.x * per + threadIdx.x / split;
  const bool live = i < n;
  float4 p = make_float4(0, 0, 0, 0), v = p;
  float ri = 0.f;
  if (live) p = pos[i], v = vel_in[i], ri = radius[i];
  const float3 me = make_float3(p.x + v.x, p.y + v.y, p.z + v.z);
  const float ri2 = ri * ri;
  float3 acc = make_float3(0.f, 0.f, 0.f);
  for (int base = 0; base < n; base += kThreads) {
    const int j = base + threadIdx.x;
    float4 q = make_float4(0, 0, 0, 0);
    if (j < n) {
      float4 a = pos[j], b = vel_in[j];
      q = make_float4(a.x + b.x, a.y + b.y, a.z + b.z, radius[j]);
    }
    tile[threadIdx.x] = q;
    __syncthreads();
    const int cnt = n - base < kThreads ? n - base : kThreads;
    if (live)
      for (int k = lane; k < cnt; k += split)
        if (base + k != i) pair_push(me, ri2, ri, tile[k], i, base + k, ndim, strength, step, seed, acc);
    __syncthreads();
  }
  part[threadIdx.x] = acc;
  __syncthreads();
  if (!live || lane != 0) return;
  for (int s = 1; s < split; ++s) {
    float3 q = part[threadIdx.x + s];
    acc.x += q.x, acc.y += q.y, acc.z += q.z;
  }
  v.x += acc.x;
  if (ndim > 1) v.y += acc.y;
  if (ndim > 2) v.z += acc.z;
  vel_out[i] = v;
}

__device__ __forceinline__ uint32_t spread3_3(uint32_t x) {  // 2 bits -> bits 0, 3
  return (x & 1u) | ((x & 2u) << 2);
}
__device__ __forceinline__ uint32_t spread2_3(uint32_t x) {  // 3 bits -> bits 0, 2, 4
  return (x & 1u) | ((x & 2u) << 1) | ((x & 4u) << 2);
}

// Table slot of a cell: hashed block offset + the cell's Morton index inside its block.
__device__ __forceinline__ uint32_t cell_slot(int cx, int cy, int cz, int ndim, uint32_t mask) {
  uint32_t bx, by = 0, bz = 0, w;
  if (ndim == 3) {
    bx = (uint32_t)cx >> 2, by = (uint32_t)cy >> 2, bz = (uint32_t)cz >> 2;
    w = spread3_3(cx & 3) | spread3_3(cy & 3) << 1 | spread3_3(cz & 3) << 2;
  } else if (ndim == 2) {
    bx = (uint32_t)cx >> 3, by = (uint32_t)cy >> 3;
    w = spread2_3(cx & 7) | spread2_3(cy & 7) << 1;
  } else {
    bx = (uint32_t)cx >> 6;
    w = cx & 63;
  }
  const uint32_t h = fl::mix32(bx ^ fl::mix32(by ^ fl::mix32(bz + 0x9e3779b9u)));
  return ((h << 6) + w) & mask;
}

__device__ __forceinline__ int cell_coord(float s, float inv) {
  return (int)fminf(fmaxf(floorf(s * inv), -1073741824.f), 1073741824.f);
}

constexpr int kKeyThreads = 1024;

__global__ void __launch_bounds__(kKeyThreads) k_grid_keys(const float4* __restrict__ pos,
                                                        const float4* __restrict__ vel, int n,
                                                        int ndim, float inv, int bits,
                                                        uint64_t* __restrict__ keys,
                                                        uint32_t* __restrict__ vals,
                                                        uint32_t* __restrict__ hist, int lo_bit) {
  __shared__ uint32_t sh[8 * 256];
  for (int i = threadIdx.x; i < 8 * 256; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  const int passes = (64 - lo_bit + 7) / 8;
  const uint32_t mask = (1u << bits) - 1;
  const int stride = gridDim.x * blockDim.x;
  for (int base = blockIdx.x * blockDim.x; base < n; base += stride) {
    const int i = base + threadIdx.x;
    const bool ok = i < n;
    uint64_t key = 0;
    if (ok) {
      float4 p = pos[i], v = vel[i];
      int cx = cell_coord(p.x + v.x, inv);
      int cy = ndim > 1 ? cell_coord(p.y + v.y, inv) : 0;
      int cz = ndim > 2 ? cell_coord(p.z + v.z, inv) : 0;
      key = (uint64_t)cell_slot(cx, cy, cz, ndim, mask) << (64 - bits);
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

// Run starts, and the sorted nodes' snapshot position and radius.
__global__ void __launch_bounds__(kThreads) k_grid_begin(const uint64_t* __restrict__ skeys,
                                                         const uint32_t* __restrict__ perm,
                                                         const float4* __restrict__ pos,
                                                         const float4* __restrict__ vel,
                                                         const float* __restrict__ radius, int n,
                                                         int bits, uint32_t* __restrict__ starts,
                                                         float4* __restrict__ sorted) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const uint64_t k = skeys[s];
  if (s == 0 || skeys[s - 1] != k) starts[(uint32_t)(k >> (64 - bits))] = (uint32_t)s;
  const uint32_t i = perm[s];
  const float4 p = pos[i], v = vel[i];
  sorted[s] = make_float4(p.x + v.x, p.y + v.y, p.z + v.z, radius[i]);
}

__global__ void __launch_bounds__(kThreads) k_grid_query(
    const uint64_t* __restrict__ skeys, const uint32_t* __restrict__ perm,
    const uint32_t* __restrict__ starts, const float4* __restrict__ sorted,
    const float4* __restrict__ vel_in, float4* __restrict__ vel_out, int n, int ndim, int bits,
    float inv, float strength, uint32_t step, uint32_t seed, const FlTick* __restrict__ tk) {
  if (tk) step = tk->step, seed = tk->seed;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const float4 me4 = sorted[s];
  const uint32_t i = perm[s];
  const float3 me = make_float3(me4.x, me4.y, me4.z);
  const float ri = me4.w, ri2 = ri * ri;
  const uint32_t mask = (1u << bits) - 1;
  const int hx = cell_coord(me.x, inv), hy = ndim > 1 ? cell_coord(me.y, inv) : 0,
            hz = ndim > 2 ? cell_coord(me.z, inv) : 0;
  const int ry = ndim > 1 ? 1 : 0, rz = ndim > 2 ? 1 : 0;
  uint32_t seen[27];
  int nseen = 0;
  float3 acc = make_float3(0.f, 0.f, 0.f);
  for (int dz = -rz; dz <= rz; ++dz)
    for (int dy = -ry; dy <= ry; ++dy)
      for (int dx = -1; dx <= 1; ++dx) {
        const uint32_t slot = cell_slot(hx + dx, hy + dy, hz + dz, ndim, mask);
        bool again = false;
        for (int q = 0; q < nseen; ++q) again |= seen[q] == slot;
        if (again) continue;
        seen[nseen++] = slot;
        const uint32_t start = starts[slot];
        const uint64_t key = (uint64_t)slot << (64 - bits);
        if (start >= (uint32_t)n || skeys[start] != key || (start > 0 && skeys[start - 1] == key))
          continue;
        for (uint32_t t = start; t < (uint32_t)n && skeys[t] == key; ++t)
          if (t != (uint32_t)s) pair_push(me, ri2, ri, sorted[t], i, perm[t], ndim, strength, step, seed, acc);
      }
  float4 v = vel_in[i];
  v.x += acc.x;
  if (ndim > 1) v.y += acc.y;
  if (ndim > 2) v.z += acc.z;
  vel_out[i] = v;
}

// ---- batches: one grid over all the graphs of a batch, each with its own cell side

// The slot of a graph's cell: as cell_slot, the graph mixed into the hash of the block, so that
// different graphs' cells spread over the table (two sharing a slot only cost tests, and a node
// never pairs with another graph's).
__device__ __forceinline__ uint32_t bcell_slot(int cx, int cy, int cz, int ndim, uint32_t mask,
                                               uint32_t g) {
  uint32_t bx, by = 0, bz = 0, w;
  if (ndim == 3) {
    bx = (uint32_t)cx >> 2, by = (uint32_t)cy >> 2, bz = (uint32_t)cz >> 2;
    w = spread3_3(cx & 3) | spread3_3(cy & 3) << 1 | spread3_3(cz & 3) << 2;
  } else if (ndim == 2) {
    bx = (uint32_t)cx >> 3, by = (uint32_t)cy >> 3;
    w = spread2_3(cx & 7) | spread2_3(cy & 7) << 1;
  } else {
    bx = (uint32_t)cx >> 6;
    w = cx & 63;
  }
  const uint32_t h = fl::mix32(bx ^ fl::mix32(by ^ fl::mix32(bz ^ fl::mix32(g + 0x9e3779b9u))));
  return ((h << 6) + w) & mask;
}

// A node takes part in iteration `iter` when its graph has that many collide iterations and
// does not sit the tick out.
__device__ __forceinline__ bool bcollides(const FlGraph& g, int iter) {
  return g.citer > iter && !g.frozen;
}

__global__ void __launch_bounds__(kKeyThreads) k_bgrid_keys(
    const float4* __restrict__ pos, const float4* __restrict__ vel, int n, int ndim,
    const uint32_t* __restrict__ gid, const FlGraph* __restrict__ gr, int iter, int bits,
    uint64_t* __restrict__ keys, uint32_t* __restrict__ vals, uint32_t* __restrict__ hist,
    int lo_bit) {
  __shared__ uint32_t sh[8 * 256];
  for (int i = threadIdx.x; i < 8 * 256; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  const int passes = (64 - lo_bit + 7) / 8;
  const uint32_t mask = (1u << bits) - 1;
  const int stride = gridDim.x * blockDim.x;
  for (int base = blockIdx.x * blockDim.x; base < n; base += stride) {
    const int i = base + threadIdx.x;
    const bool ok = i < n;
    uint64_t key = ~0ull;  // not taking part: after every cell
    if (ok) {
      const uint32_t g = gid[i];
      const FlGraph& G = gr[g];
      if (bcollides(G, iter)) {
        const float4 p = pos[i], v = vel[i];
        const int cx = cell_coord(p.x + v.x, G.cinv);
        const int cy = ndim > 1 ? cell_coord(p.y + v.y, G.cinv) : 0;
        const int cz = ndim > 2 ? cell_coord(p.z + v.z, G.cinv) : 0;
        key = (uint64_t)bcell_slot(cx, cy, cz, ndim, mask, g) << (63 - bits);
      }
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

// Run starts of the cells, and each sorted node's snapshot position, radius and graph.
__global__ void __launch_bounds__(kThreads) k_bgrid_begin(
    const uint64_t* __restrict__ skeys, const uint32_t* __restrict__ perm,
    const float4* __restrict__ pos, const float4* __restrict__ vel,
    const float* __restrict__ radius, const uint32_t* __restrict__ gid, int n, int bits,
    uint32_t* __restrict__ starts, float4* __restrict__ sorted, uint32_t* __restrict__ sgid) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const uint64_t k = skeys[s];
  if (k == ~0ull) return;  // not taking part (and sorted after every node that does)
  if (s == 0 || skeys[s - 1] != k) starts[(uint32_t)(k >> (63 - bits))] = (uint32_t)s;
  const uint32_t i = perm[s];
  const float4 p = pos[i], v = vel[i];
  sorted[s] = make_float4(p.x + v.x, p.y + v.y, p.z + v.z, radius[i]);
  sgid[s] = gid[i];
}

// Each node's pushes from the overlapping nodes of its own graph in the 3^d cells around its
// own (the jiggle's ids and step are the graph's own: the same alone or in any batch).
__global__ void __launch_bounds__(kThreads) k_bgrid_query(
    const uint64_t* __restrict__ skeys, const uint32_t* __restrict__ perm,
    const uint32_t* __restrict__ starts, const float4* __restrict__ sorted,
    const uint32_t* __restrict__ sgid, const FlGraph* __restrict__ gr,
    const float4* __restrict__ vel_in, float4* __restrict__ vel_out, int n, int ndim, int bits,
    const FlTick* __restrict__ tk) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const uint32_t i = perm[s];
  float4 v = vel_in[i];
  const uint64_t mykey = skeys[s];
  if (mykey != ~0ull) {
    const uint32_t g = sgid[s];
    const FlGraph& G = gr[g];
    const uint32_t first = (uint32_t)G.first, step = tk->step + G.tick0, seed = tk->seed;
    const float4 me4 = sorted[s];
    const float3 me = make_float3(me4.x, me4.y, me4.z);
    const float ri = me4.w, ri2 = ri * ri;
    const uint32_t mask = (1u << bits) - 1;
    const int hx = cell_coord(me.x, G.cinv), hy = ndim > 1 ? cell_coord(me.y, G.cinv) : 0,
              hz = ndim > 2 ? cell_coord(me.z, G.cinv) : 0;
    const int ry = ndim > 1 ? 1 : 0, rz = ndim > 2 ? 1 : 0;
    uint32_t seen[27];
    int nseen = 0;
    float3 acc = make_float3(0.f, 0.f, 0.f);
    for (int dz = -rz; dz <= rz; ++dz)
      for (int dy = -ry; dy <= ry; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
          const uint32_t slot = bcell_slot(hx + dx, hy + dy, hz + dz, ndim, mask, g);
          bool again = false;
          for (int q = 0; q < nseen; ++q) again |= seen[q] == slot;
          if (again) continue;
          seen[nseen++] = slot;
          const uint32_t start = starts[slot];
          const uint64_t key = (uint64_t)slot << (63 - bits);
          if (start >= (uint32_t)n || skeys[start] != key || (start > 0 && skeys[start - 1] == key))
            continue;
          for (uint32_t t = start; t < (uint32_t)n && skeys[t] == key; ++t)
            if (t != (uint32_t)s && sgid[t] == g)
              pair_push(me, ri2, ri, sorted[t], i - first, perm[t] - first, ndim, G.cstr, step,
                        seed, acc);
        }
    v.x += acc.x;
    if (ndim > 1) v.y += acc.y;
    if (ndim > 2) v.z += acc.z;
  }
  vel_out[i] = v;
}

}  // namespace

void fl_launch_bgrid_keys(const float4* pos, const float4* vel, int n, int ndim,
                          const uint32_t* gid, const FlGraph* gr, int iter, int bits,
                          uint64_t* keys, uint32_t* vals, uint32_t* hist, int lo_bit,
                          cudaStream_t st) {
  int g = (n + kKeyThreads - 1) / kKeyThreads;  // as fl_launch_grid_keys
  if (g > 2 * fl_sms()) g = 2 * fl_sms();
  if (g < 1) g = 1;
  k_bgrid_keys<<<g, kKeyThreads, 0, st>>>(pos, vel, n, ndim, gid, gr, iter, bits, keys, vals,
                                          hist, lo_bit);
}

void fl_launch_bgrid_query(const FlGridBufs* g, const uint64_t* skeys, const uint32_t* perm,
                           const float4* pos, const float4* vel_in, float4* vel_out,
                           const float* radius, int ndim, const uint32_t* gid,
                           const FlGraph* gr, uint32_t* sgid, const FlTick* tk, cudaStream_t st,
                           int64_t* launches) {
  const int n = g->n, blocks = (n + kThreads - 1) / kThreads;
  k_bgrid_begin<<<blocks, kThreads, 0, st>>>(skeys, perm, pos, vel_in, radius, gid, n, g->bits,
                                             g->starts, g->sorted, sgid);
  k_bgrid_query<<<blocks, kThreads, 0, st>>>(skeys, perm, g->starts, g->sorted, sgid, gr, vel_in,
                                             vel_out, n, ndim, g->bits, tk);
  *launches += 2;
}

void fl_launch_collide_allpairs(const float4* pos, const float4* vel_in, float4* vel_out,
                                const float* radius, int n, int ndim, float strength,
                                uint32_t step, uint32_t seed, cudaStream_t st, const FlTick* tk) {
  int split = 1;
  while (split < 16 && (int64_t)n * split < (1 << 18)) split *= 2;
  const int per = kThreads / split;
  const int g = (n + per - 1) / per;
  k_collide_allpairs<<<g < 1 ? 1 : g, kThreads, 0, st>>>(pos, vel_in, vel_out, radius, n, ndim,
                                                         strength, step, seed, split, tk);
}

size_t fl_grid_bytes(int64_t n) {
  int bits = 8;
  while ((int64_t(1) << bits) < 2 * n) ++bits;
  return align256(4 * ((size_t)1 << bits)) + align256(16 * (size_t)(n > 0 ? n : 1));
}

void fl_grid_carve(FlGridBufs* g, void* base, int64_t n) {
  int bits = 8;
  while ((int64_t(1) << bits) < 2 * n) ++bits;
  char* p = static_cast<char*>(base);
  g->n = (int)n, g->bits = bits;
  g->starts = (uint32_t*)p, p += align256(4 * ((size_t)1 << bits));
  g->sorted = (float4*)p;
}

void fl_launch_grid_keys(const float4* pos, const float4* vel, int n, int ndim, float inv_cell,
                         int bits, uint64_t* keys, uint32_t* vals, uint32_t* hist, int lo_bit,
                         cudaStream_t st) {
  // few, large blocks: each flushes its histograms with global atomics
  int g = (n + kKeyThreads - 1) / kKeyThreads;
  if (g > 2 * fl_sms()) g = 2 * fl_sms();
  if (g < 1) g = 1;
  k_grid_keys<<<g, kKeyThreads, 0, st>>>(pos, vel, n, ndim, inv_cell, bits, keys, vals, hist, lo_bit);
}

void fl_launch_grid_query(const FlGridBufs* g, const uint64_t* skeys, const uint32_t* perm,
                          const float4* pos, const float4* vel_in, float4* vel_out,
                          const float* radius, int ndim, float inv_cell, float strength,
                          uint32_t step, uint32_t seed, cudaStream_t st, int64_t* launches,
                          const FlTick* tk) {
  const int n = g->n, blocks = (n + kThreads - 1) / kThreads;
  k_grid_begin<<<blocks, kThreads, 0, st>>>(skeys, perm, pos, vel_in, radius, n, g->bits, g->starts,
                                            g->sorted);
  k_grid_query<<<blocks, kThreads, 0, st>>>(skeys, perm, g->starts, g->sorted, vel_in, vel_out, n,
                                            ndim, g->bits, inv_cell, strength, step, seed, tk);
  *launches += 2;
}
