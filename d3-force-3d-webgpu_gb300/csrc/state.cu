// Per-node streaming kernels: the bounding-box / centre reduction, the centre shift, the fused
// integrate, and the per-node forces (radial, x/y/z). All HBM-bound; one float4 per node.
#include "kernels.h"

namespace {

constexpr int kThreads = 256;

inline int grid_for(int n, int per_block) {
  int g = (n + per_block - 1) / per_block;
  if (g < 1) g = 1;
  return g;
}

// Knuth's TwoSum: s + x = t + e exactly, t = fl(s + x).
__device__ __forceinline__ void two_sum(float s, float x, float& t, float& e) {
  t = s + x;
  const float bp = t - s;
  e = (s - (t - bp)) + (x - bp);
}

// Bounding box (ordered-uint atomics) and sum of the positions, one pass.
// d3 computes the cube from the extent of the points (d3-octree cover) and the centre force
// sums positions in FP64 (src/center.js:8-26); both come from this one read. The sums are exact
// fixed-point integers (fl::fx128: 128 bits, 2^-40 resolution), so they do not depend on the
// order of the additions: the same positions give the same mean bit for bit, whatever the grid.
// One thread's share of the reduction: box and exact sums of the positions it saw.
struct Partial {
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  __int128 s[3] = {0, 0, 0};
  uint32_t bad = 0;
  __device__ __forceinline__ void add(float4 p, int ndim, int want_sum) {
    const float c[3] = {p.x, p.y, p.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      lo[k] = fminf(lo[k], c[k]);
      hi[k] = fmaxf(hi[k], c[k]);
      if (want_sum && k < ndim) s[k] += fl::fx128(c[k], bad);
    }
  }
};

// The block's partials into red: warp shuffles, then one atomic per axis and quantity.
__device__ void flush_partial(const Partial& q, int ndim, int want_box, int want_sum,
                              FlReduce* red);

__global__ void __launch_bounds__(kThreads) k_reduce(const float4* __restrict__ pos, int n,
                                                     int ndim, int want_box, int want_sum,
                                                     FlReduce* red) {
  Partial q;
  // a few blocks, many positions per thread: the warp shuffles and atomics of the reduction
  // are paid once per warp, not per handful of positions
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    q.add(pos[i], ndim, want_sum);
  flush_partial(q, ndim, want_box, want_sum, red);
}

__device__ void flush_partial(const Partial& q, int ndim, int want_box, int want_sum,
                              FlReduce* red) {
  float lo[3] = {q.lo[0], q.lo[1], q.lo[2]}, hi[3] = {q.hi[0], q.hi[1], q.hi[2]};
  __int128 sum[3] = {q.s[0], q.s[1], q.s[2]};
  uint32_t bad = q.bad;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lo[k] = fminf(lo[k], __shfl_xor_sync(FL_FULL, lo[k], o));
      hi[k] = fmaxf(hi[k], __shfl_xor_sync(FL_FULL, hi[k], o));
      if (want_sum) sum[k] += fl::shfl_xor128(sum[k], o);
    }
  }
  if (want_sum) bad = __reduce_add_sync(FL_FULL, bad);
  __shared__ float s_lo[3][kThreads / 32], s_hi[3][kThreads / 32];
  __shared__ __int128 s_sum[3][kThreads / 32];
  __shared__ uint32_t s_bad[kThreads / 32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    for (int k = 0; k < 3; ++k) s_lo[k][warp] = lo[k], s_hi[k][warp] = hi[k], s_sum[k][warp] = sum[k];
    s_bad[warp] = bad;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    int k = threadIdx.x;
    float a = INFINITY, b = -INFINITY;
    __int128 s = 0;
    uint32_t nb = 0;
    for (int w = 0; w < kThreads / 32; ++w) {
      a = fminf(a, s_lo[k][w]), b = fmaxf(b, s_hi[k][w]), s += s_sum[k][w];
      nb += s_bad[w];
    }
    if (k < ndim) {
      if (want_box) {  // lo holds ~ordered(min), so a zeroed record is an empty box
        atomicMax(&red->lo[k], ~fl::ordered(a));
        atomicMax(&red->hi[k], fl::ordered(b));
      }
      if (want_sum) fl::atomic_add128(&red->sum_lo[k], &red->sum_hi[k], s);
    }
    if (want_sum && k == 0 && nb) atomicAdd(&red->bad, nb);
  }
}

// Per-graph bounding boxes and position sums of a batch. Nodes are grouped by graph, so graph
// ids do not decrease along the nodes: a block takes kBreduceItems * kThreads consecutive nodes;
// in each of its warps every run of equal ids is reduced toward its first lane (shuffles that
// stop at the run's end), which adds the run to the block's table of the graphs it covers
// (shared-memory atomics); the table then goes to the graphs' records with one global atomic
// per graph, axis and quantity. A run whose graph falls past the table (a block over many tiny
// graphs) goes to its record directly.
constexpr int kBreduceItems = 8, kBreduceSlots = 16;
__global__ void __launch_bounds__(kThreads) k_breduce(const float4* __restrict__ pos, int n,
                                                      int ndim, const uint32_t* __restrict__ gid,
                                                      FlReduce* red) {
  __shared__ uint32_t s_lo[kBreduceSlots][3], s_hi[kBreduceSlots][3];
  __shared__ unsigned long long s_slo[kBreduceSlots][3], s_shi[kBreduceSlots][3];
  __shared__ uint32_t s_bad[kBreduceSlots];
  const int lane = threadIdx.x & 31;
  const int64_t first = (int64_t)blockIdx.x * kThreads * kBreduceItems;
  const uint32_t g0 = gid[first < n ? first : n - 1];
  for (int i = threadIdx.x; i < kBreduceSlots * 3; i += kThreads) {
    (&s_lo[0][0])[i] = 0u, (&s_hi[0][0])[i] = 0u, (&s_slo[0][0])[i] = 0ull, (&s_shi[0][0])[i] = 0ull;
  }
  for (int i = threadIdx.x; i < kBreduceSlots; i += kThreads) s_bad[i] = 0u;
  __syncthreads();
  for (int it = 0; it < kBreduceItems; ++it) {
    const int64_t i = first + (int64_t)it * kThreads + threadIdx.x;
    const bool ok = i < n;
    const uint32_t g = ok ? gid[i] : 0xffffffffu;
    float4 p = ok ? pos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    uint32_t bad = 0;
    float lo[3] = {p.x, p.y, p.z}, hi[3] = {p.x, p.y, p.z};
    __int128 sm[3] = {fl::fx128(p.x, bad), ndim > 1 ? fl::fx128(p.y, bad) : 0,
                      ndim > 2 ? fl::fx128(p.z, bad) : 0};
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t go = __shfl_down_sync(FL_FULL, g, o);
      const bool same = lane + o < 32 && go == g;
      const uint32_t bo = __shfl_down_sync(FL_FULL, bad, o);
      if (same) bad += bo;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float a = __shfl_down_sync(FL_FULL, lo[k], o), b = __shfl_down_sync(FL_FULL, hi[k], o);
        const __int128 c = fl::shfl_down128(sm[k], o);
        if (same) lo[k] = fminf(lo[k], a), hi[k] = fmaxf(hi[k], b), sm[k] += c;
      }
    }
    const uint32_t gp = __shfl_up_sync(FL_FULL, g, 1);
    if (!ok || (lane > 0 && gp == g)) continue;  // not the first lane of its run
    const uint32_t slot = g - g0;
    if (slot < (uint32_t)kBreduceSlots) {
      for (int k = 0; k < ndim; ++k) {
        atomicMax(&s_lo[slot][k], ~fl::ordered(lo[k]));
        atomicMax(&s_hi[slot][k], fl::ordered(hi[k]));
        fl::atomic_add128(&s_slo[slot][k], &s_shi[slot][k], sm[k]);
      }
      if (bad) atomicAdd(&s_bad[slot], bad);
    } else {
      FlReduce* r = red + g;
      for (int k = 0; k < ndim; ++k) {
        atomicMax(&r->lo[k], ~fl::ordered(lo[k]));
        atomicMax(&r->hi[k], fl::ordered(hi[k]));
        fl::atomic_add128(&r->sum_lo[k], &r->sum_hi[k], sm[k]);
      }
      if (bad) atomicAdd(&r->bad, bad);
    }
  }
  __syncthreads();
  // the table: one thread per graph and axis (a zero low word: no run of that graph here)
  for (int t = threadIdx.x; t < kBreduceSlots * 3; t += kThreads) {
    const int slot = t / 3, k = t % 3;
    if (k >= ndim || s_lo[slot][k] == 0u) continue;
    FlReduce* r = red + (g0 + slot);
    atomicMax(&r->lo[k], s_lo[slot][k]);
    atomicMax(&r->hi[k], s_hi[slot][k]);
    const __int128 v = (__int128)(((unsigned __int128)s_shi[slot][k] << 64) | s_slo[slot][k]);
    fl::atomic_add128(&r->sum_lo[k], &r->sum_hi[k], v);
    if (k == 0 && s_bad[slot]) atomicAdd(&r->bad, s_bad[slot]);
  }
}

// The centre force's shift, (mean - c) * strength per active axis, computed in FP64 once per
// block and shared as a pair of floats (hi + lo), which the threads subtract in FP32.
__device__ __forceinline__ void center_shift(const FlReduce* red, int n, int ndim, double cx,
                                             double cy, double cz, double strength, float2* sh) {
  __shared__ float2 s_shift[3];
  if (threadIdx.x < 3) {
    const int k = threadIdx.x;
    const double c = k == 0 ? cx : k == 1 ? cy : cz;
    const double d = k < ndim ? (fl::sum_of(*red, k) / n - c) * strength : 0.0;
    const float h = (float)d;
    s_shift[k] = make_float2(h, (float)(d - (double)h));
  }
  __syncthreads();
  sh[0] = s_shift[0], sh[1] = s_shift[1], sh[2] = s_shift[2];
}

// x - (hi + lo), rounded once in all but the rarest cases: the first subtraction's rounding
// error is recovered exactly (TwoSum) and folded in with lo
__device__ __forceinline__ float sub_shift(float x, float2 s) {
  float t, e;
  two_sum(x, -s.x, t, e);
  return t + (e - s.y);
}

__global__ void k_center_apply(float4* __restrict__ pos, int n, int ndim, const FlReduce* red,
                               double cx, double cy, double cz, double strength) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  float2 sh[3];
  center_shift(red, n, ndim, cx, cy, cz, strength, sh);
  if (i >= n) return;
  float4 p = pos[i];
  p.x = sub_shift(p.x, sh[0]);
  p.y = sub_shift(p.y, sh[1]);
  p.z = sub_shift(p.z, sh[2]);
  pos[i] = p;
}

// src/simulation.js:61-73 (and src/gpu/wgsl.js INTEGRATE): v *= decay; p += v; a pinned axis
// takes p = fixed, v = 0. With the centre force fused (it was the last force), positions are
// first shifted by it, as the reference applies it before integrating.
// One node of k_integrate (no batch): decay, move, shift by the centre force, pins.
__device__ __forceinline__ void integrate_node(float4& p, float4& v, const float4* __restrict__ fix,
                                               uint32_t m, int i, int ndim, float decay,
                                               bool shift, const float2* sh) {
  if (shift) {
    p.x = sub_shift(p.x, sh[0]);
    p.y = sub_shift(p.y, sh[1]);
    p.z = sub_shift(p.z, sh[2]);
  }
  v.x *= decay, v.y *= decay, v.z *= decay;
  p.x += v.x, p.y += v.y, p.z += v.z;
  if (m) {
    float4 f = fix[i];
    if (m & 1u) p.x = f.x, v.x = 0.f;
    if (m & 2u) p.y = f.y, v.y = 0.f;
    if (m & 4u) p.z = f.z, v.z = 0.f;
  }
  if (ndim < 3) p.z = 0.f, v.z = 0.f;
  if (ndim < 2) p.y = 0.f, v.y = 0.f;
  p.w = 0.f, v.w = 0.f;
}

// k_integrate that also reduces the new positions (box and/or sums) into `out`: the next
// tick's k_reduce, fused. A grid-stride loop over few blocks, as k_reduce.
__global__ void __launch_bounds__(kThreads) k_integrate_reduce(
    float4* __restrict__ pos, float4* __restrict__ vel, const float4* __restrict__ fix,
    const uint32_t* __restrict__ mask, int n, int ndim, float decay, const FlReduce* red,
    double cx, double cy, double cz, double strength, const FlTick* __restrict__ tk,
    FlReduce* out, int want_box, int want_sum, float4* __restrict__ snap) {
  if (tk) decay = tk->decay;
  float2 sh[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
  if (red) center_shift(red, n, ndim, cx, cy, cz, strength, sh);  // block-uniform branch
  Partial q;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float4 p = pos[i], v = vel[i];
    integrate_node(p, v, fix, mask[i], i, ndim, decay, red != nullptr, sh);
    pos[i] = p;
    vel[i] = v;
    if (snap) snap[i] = make_float4(p.x + v.x, p.y + v.y, p.z + v.z, 0.f);
    q.add(p, ndim, want_sum);
  }
  flush_partial(q, ndim, want_box, want_sum, out);
}

__global__ void __launch_bounds__(kThreads) k_integrate(float4* __restrict__ pos,
                                                        float4* __restrict__ vel,
                                                        const float4* __restrict__ fix,
                                                        const uint32_t* __restrict__ mask, int n,
                                                        int ndim, float decay, const FlReduce* red,
                                                        double cx, double cy, double cz,
                                                        double strength, const FlGraph* gr,
                                                        const uint32_t* __restrict__ gid,
                                                        const FlTick* __restrict__ tk,
                                                        float4* __restrict__ snap) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (tk) decay = tk->decay;
  float2 sh[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
  if (red) center_shift(red, n, ndim, cx, cy, cz, strength, sh);  // block-uniform branch
  if (i >= n) return;
  float4 p = pos[i], v = vel[i];
  if (gr) {  // a batch: the node's graph's decay and centre shift
    const FlGraph& g = gr[gid[i]];
    if (g.frozen) return;  // sitting this tick out: state unchanged
    decay = g.decay;
    sh[0] = g.shift[0], sh[1] = g.shift[1], sh[2] = g.shift[2];
  }
  integrate_node(p, v, fix, mask[i], i, ndim, decay, red || gr, sh);
  pos[i] = p;
  vel[i] = v;
  if (snap) snap[i] = make_float4(p.x + v.x, p.y + v.y, p.z + v.z, 0.f);
}

__global__ void __launch_bounds__(kThreads) k_snapshot(const float4* __restrict__ pos,
                                                       const float4* __restrict__ vel,
                                                       float4* __restrict__ snap, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 p = pos[i], v = vel[i];
  snap[i] = make_float4(p.x + v.x, p.y + v.y, p.z + v.z, 0.f);
}

__device__ __forceinline__ float or1e6(float v) { return v != 0.f ? v : 1e-6f; }

// forceRadial (src/radial.js:16-28): d = p - c with exact-zero components replaced by 1e-6;
// v += d * (r_i - |d|) * s_i * alpha / |d|. Axes beyond numDimensions still enter |d| as
// (0 - c)||1e-6, as in the reference's CPU force (they are never moved).
__global__ void __launch_bounds__(kThreads) k_radial(const float4* __restrict__ pos,
                                                     float4* __restrict__ vel,
                                                     const float* __restrict__ radius,
                                                     const float* __restrict__ strength, int n,
                                                     int ndim, float cx, float cy, float cz,
                                                     float alpha, const FlTick* __restrict__ tk) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (tk) alpha = tk->alpha;
  if (i >= n) return;
  float4 p = pos[i];
  float dx = or1e6(p.x - cx);
  float dy = or1e6((ndim > 1 ? p.y : 0.f) - cy);
  float dz = or1e6((ndim > 2 ? p.z : 0.f) - cz);
  float r = sqrtf(dx * dx + dy * dy + dz * dz);
  float k = (radius[i] - r) * strength[i] * alpha / r;
  float4 v = vel[i];
  v.x += dx * k;
  if (ndim > 1) v.y += dy * k;
  if (ndim > 2) v.z += dz * k;
  vel[i] = v;
}

// forceX / forceY / forceZ (src/x.js:12-16): v[axis] += (target_i - p[axis]) * s_i * alpha.
__global__ void __launch_bounds__(kThreads) k_position(const float4* __restrict__ pos,
                                                       float4* __restrict__ vel,
                                                       const float* __restrict__ target,
                                                       const float* __restrict__ strength, int n,
                                                       int axis, float alpha,
                                                       const FlTick* __restrict__ tk) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (tk) alpha = tk->alpha;
  if (i >= n) return;
  float p = axis == 0 ? pos[i].x : axis == 1 ? pos[i].y : pos[i].z;
  float dv = (target[i] - p) * strength[i] * alpha;
  float4 v = vel[i];
  if (axis == 0) v.x += dv;
  else if (axis == 1) v.y += dv;
  else v.z += dv;
  vel[i] = v;
}

// Positions and velocities to `ndim` floats per node: out[0, n ndim) and out[n ndim, 2 n ndim),
// one thread per output float (coalesced writes).
__global__ void __launch_bounds__(kThreads) k_pack(const float* __restrict__ pos,
                                                   const float* __restrict__ vel, int64_t n,
                                                   int ndim, float* __restrict__ out) {
  const int64_t m = n * ndim;
  for (int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x; i < m;
       i += (int64_t)gridDim.x * kThreads) {
    const int64_t node = i / ndim, at = node * 4 + (i - node * ndim);
    if (pos) out[i] = pos[at];
    if (vel) out[m + i] = vel[at];
  }
}

// `ndim` floats per node back to float4 state: the components past ndim and w are 0, as the
// integrate leaves them.
__global__ void __launch_bounds__(kThreads) k_unpack(const float* __restrict__ src, int count,
                                                     int ndim, float4* __restrict__ dst) {
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= count) return;
  const float* s = src + (int64_t)i * ndim;
  dst[i] = make_float4(s[0], ndim > 1 ? s[1] : 0.f, ndim > 2 ? s[2] : 0.f, 0.f);
}

}  // namespace

void fl_launch_pack(const float4* pos, const float4* vel, int n, int ndim, float* out,
                    cudaStream_t st) {
  if (n <= 0) return;
  int g = grid_for(n * ndim, kThreads * 4);
  if (g > 8 * fl_sms()) g = 8 * fl_sms();
  k_pack<<<g, kThreads, 0, st>>>(reinterpret_cast<const float*>(pos),
                                 reinterpret_cast<const float*>(vel), n, ndim, out);
}

void fl_launch_unpack(const float* src, int count, int ndim, float4* dst, cudaStream_t st) {
  if (count <= 0) return;
  k_unpack<<<grid_for(count, kThreads), kThreads, 0, st>>>(src, count, ndim, dst);
}

void fl_launch_reduce(const float4* pos, int n, int ndim, int want_box, int want_sum,
                      FlReduce* red, cudaStream_t st) {
  int g = grid_for(n, kThreads * 4);
  if (g > 2 * fl_sms()) g = 2 * fl_sms();
  k_reduce<<<g, kThreads, 0, st>>>(pos, n, ndim, want_box, want_sum, red);
}

void fl_launch_center_apply(float4* pos, int n, int ndim, const FlReduce* red, double cx,
                            double cy, double cz, double strength, cudaStream_t st) {
  k_center_apply<<<grid_for(n, kThreads), kThreads, 0, st>>>(pos, n, ndim, red, cx, cy, cz, strength);
}

void fl_launch_breduce(const float4* pos, int n, int ndim, const uint32_t* gid, FlReduce* red,
                       cudaStream_t st) {
  if (n <= 0) return;
  k_breduce<<<grid_for(n, kThreads * kBreduceItems), kThreads, 0, st>>>(pos, n, ndim, gid, red);
}

void fl_launch_integrate(float4* pos, float4* vel, const float4* fix, const uint32_t* mask, int n,
                         int ndim, float decay, const FlReduce* red, double cx, double cy,
                         double cz, double strength, cudaStream_t st, const FlGraph* gr,
                         const uint32_t* gid, const FlTick* tk, FlReduce* out, int want_box,
                         int want_sum, float4* snap) {
  if (gr) snap = nullptr;  // a batch keeps no snapshot
  if (out && !gr) {
    int g = grid_for(n, kThreads * 4);
    if (g > 4 * fl_sms()) g = 4 * fl_sms();
    k_integrate_reduce<<<g, kThreads, 0, st>>>(pos, vel, fix, mask, n, ndim, decay, red, cx, cy,
                                                cz, strength, tk, out, want_box, want_sum, snap);
    return;
  }
  k_integrate<<<grid_for(n, kThreads), kThreads, 0, st>>>(pos, vel, fix, mask, n, ndim, decay, red,
                                                          cx, cy, cz, strength, gr, gid, tk, snap);
}

void fl_launch_snapshot(const float4* pos, const float4* vel, float4* snap, int n, cudaStream_t st) {
  if (n <= 0) return;
  k_snapshot<<<grid_for(n, kThreads), kThreads, 0, st>>>(pos, vel, snap, n);
}

void fl_launch_radial(const float4* pos, float4* vel, const float* radius, const float* strength,
                      int n, int ndim, float cx, float cy, float cz, float alpha, cudaStream_t st,
                      const FlTick* tk) {
  k_radial<<<grid_for(n, kThreads), kThreads, 0, st>>>(pos, vel, radius, strength, n, ndim, cx, cy,
                                                       cz, alpha, tk);
}

void fl_launch_position(const float4* pos, float4* vel, const float* target, const float* strength,
                        int n, int axis, float alpha, cudaStream_t st, const FlTick* tk) {
  k_position<<<grid_for(n, kThreads), kThreads, 0, st>>>(pos, vel, target, strength, n, axis, alpha,
                                                         tk);
}
