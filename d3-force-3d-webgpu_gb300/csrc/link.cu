// forceLink over a CSR adjacency (src/link.js:34-54, the GPU form of src/gpu/passes/link.js).
//
// Every node gathers the links it belongs to, against one snapshot of p + v (the reference's
// GPU semantics: all links see the same state, where the CPU force applies them one after
// another). The snapshot is not copied: the kernel reads p and v_in and writes v_out.
//
// Per entry (float4): other end, distance, strength, this end's share of the push (1 - bias at
// the source, bias at the target). For a link s -> t with d = (p_t + v_t) - (p_s + v_s):
//     k = (|d| - distance) / |d| * alpha * strength
//     v_t -= d * k * bias,  v_s += d * k * (1 - bias)
// Seen from either end, d_view = other - this is +d at the source and -d at the target (the
// same float up to sign, IEEE subtraction being antisymmetric), so both ends compute
// v += d_view * k * share. A zero component of d is replaced by the link's jiggle, with the
// sign of the end that sees it.
//
// With a snapshot (snap = p + v per node, written by the integrate before) the node's own state
// and every other end come from one 16-byte record: the same FP32 sums, half the bytes gathered.
//
// Load balance: a warp takes 32 consecutive rows; each lane walks its row with float4 loads.
// Rows longer than kLong (high-degree hubs) are split across the whole warp and combined with a
// warp reduction, so one hub does not stall its warp for thousands of iterations.
#include "kernels.h"

namespace {

constexpr int kThreads = 256;
constexpr int kLong = 64;

// The state p + v of node j: from the snapshot, or summed from p and v.
template <bool SNAP>
__device__ __forceinline__ float3 state_of(const float4* __restrict__ pos,
                                           const float4* __restrict__ vel,
                                           const float4* __restrict__ snap, int j) {
  if (SNAP) {
    const float4 s = __ldg(snap + j);
    return make_float3(s.x, s.y, s.z);
  }
  const float4 pj = __ldg(pos + j), vj = __ldg(vel + j);
  return make_float3(pj.x + vj.x, pj.y + vj.y, pj.z + vj.z);
}

// One entry's term, given the other end's state sj. The entry's code word (link * 2 + end) is
// read only for a zero component, which is rare: the common case streams the float4 entries alone.
__device__ __forceinline__ void link_apply(float3 sj, float3 me, float4 e,
                                           const uint32_t* __restrict__ codep, int ndim,
                                           float alpha, uint32_t step, uint32_t seed, float3& acc) {
  float dx = sj.x - me.x;
  float dy = ndim > 1 ? sj.y - me.y : 0.f;
  float dz = ndim > 2 ? sj.z - me.z : 0.f;
  if (dx == 0.f || (ndim > 1 && dy == 0.f) || (ndim > 2 && dz == 0.f)) {
    // jiggle(link): the same value at both ends, negated at the target
    const uint32_t code = __ldg(codep);
    const uint32_t link = code >> 1;
    const float sgn = (code & 1u) ? -1.f : 1.f;
    if (dx == 0.f) dx = sgn * fl::jiggle(link, 0x7fffffffu, 0, step, seed);
    if (ndim > 1 && dy == 0.f) dy = sgn * fl::jiggle(link, 0x7fffffffu, 1, step, seed);
    if (ndim > 2 && dz == 0.f) dz = sgn * fl::jiggle(link, 0x7fffffffu, 2, step, seed);
  }
  float l = sqrtf(dx * dx + dy * dy + dz * dz);
  float k = (l - e.y) / l * alpha * e.z;
  acc.x += dx * k * e.w;
  acc.y += dy * k * e.w;
  acc.z += dz * k * e.w;
}

template <bool SNAP>
__device__ __forceinline__ void link_term(const float4* __restrict__ pos,
                                          const float4* __restrict__ vel,
                                          const float4* __restrict__ snap, float3 me, float4 e,
                                          const uint32_t* __restrict__ codep, int ndim,
                                          float alpha, uint32_t step, uint32_t seed, float3& acc) {
  link_apply(state_of<SNAP>(pos, vel, snap, __float_as_int(e.x)), me, e, codep, ndim, alpha, step,
             seed, acc);
}

template <bool SNAP>
__global__ void __launch_bounds__(kThreads) k_link(const float4* __restrict__ pos,
                                                   const float4* __restrict__ vel_in,
                                                   float4* __restrict__ vel_out,
                                                   const int32_t* __restrict__ row,
                                                   const float4* __restrict__ entry,
                                                   const uint32_t* __restrict__ code, int n,
                                                   int ndim, float alpha, uint32_t step,
                                                   uint32_t seed, const FlGraph* __restrict__ gr,
                                                   const uint32_t* __restrict__ gid,
                                                   const FlTick* __restrict__ tk,
                                                   const float4* __restrict__ snap) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (tk) alpha = tk->alpha, step = tk->step, seed = tk->seed;
  const int lane = threadIdx.x & 31;
  const bool live = i < n;
  bool frozen = false;
  if (gr && live) {  // a batch: the node's graph's alpha; a graph sitting the tick out keeps v
    const FlGraph& g = gr[gid[i]];
    alpha = g.alpha, frozen = g.frozen != 0;
    step += g.tick0;  // the graph's own step (its jiggles do not depend on the batch)
  }
  int r0 = 0, r1 = 0;
  float4 v = make_float4(0, 0, 0, 0);
  float3 me = make_float3(0.f, 0.f, 0.f);
  if (live) {
    r0 = row[i], r1 = row[i + 1];
    v = vel_in[i];
    if (SNAP) {
      const float4 s = snap[i];
      me = make_float3(s.x, s.y, s.z);
    } else {
      const float4 p = pos[i];
      me = make_float3(p.x + v.x, p.y + v.y, p.z + v.z);
    }
  }
  float3 acc = make_float3(0.f, 0.f, 0.f);
  const bool longrow = !frozen && (r1 - r0) > kLong;
  if (!longrow && !frozen) {
    // two entries at a time: both loads and both gathers in flight before either term (the terms
    // still add in row order)
    int e = r0;
    for (; e + 1 < r1; e += 2) {
      const float4 ea = __ldg(entry + e), eb = __ldg(entry + e + 1);
      const float3 sa = state_of<SNAP>(pos, vel_in, snap, __float_as_int(ea.x));
      const float3 sb = state_of<SNAP>(pos, vel_in, snap, __float_as_int(eb.x));
      link_apply(sa, me, ea, code + e, ndim, alpha, step, seed, acc);
      link_apply(sb, me, eb, code + e + 1, ndim, alpha, step, seed, acc);
    }
    if (e < r1)
      link_term<SNAP>(pos, vel_in, snap, me, __ldg(entry + e), code + e, ndim, alpha, step, seed, acc);
  }
  // long rows: the warp takes them one at a time
  uint32_t longs = __ballot_sync(FL_FULL, longrow);
  while (longs) {
    const int src = __ffs(longs) - 1;
    longs &= longs - 1;
    const int a = __shfl_sync(FL_FULL, r0, src), b = __shfl_sync(FL_FULL, r1, src);
    const float3 m = make_float3(__shfl_sync(FL_FULL, me.x, src), __shfl_sync(FL_FULL, me.y, src),
                                 __shfl_sync(FL_FULL, me.z, src));
    const float am = __shfl_sync(FL_FULL, alpha, src);
    const uint32_t sm = __shfl_sync(FL_FULL, step, src);
    float3 part = make_float3(0.f, 0.f, 0.f);
    for (int e = a + lane; e < b; e += 32)
      link_term<SNAP>(pos, vel_in, snap, m, __ldg(entry + e), code + e, ndim, am, sm, seed, part);
    part.x = fl::warp_sum(part.x), part.y = fl::warp_sum(part.y), part.z = fl::warp_sum(part.z);
    if (lane == src) acc = part;
  }
  if (!live) return;
  v.x += acc.x;
  if (ndim > 1) v.y += acc.y;
  if (ndim > 2) v.z += acc.z;
  vel_out[i] = v;
}

}  // namespace

void fl_launch_link(const float4* pos, const float4* vel_in, float4* vel_out, FlLinkCsr csr, int n,
                    int ndim, float alpha, uint32_t step, uint32_t seed, cudaStream_t st,
                    const FlGraph* gr, const uint32_t* gid, const FlTick* tk,
                    const float4* snap) {
  int g = (n + kThreads - 1) / kThreads;
  if (g < 1) g = 1;
  if (snap)
    k_link<true><<<g, kThreads, 0, st>>>(pos, vel_in, vel_out, csr.row, csr.entry, csr.code, n,
                                         ndim, alpha, step, seed, gr, gid, tk, snap);
  else
    k_link<false><<<g, kThreads, 0, st>>>(pos, vel_in, vel_out, csr.row, csr.entry, csr.code, n,
                                          ndim, alpha, step, seed, gr, gid, tk, nullptr);
}
