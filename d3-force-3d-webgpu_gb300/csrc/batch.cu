// fl_batch: many independent force layouts advanced together, one launch per kernel per tick.
//
// The graphs are concatenated (nodes, links) with per-graph offsets; every kernel of a tick runs
// once over the whole batch and finds a node's graph from a graph-id array: bounding boxes and
// centre sums are reduced per graph, each graph gets its own d3 cube and Morton keys, the tree's
// sort orders the points by (graph, Morton code) so that each graph owns one contiguous range of
// the sorted order and builds its own tree there, and the walk starts each point at its own
// graph's root. Link, many-body and centre forces per graph, with per-graph alpha schedules
// (fl_batch_enqueue takes one alpha per graph and tick), theta, distances and velocity decay.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/forcegpu.h"
#include "kernels.h"
#include "tune.h"

namespace {

struct Buf {
  void* p = nullptr;
  size_t bytes = 0;
  Buf() = default;
  Buf(const Buf&) = delete;
  Buf& operator=(const Buf&) = delete;
  ~Buf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr, bytes = 0;
  }
  cudaError_t alloc(size_t b) {
    release();
    cudaError_t e = cudaMalloc(&p, b ? b : 256);
    if (e != cudaSuccess) p = nullptr;
    else bytes = b ? b : 256;
    return e;
  }
  // At least b bytes, keeping the buffer when it is large enough: freeing device memory waits
  // for the whole device (every other stream's work too), so a batch rebuilt with fewer nodes
  // reuses its buffers, and one that grows takes half as much again as it needs.
  cudaError_t reserve(size_t b) {
    if (p && b <= bytes) return cudaSuccess;
    return alloc(b + b / 2);
  }
  template <typename T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

constexpr int64_t kMaxBatchNodes = (int64_t(1) << 26) - 1;

}  // namespace

struct fl_batch {
  int32_t device = 0;
  cudaStream_t st = nullptr;
  std::string err;
  int32_t ndim = 3, graphs = 0, n = 0, m = 0;
  Buf pos, vel[2], fix, mask, gid, off, prm, red, gr, alphas, charge, row, entry, code, errw;
  Buf sort1, sort2, tree, gid_pos, groups;
  int32_t ngroups = 0;
  // collide: per-node radii, the grid (run starts, sorted snapshot, sorted graph ids) and the
  // most iterations any graph's collide force has (0: no graph collides)
  Buf radius, grid, sgid;
  FlGridBufs gb{};
  int32_t citer_max = 0;
  FlSortBufs sb{}, sb2{};
  FlTreeBufs tb{};
  int cur = 0;
  size_t alpha_cap = 0;
  uint32_t step = 0, seed = 0x9e3779b9u;
  int fx_exp = 32;
  bool closed = true, neg = false, posv = false;  // strengths: some below 0, some above
  double smax = 0;
  float sign = -1.f;
  double dmax_any = INFINITY;  // finite when some graph has a finite distanceMax
  int64_t ticks = 0, launches = 0;
  // per-tick steps in device memory and the CUDA graphs of tick blocks, as fl_sim's
  Buf tickbuf;
  int32_t tick_cap = 0;
  std::vector<FlTick> htick;
  std::vector<int32_t> hoff;  // first node of each graph, and the total
  struct Block {
    int32_t count;
    int cur_in, cur_out;
    int64_t launches;
    bool captured;
    cudaGraphExec_t exec;
  };
  std::vector<Block> blocks;
  bool use_graphs = true;
  int sort_passes = 0, walk_blocks = 0;  // tuning (FL_TUNE_SORT_PASSES, FL_TUNE_WALK_BLOCKS)
  // the side stream of the trees (overlapping the links), forked and joined by events
  cudaStream_t aux = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_tree = nullptr;
};

namespace {

int32_t bfail(fl_batch* b, int32_t code, const std::string& msg) {
  if (b) b->err = msg;
  return code;
}

int32_t bcuda(fl_batch* b, cudaError_t e, const char* what) {
  cudaGetLastError();
  return bfail(b, e == cudaErrorMemoryAllocation ? FL_E_OOM : FL_E_DEVICE,
               std::string(what) + ": " + cudaGetErrorString(e));
}

#define FB_CK(b, call)                                      \
  do {                                                      \
    cudaError_t e_ = (call);                                \
    if (e_ != cudaSuccess) return bcuda(b, e_, #call);      \
  } while (0)

int32_t bcheck(fl_batch* b) {
  if (!b) return FL_E_ARG;
  if (cudaSetDevice(b->device) != cudaSuccess) return bfail(b, FL_E_DEVICE, "cudaSetDevice failed");
  return FL_OK;
}

float4* bvel(fl_batch* b) { return b->vel[b->cur].as<float4>(); }

void clear_blocks(fl_batch* b) {
  for (auto& x : b->blocks)
    if (x.captured) cudaGraphExecDestroy(x.exec);
  b->blocks.clear();
}

// One tick of the batch: alphas of this tick are at `alpha` (device, one per graph), its step
// and seed at tk (device).
void encode_batch_tick(fl_batch* b, const double* alpha, const FlTick* tk) {
  const int n = b->n, G = b->graphs;
  cudaStream_t st = b->st;
  uint32_t* err = b->errw.as<uint32_t>();
  const uint32_t* gid = b->gid.as<uint32_t>();
  FlGraph* gr = b->gr.as<FlGraph>();
  // per-graph boxes and sums, then each graph's cube, threshold, alpha, decay and centre shift
  cudaMemsetAsync(b->red.p, 0, sizeof(FlReduce) * (size_t)G, st);
  fl_launch_breduce(b->pos.as<float4>(), n, b->ndim, gid, b->red.as<FlReduce>(), st);
  fl_launch_bgraph(G, b->ndim, b->off.as<int32_t>(), b->red.as<FlReduce>(),
                   b->prm.as<FlBatchParams>(), alpha, gr, st);
  b->launches += 2;
  // many-body trees: sort by Morton code, then (stably) by graph; one tree per graph. They
  // depend on the positions and the graphs' cubes only, so they are built on the side stream
  // while the links run on the main one
  uint64_t* skeys = nullptr;
  uint32_t* perm = nullptr;
  uint32_t* gpos = b->gid_pos.as<uint32_t>();
  FlSegs segs{G, b->off.as<int32_t>(), gid, gpos, gr, b->groups.as<uint2>(), b->ngroups};
  const bool side = b->aux != nullptr;
  if (n >= 2) {
    cudaStream_t ts = st;
    if (side) {
      cudaEventRecord(b->ev_fork, st);
      cudaStreamWaitEvent(b->aux, b->ev_fork, 0);
      ts = b->aux;
    }
    const int bits = (b->ndim == 3 ? 21 : 24) * b->ndim, lo_bit = 64 - bits;
    const int lo_sort = fl_sort_split(lo_bit, b->sort_passes);
    fl_sort_reset(&b->sb, n, (64 - lo_sort + 7) / 8, ts);
    fl_launch_bmorton(b->pos.as<float4>(), n, b->ndim, gid, gr, b->sb.keys[0], b->sb.vals[0],
                      b->sb.hist, lo_sort, ts);
    int r = fl_sort_passes(&b->sb, n, lo_sort, err, ts, &b->launches);
    r = fl_sort_runfix(&b->sb, n, lo_bit, lo_sort, r, ts, &b->launches);
    fl_sort_reset(&b->sb2, n, 2, ts);
    fl_launch_bgidkey(n, b->sb.vals[r], gid, b->off.as<int32_t>(), G, b->sb2.keys[0],
                      b->sb2.vals[0], b->sb2.hist, ts);
    const int r2 = fl_sort_passes(&b->sb2, n, 48, err, ts, &b->launches);
    skeys = b->sb.keys[1 - r];
    perm = b->sb.vals[1 - r];
    fl_launch_bgather(n, b->sb2.vals[r2], b->sb.keys[r], b->sb.vals[r], gid, skeys, perm, gpos, ts);
    b->launches += 3;
    fl_launch_build(&b->tb, skeys, perm, b->pos.as<float4>(), b->charge.as<float>(), b->closed,
                    nullptr, b->fx_exp, ts, &b->launches, segs);
    fl_launch_aggregate(&b->tb, skeys, b->closed, b->sign, nullptr, b->fx_exp, 6, err, ts,
                        &b->launches, segs);
    if (side) cudaEventRecord(b->ev_tree, ts);
  }
  // links (a snapshot: read v, write the other velocity buffer)
  if (b->m > 0) {
    FlLinkCsr csr{b->row.as<int32_t>(), b->entry.as<float4>(), b->code.as<uint32_t>()};
    fl_launch_link(b->pos.as<float4>(), bvel(b), b->vel[1 - b->cur].as<float4>(), csr, n, b->ndim,
                   0.f, b->step, b->seed, st, gr, gid, tk);
    b->cur = 1 - b->cur;
    ++b->launches;
  }
  if (n >= 2) {
    if (side) cudaStreamWaitEvent(st, b->ev_tree, 0);
    b->tb.walk_blocks = b->walk_blocks;
    fl_launch_walk(&b->tb, perm, nullptr, bvel(b), 0.f, 1.0, 0.0, b->dmax_any, b->step, b->seed,
                   err, nullptr, 32, st, segs, tk);
    ++b->launches;
  }
  // collide (every graph with a collide force, each with its own cell side and iterations),
  // against a snapshot: read v, write the other velocity buffer. Its sort reuses the trees'
  // first sort buffers, free once the walk has run.
  for (int it = 0; it < b->citer_max; ++it) {
    const int gbits = b->gb.bits, lo_bit = 63 - gbits;
    fl_sort_reset(&b->sb, n, (64 - lo_bit + 7) / 8, st);
    fl_launch_bgrid_keys(b->pos.as<float4>(), bvel(b), n, b->ndim, gid, gr, it, gbits,
                         b->sb.keys[0], b->sb.vals[0], b->sb.hist, lo_bit, st);
    const int r = fl_sort_passes(&b->sb, n, lo_bit, err, st, &b->launches);
    fl_launch_bgrid_query(&b->gb, b->sb.keys[r], b->sb.vals[r], b->pos.as<float4>(), bvel(b),
                          b->vel[1 - b->cur].as<float4>(), b->radius.as<float>(), b->ndim, gid, gr,
                          b->sgid.as<uint32_t>(), tk, st, &b->launches);
    b->cur = 1 - b->cur;
    ++b->launches;
  }
  // centre shift (per graph) and integration
  fl_launch_integrate(b->pos.as<float4>(), bvel(b), b->fix.as<float4>(), b->mask.as<uint32_t>(),
                      n, b->ndim, 1.f, nullptr, 0, 0, 0, 0, st, gr, gid);
  ++b->launches;
}

}  // namespace

extern "C" {

int32_t fl_batch_create(int32_t device, fl_batch** out) {
  if (!out) return FL_E_ARG;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
    cudaGetLastError();
    return FL_E_DEVICE;
  }
  fl_batch* b = new fl_batch();
  b->device = device;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) != cudaSuccess ||
      b->errw.alloc(256) != cudaSuccess || cudaMemset(b->errw.p, 0, 256) != cudaSuccess) {
    cudaGetLastError();
    if (b->st) cudaStreamDestroy(b->st);
    delete b;
    return FL_E_DEVICE;
  }
  if (cudaStreamCreateWithFlags(&b->aux, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->ev_tree, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();  // no side stream: the trees run on the main one
    if (b->aux) cudaStreamDestroy(b->aux);
    b->aux = nullptr;
  }
  *out = b;
  return FL_OK;
}

int32_t fl_batch_destroy(fl_batch* b) {
  if (!b) return FL_OK;
  cudaSetDevice(b->device);
  cudaStreamSynchronize(b->st);
  if (b->aux) cudaStreamSynchronize(b->aux);
  clear_blocks(b);
  cudaStreamDestroy(b->st);
  if (b->aux) cudaStreamDestroy(b->aux);
  if (b->ev_fork) cudaEventDestroy(b->ev_fork);
  if (b->ev_tree) cudaEventDestroy(b->ev_tree);
  delete b;
  return FL_OK;
}

const char* fl_batch_last_error(const fl_batch* b) { return b ? b->err.c_str() : "no batch"; }

}  // extern "C"

namespace {

// The host-side arrays of graphs [graph0, graph0 + count) of a batch, whose nodes start at node
// node0 and links at link m0: what fl_batch_set_graphs uploads for all graphs and
// fl_batch_add_graphs for the graphs it appends.
struct HostPart {
  int64_t n = 0, m = 0;
  std::vector<float> pos, vel, charge, radius;
  std::vector<uint32_t> gid;
  std::vector<int32_t> off;  // count entries: each graph's first node (global)
  std::vector<FlBatchParams> prm;
  std::vector<uint2> groups;
  std::vector<int32_t> row;  // n entries: the rows' ends (global entry offsets)
  std::vector<float> entry;
  std::vector<uint32_t> code;
  bool neg = false, posv = false, has_radius = false;
  double smax = 0, dmax_any = INFINITY;
  int32_t citer_max = 0;
};

int32_t check_descs(fl_batch* b, int32_t count, const fl_graph_desc* d, int64_t* n, int64_t* m) {
  *n = 0, *m = 0;
  for (int32_t g = 0; g < count; ++g) {
    if (d[g].n < 0 || d[g].m < 0 || (d[g].n && !d[g].pos4) || (d[g].m && (!d[g].source || !d[g].target)))
      return bfail(b, FL_E_ARG, "graph " + std::to_string(g) + ": bad sizes or arrays");
    if (!(d[g].theta2 >= 0) || !(d[g].distance_min2 >= 0) || !(d[g].distance_max2 > 0))
      return bfail(b, FL_E_ARG, "graph " + std::to_string(g) + ": bad many-body parameters");
    for (int32_t j = 0; j < d[g].m; ++j) {
      const int32_t a = d[g].source[j], c = d[g].target[j];
      if (a < 0 || a >= d[g].n || c < 0 || c >= d[g].n)
        return bfail(b, FL_E_ARG, "graph " + std::to_string(g) + " link " + std::to_string(j) + ": node not found");
    }
    *n += d[g].n, *m += d[g].m;
  }
  return FL_OK;
}

// step0: the batch's tick counter when these graphs join (a graph's jiggle step is the batch's
// plus its own tick count at joining, less step0).
void build_part(int32_t ndim, int32_t count, const fl_graph_desc* d, int64_t node0, int32_t graph0,
                int64_t m0, uint32_t step0, HostPart* hp) {
  int64_t n = 0, m = 0;
  for (int32_t g = 0; g < count; ++g) n += d[g].n, m += d[g].m;
  hp->n = n, hp->m = m;
  const size_t N = (size_t)std::max<int64_t>(n, 1);
  hp->pos.assign(4 * N, 0.f), hp->vel.assign(4 * N, 0.f);
  hp->gid.assign(N, 0u), hp->charge.assign(N, -30.f), hp->radius.assign(N, 0.f);
  hp->off.assign(count, 0), hp->prm.assign(count, FlBatchParams{});
  hp->groups.clear();
  for (int32_t g = 0, at = 0; g < count; ++g) {
    const int64_t gat = node0 + at;  // the graph's first node in the batch
    hp->off[g] = (int32_t)gat;
    const fl_graph_desc& x = d[g];
    double gmax = x.charge ? 0.0 : 30.0;
    float rmax = 0.f;  // collide: the graph's largest radius
    // the walk's point groups: the graph's sorted positions in runs of 32 from its first one (a
    // graph of one point has no tree and no group)
    if (x.n >= 2)
      for (int32_t j = 0; j < x.n; j += 32)
        hp->groups.push_back(make_uint2((uint32_t)(gat + j), (uint32_t)(gat + std::min(j + 32, x.n))));
    for (int32_t i = 0; i < x.n; ++i) {
      for (int k = 0; k < 4; ++k) {
        const float p = k < ndim ? x.pos4[4 * (size_t)i + k] : 0.f;
        hp->pos[4 * (size_t)(at + i) + k] = std::isfinite(p) ? p : 0.f;
        if (x.vel4 && k < ndim) hp->vel[4 * (size_t)(at + i) + k] = x.vel4[4 * (size_t)i + k];
      }
      hp->gid[at + i] = (uint32_t)(graph0 + g);
      if (x.radii) {  // non-numbers count as 0, as the plain engine's radii
        const float r = std::isfinite(x.radii[i]) ? x.radii[i] : 0.f;
        hp->radius[at + i] = r;
        rmax = std::max(rmax, r);
      }
      const float c = x.charge ? x.charge[i] : -30.f;
      const float cc = std::isfinite(c) ? c : 0.f;
      hp->charge[at + i] = cc;
      hp->neg = hp->neg || cc < 0.f, hp->posv = hp->posv || cc > 0.f;
      hp->smax = std::max(hp->smax, (double)std::fabs(cc));
      gmax = std::max(gmax, (double)std::fabs(cc));
    }
    // the graph's own fixed-point scale, as a lone simulation of it chooses it: its cells come
    // out the same bit for bit, alone or in any batch
    hp->prm[g] = FlBatchParams{x.theta2, x.distance_min2, x.distance_max2, x.center_x, x.center_y,
                               x.center_z, x.center_strength, 1.0 - x.velocity_decay,
                               fl_fixed_exponent(x.n, gmax * (ndim == 1 ? 8192.0 : 1.0)),
                               x.tick0 - step0, 0, 0.f, 0.f};
    // collide as the plain engine runs it: cells twice the largest radius, nothing to do
    // without a radius above 0 or a second node
    if (x.radii) hp->has_radius = true;
    if (x.radii && x.n >= 2 && rmax > 0.f && x.collide_iterations > 0) {
      hp->prm[g].citer = x.collide_iterations;
      hp->prm[g].cinv = 1.f / (2.f * rmax);
      hp->prm[g].cstr = (float)x.collide_strength;
      hp->citer_max = std::max(hp->citer_max, x.collide_iterations);
    }
    if (x.distance_max2 < 3e38) hp->dmax_any = 1.0;  // some graph has a finite distanceMax
    at += x.n;
  }
  // links: a CSR over the part's nodes, node indices made global; d3's default strength and
  // bias; each entry's code holds its link's index within its own graph (the jiggle of a link
  // is the graph's own)
  std::vector<int32_t> cnt(N + 1, 0);  // per node: its entries; then the rows' starts
  {
    int64_t at = 0;
    for (int32_t g = 0; g < count; ++g) {
      for (int32_t j = 0; j < d[g].m; ++j) ++cnt[at + d[g].source[j]], ++cnt[at + d[g].target[j]];
      at += d[g].n;
    }
  }
  hp->row.assign(N, 0);
  std::vector<int32_t> cur(N, 0);
  {
    int64_t run = 2 * m0;
    for (int64_t i = 0; i < n; ++i) cur[i] = (int32_t)(run - 2 * m0), run += cnt[i], hp->row[i] = (int32_t)run;
  }
  hp->entry.assign(4 * (size_t)std::max<int64_t>(2 * m, 1), 0.f);
  hp->code.assign((size_t)std::max<int64_t>(2 * m, 1), 0u);
  int64_t at = 0;
  for (int32_t g = 0; g < count; ++g) {
    const fl_graph_desc& x = d[g];
    for (int32_t j = 0; j < x.m; ++j) {
      const int32_t a = x.source[j], c = x.target[j];
      const int32_t ga = (int32_t)(node0 + at + a), gc = (int32_t)(node0 + at + c);
      const float dist = x.link_distance ? x.link_distance[j] : 30.f;
      // src/link.js:73-75, :36-38: bias = count(source) / (count(source) + count(target)),
      // strength = 1 / min(count(source), count(target))
      const int32_t ca = cnt[at + a], cc = cnt[at + c];
      const float bias = x.link_bias ? x.link_bias[j] : (float)((double)ca / (ca + cc));
      const float str = x.link_strength ? x.link_strength[j] : (float)(1.0 / std::min(ca, cc));
      int32_t e = cur[at + a]++;
      std::memcpy(&hp->entry[4 * (size_t)e], &gc, 4);
      hp->entry[4 * (size_t)e + 1] = dist, hp->entry[4 * (size_t)e + 2] = str;
      hp->entry[4 * (size_t)e + 3] = (float)(1.0 - (double)bias);
      hp->code[e] = 2u * (uint32_t)j;
      e = cur[at + c]++;
      std::memcpy(&hp->entry[4 * (size_t)e], &ga, 4);
      hp->entry[4 * (size_t)e + 1] = dist, hp->entry[4 * (size_t)e + 2] = str;
      hp->entry[4 * (size_t)e + 3] = bias;
      hp->code[e] = 2u * (uint32_t)j + 1u;
    }
    at += x.n;
  }
}

// The per-node and per-tick scratch of a batch of n nodes (recomputed every tick: no contents
// to keep), and the collide grid.
int32_t size_scratch(fl_batch* b) {
  const int64_t n = b->n;
  const size_t N = (size_t)std::max<int64_t>(n, 1);
  FB_CK(b, b->gid_pos.reserve(4 * N));
  FB_CK(b, b->red.reserve(sizeof(FlReduce) * (size_t)b->graphs));
  FB_CK(b, b->gr.reserve(sizeof(FlGraph) * (size_t)b->graphs));
  FB_CK(b, b->sort1.reserve(fl_sort_bytes(n)));
  FB_CK(b, b->sort2.reserve(fl_sort_bytes(n)));
  FB_CK(b, b->tree.reserve(fl_tree_bytes(n)));
  fl_sort_carve(&b->sb, b->sort1.p, n);
  fl_sort_carve(&b->sb2, b->sort2.p, n);
  fl_tree_carve(&b->tb, b->tree.p, n, b->ndim);
  if (b->citer_max) {
    FB_CK(b, b->grid.reserve(fl_grid_bytes(n)));
    FB_CK(b, b->sgid.reserve(4 * N));
    fl_grid_carve(&b->gb, b->grid.p, n);
  }
  return FL_OK;
}

// At least `bytes` bytes in buf, keeping its first `keep` bytes (copied on the batch's stream).
int32_t grow(fl_batch* b, Buf& buf, size_t bytes, size_t keep) {
  if (buf.p && bytes <= buf.bytes) return FL_OK;
  Buf nb;
  FB_CK(b, nb.alloc(bytes + bytes / 2));
  if (keep && buf.p) FB_CK(b, cudaMemcpyAsync(nb.p, buf.p, keep, cudaMemcpyDeviceToDevice, b->st));
  FB_CK(b, cudaStreamSynchronize(b->st));
  std::swap(buf.p, nb.p);
  std::swap(buf.bytes, nb.bytes);
  return FL_OK;  // nb frees the old buffer
}

// Upload part hp at nodes [node0, ...), graphs [graph0, ...), entries [2 m0, ...) (the buffers
// already hold room for them), and fold its flags into the batch's.
int32_t upload_part(fl_batch* b, const HostPart& hp, int64_t node0, int32_t graph0, int64_t m0,
                    int32_t count) {
  cudaStream_t st = b->st;
  const size_t n = (size_t)hp.n;
  if (n) {
    FB_CK(b, cudaMemcpyAsync(b->pos.as<float4>() + node0, hp.pos.data(), 16 * n, cudaMemcpyHostToDevice, st));
    FB_CK(b, cudaMemcpyAsync(bvel(b) + node0, hp.vel.data(), 16 * n, cudaMemcpyHostToDevice, st));
    FB_CK(b, cudaMemsetAsync(b->fix.as<float4>() + node0, 0, 16 * n, st));
    FB_CK(b, cudaMemsetAsync(b->mask.as<uint32_t>() + node0, 0, 4 * n, st));
    FB_CK(b, cudaMemcpyAsync(b->gid.as<uint32_t>() + node0, hp.gid.data(), 4 * n, cudaMemcpyHostToDevice, st));
    FB_CK(b, cudaMemcpyAsync(b->charge.as<float>() + node0, hp.charge.data(), 4 * n, cudaMemcpyHostToDevice, st));
    if (b->radius.p)
      FB_CK(b, cudaMemcpyAsync(b->radius.as<float>() + node0, hp.radius.data(), 4 * n, cudaMemcpyHostToDevice, st));
    FB_CK(b, cudaMemcpyAsync(b->row.as<int32_t>() + node0 + 1, hp.row.data(), 4 * n, cudaMemcpyHostToDevice, st));
  }
  FB_CK(b, cudaMemcpyAsync(b->off.as<int32_t>() + graph0, hp.off.data(), 4 * (size_t)count,
                           cudaMemcpyHostToDevice, st));
  const int32_t end = (int32_t)(node0 + hp.n);
  FB_CK(b, cudaMemcpyAsync(b->off.as<int32_t>() + graph0 + count, &end, 4, cudaMemcpyHostToDevice, st));
  FB_CK(b, cudaMemcpyAsync(b->prm.as<FlBatchParams>() + graph0, hp.prm.data(),
                           sizeof(FlBatchParams) * (size_t)count, cudaMemcpyHostToDevice, st));
  if (!hp.groups.empty())
    FB_CK(b, cudaMemcpyAsync(b->groups.as<uint2>() + (b->ngroups - hp.groups.size()), hp.groups.data(),
                             8 * hp.groups.size(), cudaMemcpyHostToDevice, st));
  if (hp.m) {
    FB_CK(b, cudaMemcpyAsync(b->entry.as<float4>() + 2 * m0, hp.entry.data(), 32 * (size_t)hp.m,
                             cudaMemcpyHostToDevice, st));
    FB_CK(b, cudaMemcpyAsync(b->code.as<uint32_t>() + 2 * m0, hp.code.data(), 8 * (size_t)hp.m,
                             cudaMemcpyHostToDevice, st));
  }
  b->hoff.resize((size_t)graph0);
  b->hoff.insert(b->hoff.end(), hp.off.begin(), hp.off.end());
  b->hoff.push_back(end);
  // the host vectors may go out of scope at return: wait for the copies that read them
  FB_CK(b, cudaStreamSynchronize(st));
  return FL_OK;
}

}  // namespace

extern "C" {

int32_t fl_batch_set_graphs(fl_batch* b, int32_t ndim, int32_t graphs, const fl_graph_desc* d) {
  int32_t rc = bcheck(b);
  if (rc) return rc;
  if (ndim < 1 || ndim > 3) return bfail(b, FL_E_ARG, "ndim must be 1, 2 or 3");
  if (graphs < 1 || graphs > 65535 || !d) return bfail(b, FL_E_ARG, "graphs must be 1..65535");
  int64_t n = 0, m = 0;
  if ((rc = check_descs(b, graphs, d, &n, &m))) return rc;
  if (n > kMaxBatchNodes) return bfail(b, FL_E_ARG, "too many nodes in one batch");
  if (m > (int64_t(1) << 30)) return bfail(b, FL_E_ARG, "too many links in one batch");
  FB_CK(b, cudaStreamSynchronize(b->st));
  clear_blocks(b);
  HostPart hp;
  build_part(ndim, graphs, d, 0, 0, 0, 0u, &hp);
  b->ndim = ndim, b->graphs = graphs, b->n = (int32_t)n, b->m = (int32_t)m;
  b->cur = 0;
  b->step = 0;
  b->neg = hp.neg, b->posv = hp.posv, b->smax = hp.smax;
  b->closed = !(hp.neg && hp.posv);
  b->sign = hp.neg ? -1.f : 1.f;
  b->fx_exp = fl_fixed_exponent(n, hp.smax * (ndim == 1 ? 8192.0 : 1.0));
  b->dmax_any = hp.dmax_any;
  b->citer_max = hp.citer_max;
  b->ngroups = (int32_t)hp.groups.size();
  // device buffers: the batch's state and graphs
  const size_t N = (size_t)std::max<int64_t>(n, 1), E = (size_t)std::max<int64_t>(2 * m, 1);
  FB_CK(b, b->pos.reserve(16 * N));
  FB_CK(b, b->vel[0].reserve(16 * N));
  FB_CK(b, b->vel[1].reserve(16 * N));
  FB_CK(b, b->fix.reserve(16 * N));
  FB_CK(b, b->mask.reserve(4 * N));
  FB_CK(b, b->gid.reserve(4 * N));
  FB_CK(b, b->charge.reserve(4 * N));
  if (hp.has_radius) FB_CK(b, b->radius.reserve(4 * N));
  else b->radius.release();
  FB_CK(b, b->off.reserve(4 * (size_t)(graphs + 1)));
  FB_CK(b, b->prm.reserve(sizeof(FlBatchParams) * (size_t)graphs));
  FB_CK(b, b->row.reserve(4 * ((size_t)n + 1)));
  FB_CK(b, b->entry.reserve(16 * E));
  FB_CK(b, b->code.reserve(4 * E));
  FB_CK(b, b->groups.reserve(8 * std::max<size_t>(hp.groups.size(), 1)));
  if ((rc = size_scratch(b))) return rc;
  const int32_t zero = 0;
  FB_CK(b, cudaMemcpyAsync(b->row.p, &zero, 4, cudaMemcpyHostToDevice, b->st));
  FB_CK(b, cudaMemsetAsync(b->vel[1].p, 0, 16 * N, b->st));
  return upload_part(b, hp, 0, 0, 0, graphs);
}

int32_t fl_batch_add_graphs(fl_batch* b, int32_t count, const fl_graph_desc* d) {
  int32_t rc = bcheck(b);
  if (rc) return rc;
  if (!b->graphs) return bfail(b, FL_E_STATE, "no graphs set: fl_batch_set_graphs first");
  if (count < 1 || b->graphs + (int64_t)count > 65535 || !d)
    return bfail(b, FL_E_ARG, "count must keep the batch at 1..65535 graphs");
  int64_t n = 0, m = 0;
  if ((rc = check_descs(b, count, d, &n, &m))) return rc;
  const int64_t n0 = b->n, m0 = b->m;
  const int32_t g0 = b->graphs;
  if (n0 + n > kMaxBatchNodes) return bfail(b, FL_E_ARG, "too many nodes in one batch");
  if (m0 + m > (int64_t(1) << 30)) return bfail(b, FL_E_ARG, "too many links in one batch");
  FB_CK(b, cudaStreamSynchronize(b->st));
  clear_blocks(b);
  HostPart hp;
  build_part(b->ndim, count, d, n0, g0, m0, b->step, &hp);
  const int64_t N1 = std::max<int64_t>(n0 + n, 1), E1 = std::max<int64_t>(2 * (m0 + m), 1);
  // the kept state grows in place of a rebuild: positions, the current velocities, pins,
  // graph ids, charges, radii, links, offsets, parameters, walk groups
  if ((rc = grow(b, b->pos, 16 * N1, 16 * n0))) return rc;
  if ((rc = grow(b, b->vel[b->cur], 16 * N1, 16 * n0))) return rc;
  if ((rc = grow(b, b->vel[1 - b->cur], 16 * N1, 0))) return rc;
  if ((rc = grow(b, b->fix, 16 * N1, 16 * n0))) return rc;
  if ((rc = grow(b, b->mask, 4 * N1, 4 * n0))) return rc;
  if ((rc = grow(b, b->gid, 4 * N1, 4 * n0))) return rc;
  if ((rc = grow(b, b->charge, 4 * N1, 4 * n0))) return rc;
  if (hp.has_radius || b->radius.p) {
    const bool had = b->radius.p != nullptr;
    if ((rc = grow(b, b->radius, 4 * N1, had ? 4 * n0 : 0))) return rc;
    if (!had && n0) FB_CK(b, cudaMemsetAsync(b->radius.p, 0, 4 * n0, b->st));
  }
  if ((rc = grow(b, b->off, 4 * (size_t)(g0 + count + 1), 4 * (size_t)(g0 + 1)))) return rc;
  if ((rc = grow(b, b->prm, sizeof(FlBatchParams) * (size_t)(g0 + count), sizeof(FlBatchParams) * (size_t)g0))) return rc;
  if ((rc = grow(b, b->row, 4 * (size_t)(N1 + 1), 4 * (size_t)(n0 + 1)))) return rc;
  if ((rc = grow(b, b->entry, 16 * (size_t)E1, 32 * (size_t)m0))) return rc;
  if ((rc = grow(b, b->code, 4 * (size_t)E1, 8 * (size_t)m0))) return rc;
  const size_t ng1 = (size_t)b->ngroups + hp.groups.size();
  if ((rc = grow(b, b->groups, 8 * std::max<size_t>(ng1, 1), 8 * (size_t)b->ngroups))) return rc;
  b->graphs = g0 + count, b->n = (int32_t)(n0 + n), b->m = (int32_t)(m0 + m);
  b->ngroups = (int32_t)ng1;
  b->neg = b->neg || hp.neg, b->posv = b->posv || hp.posv, b->smax = std::max(b->smax, hp.smax);
  b->closed = !(b->neg && b->posv);
  b->sign = b->neg ? -1.f : 1.f;
  b->fx_exp = fl_fixed_exponent(b->n, b->smax * (b->ndim == 1 ? 8192.0 : 1.0));
  if (hp.dmax_any < 3e38) b->dmax_any = 1.0;
  b->citer_max = std::max(b->citer_max, hp.citer_max);
  if ((rc = size_scratch(b))) return rc;
  return upload_part(b, hp, n0, g0, m0, count);
}

int32_t fl_batch_set_seed(fl_batch* b, uint32_t seed) {
  int32_t rc = bcheck(b);
  if (rc) return rc;
  b->seed = seed;
  return FL_OK;
}

int32_t fl_batch_set_tuning(fl_batch* b, int32_t key, int32_t value) {
  int32_t rc = bcheck(b);
  if (rc) return rc;
  clear_blocks(b);
  switch (key) {
    case FL_TUNE_GRAPHS:
      if (value != 0 && value != 1) return bfail(b, FL_E_ARG, "graphs must be 0 or 1");
      b->use_graphs = value != 0;
      return FL_OK;
    case FL_TUNE_SORT_PASSES:
      if (value < 0 || value > 8) return bfail(b, FL_E_ARG, "sort passes must be 0..8");
      b->sort_passes = value;
      return FL_OK;
    case FL_TUNE_WALK_BLOCKS:
      if (value < 0 || value > 32) return bfail(b, FL_E_ARG, "walk blocks per SM must be 0..32");
      b->walk_blocks = value;
      return FL_OK;
    default:
      return bfail(b, FL_E_ARG, "unknown tuning key for a batch");
  }
}

int32_t fl_batch_enqueue(fl_batch* b, const double* alphas, int32_t ticks) {
  int32_t rc = bcheck(b);
  if (rc) return rc;
  if (!b->graphs) return bfail(b, FL_E_STATE, "no graphs set");
  if (ticks < 0 || (ticks && !alphas)) return bfail(b, FL_E_ARG, "bad alphas");
  if (!ticks) return FL_OK;
  const size_t need = (size_t)ticks * (size_t)b->graphs;
  if (need > b->alpha_cap || ticks > b->tick_cap) {
    FB_CK(b, cudaStreamSynchronize(b->st));
    clear_blocks(b);  // captured blocks point into the old buffers
    if (need > b->alpha_cap) {
      FB_CK(b, b->alphas.alloc(8 * need));
      b->alpha_cap = need;
    }
    if (ticks > b->tick_cap) {
      FB_CK(b, b->tickbuf.alloc(sizeof(FlTick) * (size_t)ticks));
      b->tick_cap = ticks;
    }
  }
  // copied on the stream, so after every tick already queued has read the previous values
  FB_CK(b, cudaMemcpyAsync(b->alphas.p, alphas, 8 * need, cudaMemcpyHostToDevice, b->st));
  b->htick.resize(ticks);
  for (int32_t k = 0; k < ticks; ++k) b->htick[k] = FlTick{0.f, 1.f, b->step + (uint32_t)k, b->seed};
  FB_CK(b, cudaMemcpyAsync(b->tickbuf.p, b->htick.data(), sizeof(FlTick) * (size_t)ticks,
                           cudaMemcpyHostToDevice, b->st));
  auto encode = [&]() {
    for (int32_t k = 0; k < ticks; ++k)
      encode_batch_tick(b, b->alphas.as<double>() + (size_t)k * b->graphs, b->tickbuf.as<FlTick>() + k);
  };
  // a block of ticks seen before runs as one CUDA graph (captured the second time)
  fl_batch::Block* x = nullptr;
  if (b->use_graphs)
    for (auto& y : b->blocks)
      if (y.count == ticks && y.cur_in == b->cur) x = &y;
  if (x && x->captured) {
    FB_CK(b, cudaGraphLaunch(x->exec, b->st));
    b->cur = x->cur_out;
    b->launches += x->launches;
  } else if (x) {
    const int cur0 = b->cur;
    const int64_t l0 = b->launches;
    cudaGraph_t g = nullptr;
    bool ok = cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
      encode();
      ok = cudaStreamEndCapture(b->st, &g) == cudaSuccess && g;
    }
    if (ok) {
      ok = cudaGraphInstantiate(&x->exec, g, 0) == cudaSuccess;
      cudaGraphDestroy(g);
    }
    if (ok) {
      x->captured = true;
      FB_CK(b, cudaGraphLaunch(x->exec, b->st));
    } else {
      cudaGetLastError();
      if (g) cudaGraphDestroy(g);
      b->use_graphs = false;
      b->cur = cur0;
      b->launches = l0;
      encode();
    }
  } else {
    const int cur0 = b->cur;
    const int64_t l0 = b->launches;
    encode();
    if (b->use_graphs) {
      if (b->blocks.size() >= 8) {
        if (b->blocks.front().captured) cudaGraphExecDestroy(b->blocks.front().exec);
        b->blocks.erase(b->blocks.begin());
      }
      b->blocks.push_back(fl_batch::Block{ticks, cur0, b->cur, b->launches - l0, false, nullptr});
    }
  }
  b->step += (uint32_t)ticks;
  b->ticks += ticks;
  FB_CK(b, cudaGetLastError());
  return FL_OK;
}

int32_t fl_batch_sync(fl_batch* b, float* pos4_out, float* vel4_out) {
  int32_t rc = bcheck(b);
  if (rc) return rc;
  if (b->n && pos4_out)
    FB_CK(b, cudaMemcpyAsync(pos4_out, b->pos.p, 16 * (size_t)b->n, cudaMemcpyDeviceToHost, b->st));
  if (b->n && vel4_out)
    FB_CK(b, cudaMemcpyAsync(vel4_out, bvel(b), 16 * (size_t)b->n, cudaMemcpyDeviceToHost, b->st));
  uint32_t w = 0;
  FB_CK(b, cudaMemcpyAsync(&w, b->errw.p, 4, cudaMemcpyDeviceToHost, b->st));
  FB_CK(b, cudaStreamSynchronize(b->st));
  if (w) {
    cudaMemsetAsync(b->errw.p, 0, 4, b->st);
    if (w & FL_ERR_LOOKBACK) return bfail(b, FL_E_TIMEOUT, "a device-side look-back wait gave up");
    return bfail(b, FL_E_OVERFLOW, "a tree was malformed or a walk overflowed");
  }
  return FL_OK;
}

int32_t fl_batch_autotune(fl_batch* b, int32_t ticks, double alpha, const char* cache_path,
                          fl_tune_result* out) {
  int32_t rc = bcheck(b);
  if (rc) return rc;
  if (!out) return bfail(b, FL_E_ARG, "out is NULL");
  if (ticks < 1 || !(alpha >= 0.0)) return bfail(b, FL_E_ARG, "ticks must be >= 1 and alpha >= 0");
  *out = fl_tune_result{32, b->sort_passes, b->walk_blocks, 100, 0, 0, 0, 0};
  const int n = b->n;
  if (!b->graphs || n < 2) return FL_OK;
  const int bits = (b->ndim == 3 ? 21 : 24) * b->ndim, lo_bit = 64 - bits;
  std::vector<int> passes{0}, seen{fl_sort_split(lo_bit, 0)};
  for (int c : {3, 5, 8}) {
    const int lo = fl_sort_split(lo_bit, c);
    if (std::find(seen.begin(), seen.end(), lo) == seen.end()) seen.push_back(lo), passes.push_back(c);
  }
  std::vector<FlTuneKnob> knobs{{FL_TUNE_SORT_PASSES, "sort_passes", passes, 0},
                                {FL_TUNE_WALK_BLOCKS, "walk_blocks", {0, 8, 6, 4}, 0}};
  const std::string key = fl_tune_arch() + " batch ndim=" + std::to_string(b->ndim) +
                          " log2graphs=" + std::to_string((int)std::floor(std::log2((double)b->graphs))) +
                          " log2n=" + std::to_string((int)std::floor(std::log2((double)n))) +
                          " links=" + std::to_string(b->m > 0 ? 1 : 0) +
                          " graphs=" + std::to_string((int)b->use_graphs);
  FB_CK(b, cudaStreamSynchronize(b->st));
  Buf snap;
  const size_t v4 = 16 * (size_t)n;
  FB_CK(b, snap.alloc(2 * v4));
  FB_CK(b, cudaMemcpyAsync(snap.p, b->pos.p, v4, cudaMemcpyDeviceToDevice, b->st));
  FB_CK(b, cudaMemcpyAsync(snap.as<char>() + v4, bvel(b), v4, cudaMemcpyDeviceToDevice, b->st));
  const uint32_t step0 = b->step;
  const int64_t ticks0 = b->ticks, launches0 = b->launches;
  auto restore = [&]() -> int32_t {
    FB_CK(b, cudaMemcpyAsync(b->pos.p, snap.p, v4, cudaMemcpyDeviceToDevice, b->st));
    FB_CK(b, cudaMemcpyAsync(b->vel[0].p, snap.as<char>() + v4, v4, cudaMemcpyDeviceToDevice, b->st));
    b->cur = 0;
    b->step = step0;
    return FL_OK;
  };
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  FB_CK(b, cudaEventCreate(&e0));
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return bfail(b, FL_E_DEVICE, "cudaEventCreate");
  }
  const std::vector<double> al((size_t)ticks * (size_t)b->graphs, alpha);
  auto time = [&](double* ms) -> int {  // as fl_autotune: direct, captured, then timed
    for (int rep = 0; rep < 3; ++rep) {
      int32_t r = restore();
      if (r) return r;
      if (rep == 2) FB_CK(b, cudaEventRecord(e0, b->st));
      if ((r = fl_batch_enqueue(b, al.data(), ticks)) != FL_OK) return r;
      if (rep == 2) FB_CK(b, cudaEventRecord(e1, b->st));
    }
    int32_t r = fl_batch_sync(b, nullptr, nullptr);
    if (r) return r;
    float t = 0.f;
    FB_CK(b, cudaEventElapsedTime(&t, e0, e1));
    *ms = (double)t / ticks;
    return FL_OK;
  };
  auto set = [&](int k, int v) -> int { return fl_batch_set_tuning(b, k, v); };
  FlTuneOutcome o;
  rc = fl_tune_search(cache_path, key, knobs, set, time, &o);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const int32_t rr = restore();
  if (!rc) rc = rr;
  cudaError_t e = cudaStreamSynchronize(b->st);
  b->ticks = ticks0, b->launches = launches0;
  if (rc) return rc;
  if (e != cudaSuccess) return bcuda(b, e, "cudaStreamSynchronize");
  *out = fl_tune_result{32, b->sort_passes, b->walk_blocks, 100, o.best_ms, o.default_ms,
                        o.candidates, o.cached ? 1 : 0};
  return FL_OK;
}

int32_t fl_batch_read(fl_batch* b, int32_t first, int32_t count, float* pos4_out,
                      float* vel4_out) {
  int32_t rc = bcheck(b);
  if (rc) return rc;
  if (first < 0 || count < 0 || first + (int64_t)count > b->graphs)
    return bfail(b, FL_E_ARG, "graph range out of bounds");
  const int32_t a = count ? b->hoff[first] : 0, e = count ? b->hoff[first + count] : 0;
  const size_t bytes = 16 * (size_t)(e - a);
  if (bytes && pos4_out)
    FB_CK(b, cudaMemcpyAsync(pos4_out, b->pos.as<float4>() + a, bytes, cudaMemcpyDeviceToHost, b->st));
  if (bytes && vel4_out)
    FB_CK(b, cudaMemcpyAsync(vel4_out, bvel(b) + a, bytes, cudaMemcpyDeviceToHost, b->st));
  uint32_t w = 0;
  FB_CK(b, cudaMemcpyAsync(&w, b->errw.p, 4, cudaMemcpyDeviceToHost, b->st));
  FB_CK(b, cudaStreamSynchronize(b->st));
  if (w) {
    cudaMemsetAsync(b->errw.p, 0, 4, b->st);
    if (w & FL_ERR_LOOKBACK) return bfail(b, FL_E_TIMEOUT, "a device-side look-back wait gave up");
    return bfail(b, FL_E_OVERFLOW, "a tree was malformed or a walk overflowed");
  }
  return FL_OK;
}

int32_t fl_batch_query(fl_batch* b, int32_t what, int64_t* out) {
  int32_t rc = bcheck(b);
  if (rc) return rc;
  if (!out) return bfail(b, FL_E_ARG, "null output");
  switch (what) {
    case FL_Q_LAUNCHES: *out = b->launches; break;
    case FL_Q_TICKS: *out = b->ticks; break;
    case FL_Q_NODES: *out = b->n; break;
    case FL_Q_DEVICE_BYTES: {
      const Buf* all[] = {&b->pos, &b->vel[0], &b->vel[1], &b->fix, &b->mask, &b->gid, &b->off,
                          &b->prm, &b->red, &b->gr, &b->alphas, &b->charge, &b->row, &b->entry,
                          &b->code, &b->sort1, &b->sort2, &b->tree, &b->gid_pos,
                          &b->groups, &b->radius, &b->grid, &b->sgid};
      size_t s = 0;
      for (const Buf* x : all) s += x->bytes;
      *out = (int64_t)s;
      break;
    }
    default: return bfail(b, FL_E_ARG, "unknown query");
  }
  return FL_OK;
}

int32_t fl_batch_stream(fl_batch* b, void** stream) {
  if (!b || !stream) return FL_E_ARG;
  *stream = (void*)b->st;
  return FL_OK;
}

}  // extern "C"
