// The engine behind include/forcegpu.h: node state resident on the device, the force plan, and
// the per-tick launch sequence on one CUDA stream.
//
// The reference encodes each tick as WebGPU dispatches, force by force in insertion order, then
// integrate (src/gpu/engine.js:351-391). Here each tick is the same sequence of CUDA kernels,
// with three GB300-side changes: no snapshot copies (link and collide read p and v and write a
// second velocity buffer, swapped afterwards); the bounding box of the tree and the centre
// force's FP64 mean come from one read of the positions at the start of the tick; and when the
// centre force is the last force its shift is applied inside the integrate kernel.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/forcegpu.h"
#include "kernels.h"
#include "tune.h"

namespace {

constexpr int64_t kMaxNodes = (int64_t(1) << 26) - 1;  // child slot / stack index width
constexpr double kExactTheta2 = 1e-6;                  // src/gpu/passes/manyBody.js:20-21
constexpr int kGridMin = 8192;                         // pairs by grid from this many nodes
constexpr int kRecursionFp64Depth = 6;  // the recursion sums cells above this depth in FP64

struct DevMem {
  void* p = nullptr;
  size_t bytes = 0;
  DevMem() = default;
  DevMem(const DevMem&) = delete;
  DevMem& operator=(const DevMem&) = delete;
  ~DevMem() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  cudaError_t alloc(size_t b) {
    release();
    if (b == 0) b = 256;
    cudaError_t e = cudaMalloc(&p, b);
    if (e != cudaSuccess) {
      p = nullptr;
      return e;
    }
    bytes = b;
    return cudaSuccess;
  }
  template <typename T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

struct Pass {
  int32_t type = 0;
  uint64_t key = 0;
  bool fresh = true;     // no version seen yet
  uint32_t version = 0;  // last version uploaded
  fl_force_desc d{};     // scalars of the last update
  DevMem a, b;           // per-node arrays
  DevMem row, entry, code;
  int32_t m = 0;
  float rmax = 0.f;
  DevMem scratch;  // tree / sort / grid buffers
  FlSortBufs sb{};
  FlTreeBufs tb{};
  FlGridBufs gb{};
  DevMem red;  // a private reduction record (a centre not fused, or a tree after a centre)
  DevMem cube;
  int alloc_n = -1;
  int sorted_in = -1;  // sort buffer holding the last tick's sorted pairs (-1: no tree yet)
  bool mixed = false;  // many-body strengths of both signs (cells need the full recursion)
  float sign = -1.f;   // the one sign of the strengths otherwise
  int fx_exp = 32;     // scale exponent of the fixed-point cell sums
};

struct ProfRec {
  int group;
  cudaEvent_t a, b;
};

const char* kGroupNames[] = {"reduce", "morton", "sort", "build", "aggregate", "walk", "allpairs",
                             "link", "collide_keys", "collide_sort", "collide_query",
                             "collide_allpairs", "center", "radial", "position", "integrate"};
enum {
  G_REDUCE, G_MORTON, G_SORT, G_BUILD, G_AGGREGATE, G_WALK, G_ALLPAIRS, G_LINK, G_CKEYS, G_CSORT,
  G_CQUERY, G_CALLPAIRS, G_CENTER, G_RADIAL, G_POSITION, G_INTEGRATE, G_COUNT
};

}  // namespace

struct fl_sim {
  int32_t device = 0;
  cudaStream_t st = nullptr;
  // a second stream for the many-body tree's construction, which depends on the positions only
  // and so overlaps with the forces before it; joined before the walk
  cudaStream_t aux = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_tree = nullptr;
  // a third stream for the tree's internal nodes and octant masks, which need only the sorted
  // keys: they run beside the sorted points' records, joined before the cells
  cudaStream_t aux2 = nullptr;
  cudaEvent_t ev_fork2 = nullptr, ev_nodes = nullptr;
  std::string err;
  int32_t n = 0, ndim = 2;
  DevMem pos, vel[2], fix, mask, errw;
  DevMem pack;  // staging of the packed transfers: ndim floats of position, then of velocity
  int cur = 0;
  // the box and sums of the tick's starting positions: reds[red_cur]; the integrate of the tick
  // before fills it (pre_valid) unless the positions changed since
  DevMem reds[2];
  int red_cur = 0;
  bool pre_valid = false;
  // p + v of every node when the tick's first pass is a link: that link's snapshot, written by the
  // integrate of the tick before (snap_valid) unless the state changed since
  DevMem snap;
  bool snap_valid = false;
  std::vector<std::unique_ptr<Pass>> plan;
  uint32_t seed = 0, step = 0;
  int64_t ticks = 0, launches = 0;
  int walk_group = 0;  // points per tree-walk traversal (tuning: 1, 16 or 32; 0 = by size)
  // per-tick values in device memory and the CUDA graphs of tick blocks (fl_enqueue)
  const FlTick* tkp = nullptr;  // the tick being encoded (null: parameters)
  DevMem tickbuf;
  int32_t tick_cap = 0;
  std::vector<FlTick> htick;
  struct Block {
    int32_t count;
    int cur_in, cur_out, red_in, red_out;
    bool pre_in, pre_out, snap_in, snap_out;
    int64_t launches;
    bool captured;
    cudaGraphExec_t exec;
  };
  std::vector<Block> blocks;
  std::vector<double> plan_sig;
  bool use_graphs = true;
  int cell_sums = 0;    // tuning FL_TUNE_CELL_SUMS
  int sort_passes = 0;  // tuning FL_TUNE_SORT_PASSES (0: the default)
  int walk_blocks = 0;  // tuning FL_TUNE_WALK_BLOCKS (0: as many as fit)
  int collide_cell = 100;  // tuning FL_TUNE_COLLIDE_CELL (percent of the largest diameter)
  uint32_t test_lookback = 0;  // tuning FL_TUNE_TEST_LOOKBACK (0: off)
  bool profiling = false;
  int prof_level = 0;
  DevMem wstats;  // walk counters (profiling level 2)
  std::vector<ProfRec> prof_pending;
  std::vector<cudaEvent_t> ev_pool;
  double prof_ms[G_COUNT] = {};
  int64_t prof_count[G_COUNT] = {};
};

namespace {

// the message of the last failed call that takes no simulation (fl_create, the sorts), one per
// host thread: two threads failing at once do not race on it
thread_local std::string g_create_error;

int32_t fail(fl_sim* s, int32_t code, const std::string& msg) {
  if (s) s->err = msg;
  else g_create_error = msg;
  return code;
}

int32_t cuda_fail(fl_sim* s, cudaError_t e, const char* what) {
  cudaGetLastError();
  return fail(s, e == cudaErrorMemoryAllocation ? FL_E_OOM : FL_E_DEVICE,
              std::string(what) + ": " + cudaGetErrorString(e));
}

#define FL_CK(s, call)                                 \
  do {                                                 \
    cudaError_t e_ = (call);                           \
    if (e_ != cudaSuccess) return cuda_fail(s, e_, #call); \
  } while (0)

cudaEvent_t take_event(fl_sim* s) {
  if (!s->ev_pool.empty()) {
    cudaEvent_t e = s->ev_pool.back();
    s->ev_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}

// Times a group of kernels with events on the simulation's stream (when profiling).
struct Scope {
  fl_sim* s;
  int group;
  cudaStream_t st;
  cudaEvent_t a = nullptr;
  Scope(fl_sim* s_, int g, cudaStream_t st_ = nullptr) : s(s_), group(g), st(st_ ? st_ : s_->st) {
    if (s->profiling) {
      a = take_event(s);
      cudaEventRecord(a, st);
    }
  }
  ~Scope() {
    if (a) {
      cudaEvent_t b = take_event(s);
      cudaEventRecord(b, st);
      s->prof_pending.push_back({group, a, b});
    }
  }
};

void drain_profile(fl_sim* s) {
  for (auto& r : s->prof_pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
      s->prof_ms[r.group] += ms;
      s->prof_count[r.group] += 1;
    }
    s->ev_pool.push_back(r.a);
    s->ev_pool.push_back(r.b);
  }
  s->prof_pending.clear();
}

float4* vel_cur(fl_sim* s) { return s->vel[s->cur].as<float4>(); }
FlReduce* red_of(fl_sim* s) { return s->reds[s->red_cur].as<FlReduce>(); }
float4* vel_next(fl_sim* s) { return s->vel[1 - s->cur].as<float4>(); }

// Host-side CSR of the links (src/gpu/passes/link.js:65-101): per node, its links in link order;
// each entry carries the other end, distance, strength and this end's share of the push.
int32_t upload_links(fl_sim* s, Pass* p, const fl_force_desc* d) {
  const int32_t n = s->n, m = d->m;
  if (m < 0 || (m > 0 && (!d->source || !d->target))) return fail(s, FL_E_ARG, "link: bad link arrays");
  std::vector<int32_t> row(n + 1, 0);
  for (int32_t k = 0; k < m; ++k) {
    int32_t a = d->source[k], b = d->target[k];
    if (a < 0 || a >= n || b < 0 || b >= n)
      return fail(s, FL_E_ARG, "link " + std::to_string(k) + ": node not found");
    ++row[a + 1], ++row[b + 1];
  }
  for (int32_t i = 0; i < n; ++i) row[i + 1] += row[i];
  std::vector<int32_t> cur(row.begin(), row.end() - 1);
  std::vector<float> entry(4 * (size_t)std::max(2 * m, 1));
  std::vector<uint32_t> code((size_t)std::max(2 * m, 1));
  for (int32_t k = 0; k < m; ++k) {
    const float dist = d->link_distance ? d->link_distance[k] : 30.f;
    const float str = d->link_strength ? d->link_strength[k] : 1.f;
    const float bias = d->link_bias ? d->link_bias[k] : 0.5f;
    const int32_t a = d->source[k], b = d->target[k];
    int32_t e = cur[a]++;
    std::memcpy(&entry[4 * (size_t)e], &b, 4);
    entry[4 * (size_t)e + 1] = dist, entry[4 * (size_t)e + 2] = str;
    entry[4 * (size_t)e + 3] = (float)(1.0 - (double)bias);
    code[e] = 2u * (uint32_t)k;
    e = cur[b]++;
    std::memcpy(&entry[4 * (size_t)e], &a, 4);
    entry[4 * (size_t)e + 1] = dist, entry[4 * (size_t)e + 2] = str;
    entry[4 * (size_t)e + 3] = bias;
    code[e] = 2u * (uint32_t)k + 1u;
  }
  FL_CK(s, p->row.alloc(4 * (size_t)(n + 1)));
  FL_CK(s, p->entry.alloc(16 * (size_t)std::max(2 * m, 1)));
  FL_CK(s, p->code.alloc(4 * (size_t)std::max(2 * m, 1)));
  FL_CK(s, cudaMemcpy(p->row.p, row.data(), 4 * (size_t)(n + 1), cudaMemcpyHostToDevice));
  if (m) {
    FL_CK(s, cudaMemcpy(p->entry.p, entry.data(), 32 * (size_t)m, cudaMemcpyHostToDevice));
    FL_CK(s, cudaMemcpy(p->code.p, code.data(), 8 * (size_t)m, cudaMemcpyHostToDevice));
  }
  p->m = m;
  return FL_OK;
}

int32_t upload_nodes(fl_sim* s, DevMem& dst, const float* src, float fill, bool finite_only) {
  std::vector<float> h((size_t)std::max(s->n, 1), fill);
  if (src)
    for (int32_t i = 0; i < s->n; ++i) {
      float v = src[i];
      h[i] = (finite_only && !std::isfinite(v)) ? 0.f : v;
    }
  FL_CK(s, dst.alloc(4 * h.size()));
  FL_CK(s, cudaMemcpy(dst.p, h.data(), 4 * h.size(), cudaMemcpyHostToDevice));
  return FL_OK;
}

// Tree / sort / grid buffers of a pass, for the current node count.
int32_t ensure_scratch(fl_sim* s, Pass* p) {
  if (p->alloc_n == s->n) return FL_OK;
  const int64_t n = s->n;
  size_t bytes = fl_sort_bytes(n);
  if (p->type == FL_FORCE_MANYBODY) bytes += fl_tree_bytes(n) + 256;
  if (p->type == FL_FORCE_COLLIDE) bytes += fl_grid_bytes(n) + 256;
  FL_CK(s, p->scratch.alloc(bytes));
  // zero: the sort's counters and look-back words and the walk's group counter start at 0 (each
  // sort and walk leaves them at 0 again)
  FL_CK(s, cudaMemset(p->scratch.p, 0, bytes));
  char* base = p->scratch.as<char>();
  fl_sort_carve(&p->sb, base, n);
  base += (fl_sort_bytes(n) + 255) & ~(size_t)255;
  if (p->type == FL_FORCE_MANYBODY) fl_tree_carve(&p->tb, base, n, s->ndim);
  if (p->type == FL_FORCE_COLLIDE) fl_grid_carve(&p->gb, base, n);
  FL_CK(s, p->red.alloc(sizeof(FlReduce)));
  FL_CK(s, p->cube.alloc(64));
  p->alloc_n = s->n;
  return FL_OK;
}

int32_t update_pass(fl_sim* s, Pass* p, const fl_force_desc* d) {
  const bool changed = p->fresh || d->version != p->version;
  p->d = *d;
  p->d.node_a = p->d.node_b = nullptr;
  p->d.source = p->d.target = nullptr;
  p->d.link_distance = p->d.link_strength = p->d.link_bias = nullptr;
  if (d->iterations < 0) return fail(s, FL_E_ARG, "iterations must be >= 0");
  if (!p->red.p) FL_CK(s, p->red.alloc(sizeof(FlReduce)));  // every pass may reduce
  if (!p->cube.p) FL_CK(s, p->cube.alloc(64));
  if (!changed) return FL_OK;
  int32_t rc = FL_OK;
  switch (d->type) {
    case FL_FORCE_MANYBODY: {
      rc = upload_nodes(s, p->a, d->node_a, -30.f, true);
      bool neg = !d->node_a, pos = false;
      double smax = d->node_a ? 0.0 : 30.0;
      if (d->node_a)
        for (int32_t i = 0; i < s->n; ++i) {
          const float v = d->node_a[i];
          if (!std::isfinite(v)) continue;
          neg = neg || v < 0.f, pos = pos || v > 0.f;
          smax = std::max(smax, (double)std::fabs(v));
        }
      p->mixed = neg && pos;
      p->sign = neg ? -1.f : 1.f;
      // the largest point weight |s| c^leafDepth: c < 1 in 3D, 1 in 2D, sqrt(2) in 1D
      p->fx_exp = fl_fixed_exponent(s->n, smax * (s->ndim == 1 ? 8192.0 : 1.0));
      break;
    }
    case FL_FORCE_LINK:
      rc = upload_links(s, p, d);
      break;
    case FL_FORCE_COLLIDE: {
      rc = upload_nodes(s, p->a, d->node_a, 1.f, true);
      float rmax = 0.f;
      if (d->node_a)
        for (int32_t i = 0; i < s->n; ++i)
          if (std::isfinite(d->node_a[i]) && d->node_a[i] > rmax) rmax = d->node_a[i];
      p->rmax = d->node_a ? rmax : (s->n ? 1.f : 0.f);
      break;
    }
    case FL_FORCE_CENTER:
      break;
    case FL_FORCE_RADIAL:
    case FL_FORCE_POSITION:
      rc = upload_nodes(s, p->a, d->node_a, 0.f, false);
      if (rc == FL_OK) rc = upload_nodes(s, p->b, d->node_b, 0.1f, true);
      break;
    default:
      return fail(s, FL_E_UNSUPPORTED, "force type " + std::to_string(d->type) + " has no GPU pass");
  }
  if (rc != FL_OK) return rc;
  if ((p->type == FL_FORCE_MANYBODY || p->type == FL_FORCE_COLLIDE) && s->n > 0) {
    rc = ensure_scratch(s, p);
    if (rc != FL_OK) return rc;
  }
  p->fresh = false;
  p->version = d->version;
  return FL_OK;
}

bool is_tree(const Pass* p) {
  return p->type == FL_FORCE_MANYBODY && p->d.theta2 > kExactTheta2;
}

// ---------------------------------------------------------------- the tick

// The many-body tree of pass p from the current positions (box: their bounding box, or null to
// reduce it here), on stream st. The sort's histograms, tickets and look-back words are zero
// before the sort (zeroed with the scratch, then after every sort, on the tree's shorter branch,
// off the critical path); `zero` (may be null), a reduction record the tick's integrate fills
// later, is zeroed on that branch too.
void encode_tree(fl_sim* s, Pass* p, const FlReduce* box, cudaStream_t st, FlReduce* zero = nullptr) {
  const int n = s->n;
  FlTreeBufs* t = &p->tb;
  const float* strength = p->a.as<float>();
  const int lo_bit = 64 - t->bits, lo_sort = fl_sort_split(lo_bit, s->sort_passes);
  if (!box) {
    Scope sc(s, G_REDUCE, st);
    cudaMemsetAsync(p->red.p, 0, sizeof(FlReduce), st);
    fl_launch_reduce(s->pos.as<float4>(), n, s->ndim, 1, 0, p->red.as<FlReduce>(), st);
    ++s->launches;
    box = p->red.as<FlReduce>();
  }
  // a small layout's keys are sorted in one launch (unless digit passes were asked for), so
  // the keys need no digit histograms (lo_bit 64: none)
  const bool by_rank = n <= kSortRankMax && s->sort_passes == 0;
  const int passes = (64 - lo_sort + 7) / 8;
  auto clean = [&](cudaStream_t cs) {  // what the next sort and the integrate want at zero
    if (!by_rank) fl_sort_reset(&p->sb, n, passes, cs);
    if (zero) cudaMemsetAsync(zero, 0, sizeof(FlReduce), cs);
  };
  {
    Scope sc(s, G_MORTON, st);
    fl_launch_morton(s->pos.as<float4>(), n, s->ndim, box, p->sb.keys[0], p->sb.vals[0],
                     by_rank ? nullptr : p->sb.hist, by_rank ? 64 : lo_sort, p->cube.as<float>(),
                     st);
    ++s->launches;
  }
  int r;
  {
    Scope sc(s, G_SORT, st);
    if (by_rank) {
      r = fl_sort_rank(&p->sb, n, st, &s->launches);
    } else {
      p->sb.test_spins = s->test_lookback;
      r = fl_sort_passes(&p->sb, n, lo_sort, s->errw.as<uint32_t>(), st, &s->launches);
      r = fl_sort_runfix(&p->sb, n, lo_bit, lo_sort, r, st, &s->launches);
    }
    p->sorted_in = r;
  }
  if (!(s->aux2 && !s->profiling)) clean(st);
  // the closed form (exact fixed-point sums) when the strengths share one sign, unless a
  // recursion was asked for
  const bool closed = !p->mixed && s->cell_sums == FL_CELLS_AUTO;
  const int fp64_depth = s->cell_sums == FL_CELLS_FP32 ? 0 : kRecursionFp64Depth;
  if (s->aux2 && !s->profiling) {
    // the internal nodes and the heads' octant masks on the third stream, beside the points
    cudaEventRecord(s->ev_fork2, st);
    cudaStreamWaitEvent(s->aux2, s->ev_fork2, 0);
    fl_launch_build_nodes(t, p->sb.keys[r], p->sb.vals[r], s->pos.as<float4>(), strength,
                          p->cube.as<float>(), p->fx_exp, s->aux2, &s->launches);
    fl_launch_frontier(t, p->sb.keys[r], s->errw.as<uint32_t>(), s->aux2, &s->launches);
    cudaEventRecord(s->ev_nodes, s->aux2);
    fl_launch_build_points(t, p->sb.keys[r], p->sb.vals[r], s->pos.as<float4>(), strength,
                           closed, p->cube.as<float>(), p->fx_exp, st, &s->launches);
    clean(st);
    cudaStreamWaitEvent(st, s->ev_nodes, 0);
    fl_launch_cells(t, closed, p->sign, p->cube.as<float>(), p->fx_exp, fp64_depth,
                    s->errw.as<uint32_t>(), st, &s->launches);
    return;
  }
  {
    Scope sc(s, G_BUILD, st);
    fl_launch_build(t, p->sb.keys[r], p->sb.vals[r], s->pos.as<float4>(), strength, closed,
                    p->cube.as<float>(), p->fx_exp, st, &s->launches);
  }
  {
    Scope sc(s, G_AGGREGATE, st);
    fl_launch_aggregate(t, p->sb.keys[r], closed, p->sign, p->cube.as<float>(), p->fx_exp,
                        fp64_depth, s->errw.as<uint32_t>(), st, &s->launches);
  }
}

// The many-body force of pass p: its tree (unless built already, on the side stream) and walk.
void encode_manybody(fl_sim* s, Pass* p, float alpha, const FlReduce* box, bool built) {
  const int n = s->n;
  if (n < 2) return;  // a lone node feels nothing
  const float* strength = p->a.as<float>();
  if (!is_tree(p)) {
    Scope sc(s, G_ALLPAIRS);
    const float dmax2 = p->d.distance_max2 > 3e38 ? INFINITY : (float)p->d.distance_max2;
    fl_launch_allpairs(s->pos.as<float4>(), strength, vel_cur(s), n, s->ndim, alpha,
                       (float)p->d.distance_min2, dmax2, s->step, s->seed, s->st, s->tkp);
    ++s->launches;
    return;
  }
  if (built) cudaStreamWaitEvent(s->st, s->ev_tree, 0);
  else encode_tree(s, p, box, s->st);
  {
    Scope sc(s, G_WALK);
    p->tb.walk_blocks = s->walk_blocks;
    fl_launch_walk(&p->tb, p->sb.vals[p->sorted_in], p->cube.as<float>(), vel_cur(s), alpha,
                   p->d.theta2, p->d.distance_min2, p->d.distance_max2, s->step, s->seed,
                   s->errw.as<uint32_t>(),
                   s->prof_level >= 2 ? s->wstats.as<unsigned long long>() : nullptr,
                   s->walk_group, s->st, FlSegs{}, s->tkp);
    ++s->launches;
  }
}

void encode_collide(fl_sim* s, Pass* p) {
  const int n = s->n;
  if (n < 2 || !(p->rmax > 0.f)) return;  // nothing can collide
  const float strength = (float)p->d.strength;
  for (int k = 0; k < p->d.iterations; ++k) {
    if (n < kGridMin) {
      Scope sc(s, G_CALLPAIRS);
      fl_launch_collide_allpairs(s->pos.as<float4>(), vel_cur(s), vel_next(s), p->a.as<float>(),
                                 n, s->ndim, strength, s->step, s->seed, s->st, s->tkp);
      ++s->launches;
    } else {
      FlGridBufs* g = &p->gb;
      const int lo_bit = 64 - g->bits;
      const float inv = 1.f / (2.f * p->rmax * (float)s->collide_cell * 0.01f);
      {
        Scope sc(s, G_CKEYS);
        fl_sort_reset(&p->sb, n, (64 - lo_bit + 7) / 8, s->st);
        fl_launch_grid_keys(s->pos.as<float4>(), vel_cur(s), n, s->ndim, inv, g->bits,
                            p->sb.keys[0], p->sb.vals[0], p->sb.hist, lo_bit, s->st);
        ++s->launches;
      }
      int r;
      {
        Scope sc(s, G_CSORT);
        r = fl_sort_passes(&p->sb, n, lo_bit, s->errw.as<uint32_t>(), s->st, &s->launches);
      }
      {
        Scope sc(s, G_CQUERY);
        fl_launch_grid_query(g, p->sb.keys[r], p->sb.vals[r], s->pos.as<float4>(), vel_cur(s),
                             vel_next(s), p->a.as<float>(), s->ndim, inv, strength, s->step,
                             s->seed, s->st, &s->launches, s->tkp);
      }
    }
    s->cur = 1 - s->cur;
  }
}

void encode_tick(fl_sim* s, float alpha, float decay) {
  const int n = s->n;
  auto& plan = s->plan;
  const int np = (int)plan.size();
  // the centre force, when last, is fused into integrate; its mean is of the positions at the
  // start of the tick (no force before it moves positions, only velocities)
  int centers = 0;
  for (auto& p : plan) centers += p->type == FL_FORCE_CENTER;
  const bool fuse_center = np > 0 && plan[np - 1]->type == FL_FORCE_CENTER && centers == 1;
  // a tree before any centre force reads the positions of the start of the tick too
  bool tree_at_start = false;
  for (auto& p : plan) {
    if (p->type == FL_FORCE_CENTER) break;
    if (is_tree(p.get()) && n >= 2) tree_at_start = true;
  }
  const bool pre = fuse_center || tree_at_start;
  if (pre && !s->pre_valid) {  // else the last tick's integrate reduced these positions
    Scope sc(s, G_REDUCE);
    cudaMemsetAsync(red_of(s), 0, sizeof(FlReduce), s->st);
    fl_launch_reduce(s->pos.as<float4>(), n, s->ndim, tree_at_start, fuse_center, red_of(s),
                     s->st);
    ++s->launches;
  }
  // the first tree before any centre force is built from the tick's starting positions, which
  // nothing changes until then: on the side stream, overlapping with the forces before it
  int early = -1;
  if (tree_at_start && s->aux)
    for (int k = 0; k < np; ++k) {
      if (plan[k]->type == FL_FORCE_CENTER) break;
      if (is_tree(plan[k].get())) {
        early = k;
        break;
      }
    }
  // the record the integrate reduces the new positions into (zeroed beside the early tree)
  FlReduce* next = pre ? s->reds[1 - s->red_cur].as<FlReduce>() : nullptr;
  bool next_zeroed = false;
  if (early >= 0) {
    cudaEventRecord(s->ev_fork, s->st);
    cudaStreamWaitEvent(s->aux, s->ev_fork, 0);
    encode_tree(s, plan[early].get(), red_of(s), s->aux, next);
    next_zeroed = next != nullptr;
    cudaEventRecord(s->ev_tree, s->aux);
  }
  bool before_center = true;
  for (int k = 0; k < np; ++k) {
    Pass* p = plan[k].get();
    switch (p->type) {
      case FL_FORCE_MANYBODY:
        encode_manybody(s, p, alpha, before_center && tree_at_start ? red_of(s) : nullptr,
                        k == early);
        break;
      case FL_FORCE_LINK:
        if (p->m == 0) break;
        for (int it = 0; it < p->d.iterations; ++it) {
          Scope sc(s, G_LINK);
          FlLinkCsr csr{p->row.as<int32_t>(), p->entry.as<float4>(), p->code.as<uint32_t>()};
          // the tick's first pass reads the snapshot the last integrate wrote (or makes it)
          const bool snapped = k == 0 && it == 0;
          if (snapped && !s->snap_valid) {
            fl_launch_snapshot(s->pos.as<float4>(), vel_cur(s), s->snap.as<float4>(), n, s->st);
            ++s->launches;
          }
          fl_launch_link(s->pos.as<float4>(), vel_cur(s), vel_next(s), csr, n, s->ndim, alpha,
                         s->step, s->seed, s->st, nullptr, nullptr, s->tkp,
                         snapped ? s->snap.as<float4>() : nullptr);
          ++s->launches;
          s->cur = 1 - s->cur;
        }
        break;
      case FL_FORCE_COLLIDE:
        encode_collide(s, p);
        break;
      case FL_FORCE_CENTER:
        before_center = false;
        if (fuse_center && k == np - 1) break;
        {
          Scope sc(s, G_CENTER);
          cudaMemsetAsync(p->red.p, 0, sizeof(FlReduce), s->st);
          fl_launch_reduce(s->pos.as<float4>(), n, s->ndim, 0, 1, p->red.as<FlReduce>(), s->st);
          fl_launch_center_apply(s->pos.as<float4>(), n, s->ndim, p->red.as<FlReduce>(), p->d.x,
                                 p->d.y, p->d.z, p->d.strength, s->st);
          s->launches += 2;
        }
        break;
      case FL_FORCE_RADIAL: {
        Scope sc(s, G_RADIAL);
        fl_launch_radial(s->pos.as<float4>(), vel_cur(s), p->a.as<float>(), p->b.as<float>(), n,
                         s->ndim, (float)p->d.x, (float)p->d.y, (float)p->d.z, alpha, s->st, s->tkp);
        ++s->launches;
        break;
      }
      case FL_FORCE_POSITION:
        if (p->d.axis < 0 || p->d.axis >= s->ndim) break;  // forceZ in 2D: nothing to act on
        {
          Scope sc(s, G_POSITION);
          fl_launch_position(s->pos.as<float4>(), vel_cur(s), p->a.as<float>(), p->b.as<float>(),
                             n, p->d.axis, alpha, s->st, s->tkp);
          ++s->launches;
        }
        break;
    }
  }
  {
    Scope sc(s, G_INTEGRATE);
    const Pass* c = fuse_center ? plan[np - 1].get() : nullptr;
    // the next tick needs the same reduction of the positions this integrate writes
    if (next && !next_zeroed) cudaMemsetAsync(next, 0, sizeof(FlReduce), s->st);
    // the next tick's link snapshot, when a link is its first pass
    const bool snap = np > 0 && plan[0]->type == FL_FORCE_LINK && plan[0]->m > 0;
    fl_launch_integrate(s->pos.as<float4>(), vel_cur(s), s->fix.as<float4>(),
                        s->mask.as<uint32_t>(), n, s->ndim, decay, c ? red_of(s) : nullptr,
                        c ? c->d.x : 0, c ? c->d.y : 0, c ? c->d.z : 0, c ? c->d.strength : 0,
                        s->st, nullptr, nullptr, s->tkp, next, tree_at_start, fuse_center,
                        snap ? s->snap.as<float4>() : nullptr);
    ++s->launches;
    if (next) s->red_cur = 1 - s->red_cur;
    s->pre_valid = next != nullptr;
    s->snap_valid = snap;
  }
}

// Captured tick blocks depend on the passes' buffers and scalars: forget them on any change.
void clear_blocks(fl_sim* s) {
  for (auto& b : s->blocks)
    if (b.captured) cudaGraphExecDestroy(b.exec);
  s->blocks.clear();
}

// What a captured block bakes in: every pass's identity, version, scalars and buffers.
std::vector<double> plan_signature(const fl_sim* s) {
  std::vector<double> v;
  for (auto& p : s->plan) {
    const fl_force_desc& d = p->d;
    const double f[] = {(double)p->type, (double)p->key, (double)p->version, (double)d.iterations,
                        (double)d.axis, d.distance_min2, d.distance_max2, d.theta2, d.strength,
                        d.x, d.y, d.z, (double)p->m, (double)p->rmax, (double)p->alloc_n,
                        (double)(uintptr_t)p->a.p, (double)(uintptr_t)p->b.p,
                        (double)(uintptr_t)p->row.p, (double)(uintptr_t)p->scratch.p};
    v.insert(v.end(), f, f + sizeof f / sizeof f[0]);
  }
  return v;
}

int32_t check_sim(fl_sim* s) {
  if (!s) return FL_E_ARG;
  cudaError_t e = cudaSetDevice(s->device);
  if (e != cudaSuccess) return cuda_fail(s, e, "cudaSetDevice");
  return FL_OK;
}

int32_t collect_errors(fl_sim* s) {
  uint32_t w = 0;
  FL_CK(s, cudaMemcpy(&w, s->errw.p, 4, cudaMemcpyDeviceToHost));
  if (w) {
    FL_CK(s, cudaMemset(s->errw.p, 0, 4));
    if (w & FL_ERR_LOOKBACK) return fail(s, FL_E_TIMEOUT, "a device-side look-back wait gave up");
    if (w & FL_ERR_STACK) return fail(s, FL_E_OVERFLOW, "the tree walk ran out of stack");
    return fail(s, FL_E_OVERFLOW, "the tree aggregation found a malformed tree");
  }
  return FL_OK;
}

}  // namespace

// The message fl_last_error(NULL) returns, set by entry points that take no simulation.
void fl_set_sim_free_error(const std::string& msg) { g_create_error = msg; }

extern "C" {

int32_t fl_create(int32_t device, fl_sim** out) {
  if (!out) return fail(nullptr, FL_E_ARG, "out is NULL");
  *out = nullptr;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    cudaGetLastError();
    return fail(nullptr, FL_E_DEVICE,
                std::string("no CUDA device: ") + (e != cudaSuccess ? cudaGetErrorString(e) : "0 devices"));
  }
  if (device < 0 || device >= count) return fail(nullptr, FL_E_ARG, "device ordinal out of range");
  std::unique_ptr<fl_sim> s(new fl_sim());
  s->device = device;
  e = cudaSetDevice(device);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaSetDevice");
  e = cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "cudaStreamCreate");
  if (cudaStreamCreateWithFlags(&s->aux, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&s->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&s->ev_tree, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();  // no side stream: every pass runs on the main one
    if (s->aux) cudaStreamDestroy(s->aux);
    s->aux = nullptr;
  }
  if (cudaStreamCreateWithFlags(&s->aux2, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&s->ev_fork2, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&s->ev_nodes, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();  // no third stream: the tree's halves run one after the other
    if (s->aux2) cudaStreamDestroy(s->aux2);
    s->aux2 = nullptr;
  }
  for (auto& r : s->reds)
    if ((e = r.alloc(sizeof(FlReduce))) != cudaSuccess) return cuda_fail(nullptr, e, "cudaMalloc");
  if ((e = s->errw.alloc(256)) != cudaSuccess) return cuda_fail(nullptr, e, "cudaMalloc");
  if ((e = cudaMemset(s->errw.p, 0, 256)) != cudaSuccess) return cuda_fail(nullptr, e, "cudaMemset");
  *out = s.release();
  return FL_OK;
}

int32_t fl_destroy(fl_sim* s) {
  if (!s) return FL_OK;
  cudaSetDevice(s->device);
  cudaStreamSynchronize(s->st);
  for (auto& r : s->prof_pending) cudaEventDestroy(r.a), cudaEventDestroy(r.b);
  for (auto e : s->ev_pool) cudaEventDestroy(e);
  if (s->aux) cudaStreamSynchronize(s->aux);
  if (s->aux2) cudaStreamSynchronize(s->aux2);
  clear_blocks(s);
  s->plan.clear();
  cudaStream_t st = s->st, aux = s->aux, aux2 = s->aux2;
  if (s->ev_fork) cudaEventDestroy(s->ev_fork);
  if (s->ev_tree) cudaEventDestroy(s->ev_tree);
  if (s->ev_fork2) cudaEventDestroy(s->ev_fork2);
  if (s->ev_nodes) cudaEventDestroy(s->ev_nodes);
  delete s;  // frees the device buffers
  if (st) cudaStreamDestroy(st);
  if (aux) cudaStreamDestroy(aux);
  if (aux2) cudaStreamDestroy(aux2);
  return FL_OK;
}

const char* fl_last_error(const fl_sim* s) { return s ? s->err.c_str() : g_create_error.c_str(); }

int32_t fl_fits(fl_sim* s, int64_t count, int32_t* fits) {
  int32_t rc = check_sim(s);
  if (rc) return rc;
  if (!fits || count < 0) return fail(s, FL_E_ARG, "bad arguments");
  size_t freeb = 0, total = 0;
  FL_CK(s, cudaMemGetInfo(&freeb, &total));
  // state 16 * 4 + 4 B, tree and sort ~ 200 B, per node, with a margin
  const double need = (double)count * 300.0;
  *fits = count <= kMaxNodes && need < 0.9 * (double)(freeb + s->pos.bytes * 8);
  return FL_OK;
}

int32_t fl_set_nodes(fl_sim* s, int32_t n, int32_t ndim, const float* pos4, const float* vel4,
                     const float* fix4, const uint32_t* mask) {
  int32_t rc = check_sim(s);
  if (rc) return rc;
  if (n < 0 || n > kMaxNodes) return fail(s, FL_E_ARG, "node count out of range");
  clear_blocks(s);
  if (n > 0 && !pos4) return fail(s, FL_E_ARG, "positions are NULL");
  FL_CK(s, cudaStreamSynchronize(s->st));
  s->plan.clear();
  s->n = n;
  s->ndim = std::min(3, std::max(1, (int)ndim));
  s->cur = 0;
  s->pre_valid = s->snap_valid = false;
  const size_t v4 = 16 * (size_t)std::max(n, 1);
  FL_CK(s, s->pos.alloc(v4));
  FL_CK(s, s->vel[0].alloc(v4));
  FL_CK(s, s->vel[1].alloc(v4));
  FL_CK(s, s->snap.alloc(v4));
  FL_CK(s, s->fix.alloc(v4));
  FL_CK(s, s->mask.alloc(4 * (size_t)std::max(n, 1)));
  FL_CK(s, s->pack.alloc(8 * (size_t)s->ndim * (size_t)std::max(n, 1)));
  if (n) {
    FL_CK(s, cudaMemcpy(s->pos.p, pos4, 16 * (size_t)n, cudaMemcpyHostToDevice));
    if (vel4) FL_CK(s, cudaMemcpy(s->vel[0].p, vel4, 16 * (size_t)n, cudaMemcpyHostToDevice));
    else FL_CK(s, cudaMemset(s->vel[0].p, 0, 16 * (size_t)n));
    if (fix4) FL_CK(s, cudaMemcpy(s->fix.p, fix4, 16 * (size_t)n, cudaMemcpyHostToDevice));
    else FL_CK(s, cudaMemset(s->fix.p, 0, 16 * (size_t)n));
    if (mask) FL_CK(s, cudaMemcpy(s->mask.p, mask, 4 * (size_t)n, cudaMemcpyHostToDevice));
    else FL_CK(s, cudaMemset(s->mask.p, 0, 4 * (size_t)n));
  }
  return FL_OK;
}

int32_t fl_upload_all(fl_sim* s, const float* pos4, const float* vel4, const float* fix4,
                      const uint32_t* mask) {
  int32_t rc = check_sim(s);
  if (rc) return rc;
  if (s->n > 0 && !pos4) return fail(s, FL_E_ARG, "positions are NULL");
  FL_CK(s, cudaStreamSynchronize(s->st));
  // the state starts over in the first velocity and reduction buffers, as after fl_set_nodes,
  // so that a tick block captured from that start replays from this one
  s->cur = 0;
  s->red_cur = 0;
  s->pre_valid = s->snap_valid = false;
  const size_t b4 = 16 * (size_t)s->n;
  if (s->n) {
    FL_CK(s, cudaMemcpyAsync(s->pos.p, pos4, b4, cudaMemcpyHostToDevice, s->st));
    if (vel4) FL_CK(s, cudaMemcpyAsync(s->vel[0].p, vel4, b4, cudaMemcpyHostToDevice, s->st));
    else FL_CK(s, cudaMemsetAsync(s->vel[0].p, 0, b4, s->st));
    if (fix4) FL_CK(s, cudaMemcpyAsync(s->fix.p, fix4, b4, cudaMemcpyHostToDevice, s->st));
    else FL_CK(s, cudaMemsetAsync(s->fix.p, 0, b4, s->st));
    if (mask)
      FL_CK(s, cudaMemcpyAsync(s->mask.p, mask, 4 * (size_t)s->n, cudaMemcpyHostToDevice, s->st));
    else FL_CK(s, cudaMemsetAsync(s->mask.p, 0, 4 * (size_t)s->n, s->st));
  }
  FL_CK(s, cudaStreamSynchronize(s->st));
  return FL_OK;
}

int32_t fl_update_positions(fl_sim* s, int32_t first, int32_t count, const float* pos4) {
  int32_t rc = check_sim(s);
  if (rc) return rc;
  if (first < 0 || count < 0 || first + (int64_t)count > s->n || (count && !pos4))
    return fail(s, FL_E_ARG, "range out of bounds");
  if (count)
    FL_CK(s, cudaMemcpyAsync(s->pos.as<float4>() + first, pos4, 16 * (size_t)count,
                             cudaMemcpyHostToDevice, s->st));
  s->pre_valid = s->snap_valid = false;  // the next tick reduces the positions afresh (count 0: written on the device)
  FL_CK(s, cudaStreamSynchronize(s->st));
  return FL_OK;
}

// The packed upload, queued on the stream; `wait` makes the call return after it has run.
static int32_t update_packed(fl_sim* s, int32_t first, int32_t count, const float* pos, bool wait) {
  int32_t rc = check_sim(s);
  if (rc) return rc;
  if (first < 0 || count < 0 || first + (int64_t)count > s->n || (count && !pos))
    return fail(s, FL_E_ARG, "range out of bounds");
  if (count) {
    FL_CK(s, cudaMemcpyAsync(s->pack.p, pos, 4 * (size_t)s->ndim * count, cudaMemcpyHostToDevice,
                             s->st));
    fl_launch_unpack(s->pack.as<float>(), count, s->ndim, s->pos.as<float4>() + first, s->st);
    ++s->launches;
  }
  s->pre_valid = s->snap_valid = false;
  if (wait) FL_CK(s, cudaStreamSynchronize(s->st));
  return FL_OK;
}

int32_t fl_update_positions_packed(fl_sim* s, int32_t first, int32_t count, const float* pos) {
  return update_packed(s, first, count, pos, true);
}

int32_t fl_update_positions_packed_async(fl_sim* s, int32_t first, int32_t count,
                                         const float* pos) {
  return update_packed(s, first, count, pos, false);
}

int32_t fl_update_velocities(fl_sim* s, int32_t first, int32_t count, const float* vel4) {
  int32_t rc = check_sim(s);
  if (rc) return rc;
  if (first < 0 || count < 0 || first + (int64_t)count > s->n || (count && !vel4))
    return fail(s, FL_E_ARG, "range out of bounds");
  if (count)
    FL_CK(s, cudaMemcpyAsync(vel_cur(s) + first, vel4, 16 * (size_t)count, cudaMemcpyHostToDevice,
                             s->st));
  FL_CK(s, cudaStreamSynchronize(s->st));
  s->snap_valid = false;  // the link's snapshot holds p + v (count 0: written on the device)
  return FL_OK;
}

int32_t fl_update_pins(fl_sim* s, int32_t first, int32_t count, const float* fix4,
                       const uint32_t* mask) {
  int32_t rc = check_sim(s);
  if (rc) return rc;
  if (first < 0 || count < 0 || first + (int64_t)count > s->n || (count && (!fix4 || !mask)))
    return fail(s, FL_E_ARG, "range out of bounds");
  if (count) {
    FL_CK(s, cudaMemcpyAsync(s->fix.as<float4>() + first, fix4, 16 * (size_t)count,
                             cudaMemcpyHostToDevice, s->st));
    FL_CK(s, cudaMemcpyAsync(s->mask.as<uint32_t>() + first, mask, 4 * (size_t)count,
                             cudaMemcpyHostToDevice, s->st));
  }
  FL_CK(s, cudaStreamSynchronize(s->st));
  return FL_OK;
}

int32_t fl_set_forces(fl_sim* s, int32_t count, const fl_force_desc* descs) {
  int32_t rc = check_sim(s);
  if (rc) return rc;
  if (count < 0 || (count && !descs)) return fail(s, FL_E_ARG, "bad force list");
  for (int32_t i = 0; i < count; ++i)
    if (descs[i].type < FL_FORCE_MANYBODY || descs[i].type > FL_FORCE_POSITION)
      return fail(s, FL_E_UNSUPPORTED, "force " + std::to_string(i) + " (type " +
                                           std::to_string(descs[i].type) + ") has no GPU pass");
  // the same passes with the same per-node arrays: only scalars change, nothing in flight is
  // touched, so no wait is needed; otherwise passes may be replaced below
  bool same = count == (int32_t)s->plan.size();
  for (int32_t i = 0; same && i < count; ++i) {
    const Pass* p = s->plan[i].get();
    same = p->key == descs[i].key && p->type == descs[i].type && !p->fresh &&
           p->version == descs[i].version;
  }
  if (!same) FL_CK(s, cudaStreamSynchronize(s->st));
  std::vector<std::unique_ptr<Pass>> old = std::move(s->plan);
  std::vector<std::unique_ptr<Pass>> next;
  for (int32_t i = 0; i < count; ++i) {
    std::unique_ptr<Pass> p;
    for (auto& o : old)
      if (o && o->key == descs[i].key && o->type == descs[i].type) {
        p = std::move(o);
        break;
      }
    if (!p) {
      p.reset(new Pass());
      p->type = descs[i].type;
      p->key = descs[i].key;
    }
    rc = update_pass(s, p.get(), &descs[i]);
    if (rc != FL_OK) {
      s->plan.clear();
      return rc;
    }
    next.push_back(std::move(p));
  }
  s->plan = std::move(next);
  std::vector<double> sig = plan_signature(s);
  if (sig != s->plan_sig) {
    clear_blocks(s);
    s->plan_sig = std::move(sig);
    s->pre_valid = s->snap_valid = false;  // the reduction the new passes want may differ
  }
  return FL_OK;
}

int32_t fl_set_seed(fl_sim* s, uint32_t seed) {
  int32_t rc = check_sim(s);
  if (rc) return rc;
  s->seed = seed;
  return FL_OK;
}

int32_t fl_enqueue(fl_sim* s, const double* alphas, int32_t count, double decay) {
  int32_t rc = check_sim(s);
  if (rc) return rc;
  if (count < 0 || (count && !alphas)) return fail(s, FL_E_ARG, "bad alphas");
  if (s->n == 0 || count == 0) return FL_OK;
  // the ticks' alphas, steps and seed, copied on the stream (after every tick already queued)
  if (count > s->tick_cap) {
    FL_CK(s, cudaStreamSynchronize(s->st));
    clear_blocks(s);  // captured blocks point into the old buffer
    FL_CK(s, s->tickbuf.alloc(sizeof(FlTick) * (size_t)count));
    s->tick_cap = count;
  }
  s->htick.resize(count);
  for (int32_t k = 0; k < count; ++k)
    s->htick[k] = FlTick{(float)alphas[k], (float)decay, s->step + (uint32_t)k, s->seed};
  FL_CK(s, cudaMemcpyAsync(s->tickbuf.p, s->htick.data(), sizeof(FlTick) * (size_t)count,
                           cudaMemcpyHostToDevice, s->st));
  const FlTick* tk = s->tickbuf.as<FlTick>();
  auto encode = [&]() {
    for (int32_t k = 0; k < count; ++k) {
      s->tkp = tk + k;
      encode_tick(s, (float)alphas[k], (float)decay);
    }
    s->tkp = nullptr;
  };
  // a block of ticks seen before (same length, same velocity buffer to start from) runs as one
  // CUDA graph: captured the second time it is seen, replayed from then on
  fl_sim::Block* b = nullptr;
  if (s->use_graphs && !s->profiling)
    for (auto& x : s->blocks)
      if (x.count == count && x.cur_in == s->cur && x.red_in == s->red_cur &&
          x.pre_in == s->pre_valid && x.snap_in == s->snap_valid)
        b = &x;
  if (b && b->captured) {
    FL_CK(s, cudaGraphLaunch(b->exec, s->st));
    s->cur = b->cur_out, s->red_cur = b->red_out, s->pre_valid = b->pre_out;
    s->snap_valid = b->snap_out;
    s->launches += b->launches;
  } else if (b) {
    const int cur0 = s->cur, red0 = s->red_cur;
    const bool pre0 = s->pre_valid, snap0 = s->snap_valid;
    const int64_t l0 = s->launches;
    cudaGraph_t g = nullptr;
    bool ok = cudaStreamBeginCapture(s->st, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
      encode();
      ok = cudaStreamEndCapture(s->st, &g) == cudaSuccess && g;
    }
    if (ok) {
      ok = cudaGraphInstantiate(&b->exec, g, 0) == cudaSuccess;
      cudaGraphDestroy(g);
    }
    if (ok) {
      b->captured = true;
      FL_CK(s, cudaGraphLaunch(b->exec, s->st));
    } else {  // graphs unavailable: launch the ticks directly from now on
      cudaGetLastError();
      if (g) cudaGraphDestroy(g);
      s->use_graphs = false;
      s->cur = cur0, s->red_cur = red0, s->pre_valid = pre0, s->snap_valid = snap0;
      s->launches = l0;
      encode();
    }
  } else {
    const int cur0 = s->cur, red0 = s->red_cur;
    const bool pre0 = s->pre_valid, snap0 = s->snap_valid;
    const int64_t l0 = s->launches;
    encode();
    if (s->use_graphs && !s->profiling) {
      if (s->blocks.size() >= 8) {
        if (s->blocks.front().captured) cudaGraphExecDestroy(s->blocks.front().exec);
        s->blocks.erase(s->blocks.begin());
      }
      s->blocks.push_back(fl_sim::Block{count, cur0, s->cur, red0, s->red_cur, pre0, s->pre_valid,
                                        snap0, s->snap_valid, s->launches - l0, false, nullptr});
    }
  }
  s->step += (uint32_t)count;
  s->ticks += count;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(s, e, "kernel launch");
  return FL_OK;
}

int32_t fl_idle(fl_sim* s) {
  int32_t rc = check_sim(s);
  if (rc) return rc;
  FL_CK(s, cudaStreamSynchronize(s->st));
  if (s->profiling) drain_profile(s);
  return collect_errors(s);
}

int32_t fl_sync(fl_sim* s, float* pos4_out, float* vel4_out) {
  int32_t rc = check_sim(s);
  if (rc) return rc;
  if (s->n && pos4_out)
    FL_CK(s, cudaMemcpyAsync(pos4_out, s->pos.p, 16 * (size_t)s->n, cudaMemcpyDeviceToHost, s->st));
  if (s->n && vel4_out)
    FL_CK(s, cudaMemcpyAsync(vel4_out, vel_cur(s), 16 * (size_t)s->n, cudaMemcpyDeviceToHost, s->st));
  FL_CK(s, cudaStreamSynchronize(s->st));
  if (s->profiling) drain_profile(s);
  return collect_errors(s);
}

int32_t fl_sync_packed(fl_sim* s, float* pos_out, float* vel_out) {
  int32_t rc = check_sim(s);
  if (rc) return rc;
  if (s->n && (pos_out || vel_out)) {
    const size_t m = (size_t)s->n * s->ndim;
    fl_launch_pack(pos_out ? s->pos.as<float4>() : nullptr, vel_out ? vel_cur(s) : nullptr, s->n,
                   s->ndim, s->pack.as<float>(), s->st);
    ++s->launches;
    if (pos_out)
      FL_CK(s, cudaMemcpyAsync(pos_out, s->pack.p, 4 * m, cudaMemcpyDeviceToHost, s->st));
    if (vel_out)
      FL_CK(s, cudaMemcpyAsync(vel_out, s->pack.as<float>() + m, 4 * m, cudaMemcpyDeviceToHost,
                               s->st));
  }
  FL_CK(s, cudaStreamSynchronize(s->st));
  if (s->profiling) drain_profile(s);
  return collect_errors(s);
}

int32_t fl_busy(fl_sim* s, int32_t* busy) {
  int32_t rc = check_sim(s);
  if (rc) return rc;
  if (!busy) return fail(s, FL_E_ARG, "busy is NULL");
  cudaError_t e = cudaStreamQuery(s->st);
  if (e != cudaSuccess && e != cudaErrorNotReady) return cuda_fail(s, e, "cudaStreamQuery");
  *busy = e == cudaErrorNotReady;
  return FL_OK;
}

int32_t fl_buffers(fl_sim* s, fl_buffer_info* out) {
  int32_t rc = check_sim(s);
  if (rc) return rc;
  if (!out) return fail(s, FL_E_ARG, "out is NULL");
  out->positions = s->pos.p;
  out->velocities = vel_cur(s);
  out->count = s->n;
  out->stride = 16;
  return FL_OK;
}

int32_t fl_set_tuning(fl_sim* s, int32_t key, int32_t value) {
  int32_t rc = check_sim(s);
  if (rc) return rc;
  clear_blocks(s);
  switch (key) {
    case FL_TUNE_WALK_GROUP:
      if (value != 0 && value != 1 && value != 16 && value != 32)
        return fail(s, FL_E_ARG, "walk group must be 0, 1, 16 or 32");
      s->walk_group = value;
      return FL_OK;
    case FL_TUNE_CELL_SUMS:
      if (value != FL_CELLS_AUTO && value != FL_CELLS_FP64_TOP && value != FL_CELLS_FP32)
        return fail(s, FL_E_ARG, "cell sums must be FL_CELLS_AUTO, FL_CELLS_FP64_TOP or FL_CELLS_FP32");
      s->cell_sums = value;
      return FL_OK;
    case FL_TUNE_GRAPHS:
      if (value != 0 && value != 1) return fail(s, FL_E_ARG, "graphs must be 0 or 1");
      s->use_graphs = value != 0;
      return FL_OK;
    case FL_TUNE_SORT_PASSES:
      if (value < 0 || value > 8) return fail(s, FL_E_ARG, "sort passes must be 0..8");
      s->sort_passes = value;
      return FL_OK;
    case FL_TUNE_WALK_BLOCKS:
      if (value < 0 || value > 32) return fail(s, FL_E_ARG, "walk blocks per SM must be 0..32");
      s->walk_blocks = value;
      return FL_OK;
    case FL_TUNE_COLLIDE_CELL:
      if (value < 100 || value > 1000) return fail(s, FL_E_ARG, "collide cell must be 100..1000 percent");
      s->collide_cell = value;
      return FL_OK;
    case FL_TUNE_TEST_LOOKBACK:
      if (value < 0 || value > 65536) return fail(s, FL_E_ARG, "test look-back polls must be 0..65536");
      s->test_lookback = (uint32_t)value;
      return FL_OK;
    default:
      return fail(s, FL_E_ARG, "unknown tuning key");
  }
}

int32_t fl_autotune(fl_sim* s, int32_t ticks, double alpha, double decay,
                    const char* cache_path, fl_tune_result* out) {
  int32_t rc = check_sim(s);
  if (rc) return rc;
  if (!out) return fail(s, FL_E_ARG, "out is NULL");
  if (ticks < 1) return fail(s, FL_E_ARG, "ticks must be >= 1");
  const int n = s->n;
  bool tree = false, grid = false;
  int key_bits = 0;
  std::string forces;
  for (auto& p : s->plan) {
    forces += std::to_string(p->type);
    if (is_tree(p.get()) && n >= 2) tree = true, key_bits = p->tb.bits, forces += 't';
    if (p->type == FL_FORCE_COLLIDE && n >= kGridMin && p->rmax > 0.f) grid = true, forces += 'g';
    forces += ',';
  }
  std::vector<FlTuneKnob> knobs;
  if (tree) {
    // digit-pass counts that give distinct splits of the key, the default (0) first
    std::vector<int> passes{0};
    const int lo_bit = 64 - key_bits;
    std::vector<int> seen{fl_sort_split(lo_bit, 0)};
    for (int c : {3, 5, 8}) {
      const int lo = fl_sort_split(lo_bit, c);
      if (std::find(seen.begin(), seen.end(), lo) == seen.end()) seen.push_back(lo), passes.push_back(c);
    }
    knobs.push_back({FL_TUNE_SORT_PASSES, "sort_passes", passes, 0});
    // the default by size first, then the other groups
    std::vector<int> groups{0};
    for (int g : {32, 16, 1})
      if (g != fl_walk_group_for(n)) groups.push_back(g);
    knobs.push_back({FL_TUNE_WALK_GROUP, "walk_group", groups, 0});
    knobs.push_back({FL_TUNE_WALK_BLOCKS, "walk_blocks", {0, 8, 6, 4}, 0});
  }
  if (grid) knobs.push_back({FL_TUNE_COLLIDE_CELL, "collide_cell", {100, 150, 200}, 100});
  *out = fl_tune_result{s->walk_group, s->sort_passes, s->walk_blocks, s->collide_cell, 0, 0, 0, 0};
  if (knobs.empty() || n < 2) return FL_OK;  // nothing to choose
  const std::string key = fl_tune_arch() + " sim ndim=" + std::to_string(s->ndim) +
                          " log2n=" + std::to_string((int)std::floor(std::log2((double)n))) +
                          " forces=" + forces + " graphs=" + std::to_string((int)s->use_graphs);
  // the state to come back to
  FL_CK(s, cudaStreamSynchronize(s->st));
  DevMem snap;
  FL_CK(s, snap.alloc(32 * (size_t)n));
  const size_t v4 = 16 * (size_t)n;
  FL_CK(s, cudaMemcpyAsync(snap.p, s->pos.p, v4, cudaMemcpyDeviceToDevice, s->st));
  FL_CK(s, cudaMemcpyAsync(snap.as<char>() + v4, vel_cur(s), v4, cudaMemcpyDeviceToDevice, s->st));
  const uint32_t step0 = s->step;
  const int64_t ticks0 = s->ticks, launches0 = s->launches;
  auto restore = [&]() -> int32_t {
    FL_CK(s, cudaMemcpyAsync(s->pos.p, snap.p, v4, cudaMemcpyDeviceToDevice, s->st));
    FL_CK(s, cudaMemcpyAsync(s->vel[0].p, snap.as<char>() + v4, v4, cudaMemcpyDeviceToDevice, s->st));
    s->cur = 0;
    s->step = step0;
    s->pre_valid = s->snap_valid = false;
    return FL_OK;
  };
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  FL_CK(s, cudaEventCreate(&e0));
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return fail(s, FL_E_DEVICE, "cudaEventCreate");
  }
  const std::vector<double> al((size_t)ticks, alpha);
  // a configuration's time: its block of ticks run three times from the same state (the first
  // direct, the second captured, the third timed: as an application's steady state runs it)
  auto time = [&](double* ms) -> int {
    for (int rep = 0; rep < 3; ++rep) {
      int32_t r = restore();
      if (r) return r;
      if (rep == 2 && cudaEventRecord(e0, s->st) != cudaSuccess) return cuda_fail(s, cudaGetLastError(), "cudaEventRecord");
      if ((r = fl_enqueue(s, al.data(), ticks, decay)) != FL_OK) return r;
      if (rep == 2 && cudaEventRecord(e1, s->st) != cudaSuccess) return cuda_fail(s, cudaGetLastError(), "cudaEventRecord");
    }
    FL_CK(s, cudaEventSynchronize(e1));
    int32_t r = collect_errors(s);
    if (r) return r;
    float t = 0.f;
    FL_CK(s, cudaEventElapsedTime(&t, e0, e1));
    *ms = (double)t / ticks;
    return FL_OK;
  };
  auto set = [&](int k, int v) -> int { return fl_set_tuning(s, k, v); };
  FlTuneOutcome o;
  rc = fl_tune_search(cache_path, key, knobs, set, time, &o);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const int32_t rr = restore();
  if (!rc) rc = rr;
  cudaError_t e = cudaStreamSynchronize(s->st);
  s->ticks = ticks0, s->launches = launches0;
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_fail(s, e, "cudaStreamSynchronize");
  *out = fl_tune_result{s->walk_group, s->sort_passes, s->walk_blocks, s->collide_cell,
                        o.best_ms, o.default_ms, o.candidates, o.cached ? 1 : 0};
  return FL_OK;
}

int32_t fl_stream(fl_sim* s, void** stream) {
  if (!s || !stream) return FL_E_ARG;
  *stream = (void*)s->st;
  return FL_OK;
}

int32_t fl_query(fl_sim* s, int32_t what, int64_t* out) {
  int32_t rc = check_sim(s);
  if (rc) return rc;
  if (!out) return fail(s, FL_E_ARG, "out is NULL");
  switch (what) {
    case FL_Q_LAUNCHES: *out = s->launches; break;
    case FL_Q_TICKS: *out = s->ticks; break;
    case FL_Q_NODES: *out = s->n; break;
    case FL_Q_ERRWORD: {
      uint32_t w = 0;
      FL_CK(s, cudaMemcpy(&w, s->errw.p, 4, cudaMemcpyDeviceToHost));
      *out = w;
      break;
    }
    case FL_Q_DEVICE_BYTES: {
      size_t b = s->pos.bytes + s->vel[0].bytes + s->vel[1].bytes + s->fix.bytes + s->mask.bytes;
      for (auto& p : s->plan)
        b += p->a.bytes + p->b.bytes + p->row.bytes + p->entry.bytes + p->code.bytes + p->scratch.bytes;
      *out = (int64_t)b;
      break;
    }
    case FL_Q_WALK_TESTS:
    case FL_Q_WALK_USEFUL:
    case FL_Q_WALK_MAX_STACK:
    case FL_Q_WALK_OPENS:
    case FL_Q_WALK_APPLIES:
    case FL_Q_WALK_RARE: {
      unsigned long long w[6] = {0, 0, 0, 0, 0, 0};
      if (s->wstats.p) {
        FL_CK(s, cudaStreamSynchronize(s->st));
        FL_CK(s, cudaMemcpy(w, s->wstats.p, sizeof w, cudaMemcpyDeviceToHost));
      }
      *out = (int64_t)w[what - FL_Q_WALK_TESTS];
      break;
    }
    default: return fail(s, FL_E_ARG, "unknown query");
  }
  return FL_OK;
}

int32_t fl_profile(fl_sim* s, int32_t enable) {
  int32_t rc = check_sim(s);
  if (rc) return rc;
  FL_CK(s, cudaStreamSynchronize(s->st));
  drain_profile(s);
  s->profiling = enable != 0;
  s->prof_level = enable;
  for (int g = 0; g < G_COUNT; ++g) s->prof_ms[g] = 0, s->prof_count[g] = 0;
  if (enable >= 2) {
    if (!s->wstats.p) FL_CK(s, s->wstats.alloc(256));
    FL_CK(s, cudaMemset(s->wstats.p, 0, 48));
  }
  return FL_OK;
}

int32_t fl_profile_read(fl_sim* s, int32_t cap, const char** names, double* ms, int64_t* launches,
                        int32_t* count) {
  int32_t rc = check_sim(s);
  if (rc) return rc;
  FL_CK(s, cudaStreamSynchronize(s->st));
  drain_profile(s);
  int32_t k = 0;
  for (int g = 0; g < G_COUNT; ++g) {
    if (!s->prof_count[g]) continue;
    if (k < cap) {
      if (names) names[k] = kGroupNames[g];
      if (ms) ms[k] = s->prof_ms[g];
      if (launches) launches[k] = s->prof_count[g];
    }
    ++k;
  }
  if (count) *count = k;
  return FL_OK;
}

int32_t fl_radix_sort(const uint64_t* keys, const uint32_t* vals, int64_t n, int32_t lo_bit,
                      uint64_t* keys_out, uint32_t* vals_out) {
  if (n < 0 || lo_bit < 0 || lo_bit > 63 || (n && (!keys || !vals || !keys_out || !vals_out)))
    return fail(nullptr, FL_E_ARG, "fl_radix_sort: bad arguments");
  if (n == 0) return FL_OK;
  if (n > (int64_t(1) << 30) - 1) return fail(nullptr, FL_E_ARG, "fl_radix_sort: too many pairs");
  DevMem buf, errw;
  cudaError_t e;
  if ((e = buf.alloc(fl_sort_bytes(n))) != cudaSuccess) return cuda_fail(nullptr, e, "cudaMalloc");
  if ((e = errw.alloc(256)) != cudaSuccess) return cuda_fail(nullptr, e, "cudaMalloc");
  FlSortBufs sb;
  fl_sort_carve(&sb, buf.p, n);
  int64_t launches = 0;
  cudaStream_t st = 0;
  const int passes = (64 - lo_bit + 7) / 8;
  if ((e = cudaMemset(errw.p, 0, 4)) != cudaSuccess) return cuda_fail(nullptr, e, "cudaMemset");
  if ((e = cudaMemcpy(sb.keys[0], keys, 8 * (size_t)n, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(sb.vals[0], vals, 4 * (size_t)n, cudaMemcpyHostToDevice)) != cudaSuccess)
    return cuda_fail(nullptr, e, "cudaMemcpy");
  fl_sort_reset(&sb, n, passes, st);
  fl_sort_histogram(&sb, n, lo_bit, st, &launches);
  const int r = fl_sort_passes(&sb, n, lo_bit, errw.as<uint32_t>(), st, &launches);
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(nullptr, e, "sort launch");
  uint32_t w = 0;
  if ((e = cudaMemcpy(keys_out, sb.keys[r], 8 * (size_t)n, cudaMemcpyDeviceToHost)) != cudaSuccess ||
      (e = cudaMemcpy(vals_out, sb.vals[r], 4 * (size_t)n, cudaMemcpyDeviceToHost)) != cudaSuccess ||
      (e = cudaMemcpy(&w, errw.p, 4, cudaMemcpyDeviceToHost)) != cudaSuccess)
    return cuda_fail(nullptr, e, "cudaMemcpy");
  if (w) return fail(nullptr, FL_E_TIMEOUT, "a device-side look-back wait gave up");
  return FL_OK;
}

int32_t fl_debug_tree(fl_sim* s, int32_t index, uint64_t* keys, uint32_t* perm, uint32_t* left,
                      uint32_t* right, uint8_t* depth, float* cube5) {
  int32_t rc = check_sim(s);
  if (rc) return rc;
  if (index < 0 || index >= (int32_t)s->plan.size()) return fail(s, FL_E_ARG, "no such force");
  Pass* p = s->plan[index].get();
  if (p->type != FL_FORCE_MANYBODY || p->sorted_in < 0 || s->n < 2)
    return fail(s, FL_E_STATE, "no tree was built for this force");
  FL_CK(s, cudaStreamSynchronize(s->st));
  const size_t n = (size_t)s->n, m = n - 1;
  const int r = p->sorted_in;
  if (keys) FL_CK(s, cudaMemcpy(keys, p->sb.keys[r], 8 * n, cudaMemcpyDeviceToHost));
  if (perm) FL_CK(s, cudaMemcpy(perm, p->sb.vals[r], 4 * n, cudaMemcpyDeviceToHost));
  if (left) FL_CK(s, cudaMemcpy(left, p->tb.left, 4 * m, cudaMemcpyDeviceToHost));
  if (right) FL_CK(s, cudaMemcpy(right, p->tb.right, 4 * m, cudaMemcpyDeviceToHost));
  if (depth) FL_CK(s, cudaMemcpy(depth, p->tb.depth, m, cudaMemcpyDeviceToHost));
  if (cube5) FL_CK(s, cudaMemcpy(cube5, p->cube.p, 20, cudaMemcpyDeviceToHost));
  return FL_OK;
}

int32_t fl_debug_links(fl_sim* s, int32_t index, int32_t* row, int32_t* other, uint32_t* code) {
  int32_t rc = check_sim(s);
  if (rc) return rc;
  if (index < 0 || index >= (int32_t)s->plan.size()) return fail(s, FL_E_ARG, "no such force");
  const Pass* p = s->plan[index].get();
  if (p->type != FL_FORCE_LINK || !p->row.p) return fail(s, FL_E_STATE, "force is not a link force");
  FL_CK(s, cudaStreamSynchronize(s->st));
  const size_t e = 2 * (size_t)p->m;
  if (row) FL_CK(s, cudaMemcpy(row, p->row.p, 4 * ((size_t)s->n + 1), cudaMemcpyDeviceToHost));
  if (code && e) FL_CK(s, cudaMemcpy(code, p->code.p, 4 * e, cudaMemcpyDeviceToHost));
  if (other && e)  // the other end's index is the first word of each float4 entry
    FL_CK(s, cudaMemcpy2D(other, 4, p->entry.p, 16, 4, e, cudaMemcpyDeviceToHost));
  return FL_OK;
}

}  // extern "C"
