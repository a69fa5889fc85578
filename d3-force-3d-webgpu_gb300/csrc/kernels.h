// Host-side launchers of the engine's kernels (one translation unit each group).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

// One tick's varying values, which the kernels read from device memory when given (null: the
// values passed as parameters), so that a CUDA graph captured for a block of ticks can be
// replayed with the next block's alphas.
struct FlTick {
  float alpha, decay;
  uint32_t step, seed;
};

// ---------------------------------------------------------------- batches of graphs
// One graph's values for a tick of a batch (device). The first five floats have the layout of a
// single simulation's cube record (origin x, y, z, size, log2 size).
struct FlGraph {
  float origin[3], size, lg;
  float T0;               // size^2 / theta^2: the walk's threshold at depth 0
  float dmin2, dmax2;     // many-body distanceMin^2, distanceMax^2
  float alpha, decay;     // this tick's alpha; velocity multiplier
  float2 shift[3];        // the centre force's shift per axis (hi + lo), 0 without one
  int32_t first, count;   // nodes [first, first + count)
  int32_t frozen;         // 1: the graph sits this tick out (its alpha was given as negative)
  int32_t fx;             // scale exponent of the graph's fixed-point cell sums
  uint32_t tick0;         // the graph's own tick count when the batch started (jiggle steps)
  int32_t citer;          // collide: iterations (0: the graph has no collide force)
  float cinv, cstr;       // collide: 1 / grid cell side (2 x largest radius); strength
  uint32_t pad;
};
// A batch of independent graphs, concatenated: graph g owns nodes [off[g], off[g+1]) and, after
// the tree's sort (by graph, then Morton code), the same range of sorted positions. Kernels
// take it by value; graphs == 0 means a single simulation.
struct FlSegs {
  int graphs;
  const int32_t* off;        // [graphs + 1]
  const uint32_t* gid_node;  // [n] graph of each node
  const uint32_t* gid_pos;   // [n] graph of each sorted position
  const FlGraph* g;          // [graphs]
  // the tree walk's point groups: sorted positions [x, y), up to 32 of one graph each, so that a
  // graph's groups (and so every sum of its walk) are the same whatever else is in the batch
  const uint2* groups;       // [ngroups]
  int ngroups;
};

// A graph's fixed parameters in a batch: many-body theta^2, distanceMin^2, distanceMax^2; the
// centre force's point and strength (0: none); the velocity multiplier (1 - velocityDecay).
struct FlBatchParams {
  double theta2, dmin2, dmax2;
  double cx, cy, cz, cstrength;
  double decay;
  int32_t fx;      // scale exponent of the fixed-point cell sums, from the graph's own size and
                   // strengths (as a lone simulation of that graph chooses it)
  uint32_t tick0;  // the graph's tick count when the batch started
  int32_t citer;   // collide force: iterations (0: none), 1 / cell side, strength
  float cinv, cstr;
};
void fl_launch_breduce(const float4* pos, int n, int ndim, const uint32_t* gid, FlReduce* red,
                       cudaStream_t st);
void fl_launch_bgraph(int graphs, int ndim, const int32_t* off, const FlReduce* red,
                      const FlBatchParams* prm, const double* alpha, FlGraph* gr, cudaStream_t st);
void fl_launch_bmorton(const float4* pos, int n, int ndim, const uint32_t* gid, const FlGraph* gr,
                       uint64_t* keys, uint32_t* vals, uint32_t* hist, int lo_bit, cudaStream_t st);
void fl_launch_bgidkey(int n, const uint32_t* mperm, const uint32_t* gid, const int32_t* off,
                       int graphs, uint64_t* keys, uint32_t* vals, uint32_t* hist, cudaStream_t st);
void fl_launch_bgather(int n, const uint32_t* order2, const uint64_t* mkeys, const uint32_t* mperm,
                       const uint32_t* gid, uint64_t* skeys, uint32_t* perm, uint32_t* gid_pos,
                       cudaStream_t st);

// ---------------------------------------------------------------- radix sort (sort.cu)
// Stable LSD sort of (uint64 key, uint32 value) pairs on the key bits [lo_bit, 64), 8 bits per
// pass: one histogram pass fused into the key producer (or run on its own), then one onesweep
// pass per digit (warp match ranking, decoupled look-back over tiles, staged coalesced scatter).
struct FlSortBufs {
  uint64_t* keys[2];
  uint32_t* vals[2];
  uint32_t* hist;      // [8][256] digit counts per pass
  uint32_t* status;    // [passes][tiles][256] look-back words (tiles of this sort's tile size)
  uint32_t* counters;  // [kSortCounters]: tile tickets of up to 8 passes, then the run fix-up's
  uint32_t* longs;     // [longs_cap] first positions of the runs the fix-up sorts in one block
  uint32_t longs_cap;
  int64_t cap;         // pairs the buffers hold
  int64_t tiles_cap;   // tiles of kSortTileSmall pairs the look-back words have room for
  // 0, or a test of the bounded look-back: every wait gives up after this many polls, and the
  // first digit pass withholds tile 0's counts, so that the waits run out (the tiles that gave
  // up count their predecessors' keys themselves: the result stays exact, FL_ERR_LOOKBACK is set)
  uint32_t test_spins;
};
constexpr int kSortCounters = 16;
// A onesweep tile: 256 threads x kSortItems pairs for up to kSortSmallMax pairs (small sorts
// take more, shorter tiles: the time of a pass is that of one tile's steps); above, 1024 threads
// x 5 to kSortItems pairs, as few as give every SM a tile (fl_sort_tile).
constexpr int kSortThreads = 1024, kSortThreadsSmall = 256, kSortItems = 8;
constexpr int kSortTileSmall = kSortThreadsSmall * kSortItems;
constexpr int64_t kSortSmallMax = 131072;
int fl_sort_tile(int64_t n);  // pairs per tile for a sort of n pairs
int fl_sms();        // SMs of the current device (cached per device)
size_t fl_sort_bytes(int64_t n);
// Carve the buffers out of one allocation of fl_sort_bytes(n) bytes.
void fl_sort_carve(FlSortBufs* b, void* base, int64_t n);
// Zero the histogram, the tickets and the look-back words for `passes` passes.
void fl_sort_reset(const FlSortBufs* b, int64_t n, int passes, cudaStream_t st);
// Histogram of the keys in keys[0] (when the producer did not fuse it).
void fl_sort_histogram(const FlSortBufs* b, int64_t n, int lo_bit, cudaStream_t st, int64_t* launches);
// Run the passes from keys[0]/vals[0]; returns which buffer (0/1) holds the result.
int fl_sort_passes(const FlSortBufs* b, int64_t n, int lo_bit, uint32_t* err, cudaStream_t st,
                   int64_t* launches);
// The tree's key sort in two steps: `passes` digit passes over the top key bits
// [fl_sort_split(lo_bit, passes), 64) (0: 4 passes), then fl_sort_runfix, which puts each run of
// pairs equal in those bits in (key, value) order: together the stable sort on [lo_bit, 64) of
// pairs whose values start as 0, 1, 2, ... fl_sort_runfix returns the buffer holding the result.
int fl_sort_split(int lo_bit, int passes = 0);
int fl_sort_runfix(const FlSortBufs* b, int64_t n, int lo_bit, int lo_sort, int cur,
                   cudaStream_t st, int64_t* launches);
// Up to this many pairs, the tree sorts its keys in one launch (fl_sort_rank): each pair's place
// counted against every key, the stable order of the digit passes and the run fix-up.
constexpr int64_t kSortRankMax = 6144;
// The stable sort of 1 <= n <= kSortRankMax pairs, keys[0]/vals[0] -> keys[1]/vals[1]; returns
// the buffer holding the result (1), or 0 without a launch for other n.
int fl_sort_rank(const FlSortBufs* b, int64_t n, cudaStream_t st, int64_t* launches);

// ---------------------------------------------------------------- state kernels (state.cu)
void fl_launch_reduce(const float4* pos, int n, int ndim, int want_box, int want_sum,
                      FlReduce* red, cudaStream_t st);
void fl_launch_center_apply(float4* pos, int n, int ndim, const FlReduce* red, double cx,
                            double cy, double cz, double strength, cudaStream_t st);
// v *= decay; p += v; pinned axes: p = fix, v = 0. When red != NULL, first shifts p by the
// centre force of (cx, cy, cz, strength) computed from red->sum (the centre force fused).
// In a batch (gr, gid non-null) each node takes its graph's decay and centre shift.
// With `out` (not in a batch), the new positions are also reduced into it (box and/or sums, as
// fl_launch_reduce): the next tick's reduction, fused. With `snap` (not in a batch), p + v of the
// new state is written there: the next tick's link snapshot (fl_launch_snapshot).
void fl_launch_integrate(float4* pos, float4* vel, const float4* fix, const uint32_t* mask, int n,
                         int ndim, float decay, const FlReduce* red, double cx, double cy,
                         double cz, double strength, cudaStream_t st, const FlGraph* gr = nullptr,
                         const uint32_t* gid = nullptr, const FlTick* tk = nullptr,
                         FlReduce* out = nullptr, int want_box = 0, int want_sum = 0,
                         float4* snap = nullptr);
// snap = p + v per node (xyz; w 0): the state the link force reads, one record per node, so that
// a link end gathers one 16-byte record of the other node instead of two.
void fl_launch_snapshot(const float4* pos, const float4* vel, float4* snap, int n, cudaStream_t st);
// Positions and velocities (either may be NULL) to `ndim` floats per node in out: positions at
// [0, n ndim), velocities at [n ndim, 2 n ndim). And back: ndim floats per node to float4 (the
// rest 0) at dst[0, count).
void fl_launch_pack(const float4* pos, const float4* vel, int n, int ndim, float* out,
                    cudaStream_t st);
void fl_launch_unpack(const float* src, int count, int ndim, float4* dst, cudaStream_t st);
void fl_launch_radial(const float4* pos, float4* vel, const float* radius, const float* strength,
                      int n, int ndim, float cx, float cy, float cz, float alpha, cudaStream_t st,
                      const FlTick* tk = nullptr);
void fl_launch_position(const float4* pos, float4* vel, const float* target, const float* strength,
                        int n, int axis, float alpha, cudaStream_t st, const FlTick* tk = nullptr);

// ---------------------------------------------------------------- link (link.cu)
struct FlLinkCsr {
  const int32_t* row;      // [n + 1]
  const float4* entry;     // [2m] (other node as int bits, distance, strength, bias share)
  const uint32_t* code;    // [2m] link * 2 + (this node is the target)
};
// In a batch (gr, gid non-null) each node's links use its graph's alpha. With `snap` (p + vel_in
// per node, fl_launch_snapshot) the kernel reads the nodes' state from it instead of pos and
// vel_in: the same sums, half the gathered bytes.
void fl_launch_link(const float4* pos, const float4* vel_in, float4* vel_out, FlLinkCsr csr, int n,
                    int ndim, float alpha, uint32_t step, uint32_t seed, cudaStream_t st,
                    const FlGraph* gr = nullptr, const uint32_t* gid = nullptr,
                    const FlTick* tk = nullptr, const float4* snap = nullptr);

// ---------------------------------------------------------------- many-body (tree.cu)
struct FlTreeBufs {
  int n, ndim, levels, bits;
  uint32_t* left;        // [n-1] child: internal index, or 0x80000000 | sorted leaf
  uint32_t* right;       // [n-1]
  uint32_t* parent;      // [n-1] parent of internal nodes; [0] unused
  uint32_t* leaf_parent; // [n]
  uint32_t* range;       // [2(n-1)] first, last sorted leaf of each internal node
  uint8_t* depth;        // [n-1] d3 depth of each internal node's cell
  uint32_t* count;       // [n-1] children of a head (0 for other nodes)
  uint32_t* first;       // [n-1] first child slot of a head
  uint32_t* flag;        // [n] mixed-sign recursion: arrivals of each head's child cells; [n-1] the start count
  uint32_t* up_list;     // [n-1] mixed-sign recursion: the heads without child cells
  float4* cell;          // [n-1] head: centroid, value at its own depth
  float4* leaf;          // [n] sorted points: position, strength
  float4* child_data;    // [2n] slot: centroid or position, value at own depth / strength
  uint2* child_meta;     // [2n] slot: (first child slot, count | depth << 26) or (sorted index, ~0)
  double* slot64;        // [2n] slot of a cell: d3's FP64 value at its depth (mixed-sign recursion)
  void* scan_scratch;
  double* wsum;          // [5n] per sorted point |a|, |a| x, |a| y, |a| z, a; then their prefix sums
  double* wtiles;        // [5 tiles] partial sums of the prefix scan
  uint32_t* omask;       // [n-1] occupied octants of each head's cell; << 16, those of its child cells
  uint32_t* head_of;     // [2n-1] d3 child: its head | octant << 27 | 1 << 31 (internal, then points)
  uint4* spill;          // the walk stacks' overflow, one region per warp slot of its grid
  uint32_t* work;        // the walk's next group of 32 points to hand out
  int walk_slots;        // warp slots of the persistent walk grid
  int walk_blocks;       // blocks per SM of that grid (0: as many as fit)
  int sms;               // SMs of the device
};
struct FlWalkParams {
  float thresh[32];   // (cube size / 2^k)^2 / theta^2
  float damp[32];     // sqrt(4 / 2^dims)^j
  float dmin2, dmax2;
  int ndim;
  uint32_t step, seed;
};
size_t fl_tree_bytes(int64_t n);
// Warp slots of the persistent walk grid for n points on the current device.
int fl_walk_slots(int64_t n);
void fl_tree_carve(FlTreeBufs* t, void* base, int64_t n, int ndim);
// Bounding box -> d3 cube -> Morton keys (left-aligned) + values = node index, fused with the
// sort's digit histogram. Also sets the walk's per-depth thresholds on the device.
void fl_launch_morton(const float4* pos, int n, int ndim, const FlReduce* red, uint64_t* keys,
                      uint32_t* vals, uint32_t* hist, int lo_bit, float* cube_out,
                      cudaStream_t st);
// Karras build + sorted leaves (position, strength) gather; with `closed`, the FP64 point
// records of the closed-form cell sums.
// The two halves of fl_launch_build, for streams of their own: the sorted points with their
// fixed-point records (and the records' top prefix), and the Karras internal nodes.
void fl_launch_build_points(const FlTreeBufs* t, const uint64_t* skeys, const uint32_t* perm,
                            const float4* pos, const float* strength, bool closed,
                            const float* cube, int fx_exp, cudaStream_t st, int64_t* launches,
                            FlSegs segs = {});
void fl_launch_build_nodes(const FlTreeBufs* t, const uint64_t* skeys, const uint32_t* perm,
                           const float4* pos, const float* strength, const float* cube,
                           int fx_exp, cudaStream_t st, int64_t* launches, FlSegs segs = {});
// The halves of fl_launch_aggregate: the heads' octant masks (after the nodes), then the cells,
// counts and child slots (after the points and the masks).
void fl_launch_frontier(const FlTreeBufs* t, const uint64_t* skeys, uint32_t* err,
                        cudaStream_t st, int64_t* launches);
void fl_launch_cells(const FlTreeBufs* t, bool closed, float sign, const float* cube, int fx_exp,
                     int fp64_depth, uint32_t* err, cudaStream_t st, int64_t* launches,
                     FlSegs segs = {});
void fl_launch_build(const FlTreeBufs* t, const uint64_t* skeys, const uint32_t* perm,
                     const float4* pos, const float* strength, bool closed, const float* cube,
                     int fx_exp, cudaStream_t st, int64_t* launches, FlSegs segs = FlSegs{});
// Heads, child counts and slots; cell values and centroids in closed form (strengths of one
// sign, fixed-point sums at scale 2^fx_exp) or by the bottom-up recursion (both signs; FP64 sums
// for the cells above depth fp64_depth, FP32 below).
void fl_launch_aggregate(const FlTreeBufs* t, const uint64_t* skeys, bool closed, float sign,
                         const float* cube, int fx_exp, int fp64_depth, uint32_t* err,
                         cudaStream_t st, int64_t* launches, FlSegs segs = FlSegs{});
// Scale exponent of the fixed-point cell sums: no sum over n points of weight <= wmax overflows.
int fl_fixed_exponent(int64_t n, double wmax);
// stats (optional): [0] child tests made by the warps (32 per child), [1] of those, tests by a
// lane whose point needed them (the d3 traversal's own work)
// group: points per traversal (16 or 32), 1 for one point per warp with the lanes over the
// point's children (small layouts), 0 for the default by size (fl_walk_group_for)
// A batch (segs.graphs > 0): cube, alpha, theta2 and dmin2 are per graph (segs.g); dmax2 is
// only tested when finite (pass the largest of the graphs').
void fl_launch_walk(const FlTreeBufs* t, const uint32_t* perm, const float* cube, float4* vel,
                    float alpha, double theta2, double dmin2, double dmax2, uint32_t step,
                    uint32_t seed, uint32_t* err, unsigned long long* stats, int group,
                    cudaStream_t st, FlSegs segs = FlSegs{}, const FlTick* tk = nullptr);
// The walk group a layout of n points gets by default: 1 (one point per warp) up to a size at
// which groups of 32 points fill the device, else 32.
int fl_walk_group_for(int n);
// Exact all-pairs sum (theta ~ 0): O(n^2), tiled through shared memory.
void fl_launch_allpairs(const float4* pos, const float* strength, float4* vel, int n, int ndim,
                        float alpha, float dmin2, float dmax2, uint32_t step, uint32_t seed,
                        cudaStream_t st, const FlTick* tk = nullptr);

// ---------------------------------------------------------------- collide (collide.cu)
void fl_launch_collide_allpairs(const float4* pos, const float4* vel_in, float4* vel_out,
                                const float* radius, int n, int ndim, float strength,
                                uint32_t step, uint32_t seed, cudaStream_t st,
                                const FlTick* tk = nullptr);
struct FlGridBufs {
  int n, bits;
  uint32_t* starts;   // [2^bits] run start per slot (validated against the sorted keys)
  float4* sorted;     // [n] sorted snapshot position, radius
};
size_t fl_grid_bytes(int64_t n);
void fl_grid_carve(FlGridBufs* g, void* base, int64_t n);
void fl_launch_grid_keys(const float4* pos, const float4* vel, int n, int ndim, float inv_cell,
                         int bits, uint64_t* keys, uint32_t* vals, uint32_t* hist, int lo_bit,
                         cudaStream_t st);
// Collide in a batch: one grid over all graphs, cells keyed by (graph, cell); iteration `iter`
// of each graph's collide force (a graph with fewer iterations, none, or sitting the tick out
// keeps its velocities). keys[0]/vals[0] of the sort buffers take the cell keys (bit 63 clear;
// ~0 for nodes not taking part), sorted on bits [lo_bit, 64); sgid[n] holds each sorted node's
// graph.
void fl_launch_bgrid_keys(const float4* pos, const float4* vel, int n, int ndim,
                          const uint32_t* gid, const FlGraph* gr, int iter, int bits,
                          uint64_t* keys, uint32_t* vals, uint32_t* hist, int lo_bit,
                          cudaStream_t st);
void fl_launch_bgrid_query(const FlGridBufs* g, const uint64_t* skeys, const uint32_t* perm,
                           const float4* pos, const float4* vel_in, float4* vel_out,
                           const float* radius, int ndim, const uint32_t* gid,
                           const FlGraph* gr, uint32_t* sgid, const FlTick* tk, cudaStream_t st,
                           int64_t* launches);
void fl_launch_grid_query(const FlGridBufs* g, const uint64_t* skeys, const uint32_t* perm,
                          const float4* pos, const float4* vel_in, float4* vel_out,
                          const float* radius, int ndim, float inv_cell, float strength,
                          uint32_t step, uint32_t seed, cudaStream_t st, int64_t* launches,
                          const FlTick* tk = nullptr);
