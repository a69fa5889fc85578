/*
 * forcegpu.h -- C ABI of the GB300 force-layout engine (libforcegpu.so).
 *
 * The drop-in boundary for the per-tick hot path of forceSimulationGPU: every entry point here
 * replaces one call of the reference's WebGPU engine (paths within erw-1/d3-force-3d-webgpu),
 * which the JavaScript facade (src/gpu/simulation.js) drives. Plain C types only: the caller
 * owns host arrays, which are copied during the call; no pointer is kept after a call returns.
 * Every function returns an FL_* status; fl_last_error() gives the message of the last failure.
 * A simulation is single-caller; separate simulations may be used from separate threads.
 *
 * Node state layout (as the reference's GPU buffers, src/gpu/wgsl.js:1-10): positions and
 * velocities are float4 per node (x, y, z, unused w), so arrays are 4*n floats. Axes beyond
 * numDimensions stay 0. Pins: fix is float4 per node (fx, fy, fz, -), mask bit 1/2/4 = axis
 * x/y/z pinned (src/gpu/engine.js:131-134).
 */
#ifndef FORCEGPU_H
#define FORCEGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FL_ABI_VERSION 1

/* Status codes. The reference reports failures by rejecting a Promise or falling back to the
 * CPU (src/gpu/engine.js:50-59, src/gpu/simulation.js:112-116); this engine has no CPU path. */
enum {
  FL_OK = 0,
  FL_E_ARG = 1,         /* invalid argument: sizes, a link endpoint out of range, bad type */
  FL_E_OOM = 2,         /* a device allocation failed */
  FL_E_DEVICE = 3,      /* a CUDA call failed (no device, launch error, ...) */
  FL_E_TIMEOUT = 4,     /* a bounded device-side wait (scan look-back) gave up */
  FL_E_OVERFLOW = 5,    /* a device-side capacity was exceeded (tree walk stack) */
  FL_E_STATE = 6,       /* not valid in this state (no nodes, destroyed) */
  FL_E_UNSUPPORTED = 7  /* a force type with no GPU pass: the reference hands such a
                           simulation to the CPU (src/gpu/engine.js:41-48); here it is an error */
};

/* Force types: the `type` of force.gpu() (src/gpu/passes/index.js:8-16). */
enum {
  FL_FORCE_MANYBODY = 1, /* src/manyBody.js:142-144   {strengths, distanceMin2, distanceMax2, theta2} */
  FL_FORCE_LINK = 2,     /* src/link.js:127-129       {links, iterations, strengths, distances, bias} */
  FL_FORCE_COLLIDE = 3,  /* src/collide.js:134-136    {radii, strength, iterations} */
  FL_FORCE_CENTER = 4,   /* src/center.js:49-51       {x, y, z, strength} */
  FL_FORCE_RADIAL = 5,   /* src/radial.js:69-71       {radiuses, strengths, x, y, z} */
  FL_FORCE_POSITION = 6  /* src/x.js:43-45 (y.js, z.js) {axis, targets, strengths} */
};

/* One force's descriptor, the C form of force.gpu(). Arrays are read only when `version`
 * differs from the version the engine last saw for the same `key` (the reference re-uploads on
 * a version change, e.g. src/gpu/passes/manyBody.js:98-106); scalars are read on every call. */
typedef struct fl_force_desc {
  int32_t type;           /* FL_FORCE_* */
  uint32_t version;       /* bumped by the force whenever its per-node / per-link values change */
  uint64_t key;           /* identity of the force object: its pass (and uploads) persist while
                             a force with this key and type stays in the list (engine.js:320-328) */
  const float* node_a;    /* [n] manyBody strengths | collide radii | radial radiuses |
                                 position targets */
  const float* node_b;    /* [n] radial strengths | position strengths */
  int32_t m;              /* link: number of links */
  const int32_t* source;  /* link: [m] source node index */
  const int32_t* target;  /* link: [m] target node index */
  const float* link_distance; /* link: [m] */
  const float* link_strength; /* link: [m] */
  const float* link_bias;     /* link: [m] bias of the target end (src/link.js:73-75) */
  int32_t iterations;     /* link, collide */
  int32_t axis;           /* position: 0 = x, 1 = y, 2 = z */
  double distance_min2;   /* manyBody */
  double distance_max2;   /* manyBody (may be +inf) */
  double theta2;          /* manyBody; <= 1e-6 selects the exact all-pairs sum */
  double strength;        /* collide, center */
  double x, y, z;         /* center, radial */
} fl_force_desc;

typedef struct fl_sim fl_sim;

/* Device-resident state, for a renderer that draws without a readback: the reference's
 * gpuBuffers() (src/gpu/engine.js:416-420), with CUDA device pointers in place of GPUBuffers. */
typedef struct fl_buffer_info {
  void* positions;  /* float4 per node, device memory */
  void* velocities; /* float4 per node, device memory */
  int32_t count;
  int32_t stride;   /* 16 */
} fl_buffer_info;

/* Create an engine on a CUDA device (replaces requestDevice + createEngine,
 * src/gpu/device.js:19-39, src/gpu/engine.js:73). */
int32_t fl_create(int32_t device, fl_sim** out);
/* Release every device buffer (engine.destroy, src/gpu/engine.js:422-427). NULL is allowed. */
int32_t fl_destroy(fl_sim* sim);
/* Message of the last failed call on this simulation. With sim NULL: the message of the last
 * failed call on the calling thread that takes no simulation (fl_create, fl_radix_sort,
 * fl_radix_sort_noalloc), kept per host thread. The string lives until the next call on the same
 * simulation (or, with NULL, the next such failure on the same thread). */
const char* fl_last_error(const fl_sim* sim);

/* Whether `count` nodes fit this device (engine.fits, src/gpu/engine.js:332-338). */
int32_t fl_fits(fl_sim* sim, int64_t count, int32_t* fits);

/* Replace the node set and upload it (engine.setNodes + uploadAll, src/gpu/engine.js:115-145,
 * :267-310). pos4/vel4/fix4 are 4*n floats; vel4, fix4 and mask may be NULL (zeros). The
 * forces must be set again afterwards, as in the reference. n may be 0. */
int32_t fl_set_nodes(fl_sim* sim, int32_t n, int32_t ndim, const float* pos4, const float* vel4,
                     const float* fix4, const uint32_t* mask);
/* Replace the whole node state of the current node set, keeping the forces (engine.markStale +
 * uploadAll, src/gpu/engine.js:115-145, :346-349, :355): pos4/vel4/fix4 are 4*n floats of the n
 * nodes fl_set_nodes gave; vel4, fix4 and mask may be NULL (zeros). The tick counter runs on, as
 * the reference's does. A block of ticks that ran before from the state fl_set_nodes left (or
 * from an earlier fl_upload_all) runs again as the same CUDA graph after this call, so a caller
 * can restart from a saved state without recapturing. */
int32_t fl_upload_all(fl_sim* sim, const float* pos4, const float* vel4, const float* fix4,
                      const uint32_t* mask);
/* Upload nodes [first, first + count) that the caller moved (uploadPositions,
 * src/gpu/engine.js:147-156): 4*count floats. */
int32_t fl_update_positions(fl_sim* sim, int32_t first, int32_t count, const float* pos4);
/* fl_update_positions with `ndim` floats per node (x[, y[, z]]: ndim*count floats), unpacked on
 * the device, so the host link carries ndim/4 of the bytes. No counterpart in the reference,
 * whose uploadPositions writes vec4s (src/gpu/engine.js:147-156). */
int32_t fl_update_positions_packed(fl_sim* sim, int32_t first, int32_t count, const float* pos);
/* fl_update_positions_packed without the wait: the copy and the unpacking are queued on the
 * simulation's stream and the call returns at once, so that the ticks queued next follow them
 * with no host round trip in between. The caller keeps `pos` (best pinned: cudaHostAlloc or
 * cudaHostRegister) unchanged until the next fl_sync, fl_sync_packed or fl_idle returns. No
 * counterpart in the reference. */
int32_t fl_update_positions_packed_async(fl_sim* sim, int32_t first, int32_t count,
                                         const float* pos);
/* Upload changed pins of nodes [first, first + count) (uploadPinned, src/gpu/engine.js:158-169). */
int32_t fl_update_pins(fl_sim* sim, int32_t first, int32_t count, const float* fix4,
                       const uint32_t* mask);
/* Overwrite velocities of nodes [first, first + count). No counterpart in the reference, whose
 * GPU owns velocities (docs/differences.md:18); used to start a run from a captured state. */
int32_t fl_update_velocities(fl_sim* sim, int32_t first, int32_t count, const float* vel4);

/* The forces, in application order (engine.setForces, src/gpu/engine.js:312-330). */
int32_t fl_set_forces(fl_sim* sim, int32_t count, const fl_force_desc* descs);

/* Seed of the coincident-node jiggle (engine.setSeed, src/gpu/engine.js:340-343). */
int32_t fl_set_seed(fl_sim* sim, uint32_t seed);

/* Queue `count` ticks without waiting (engine.enqueue, src/gpu/engine.js:351-391). alphas are the
 * host-computed alpha of each tick (src/gpu/simulation.js:141-151); decay is the velocity
 * multiplier, 1 - velocityDecay. */
int32_t fl_enqueue(fl_sim* sim, const double* alphas, int32_t count, double decay);
/* Wait for every queued tick, then copy positions and velocities (4*n floats each; either may
 * be NULL) into the caller's arrays (engine.sync + readback, src/gpu/engine.js:218-239,
 * :406-414). Reports a device-side error raised by any tick since the previous sync. */
int32_t fl_sync(fl_sim* sim, float* pos4_out, float* vel4_out);
/* fl_sync with positions and velocities packed to `ndim` floats per node (ndim*n floats each;
 * either may be NULL), packed on the device first so that the host link carries ndim/4 of
 * fl_sync's bytes. No counterpart in the reference, whose readback maps the two vec4 buffers
 * (src/gpu/engine.js:218-239). */
int32_t fl_sync_packed(fl_sim* sim, float* pos_out, float* vel_out);
/* Wait for every queued tick, no readback (engine.idle, src/gpu/engine.js:401-404). */
int32_t fl_idle(fl_sim* sim);
/* Whether queued work is still running (engine.busy, src/gpu/engine.js:393-396). */
int32_t fl_busy(fl_sim* sim, int32_t* busy);
/* Device pointers of the state (engine.buffers), for reading (rendering): positions written
 * through them are not seen by the next tick's bounding box and centre sums, which the last
 * integrate already took, nor velocities by the next tick's link snapshot (p + v, also written
 * by the last integrate); write positions with fl_update_positions and velocities with
 * fl_update_velocities, or call fl_update_positions(sim, 0, 0, NULL) /
 * fl_update_velocities(sim, 0, 0, NULL) after writing them on the device. */
int32_t fl_buffers(fl_sim* sim, fl_buffer_info* out);

/* ---- measurement (no reference counterpart: the reference times only with performance.now()
 *      around tickAsync, examples/benchmark.html:105-132) ---- */

/* Tuning parameters (no reference counterpart; the reference's closest are its fixed
 * constants, e.g. src/gpu/passes/barnesHut.js:49-58): FL_TUNE_WALK_GROUP, points that share one
 * tree-walk traversal, 16 or 32, or 1 for one point per warp with the warp's lanes testing up to
 * 32 of its children at once (0, the default: 1 up to 32,768 nodes, else 32); FL_TUNE_CELL_SUMS, how the many-body cells' values
 * and centroids are summed: FL_CELLS_AUTO (default: exact fixed-point prefix sums when the
 * strengths share one sign, else the bottom-up recursion: d3's FP64 values bit for bit, FP64
 * centroid sums near the root), FL_CELLS_FP64_TOP (always that recursion) or FL_CELLS_FP32 (the
 * recursion all in FP32, for precision comparisons); FL_TUNE_GRAPHS, 1 (default) to run a block of ticks that fl_enqueue
 * has seen before (same length, same forces) as one CUDA graph, captured the second time it is
 * seen, or 0 to launch every kernel of every block directly; FL_TUNE_SORT_PASSES, the 8-bit digit
 * passes of the tree's radix sort, from the top of the Morton key (0 = 4, the default: the top
 * 31 bits in 3D, 32 in 2D; 8 = every bit in 3D), the bits below ordered within runs of equal top
 * bits by a fix-up pass: fewer passes, longer runs (with 0, a layout of up to 6,144 nodes sorts
 * in one launch instead, each key ranked against all others: the same order); FL_TUNE_WALK_BLOCKS, blocks per SM of the
 * persistent tree-walk grid (0 = as many as fit, the default); FL_TUNE_COLLIDE_CELL, the collide
 * grid's cell side in percent of the largest diameter (>= 100; 100 = the default).
 * fl_autotune picks these by timing. */
enum {
  FL_TUNE_WALK_GROUP = 1,
  FL_TUNE_CELL_SUMS = 2,
  FL_TUNE_GRAPHS = 3,
  FL_TUNE_SORT_PASSES = 4,
  FL_TUNE_WALK_BLOCKS = 5,
  FL_TUNE_COLLIDE_CELL = 6,
  /* A test of the bounded device-side waits, not a tuning: with value v > 0 every look-back wait
   * of the many-body tree's sort gives up after v polls, and the first digit pass of each tick
   * withholds the first tile's counts, so that the waits do run out. A tile whose wait gave up
   * counts its predecessors' keys itself (the sort stays exact, only slower) and the next
   * fl_sync / fl_idle reports FL_E_TIMEOUT. 0 (the default) turns it off. */
  FL_TUNE_TEST_LOOKBACK = 7
};
enum { FL_CELLS_AUTO = 0, FL_CELLS_FP64_TOP = 1, FL_CELLS_FP32 = 2 };
int32_t fl_set_tuning(fl_sim* sim, int32_t key, int32_t value);

/* The autotuner (no reference counterpart: the reference's block sizes, digit widths and stack
 * depths are constants). It times `ticks`-tick blocks of the current nodes and forces at the
 * given alpha and decay under candidate values of FL_TUNE_SORT_PASSES, FL_TUNE_WALK_GROUP,
 * FL_TUNE_WALK_BLOCKS and FL_TUNE_COLLIDE_CELL (those that the forces use), one knob at a time,
 * keeps the fastest, and restores the state: positions, velocities and the tick count are as
 * before the call. With a cache file (NULL: none) the result is stored under a key of the
 * device's compute capability, the dimensions, log2 of the node count and the forces, and a
 * later call with the same key applies it without timing. */
typedef struct {
  int32_t walk_group, sort_passes, walk_blocks, collide_cell;  /* the values chosen */
  double ms_per_tick;  /* with them */
  double ms_default;   /* with the defaults, timed the same way */
  int32_t candidates;  /* configurations timed (0 when read from the cache) */
  int32_t from_cache;
} fl_tune_result;
int32_t fl_autotune(fl_sim* sim, int32_t ticks, double alpha, double decay,
                    const char* cache_path, fl_tune_result* out);

/* The cudaStream_t every kernel of this simulation runs on. */
int32_t fl_stream(fl_sim* sim, void** stream);
/* Queries: FL_Q_LAUNCHES kernels launched so far, FL_Q_TICKS ticks queued so far, FL_Q_NODES,
 * FL_Q_ERRWORD the raw device error word, FL_Q_DEVICE_BYTES device memory held. Walk counters,
 * summed over the tree walks since profiling level 2 was enabled: FL_Q_WALK_TESTS child tests
 * made (one per point of the walking group and child), FL_Q_WALK_USEFUL of those, the tests a
 * point's own d3 traversal needed, FL_Q_WALK_MAX_STACK the deepest walk stack,
 * FL_Q_WALK_OPENS cells opened and FL_Q_WALK_APPLIES cells or points applied (both per point),
 * FL_Q_WALK_RARE rounds of two children that took the uncommon-case path. */
enum { FL_Q_LAUNCHES = 1, FL_Q_TICKS = 2, FL_Q_NODES = 3, FL_Q_ERRWORD = 4, FL_Q_DEVICE_BYTES = 5,
       FL_Q_WALK_TESTS = 6, FL_Q_WALK_USEFUL = 7, FL_Q_WALK_MAX_STACK = 8, FL_Q_WALK_OPENS = 9,
       FL_Q_WALK_APPLIES = 10, FL_Q_WALK_RARE = 11 };
int32_t fl_query(fl_sim* sim, int32_t what, int64_t* out);
/* Per-kernel timing with CUDA events on the simulation's stream: enable (1), or enable with
 * the walk's counters too (2); then read the summed milliseconds and launch count of each
 * kernel group since it was enabled. */
int32_t fl_profile(fl_sim* sim, int32_t enable);
/* Fills up to `cap` entries; returns the number of groups in *count. Names live as long as sim. */
int32_t fl_profile_read(fl_sim* sim, int32_t cap, const char** names, double* ms,
                        int64_t* launches, int32_t* count);

/* ---- batches: many independent layouts advanced together ----
 * No counterpart in the reference, which runs one simulation per engine (src/gpu/engine.js:73);
 * its closest relatives are the per-device engine sharing of src/gpu/device.js:4 and the
 * step batching of src/gpu/engine.js:7-9, :362-389. A batch holds G graphs, each with a link
 * force, a many-body force and an optional centre force (the forces of the reference's
 * benchmark), an optional collide force (applied after the many-body force, as the served jobs
 * list it), all in one dimensionality; every kernel of a tick runs once for the whole batch.
 * Each graph has its own alpha schedule, theta, distances, centre and velocity decay. */
typedef struct fl_graph_desc {
  int32_t n;                 /* nodes */
  int32_t m;                 /* links */
  const float* pos4;         /* [4n] start positions (x, y, z, -) */
  const float* vel4;         /* [4n] start velocities, or NULL (0) */
  const int32_t* source;     /* [m] link ends, node indices within this graph */
  const int32_t* target;     /* [m] */
  const float* link_distance; /* [m] or NULL: 30 (src/link.js:19) */
  const float* link_strength; /* [m] or NULL: 1 / min(count(source), count(target)) (src/link.js:36-38) */
  const float* link_bias;     /* [m] or NULL: count(source) / (count(source) + count(target)) (src/link.js:73-75) */
  const float* charge;       /* [n] many-body strengths, or NULL (-30) */
  double theta2, distance_min2, distance_max2;  /* many-body (d3 defaults 0.81, 1, inf) */
  double center_x, center_y, center_z, center_strength; /* centre force; strength 0: none */
  double velocity_decay;     /* d3's velocityDecay (0.4 default) */
  uint32_t tick0;            /* ticks the graph has run before (0 for a new layout): a layout
                                moved from batch to batch keeps its own tick count, which seeds
                                its coincident-node jiggles, so its result does not depend on
                                the batches it went through */
  const float* radii;        /* [n] collide radii (src/collide.js:134-136), or NULL: no collide force */
  double collide_strength;   /* collide strength (d3's default 1) */
  int32_t collide_iterations; /* collide iterations (d3's default 1) */
} fl_graph_desc;

typedef struct fl_batch fl_batch;
int32_t fl_batch_create(int32_t device, fl_batch** out);
int32_t fl_batch_destroy(fl_batch* b);
const char* fl_batch_last_error(const fl_batch* b);
/* Replace the batch's graphs (copied; the state starts from pos4 / vel4). */
int32_t fl_batch_set_graphs(fl_batch* b, int32_t ndim, int32_t graphs, const fl_graph_desc* descs);
/* Append graphs to the batch, keeping every graph it holds and their state (continuous
 * batching: a layout job joins a batch that is running without a readback of the others). The
 * appended graphs are numbered after the present ones; their descriptors are as
 * fl_batch_set_graphs's, in the batch's dimensionality, and a graph's tick0 is its own tick
 * count. No counterpart in the reference. */
int32_t fl_batch_add_graphs(fl_batch* b, int32_t count, const fl_graph_desc* descs);
int32_t fl_batch_set_seed(fl_batch* b, uint32_t seed);
/* Queue `ticks` ticks without waiting; alphas[k * graphs + g] is graph g's alpha at tick k. A
 * negative alpha makes graph g sit tick k out: its positions and velocities do not change (a
 * graph whose layout is finished while others in the batch go on). */
int32_t fl_batch_enqueue(fl_batch* b, const double* alphas, int32_t ticks);
/* Wait, then copy the concatenated positions / velocities (4 floats per node; either may be
 * NULL). Reports a device-side error raised since the previous sync. */
int32_t fl_batch_sync(fl_batch* b, float* pos4_out, float* vel4_out);
/* Wait, then read back the positions and velocities (float4 per node) of graphs
 * [first, first + count) only; NULL outputs are skipped. */
int32_t fl_batch_read(fl_batch* b, int32_t first, int32_t count, float* pos4_out,
                      float* vel4_out);
/* FL_Q_LAUNCHES, FL_Q_TICKS, FL_Q_NODES, FL_Q_DEVICE_BYTES */
int32_t fl_batch_query(fl_batch* b, int32_t what, int64_t* out);
int32_t fl_batch_stream(fl_batch* b, void** stream);
/* Tuning of a batch, as fl_set_tuning: FL_TUNE_GRAPHS, FL_TUNE_SORT_PASSES, FL_TUNE_WALK_BLOCKS. */
int32_t fl_batch_set_tuning(fl_batch* b, int32_t key, int32_t value);
/* fl_autotune for a batch: FL_TUNE_SORT_PASSES and FL_TUNE_WALK_BLOCKS, every graph at `alpha`;
 * the key adds log2 of the graph count. */
int32_t fl_batch_autotune(fl_batch* b, int32_t ticks, double alpha, const char* cache_path,
                          fl_tune_result* out);

/* ---- integer stages, exposed for bit-exact checks against a CPU rebuild ---- */

/* Stable LSD radix sort of n (key, value) pairs on key bits [lo_bit, 64), the engine's sort on
 * its own (the reference's createSort, src/gpu/sort.js:139-190, tested alone by
 * test/gpu-sort-test.js). Host arrays in and out; device memory is allocated for the call.
 * Runs on the calling thread's current CUDA device. */
int32_t fl_radix_sort(const uint64_t* keys, const uint32_t* vals, int64_t n, int32_t lo_bit,
                      uint64_t* keys_out, uint32_t* vals_out);

/* fl_radix_sort for callers that cannot allocate device memory: those whose device memory is
 * all owned by their own pool or fixed budget (a renderer's or plugin host's allocator), those
 * that must not stall the device with cudaMalloc/cudaFree, and those that must not fail for lack
 * of memory mid-frame. No counterpart in the reference. keys/vals and keys_out/vals_out are
 * DEVICE buffers of n pairs on the calling thread's current device (the outputs may be the
 * inputs, sorted in place; they must not otherwise overlap); the sort runs on `stream` (NULL:
 * the default stream) and the call returns when it has finished. Its scratch is a built-in
 * device array of about 3.6 MB, present on every device that loads this library until the
 * process exits, so n may not exceed FL_SORT_NOALLOC_MAX_PAIRS (FL_E_ARG otherwise). Every
 * call looks the array's address up in the current context (cudaGetSymbolAddress, which
 * allocates nothing); the first call in a context also loads the library's device code there:
 * make that first call before any stream capture. Calls share the array, so calls that overlap
 * on the GPU (from several host threads, or on several streams) race and corrupt each other's
 * results. */
#define FL_SORT_NOALLOC_MAX_PAIRS 262144
int32_t fl_radix_sort_noalloc(const uint64_t* keys, const uint32_t* vals, int64_t n,
                              int32_t lo_bit, uint64_t* keys_out, uint32_t* vals_out,
                              void* stream);

/* The many-body tree the last tick built for force `index` of the list (a Barnes-Hut pass,
 * src/gpu/passes/barnesHut.js:934-1126): sorted left-aligned Morton keys [n], the sort
 * permutation [n] (node index per sorted position), and per internal node [n-1] its children
 * (0x80000000 | sorted index for a point) and d3 depth; cube = {origin x, y, z, size, log2 size}.
 * Any output may be NULL. */
int32_t fl_debug_tree(fl_sim* sim, int32_t index, uint64_t* keys, uint32_t* perm, uint32_t* left,
                      uint32_t* right, uint8_t* depth, float* cube5);

/* The link CSR the engine holds for force `index` (a link force), as the reference builds it on
 * the host (src/gpu/passes/link.js:65-101): row[n + 1] offsets of each node's entries, then per
 * entry [2m] the other end's node index and its code, link * 2 + (this node is the target),
 * each node's entries in link order. Any output may be NULL. */
int32_t fl_debug_links(fl_sim* sim, int32_t index, int32_t* row, int32_t* other, uint32_t* code);

#ifdef __cplusplus
}
#endif

#endif
