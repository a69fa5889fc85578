/*
 * d3force_oracle.h -- CPU restatement (FP64) of d3-force-3d's CPU force simulation.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the checker for the GB300 engine: only the
 * tests, __graft_entry__.smoke() and the cpu_baseline / reference legs of bench.py load it.
 * The product path (d3-force-3d-webgpu_gb300/) never links, loads or calls it.
 *
 * Restated from the reference's CPU sources (paths within erw-1/d3-force-3d-webgpu):
 *   src/simulation.js   tick (:49-77), phyllotaxis init (:79-107), defaults (:28-36)
 *   src/manyBody.js     force (:21-31), accumulate (:42-71), apply (:73-115)
 *   src/link.js         force (:34-54), initialize: count, bias, default strength (:30-32, :56-79)
 *   src/collide.js      force/apply (:30-95), prepare (:97-104)
 *   src/center.js       (:8-26)   src/radial.js (:16-28)   src/x.js, y.js, z.js (:12-16)
 *   src/lcg.js (:1-9)   src/jiggle.js (:1-3)
 * and the behaviour of the third-party trees those forces build, which are not vendored in the
 * reference: d3-binarytree 1.0.1, d3-quadtree 3.0.1, d3-octree 1.0.1 (package.json:43-49,
 * yarn.lock:310-328). Their published algorithm is restated here: cover() (floor of the first
 * point, then doubling a power-of-two extent), add() (midpoint descent, coincident points chained
 * newest-first, splitting until two points separate), visit() (pre-order, children in index
 * order, index bit k = coordinate k >= midpoint) and visitAfter() (post-order).
 *
 * Pinned by the reference's CPU known-answer tests (test/simulation-test.js:10-17,
 * test/center-test.js:4-22, test/collide-test.js:5-50, test/x-test.js:5-77); see tests/golden/.
 * Many-body has no CPU known-answer test in the reference: it is pinned by self-consistency
 * (theta -> 0 equals the FP64 all-pairs sum) and by the published layout sizes.
 */
#ifndef D3FORCE_ORACLE_H
#define D3FORCE_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct osim osim;

/* Force evaluation modes. D3 = the reference CPU force exactly (sequential, tree, LCG jiggle).
 * JACOBI = every link / pair against one snapshot of p + v (the GPU's all-at-once form).
 * EXACT = FP64 sum over all pairs (no tree). */
enum { OFL_MODE_D3 = 0, OFL_MODE_JACOBI = 1, OFL_MODE_EXACT = 2 };

/* forceSimulation(nodes, numDimensions): positions that are NaN get the phyllotaxis start,
 * velocities that are NaN become 0, pinned axes (fmask bits 1/2/4) take fx/fy/fz. Any pointer
 * may be NULL (all NaN / no pins). Arrays are n*3 doubles. */
osim* ofl_create(int32_t n, int32_t ndim, const double* xyz, const double* vxyz,
                 const double* fxyz, const uint8_t* fmask);
void ofl_destroy(osim* s);

/* alpha, alphaMin, alphaDecay, alphaTarget, and the stored velocity multiplier (1 - velocityDecay) */
void ofl_set_params(osim* s, double alpha, double alpha_min, double alpha_decay,
                    double alpha_target, double velocity_multiplier);
void ofl_get_params(const osim* s, double* out5);

void ofl_set_pins(osim* s, const double* fxyz, const uint8_t* fmask);
void ofl_get_state(const osim* s, double* xyz, double* vxyz);
void ofl_set_state(osim* s, const double* xyz, const double* vxyz);
uint32_t ofl_get_lcg(const osim* s);
void ofl_set_lcg(osim* s, uint32_t state);
double ofl_random(osim* s); /* one draw of the simulation's LCG (src/lcg.js) */

/* Forces are applied in the order they are added (a Map in insertion order in the reference).
 * Per-node / per-link arrays are final values (accessors already evaluated by the caller). */
int32_t ofl_add_manybody(osim* s, const double* strengths, double distance_min2,
                         double distance_max2, double theta2, int32_t mode);
/* dist / str may be NULL: distance 30, strength 1 / min(count[source], count[target]). */
int32_t ofl_add_link(osim* s, int32_t m, const int32_t* src, const int32_t* dst,
                     const double* dist, const double* str, int32_t iterations, int32_t mode);
int32_t ofl_add_collide(osim* s, const double* radii, double strength, int32_t iterations,
                        int32_t mode);
int32_t ofl_add_center(osim* s, double x, double y, double z, double strength);
int32_t ofl_add_radial(osim* s, const double* radiuses, const double* strengths, double x,
                       double y, double z);
int32_t ofl_add_position(osim* s, int32_t axis, const double* targets, const double* strengths);
void ofl_clear_forces(osim* s);
/* the bias and default strength the link force at index k computed (m doubles each) */
void ofl_link_params(const osim* s, int32_t k, double* bias, double* strength);

void ofl_tick(osim* s, int32_t iterations);
/* Apply force k once at the given alpha (no alpha update, no integration). */
void ofl_apply_force(osim* s, int32_t k, double alpha);

/* The velocity change many-body force k would give each of `count` target nodes at the current
 * state and `alpha`, without changing the state: OFL_MODE_D3 walks d3's tree (built over all
 * nodes), OFL_MODE_EXACT sums every pair in FP64 on `threads` host threads. out3: 3 * count
 * doubles. Returns 0, or -1 for a bad force index or target. */
int32_t ofl_manybody_probe(osim* s, int32_t k, double alpha, int32_t mode, int32_t count,
                           const int32_t* targets, int32_t threads, double* out3);

/* The velocity change one iteration of collide force k in its Jacobi form (every pair against
 * one snapshot of p + v) gives each of `count` target nodes, state unchanged: the values the
 * JACOBI mode's full pass gives those nodes, at O(count * n) on `threads` host threads.
 * out3: 3 * count doubles. Returns 0, or -1 for a bad force index or target. */
int32_t ofl_collide_probe(osim* s, int32_t k, int32_t count, const int32_t* targets,
                          int32_t threads, double* out3);

/* Counters of the last many-body d3 tree walk: [0] approximated cells (internal cells that
 * passed the theta test, with a nonzero value), [1] point interactions (leaf data visited),
 * [2] cells opened (internal cells that failed the theta test). */
void ofl_walk_stats(const osim* s, int64_t* out3);

/* ---- integer rebuilds (bit-exact references for the GPU's integer stages) ---- */

/* Levels of the Morton code per dimension count (index 1..3). */
int32_t ofl_levels(int32_t ndim);
/* The d3 cube of FP32 positions (stride 4): out4 = {origin x, y, z, size}; returns log2(size). */
int32_t ofl_cube(int32_t n, int32_t ndim, const float* pos4, double* out4);
/* Morton codes in the d3 child order (bit 0 of a level = x, 1 = y, 2 = z), LEVELS levels,
 * most significant level first, in the low DIMS*LEVELS bits of each code. */
void ofl_morton(int32_t n, int32_t ndim, const float* pos4, uint64_t* codes);
/* The stable order of the codes (ties by node index). */
void ofl_sort_perm(int32_t n, const uint64_t* codes, uint32_t* perm);
/* Karras (2012) binary radix tree over sorted codes. For every internal node i < n-1:
 * left/right child (leaf flag 0x80000000 | sorted index, or internal index), and the d3 depth
 * of its cell: min(common prefix bits / DIMS, LEVELS), ties between equal codes broken by index. */
void ofl_karras(int32_t n, int32_t ndim, const uint64_t* sorted_codes, uint32_t* left,
                uint32_t* right, int32_t* depth);
/* CSR over nodes of m links: row_start (n+1), then per entry (other endpoint, link*2 + is_target),
 * each node's entries in link order. */
void ofl_csr(int32_t n, int32_t m, const int32_t* src, const int32_t* dst, int32_t* row_start,
             int32_t* other, int32_t* code);

#ifdef __cplusplus
}
#endif
#endif
