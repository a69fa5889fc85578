/* A host written in C against include/forcegpu.h alone, as a non-Python binding would use the
 * library: one 3D layout (link + many-body + centre) stepped through the C ABI, its positions
 * written to stdout. tests/test_gpu_c_host.py builds it with gcc and compares its output with
 * the same layout stepped through the Python binding.
 *
 *   abi_host N TICKS   (N nodes, a path plus chords i -> i + 7 mod N, a spiral start) */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "forcegpu.h"

#define CHECK(call)                                                               \
  do {                                                                            \
    int32_t rc_ = (call);                                                         \
    if (rc_ != FL_OK) {                                                           \
      fprintf(stderr, "%s failed (%d): %s\n", #call, rc_, fl_last_error(sim));    \
      return 1;                                                                   \
    }                                                                             \
  } while (0)

int main(int argc, char** argv) {
  const int n = argc > 1 ? atoi(argv[1]) : 1000;
  const int ticks = argc > 2 ? atoi(argv[2]) : 10;
  if (n < 2 || ticks < 1) return 2;
  fl_sim* sim = NULL;
  if (fl_create(0, &sim) != FL_OK) {
    fprintf(stderr, "fl_create: %s\n", fl_last_error(NULL));
    return 1;
  }
  /* a spiral start: radius 10 cbrt(i + 0.5), two golden-ratio-like angles */
  float* pos4 = calloc(4 * (size_t)n, sizeof(float));
  const double pi = 3.14159265358979323846;
  const double r0 = 10.0, ang = pi * (3 - sqrt(5.0)), ang2 = pi * 20 / (9 + sqrt(221.0));
  for (int i = 0; i < n; ++i) {
    const double r = r0 * cbrt(0.5 + i), a = i * ang, b = i * ang2;
    pos4[4 * i + 0] = (float)(r * sin(b) * cos(a));
    pos4[4 * i + 1] = (float)(r * cos(b));
    pos4[4 * i + 2] = (float)(r * sin(b) * sin(a));
  }
  CHECK(fl_set_nodes(sim, n, 3, pos4, NULL, NULL, NULL));
  /* links: a path 0-1-...-(n-1) plus i -> (i + 7) % n */
  const int m = (n - 1) + n;
  int32_t* src = malloc(sizeof(int32_t) * m);
  int32_t* dst = malloc(sizeof(int32_t) * m);
  float* dist = malloc(sizeof(float) * m);
  float* strength = malloc(sizeof(float) * m);
  float* bias = malloc(sizeof(float) * m);
  int* deg = calloc((size_t)n, sizeof(int));
  int k = 0;
  for (int i = 0; i + 1 < n; ++i, ++k) src[k] = i, dst[k] = i + 1;
  for (int i = 0; i < n; ++i, ++k) src[k] = i, dst[k] = (i + 7) % n;
  for (int j = 0; j < m; ++j) ++deg[src[j]], ++deg[dst[j]];
  for (int j = 0; j < m; ++j) {  /* d3's defaults (src/link.js:36-38, :73-75) */
    const int a = deg[src[j]], c = deg[dst[j]];
    dist[j] = 30.f;
    strength[j] = 1.f / (float)(a < c ? a : c);
    bias[j] = (float)a / (float)(a + c);
  }
  float* charge = malloc(sizeof(float) * n);
  for (int i = 0; i < n; ++i) charge[i] = -30.f;
  fl_force_desc d[3] = {{0}};
  d[0].type = FL_FORCE_LINK, d[0].key = 1, d[0].version = 1, d[0].iterations = 1, d[0].m = m;
  d[0].source = src, d[0].target = dst;
  d[0].link_distance = dist, d[0].link_strength = strength, d[0].link_bias = bias;
  d[1].type = FL_FORCE_MANYBODY, d[1].key = 2, d[1].version = 1, d[1].node_a = charge;
  d[1].theta2 = 0.81, d[1].distance_min2 = 1.0, d[1].distance_max2 = INFINITY;
  d[2].type = FL_FORCE_CENTER, d[2].key = 3, d[2].version = 1, d[2].strength = 1.0;
  CHECK(fl_set_forces(sim, 3, d));
  CHECK(fl_set_seed(sim, 7));
  /* d3's alpha schedule (src/simulation.js:28-32, :49-56), velocityDecay 0.4 */
  double* alphas = malloc(sizeof(double) * ticks);
  double alpha = 1.0;
  const double decay = 1 - pow(0.001, 1.0 / 300);
  for (int t = 0; t < ticks; ++t) alpha += (0.0 - alpha) * decay, alphas[t] = alpha;
  CHECK(fl_enqueue(sim, alphas, ticks, 0.6));
  float* out = malloc(sizeof(float) * 4 * (size_t)n);
  CHECK(fl_sync(sim, out, NULL));
  /* the packed readback carries the same x, y, z */
  float* packed = malloc(sizeof(float) * 3 * (size_t)n);
  CHECK(fl_sync_packed(sim, packed, NULL));
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k)
      if (packed[3 * i + k] != out[4 * i + k]) {
        fprintf(stderr, "fl_sync_packed differs from fl_sync at node %d\n", i);
        return 3;
      }
  for (int i = 0; i < n; ++i) printf("%.9g %.9g %.9g\n", out[4 * i], out[4 * i + 1], out[4 * i + 2]);
  fl_destroy(sim);
  free(pos4), free(src), free(dst), free(dist), free(strength), free(bias), free(deg);
  free(charge), free(alphas), free(out), free(packed);
  return 0;
}
