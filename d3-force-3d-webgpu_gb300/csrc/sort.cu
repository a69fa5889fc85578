// Onesweep LSD radix sort of (uint64 key, uint32 value) pairs.
//
// Replaces the reference's three-dispatch-per-digit sort (src/gpu/sort.js:4-20, 139-190) with
// the GB300 form of Adinets & Merrill's "Onesweep" (2022): the digit histograms of every pass
// come from one read of the keys (fused into the key producer where possible); each pass is one
// kernel that ranks a tile of keys (fl_sort_tile) by digit within each warp (eight ballots, one per digit
// bit, give the lanes that share a lane's digit: cheaper here than the match instruction), publishes
// the tile's digit counts, and takes its global offsets from a decoupled look-back over the
// preceding tiles (bounded: a wait gives up after FL_SPIN_LIMIT polls and raises an error bit
// instead of hanging); keys are then staged in shared memory in digit order and written out in
// coalesced runs. Stable: keys of equal digit keep their input order.
#include <atomic>

#include "kernels.h"

namespace {

constexpr uint32_t kValMask = (1u << 30) - 1;
constexpr uint32_t kFlagAgg = 1u << 30;
constexpr uint32_t kFlagPre = 2u << 30;
constexpr int kLook = 8;  // look-back words read per round (within 64 registers)

// Block-wide exclusive scan of one value per thread (kThreads); returns the exclusive prefix,
// and the block total in *total.
template <int kThreads>
__device__ uint32_t block_excl_scan(uint32_t v, uint32_t* s_warp, uint32_t* total) {
  constexpr int kWarps = kThreads / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(FL_FULL, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < kWarps ? s_warp[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(FL_FULL, w, o);
      if (lane >= o) w += y;
    }
    if (lane < kWarps) s_warp[lane] = w;  // inclusive totals of warps
  }
  __syncthreads();
  uint32_t before = (warp ? s_warp[warp - 1] : 0) + x - v;
  *total = s_warp[kWarps - 1];
  __syncthreads();
  return before;
}

__global__ void __launch_bounds__(256) k_hist(const uint64_t* __restrict__ keys, int64_t n,
                                              int lo_bit, int passes, uint32_t* hist) {
  __shared__ uint32_t sh[8 * 256];
  for (int i = threadIdx.x; i < 8 * 256; i += blockDim.x) sh[i] = 0;
  __syncthreads();
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
    int64_t i = base + threadIdx.x;
    bool ok = i < n;
    uint64_t k = ok ? keys[i] : 0;
    for (int p = 0; p < passes; ++p)
      fl::hist_add(sh + p * 256, (uint32_t)(k >> (lo_bit + 8 * p)) & 255u, ok);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < passes * 256; i += blockDim.x)
    if (sh[i]) atomicAdd(&hist[i], sh[i]);
}

// The lanes of the warp whose digit equals this lane's (d < 256), or this lane alone (!valid).
__device__ __forceinline__ uint32_t match_digit(uint32_t d, bool valid) {
  uint32_t m = __ballot_sync(FL_FULL, valid);
#pragma unroll
  for (int b = 0; b < 8; ++b) {
    const uint32_t v = __ballot_sync(FL_FULL, (d >> b) & 1u);
    m &= ((d >> b) & 1u) ? v : ~v;
  }
  return valid ? m : (1u << (threadIdx.x & 31));
}

template <int kThreads, int kItems>
__global__ void __launch_bounds__(kThreads, 1024 / kThreads) k_onesweep(
    const uint64_t* __restrict__ kin, const uint32_t* __restrict__ vin, uint64_t* __restrict__ kout,
    uint32_t* __restrict__ vout, int64_t n, int shift, const uint32_t* __restrict__ ghist,
    uint32_t* status, uint32_t* ticket, uint32_t* err, uint32_t spin_limit, int hold) {
  constexpr int kWarps = kThreads / 32, kTile = kThreads * kItems;
  extern __shared__ __align__(16) unsigned char smem[];
  uint64_t* sk = reinterpret_cast<uint64_t*>(smem);
  uint32_t* sv = reinterpret_cast<uint32_t*>(sk + kTile);
  __shared__ uint32_t s_whist[kWarps][256];
  __shared__ uint32_t s_gexcl[256];
  __shared__ uint32_t s_texcl[256];
  __shared__ uint32_t s_base[256];
  __shared__ uint32_t s_warp[kWarps];
  __shared__ uint32_t s_fall[256];
  __shared__ uint32_t s_tile;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) s_tile = atomicAdd(ticket, 1u);
  for (int i = tid; i < kWarps * 256; i += kThreads) (&s_whist[0][0])[i] = 0;
  uint32_t total;
  // digit-wise phases: threads 0..255 take one digit each (a block of 256 or more threads)
  const bool dt = tid < 256;
  const uint32_t gh = dt ? ghist[tid] : 0u;
  __syncthreads();
  const uint32_t tile = s_tile;
  const int64_t tbase = (int64_t)tile * kTile;

  uint64_t key[kItems];
  uint32_t val[kItems], dig[kItems], rank[kItems];
  const int64_t wbase = tbase + (int64_t)warp * (32 * kItems);
#pragma unroll
  for (int j = 0; j < kItems; ++j) {
    int64_t idx = wbase + j * 32 + lane;
    if (idx < n) {
      key[j] = kin[idx];
      val[j] = vin[idx];
      dig[j] = (uint32_t)(key[j] >> shift) & 255u;
    } else {
      key[j] = 0;
      val[j] = 0;
      dig[j] = 256u + lane;  // unique: ranked alone, never stored
    }
  }
  // the digits' global offsets, while the keys are on their way (a scan has barriers, which
  // would otherwise hold the loads back)
  const uint32_t gx = block_excl_scan<kThreads>(gh, s_warp, &total);  // syncs inside
  if (dt) s_gexcl[tid] = gx;
  const uint32_t lt = fl::lanemask_lt();
#pragma unroll
  for (int j = 0; j < kItems; ++j) {
    uint32_t peers = match_digit(dig[j], dig[j] < 256u);
    int leader = 31 - __clz(peers);
    uint32_t before = 0;
    if (lane == leader && dig[j] < 256u) {
      before = s_whist[warp][dig[j]];
      s_whist[warp][dig[j]] = before + __popc(peers);
    }
    before = __shfl_sync(FL_FULL, before, leader);
    rank[j] = before + __popc(peers & lt);
    __syncwarp();
  }
  __syncthreads();

  // per digit: exclusive prefix over warps, the tile's count
  const uint32_t d = dt ? (uint32_t)tid : 0u;
  uint32_t run = 0;
  uint32_t* mine = status + (size_t)tile * 256 + d;
  if (dt) {
#pragma unroll
    for (int w = 0; w < kWarps; ++w) {
      uint32_t t = s_whist[w][d];
      s_whist[w][d] = run;
      run += t;
    }
    // `hold` (a test of the bounded wait): tile 0 keeps its counts to itself in this pass
    if (!(hold && tile == 0)) fl::st_relaxed(mine, (tile == 0 ? kFlagPre : kFlagAgg) | run);
  }
  const uint32_t tx = block_excl_scan<kThreads>(run, s_warp, &total);
  if (dt) s_texcl[d] = tx;

  uint32_t prefix = 0;
  bool gave_up = false;
  if (dt && tile > 0) {
    // look back kLook tiles per round (independent loads), up to the nearest inclusive prefix:
    // all tiles of a pass start at once and publish their counts together, so the inclusive
    // prefixes spread from tile 0 while the last tiles walk back to meet them; a wide round
    // shortens that walk
    int64_t p = (int64_t)tile - 1;
    uint32_t spins = 0;
    for (;;) {
      uint32_t w[kLook];
#pragma unroll
      for (int k = 0; k < kLook; ++k)
        w[k] = p - k >= 0 ? fl::ld_relaxed(status + (size_t)(p - k) * 256 + d) : kFlagPre;
      int used = 0;
      bool done = false;
#pragma unroll
      for (int k = 0; k < kLook; ++k) {
        if (done || used < k) break;
        const uint32_t f = w[k] & ~kValMask;
        if (f == 0) break;  // not published yet: wait for it
        prefix += w[k] & kValMask;
        used = k + 1;
        done = f == kFlagPre;
      }
      if (done) break;
      if (used == 0) {
        if (++spins > spin_limit) {
          gave_up = true;
          break;
        }
        if (spins > 64) __nanosleep(100);
        continue;
      }
      p -= used;
    }
    if (!gave_up) fl::st_relaxed(mine, kFlagPre | (prefix + run));
  }
  if (dt) s_base[d] = s_gexcl[d] + prefix - s_texcl[d];
  if (__syncthreads_or(gave_up)) {
    // a wait gave up (a predecessor tile never published): the block counts the digits of every
    // key before its tile itself, reading the pass's input, which is complete. Slower, still
    // exact; the error bit reports that the wait gave up.
    if (tid < 256) s_fall[tid] = 0u;
    __syncthreads();
    for (int64_t i = tid; i < tbase; i += kThreads) atomicAdd(&s_fall[(uint32_t)(kin[i] >> shift) & 255u], 1u);
    __syncthreads();
    if (dt) {
      prefix = s_fall[d];
      s_base[d] = s_gexcl[d] + prefix - s_texcl[d];
      fl::st_relaxed(mine, kFlagPre | (prefix + run));
    }
    if (tid == 0) atomicOr(err, FL_ERR_LOOKBACK);
    __syncthreads();
  }

#pragma unroll
  for (int j = 0; j < kItems; ++j) {
    if (dig[j] < 256u) {
      uint32_t pos = s_texcl[dig[j]] + s_whist[warp][dig[j]] + rank[j];
      sk[pos] = key[j];
      sv[pos] = val[j];
    }
  }
  __syncthreads();
  const int valid = (int)((n - tbase) < kTile ? (n - tbase) : kTile);
  for (int i = tid; i < valid; i += kThreads) {
    uint64_t k = sk[i];
    uint32_t g = s_base[(uint32_t)(k >> shift) & 255u] + (uint32_t)i;
    if (g < (uint64_t)n) {  // always true: a guard against a corrupted histogram
      kout[g] = k;
      vout[g] = sv[i];
    }
  }
}

// ---- the run fix-up after a sort of the top key bits only
//
// Onesweep passes over the key bits [lo_sort, 64) leave the pairs ordered by those bits and, among
// equal ones, by value (the passes are stable and the values start as 0, 1, 2, ...). A run of keys
// equal above lo_sort is then put in (key, value) order, which makes the result that of the full
// sort on [lo_bit, 64). Such runs are rare and short for Morton keys of a layout's points: the top
// 32 bits resolve cells of 1/1600 of the cube's side. A run of up to kRunShort pairs is ranked by
// each of its threads counting the pairs before its own; a longer one is recorded, and the last
// block to finish sorts each recorded run by LSD passes of its own (no wait on other blocks: the
// last block is the one that finds every other block done).
constexpr int kRunThreads = 256;
constexpr int kRunShort = 1024;

__device__ __forceinline__ bool pair_less(uint64_t ka, uint32_t va, uint64_t kb, uint32_t vb) {
  return ka < kb || (ka == kb && va < vb);
}

// One CTA: a stable LSD sort of the pairs [0, L) of (ka, va) on the key bits [lo_bit, hi_bit),
// ping-ponging with (kb, vb); the result ends in (ka, va)'s place when `in_a`, else in (kb, vb).
__device__ void cta_sort_run(uint64_t* ka, uint32_t* va, uint64_t* kb, uint32_t* vb, int64_t L,
                             int lo_bit, int hi_bit, uint32_t* s_cnt, uint32_t* s_w) {
  constexpr int kW = kRunThreads / 32;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t lt = fl::lanemask_lt();
  uint64_t* ks = ka;
  uint32_t* vs = va;
  uint64_t* kd = kb;
  uint32_t* vd = vb;
  for (int shift = lo_bit; shift < hi_bit; shift += 8) {
    const uint32_t dmask = (1u << (hi_bit - shift < 8 ? hi_bit - shift : 8)) - 1u;
    for (int i = tid; i < 256; i += kRunThreads) s_cnt[i] = 0;
    __syncthreads();
    for (int64_t i = tid; i < L; i += kRunThreads) atomicAdd(&s_cnt[(uint32_t)(ks[i] >> shift) & dmask], 1u);
    __syncthreads();
    if (tid == 0) {  // exclusive offsets (a fallback path: a serial scan is enough)
      uint32_t run = 0;
      for (int d = 0; d < 256; ++d) {
        const uint32_t c = s_cnt[d];
        s_cnt[d] = run;
        run += c;
      }
    }
    __syncthreads();
    for (int64_t base = 0; base < L; base += kRunThreads) {
      const int64_t i = base + tid;
      const bool ok = i < L;
      const uint64_t k = ok ? ks[i] : 0;
      const uint32_t v = ok ? vs[i] : 0;
      const uint32_t d = ok ? (uint32_t)(k >> shift) & dmask : 256u + (uint32_t)lane;
      for (int j = tid; j < kW * 256; j += kRunThreads) s_w[j] = 0;
      __syncthreads();
      const uint32_t peers = __match_any_sync(FL_FULL, d);
      if (ok && (peers & lt) == 0) s_w[warp * 256 + d] = __popc(peers);
      __syncthreads();
      if (ok) {
        uint32_t pos = s_cnt[d] + __popc(peers & lt);
        for (int w = 0; w < warp; ++w) pos += s_w[w * 256 + d];
        kd[pos] = k;
        vd[pos] = v;
      }
      __syncthreads();
      for (int dd = tid; dd < 256; dd += kRunThreads) {
        uint32_t c = 0;
        for (int w = 0; w < kW; ++w) c += s_w[w * 256 + dd];
        s_cnt[dd] += c;
      }
      __syncthreads();
    }
    uint64_t* tk = ks;
    ks = kd, kd = tk;
    uint32_t* tv = vs;
    vs = vd, vd = tv;
  }
  if (ks != kb) {  // the result must end in (kb, vb)
    for (int64_t i = tid; i < L; i += kRunThreads) kb[i] = ks[i], vb[i] = vs[i];
    __syncthreads();
  }
}

// counters[1]: long runs recorded in longs[] (k_longruns sorts them and resets the count).
__global__ void __launch_bounds__(kRunThreads) k_runfix(
    const uint64_t* __restrict__ kin, const uint32_t* __restrict__ vin, uint64_t* __restrict__ kout,
    uint32_t* __restrict__ vout, int64_t n, int lo_sort, uint32_t* counters, uint32_t* longs,
    uint32_t longs_cap) {
  for (int64_t i = (int64_t)blockIdx.x * kRunThreads + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kRunThreads) {
    const uint64_t k = kin[i];
    const uint32_t v = vin[i];
    const uint64_t h = k >> lo_sort;
    const bool prev = i > 0 && (kin[i - 1] >> lo_sort) == h;
    const bool next = i + 1 < n && (kin[i + 1] >> lo_sort) == h;
    if (!prev && !next) {
      kout[i] = k, vout[i] = v;
    } else {
      int64_t s = i, e = i + 1;
      while (s > 0 && i - s < kRunShort && (kin[s - 1] >> lo_sort) == h) --s;
      while (e < n && e - s <= kRunShort && (kin[e] >> lo_sort) == h) ++e;
      const bool open = (s > 0 && (kin[s - 1] >> lo_sort) == h) || (e < n && (kin[e] >> lo_sort) == h);
      if (!open) {  // a short run: this pair's place is the run's start plus the pairs before it
        uint32_t r = 0;
        for (int64_t j = s; j < e; ++j) r += pair_less(kin[j], vin[j], k, v);
        kout[s + r] = k, vout[s + r] = v;
      } else if (!prev) {  // a long run's first pair records it
        const uint32_t slot = atomicAdd(&counters[1], 1u);
        if (slot < longs_cap) longs[slot] = (uint32_t)i;
      }
    }
  }
}

// One block: the long runs k_runfix recorded, each sorted on the bits below lo_sort (none, in
// the common case: the block reads the count and returns). Leaves the count at zero.
__global__ void __launch_bounds__(kRunThreads) k_longruns(
    uint64_t* __restrict__ kin, uint32_t* __restrict__ vin, uint64_t* __restrict__ kout,
    uint32_t* __restrict__ vout, int64_t n, int lo_bit, int lo_sort, uint32_t* counters,
    const uint32_t* longs, uint32_t longs_cap) {
  __shared__ uint32_t s_cnt[256];
  __shared__ uint32_t s_w[(kRunThreads / 32) * 256];
  const uint32_t count = counters[1];
  if (count == 0) return;
  for (uint32_t r = 0; r < count && r < longs_cap; ++r) {
    const int64_t s = longs[r];
    const uint64_t h = kin[s] >> lo_sort;
    // the run's end: the first pair past s whose top bits differ
    __shared__ unsigned long long s_end;
    if (threadIdx.x == 0) s_end = (unsigned long long)n;
    __syncthreads();
    for (int64_t base = s + 1; base < n; base += kRunThreads) {
      const int64_t j = base + threadIdx.x;
      if (j < n && (kin[j] >> lo_sort) != h) atomicMin(&s_end, (unsigned long long)j);
      if (__syncthreads_or(j < n && (kin[j] >> lo_sort) != h)) break;
    }
    const int64_t L = (int64_t)s_end - s;
    cta_sort_run(kin + s, vin + s, kout + s, vout + s, L, lo_bit, lo_sort, s_cnt, s_w);
    __syncthreads();
  }
  if (threadIdx.x == 0) counters[1] = 0u;
}

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

int64_t tiles_for(int64_t n) {
  const int64_t t = fl_sort_tile(n);
  return (n + t - 1) / t;
}
int64_t tiles_cap_for(int64_t cap) { return (cap + kSortTileSmall - 1) / kSortTileSmall; }

// True the first time it is called on the current device for `done` (a kernel's shared-memory
// limit is raised once per device, and on the first launch, which is never inside a capture).
static bool first_on_device(std::atomic<uint64_t>& done) {
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return true;
  const uint64_t bit = 1ull << dev;
  return !(done.fetch_or(bit) & bit);
}

template <int T, int I>
void launch_pass(const uint64_t* kin, const uint32_t* vin, uint64_t* kout, uint32_t* vout,
                 int64_t n, int shift, const uint32_t* ghist, uint32_t* status, uint32_t* ticket,
                 uint32_t* err, uint32_t spin_limit, int hold, cudaStream_t st) {
  static std::atomic<uint64_t> configured{0};
  const size_t dyn = (size_t)T * I * 12;
  if (first_on_device(configured))
    cudaFuncSetAttribute(k_onesweep<T, I>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
  const int64_t tiles = (n + T * I - 1) / (T * I);
  k_onesweep<T, I><<<(int)tiles, T, dyn, st>>>(kin, vin, kout, vout, n, shift, ghist, status,
                                               ticket, err, spin_limit, hold);
}
uint32_t longs_cap_for(int64_t n) { return (uint32_t)(n / (kRunShort + 1) + 1); }

constexpr int kRankWarps = 8;

// The stable sort of up to kSortRankMax pairs in one launch, for the tree of a small layout,
// where the digit passes and the run fix-up are five launches over a few thousand keys. A pair's
// place is the number of smaller keys plus the number of equal keys before it in the input.
// Block b places pairs 32 b .. 32 b + 31: the block copies every key to shared memory
// (coalesced), then lane l of every warp holds pair 32 b + l and counts over one kRankWarps-th
// of the keys (the same key in every lane: a broadcast read); the warps' counts are summed in
// shared memory.
__global__ void __launch_bounds__(kRankWarps * 32) k_ranksort(const uint64_t* __restrict__ keys,
                                                              const uint32_t* __restrict__ vals,
                                                              int n, uint64_t* __restrict__ okeys,
                                                              uint32_t* __restrict__ ovals) {
  extern __shared__ uint64_t s_keys[];  // [n]
  __shared__ uint32_t s_rank[kRankWarps][32];
  for (int j = threadIdx.x; j < n; j += kRankWarps * 32) s_keys[j] = keys[j];
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int i = blockIdx.x * 32 + lane;
  const uint64_t k = i < n ? s_keys[i] : ~0ull;
  const int per = (n + kRankWarps - 1) / kRankWarps;
  const int j0 = min(n, w * per), j1 = min(n, j0 + per);
  uint32_t rank = 0;
#pragma unroll 8
  for (int j = j0; j < j1; ++j) {
    const uint64_t kj = s_keys[j];
    rank += (uint32_t)((kj < k) | ((kj == k) & (j < i)));
  }
  s_rank[w][lane] = rank;
  __syncthreads();
  if (w == 0 && i < n) {
    uint32_t r = 0;
#pragma unroll
    for (int q = 0; q < kRankWarps; ++q) r += s_rank[q][lane];
    okeys[r] = k;
    ovals[r] = vals[i];
  }
}

}  // namespace

// Keys per thread of a pass's tiles of 1024 threads: as few as fill every SM with one tile (the
// pass then takes one wave, each tile's time growing with its keys), from 5 up to 8 (beyond
// 152 SMs x 8 x 1024 = 1.2 M keys, more than one wave of the largest tiles).
static int sort_items(int64_t n) {
  const int64_t per_sm = (int64_t)fl_sms() * kSortThreads;
  int64_t it = (n + per_sm - 1) / per_sm;
  return it < 5 ? 5 : it > kSortItems ? kSortItems : (int)it;
}

int fl_sort_tile(int64_t n) {
  return n <= kSortSmallMax ? kSortTileSmall : kSortThreads * sort_items(n);
}

// The SM count of the current device, queried once per device index. The cache entries are
// atomics: threads that race on a device's first query store the same value.
int fl_sms() {
  constexpr int kMaxDevices = 64;
  static std::atomic<int> cache[kMaxDevices];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    dev = -1;
  }
  if (dev >= 0 && dev < kMaxDevices) {
    const int c = cache[dev].load(std::memory_order_relaxed);
    if (c > 0) return c;
  }
  int v = 0;
  const int sms = dev >= 0 && cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && v > 0 ? v : 1;
  if (dev >= 0 && dev < kMaxDevices && v > 0) cache[dev].store(sms, std::memory_order_relaxed);
  return sms;
}

size_t fl_sort_bytes(int64_t n) {
  int64_t cap = n > 0 ? n : 1, tiles = tiles_cap_for(cap);
  return 2 * align256(8 * (size_t)cap) + 2 * align256(4 * (size_t)cap) + align256(8 * 256 * 4) +
         align256(kSortCounters * 4) + align256(8 * (size_t)tiles * 256 * 4) +
         align256(4 * (size_t)longs_cap_for(cap));
}

// hist, counters and the look-back words in that order: one memset clears what a sort uses
void fl_sort_carve(FlSortBufs* b, void* base, int64_t n) {
  int64_t cap = n > 0 ? n : 1, tiles = tiles_cap_for(cap);
  char* p = static_cast<char*>(base);
  for (int i = 0; i < 2; ++i) b->keys[i] = reinterpret_cast<uint64_t*>(p), p += align256(8 * (size_t)cap);
  for (int i = 0; i < 2; ++i) b->vals[i] = reinterpret_cast<uint32_t*>(p), p += align256(4 * (size_t)cap);
  b->hist = reinterpret_cast<uint32_t*>(p), p += align256(8 * 256 * 4);
  b->counters = reinterpret_cast<uint32_t*>(p), p += align256(kSortCounters * 4);
  b->status = reinterpret_cast<uint32_t*>(p), p += align256(8 * (size_t)tiles * 256 * 4);
  b->longs = reinterpret_cast<uint32_t*>(p);
  b->longs_cap = longs_cap_for(cap);
  b->cap = cap;
  b->tiles_cap = tiles;
  b->test_spins = 0;
}

void fl_sort_reset(const FlSortBufs* b, int64_t n, int passes, cudaStream_t st) {
  const int64_t tiles = tiles_for(n > 0 ? n : 1);
  const char* a = reinterpret_cast<const char*>(b->hist);
  const char* e = reinterpret_cast<const char*>(b->status + (size_t)passes * tiles * 256);
  cudaMemsetAsync(b->hist, 0, (size_t)(e - a), st);
}

void fl_sort_histogram(const FlSortBufs* b, int64_t n, int lo_bit, cudaStream_t st,
                       int64_t* launches) {
  int passes = (64 - lo_bit + 7) / 8;
  int64_t blocks = (n + 255) / 256;
  if (blocks > 4 * fl_sms()) blocks = 4 * fl_sms();
  if (blocks < 1) blocks = 1;
  k_hist<<<(int)blocks, 256, 0, st>>>(b->keys[0], n, lo_bit, passes, b->hist);
  ++*launches;
}

int fl_sort_passes(const FlSortBufs* b, int64_t n, int lo_bit, uint32_t* err, cudaStream_t st,
                   int64_t* launches) {
  int passes = (64 - lo_bit + 7) / 8;
  int cur = 0;
  if (n <= 0) return 0;
  const int64_t tiles = tiles_for(n);
  // the test of the bounded wait (b->test_spins > 0): the first pass withholds tile 0's counts
  const uint32_t limit = b->test_spins ? b->test_spins : FL_SPIN_LIMIT;
  for (int p = 0; p < passes; ++p) {
    uint32_t* status = b->status + (size_t)p * tiles * 256;
    const int hold = b->test_spins && p == 0;
#define FL_PASS(T, I)                                                                          \
  launch_pass<T, I>(b->keys[cur], b->vals[cur], b->keys[1 - cur], b->vals[1 - cur], n,            \
                    lo_bit + 8 * p, b->hist + p * 256, status, b->counters + p, err, limit, hold, st)
    switch (fl_sort_tile(n)) {
      case kSortTileSmall: FL_PASS(kSortThreadsSmall, kSortItems); break;
      case 5 * kSortThreads: FL_PASS(kSortThreads, 5); break;
      case 6 * kSortThreads: FL_PASS(kSortThreads, 6); break;
      case 7 * kSortThreads: FL_PASS(kSortThreads, 7); break;
      default: FL_PASS(kSortThreads, 8); break;
    }
#undef FL_PASS
    ++*launches;
    cur = 1 - cur;
  }
  return cur;
}

int fl_sort_rank(const FlSortBufs* b, int64_t n, cudaStream_t st, int64_t* launches) {
  if (n <= 0 || n > kSortRankMax) return 0;
  static std::atomic<uint64_t> configured{0};
  if (first_on_device(configured))
    cudaFuncSetAttribute(k_ranksort, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)(kSortRankMax * sizeof(uint64_t)));
  k_ranksort<<<(int)((n + 31) / 32), kRankWarps * 32, (size_t)n * sizeof(uint64_t), st>>>(
      b->keys[0], b->vals[0], (int)n, b->keys[1], b->vals[1]);
  ++*launches;
  return 1;
}

int fl_sort_split(int lo_bit, int passes) {
  const int full = (64 - lo_bit + 7) / 8;
  if (passes <= 0) passes = 4;
  return passes >= full ? lo_bit : lo_bit + 8 * (full - passes);
}

int fl_sort_runfix(const FlSortBufs* b, int64_t n, int lo_bit, int lo_sort, int cur,
                   cudaStream_t st, int64_t* launches) {
  if (n <= 0 || lo_sort <= lo_bit) return cur;
  int64_t blocks = (n + kRunThreads - 1) / kRunThreads;
  if (blocks > 8 * (int64_t)fl_sms()) blocks = 8 * (int64_t)fl_sms();  // one full wave
  k_runfix<<<(unsigned)blocks, kRunThreads, 0, st>>>(b->keys[cur], b->vals[cur], b->keys[1 - cur],
                                                     b->vals[1 - cur], n, lo_sort, b->counters + 8,
                                                     b->longs, b->longs_cap);
  k_longruns<<<1, kRunThreads, 0, st>>>(b->keys[cur], b->vals[cur], b->keys[1 - cur],
                                        b->vals[1 - cur], n, lo_bit, lo_sort, b->counters + 8,
                                        b->longs, b->longs_cap);
  *launches += 2;
  return 1 - cur;
}
