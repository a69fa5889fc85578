// fl_radix_sort_noalloc: the engine's radix sort for callers that cannot allocate device memory.
//
// Who needs it: code that owns every byte of device memory through its own pool or budget (a
// renderer or game engine whose allocator is fixed at start-up, a plugin host that hands out
// device buffers), code running where cudaMalloc/cudaFree would synchronise the device and
// stall other work, and code that must not fail with an out-of-memory error halfway through a
// frame. Such a caller passes device buffers it already owns; this entry point needs no more.
//
// How: the sort's scratch (one key/value ping-pong buffer, the digit histograms, the look-back
// words, the tile tickets and an error word) lives in one file-scope __device__ array of
// kScratchBytes, which the CUDA runtime places on every device that loads this library and
// keeps until the process exits. Its host-side name is only a stand-in for the device symbol,
// so every call looks the device address up with cudaGetSymbolAddress, with the caller's device
// (and context) current. The address belongs to the context that loaded the module, so it is
// not cached: after cudaDeviceReset, or under a host that makes its own driver-API context
// current, a cached address would point into memory the current context does not map. The
// lookup allocates nothing. The caller's output buffers are the other half of the ping-pong.
#include <cuda_runtime.h>

#include <string>

#include "../../include/forcegpu.h"
#include "kernels.h"

void fl_set_sim_free_error(const std::string& msg);  // engine.cu: the message of fl_last_error(NULL)

namespace {

constexpr int64_t kMaxPairs = FL_SORT_NOALLOC_MAX_PAIRS;
constexpr int64_t kTile = kSortTileSmall;  // the smallest onesweep tile: the most tiles
constexpr int64_t kTiles = (kMaxPairs + kTile - 1) / kTile;
constexpr size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t kErrOff = 0;
constexpr size_t kKeysOff = 256;
constexpr size_t kValsOff = kKeysOff + a256(8 * (size_t)kMaxPairs);
constexpr size_t kHistOff = kValsOff + a256(4 * (size_t)kMaxPairs);
constexpr size_t kStatusOff = kHistOff + a256(8 * 256 * 4);
constexpr size_t kCountersOff = kStatusOff + a256(8 * (size_t)kTiles * 256 * 4);
constexpr size_t kScratchBytes = kCountersOff + 256;  // 3.6 MB for 262,144 pairs

static __device__ __align__(256) unsigned char g_sort_scratch[kScratchBytes];

int32_t fail(int32_t code, const std::string& msg) {
  fl_set_sim_free_error("fl_radix_sort_noalloc: " + msg);
  return code;
}

int32_t cuda_fail(cudaError_t e, const char* what) {
  cudaGetLastError();
  return fail(FL_E_DEVICE, std::string(what) + ": " + cudaGetErrorString(e));
}

// The device address of the scratch array in the current context (the current device's,
// unless the host made another context current). Looked up on every call, never cached.
int32_t scratch_of_current_context(char** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_sort_scratch);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress");
  if (!p) return fail(FL_E_DEVICE, "cudaGetSymbolAddress returned no address");
  *out = static_cast<char*>(p);
  return FL_OK;
}

bool overlap(const void* a, size_t an, const void* b, size_t bn) {
  const char *x = static_cast<const char*>(a), *y = static_cast<const char*>(b);
  return x < y + bn && y < x + an;
}

}  // namespace

extern "C" int32_t fl_radix_sort_noalloc(const uint64_t* keys, const uint32_t* vals, int64_t n,
                                         int32_t lo_bit, uint64_t* keys_out, uint32_t* vals_out,
                                         void* stream) {
  if (n < 0 || lo_bit < 0 || lo_bit > 63) return fail(FL_E_ARG, "bad arguments");
  if (n > kMaxPairs)
    return fail(FL_E_ARG, "n = " + std::to_string(n) + " exceeds the maximum of " +
                              std::to_string(kMaxPairs) + " pairs (FL_SORT_NOALLOC_MAX_PAIRS)");
  if (n == 0) return FL_OK;
  if (!keys || !vals || !keys_out || !vals_out) return fail(FL_E_ARG, "null buffer");
  const size_t kb = 8 * (size_t)n, vb = 4 * (size_t)n;
  // the keys are copied to keys_out before the values to vals_out, so keys_out may not overlap
  // vals (nor, for the same reason the other way round, vals_out the keys); only identical
  // buffers may coincide: a sort in place
  if ((keys != keys_out && overlap(keys, kb, keys_out, kb)) ||
      (vals != vals_out && overlap(vals, vb, vals_out, vb)) || overlap(keys_out, kb, vals_out, vb) ||
      overlap(keys_out, kb, vals, vb) || overlap(vals_out, vb, keys, kb))
    return fail(FL_E_ARG, "input and output buffers overlap (only identical, in-place buffers may)");
  char* base = nullptr;
  int32_t rc = scratch_of_current_context(&base);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  uint32_t* err = reinterpret_cast<uint32_t*>(base + kErrOff);
  FlSortBufs sb{};
  sb.keys[0] = keys_out;
  sb.vals[0] = vals_out;
  sb.keys[1] = reinterpret_cast<uint64_t*>(base + kKeysOff);
  sb.vals[1] = reinterpret_cast<uint32_t*>(base + kValsOff);
  sb.hist = reinterpret_cast<uint32_t*>(base + kHistOff);
  sb.status = reinterpret_cast<uint32_t*>(base + kStatusOff);
  sb.counters = reinterpret_cast<uint32_t*>(base + kCountersOff);
  sb.longs = nullptr;  // no run fix-up: every digit pass runs
  sb.longs_cap = 0;
  sb.cap = n;
  sb.tiles_cap = kTiles;
  int64_t launches = 0;
  cudaError_t e;
  // every call shares the scratch and finds the last call's contents: the error word, the
  // histograms, the look-back words and the tickets must start at zero
  if ((e = cudaMemsetAsync(err, 0, 4, st)) != cudaSuccess ||
      (e = cudaMemsetAsync(base + kHistOff, 0, kScratchBytes - kHistOff, st)) != cudaSuccess)
    return cuda_fail(e, "cudaMemsetAsync");
  if (keys != keys_out && (e = cudaMemcpyAsync(keys_out, keys, kb, cudaMemcpyDeviceToDevice, st)) != cudaSuccess)
    return cuda_fail(e, "cudaMemcpyAsync");
  if (vals != vals_out && (e = cudaMemcpyAsync(vals_out, vals, vb, cudaMemcpyDeviceToDevice, st)) != cudaSuccess)
    return cuda_fail(e, "cudaMemcpyAsync");
  fl_sort_histogram(&sb, n, lo_bit, st, &launches);
  const int r = fl_sort_passes(&sb, n, lo_bit, err, st, &launches);
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "sort launch");
  if (r == 1) {  // an odd number of digit passes ends in the scratch half
    if ((e = cudaMemcpyAsync(keys_out, sb.keys[1], kb, cudaMemcpyDeviceToDevice, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(vals_out, sb.vals[1], vb, cudaMemcpyDeviceToDevice, st)) != cudaSuccess)
      return cuda_fail(e, "cudaMemcpyAsync");
  }
  uint32_t w = 0;
  if ((e = cudaMemcpyAsync(&w, err, 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return cuda_fail(e, "readback of the error word");
  if (w) return fail(FL_E_TIMEOUT, "a device-side look-back wait gave up");
  return FL_OK;
}
