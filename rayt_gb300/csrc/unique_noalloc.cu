// rayt_feedback_unique_noalloc: the feedback compaction + radix sort + unique
// of rayt_feedback_unique, for callers that must not see the library allocate.
//
// Who needs it: a host application that owns all device memory through its
// own allocator or a fixed up-front reservation (a renderer or server that
// carves HBM into pools at start-up and treats any other cudaMalloc as a
// budget violation), and frame loops that cannot afford cudaMalloc/cudaFree
// at run time (cudaFree waits for the whole device, which stalls every stream
// in flight).  rayt_feedback_unique grows a per-device scratch buffer with
// cudaMalloc on first use or when a larger n arrives; this entry point instead
// works in a fixed scratch area that lives in this file as a __device__ array.
//
// Limits and sharing:
//  * n is at most RAYT_FEEDBACK_UNIQUE_NOALLOC_MAX_WORDS (2^21 words, enough
//    for the feedback of one 1920x1080 frame); larger n is rejected with
//    RAYT_E_LIMIT before any GPU work.  The array is about 17 MiB and every
//    GPU that loads the library holds it until the process exits.
//  * Every call on a device uses the same array, so two calls whose GPU work
//    overlaps race and both results are undefined.  Calls through this entry
//    point take the library's primitives lock and return only after their
//    stream has finished, so calls from several host threads are serialised
//    like rayt_sort_i32 / rayt_scan_i32 / rayt_feedback_unique, with which
//    they also share the device error flag and the look-back epoch.  GPU work
//    the caller queued on other streams that reads or writes the array is not
//    ordered by the library.  The array keeps the previous call's contents;
//    every part the kernels expect to start at zero is cleared by each call.
//  * The first call on each device looks up the array's device address with
//    cudaGetSymbolAddress (with that device current) and zeroes the array on
//    the caller's stream, ordered before that call's kernels; make that first
//    call before any stream capture.
// No cudaMalloc, cudaFree or allocating library routine is called here.
#include <mutex>

#include "internal.h"

namespace rayt {
namespace {

constexpr int kMaxWords = RAYT_FEEDBACK_UNIQUE_NOALLOC_MAX_WORDS;
constexpr size_t kCountsBytes = 256;

// Sort/unique scratch for kMaxWords words plus 256 bytes for the result count.
// feedback_scratch_bytes() is a host function, so the size is computed from the
// same layout rules here: two key arrays of (n + 4) words rounded to 256 bytes,
// 6 x 256 histogram words, one 8-byte look-back word per 256 buckets per
// 4096-key tile (+1 tile), 16 tile counters, 4 counts, 8 key-range words and
// 256 partition cursors 128 bytes apart, each rounded to 256 bytes.
constexpr size_t Up256(size_t v) { return (v + 255) & ~(size_t)255; }
constexpr size_t kTiles = ((size_t)kMaxWords + 4095) / 4096 + 1;
constexpr size_t kScratchBytes = 2 * Up256((size_t)kMaxWords * 4 + 16) + Up256(6 * 256 * 4) +
                                 Up256(kTiles * 256 * 8) + Up256(16 * 4) + Up256(4 * 4) + Up256(8 * 4) +
                                 Up256(256 * 32 * 4);

static __device__ __align__(256) uint8_t g_noalloc_scratch[kScratchBytes + kCountsBytes];

void* g_scratch_ptr[64];

// Device address of g_noalloc_scratch on the current device (looked up once;
// the caller holds prims_mutex()).  The first lookup zeroes the array on the
// caller's stream s, so the zeroing is ordered before that call's kernels even
// when s does not synchronise with the legacy default stream.
int scratch_address(void** out, cudaStream_t s) {
  int dev = 0;
  RAYT_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(RAYT_E_ARG, "device ordinal out of range");
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    RAYT_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    // the sort's look-back words are epoch-tagged, never cleared: start from zeros
    RAYT_CUDA_TRY(cudaMemsetAsync(p, 0, sizeof(g_noalloc_scratch), s));
    register_lookback_area(p, sizeof(g_noalloc_scratch));
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return RAYT_OK;
}

}  // namespace
}  // namespace rayt

extern "C" int rayt_feedback_unique_noalloc(const int32_t* words, int n, int nodes_in_block, int32_t* unique,
                                            int* unique_count, void* stream) {
  using rayt::fail;
  if (n < 0 || !unique_count || (n > 0 && (!words || !unique)) || nodes_in_block < 0)
    return fail(RAYT_E_ARG, "rayt_feedback_unique_noalloc: bad arguments");
  if (n > rayt::kMaxWords)
    return fail(RAYT_E_LIMIT, "rayt_feedback_unique_noalloc: n exceeds RAYT_FEEDBACK_UNIQUE_NOALLOC_MAX_WORDS (2^21)");
  if (n == 0) {
    *unique_count = 0;
    return RAYT_OK;
  }
  if (rayt::feedback_scratch_bytes(n) > rayt::kScratchBytes)
    return fail(RAYT_E_LIMIT, "rayt_feedback_unique_noalloc: scratch layout larger than the static area");
  std::lock_guard<std::mutex> lock(rayt::prims_mutex());
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  void* base = nullptr;
  int rc = rayt::scratch_address(&base, s);
  if (rc != RAYT_OK) return rc;
  if ((rc = rayt::lookback_epoch_step(s)) != RAYT_OK) return rc;
  int* counts = reinterpret_cast<int*>(static_cast<uint8_t*>(base) + rayt::kScratchBytes);
  // the launcher clears the histograms, tile counters and counts it relies on
  RAYT_CUDA_TRY(rayt::feedback_unique_device(words, n, nodes_in_block, unique, counts, base, rayt::kScratchBytes, s));
  int host = 0;
  RAYT_CUDA_TRY(cudaMemcpyAsync(&host, counts, sizeof(int), cudaMemcpyDeviceToHost, s));
  RAYT_CUDA_TRY(cudaStreamSynchronize(s));
  int flag = 0;
  RAYT_CUDA_TRY(cudaMemcpy(&flag, rayt::device_error_flag(), sizeof(int), cudaMemcpyDeviceToHost));
  if (flag) {
    const int zero = 0;
    cudaMemcpy(rayt::device_error_flag(), &zero, sizeof(int), cudaMemcpyHostToDevice);
    return fail(RAYT_E_TIMEOUT, "rayt_feedback_unique_noalloc: a bounded device wait gave up");
  }
  *unique_count = host;
  return RAYT_OK;
}
