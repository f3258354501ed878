// C ABI of the stand-alone feedback primitives (GPUSort, GPUScan and the
// feedback extractor's GetUnique).  Scratch memory is a per-device buffer the
// library grows on demand and keeps; calls are serialised by one mutex, so
// concurrent host threads do not share it mid-operation.
#include <mutex>
#include "internal.h"

namespace rayt {
namespace {
struct Scratch {
  void* ptr = nullptr;
  size_t bytes = 0;
};
Scratch g_scratch[64];

// Look-back epoch bookkeeping per device: calls since the tables were last
// cleared (= the device epoch), and the static area of the allocation-free
// entry point.
constexpr uint32_t kEpochLimit = (1u << 27) - 1;
uint32_t g_epoch_calls[64];
Scratch g_static_area[64];

int current_device(int* dev) {
  RAYT_CUDA_TRY(cudaGetDevice(dev));
  if (*dev < 0 || *dev >= 64) return fail(RAYT_E_ARG, "device ordinal out of range");
  return RAYT_OK;
}
}  // namespace

std::mutex& prims_mutex() {
  static std::mutex mu;
  return mu;
}

void register_lookback_area(void* p, size_t bytes) {
  int dev = 0;
  if (current_device(&dev) != RAYT_OK) return;
  g_static_area[dev].ptr = p;
  g_static_area[dev].bytes = bytes;
}

int lookback_epoch_step(cudaStream_t s) {
  int dev = 0;
  int rc = current_device(&dev);
  if (rc != RAYT_OK) return rc;
  if (g_epoch_calls[dev] >= kEpochLimit) {
    // the next epoch would reuse a tag that old look-back words may still
    // carry: zero every table (a zero word is never "published") and restart
    for (const Scratch* a : {&g_scratch[dev], &g_static_area[dev]})
      if (a->ptr) RAYT_CUDA_TRY(cudaMemsetAsync(a->ptr, 0, a->bytes, s));
    RAYT_CUDA_TRY(set_lookback_epoch(0, s));
    g_epoch_calls[dev] = 0;
  }
  ++g_epoch_calls[dev];
  return RAYT_OK;
}

namespace {

int get_scratch(size_t bytes, void** out, cudaStream_t stream) {
  int dev = 0;
  RAYT_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(RAYT_E_ARG, "device ordinal out of range");
  Scratch& s = g_scratch[dev];
  if (s.bytes < bytes) {
    if (s.ptr) {
      RAYT_CUDA_TRY(cudaDeviceSynchronize());
      cudaFree(s.ptr);
      s.ptr = nullptr;
      s.bytes = 0;
    }
    if (cudaMalloc(&s.ptr, bytes) != cudaSuccess) return fail(RAYT_E_OOM, "scratch allocation failed");
    s.bytes = bytes;
    // the sort's look-back words are epoch-tagged, never cleared: start from
    // zeros, ordered before the call's kernels on the caller's stream
    RAYT_CUDA_TRY(cudaMemsetAsync(s.ptr, 0, bytes, stream));
  }
  *out = s.ptr;
  return RAYT_OK;
}

int check_device_error(cudaStream_t s) {
  RAYT_CUDA_TRY(cudaStreamSynchronize(s));
  int flag = 0;
  RAYT_CUDA_TRY(cudaMemcpy(&flag, device_error_flag(), 4, cudaMemcpyDeviceToHost));
  if (flag) {
    int zero = 0;
    cudaMemcpy(device_error_flag(), &zero, 4, cudaMemcpyHostToDevice);
    return fail(RAYT_E_TIMEOUT, "a bounded device wait gave up (look-back did not complete)");
  }
  return RAYT_OK;
}

// rayt_feedback_unique's device work (4 memsets and 12 kernels, most of them
// short or returning at once) as one CUDA graph, replayed while the call's
// arguments repeat (a frame loop calls with the same buffers every frame):
// one graph launch instead of 16 stream operations.  The count and the
// device error flag come back in one copy into pinned memory.
struct UniqueGraph {
  const int32_t* words = nullptr;
  int n = 0, nib = 0;
  int32_t* out = nullptr;
  void* scratch = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t capture = nullptr;  // private stream the graph is captured on
  int* host = nullptr;             // pinned: [0] unique count, [1] error flag
};
UniqueGraph g_unique[64];

// Launches the device work of one call on s: the cached graph when the
// arguments match, else a newly captured one; direct launches if capture
// fails.  Then queues the read-back of the count and the error flag.
int unique_launch(int dev, const int32_t* words, int n, int nib, int32_t* out, void* scratch, size_t bytes,
                  int* counts, cudaStream_t s, int** host) {
  UniqueGraph& g = g_unique[dev];
  if (!g.host) RAYT_CUDA_TRY(cudaHostAlloc(&g.host, 2 * sizeof(int), cudaHostAllocDefault));
  if (!g.capture) RAYT_CUDA_TRY(cudaStreamCreateWithFlags(&g.capture, cudaStreamNonBlocking));
  const bool same = g.exec && g.words == words && g.n == n && g.nib == nib && g.out == out && g.scratch == scratch;
  if (!same) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g.exec = nullptr;
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(g.capture, cudaStreamCaptureModeRelaxed) == cudaSuccess) {
      const cudaError_t le = feedback_unique_device(words, n, nib, out, counts, scratch, bytes, g.capture);
      const cudaError_t ce = cudaStreamEndCapture(g.capture, &graph);
      if (le == cudaSuccess && ce == cudaSuccess && graph &&
          cudaGraphInstantiate(&g.exec, graph, 0) != cudaSuccess)
        g.exec = nullptr;
      if (graph) cudaGraphDestroy(graph);
    }
    cudaGetLastError();  // a failed capture leaves its error behind; the launches below report their own
    g.words = words, g.n = n, g.nib = nib, g.out = out, g.scratch = scratch;
  }
  if (g.exec) RAYT_CUDA_TRY(cudaGraphLaunch(g.exec, s));
  else RAYT_CUDA_TRY(feedback_unique_device(words, n, nib, out, counts, scratch, bytes, s));
  RAYT_CUDA_TRY(cudaMemcpyAsync(g.host, counts, sizeof(int), cudaMemcpyDeviceToHost, s));
  RAYT_CUDA_TRY(cudaMemcpyAsync(g.host + 1, device_error_flag(), sizeof(int), cudaMemcpyDeviceToHost, s));
  *host = g.host;
  return RAYT_OK;
}
}  // namespace
}  // namespace rayt

using rayt::fail;

extern "C" {

int rayt_sort_i32(int32_t* data, int n, void* stream) {
  if (n < 0 || (n > 0 && !data)) return fail(RAYT_E_ARG, "rayt_sort_i32: bad arguments");
  if (n >= (1 << 30)) return fail(RAYT_E_LIMIT, "rayt_sort_i32: n must be below 2^30");
  if (n <= 1) return RAYT_OK;
  std::lock_guard<std::mutex> lock(rayt::prims_mutex());
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  void* scratch = nullptr;
  const size_t bytes = rayt::sort_scratch_bytes(n);
  int rc = rayt::get_scratch(bytes, &scratch, s);
  if (rc != RAYT_OK) return rc;
  if ((rc = rayt::lookback_epoch_step(s)) != RAYT_OK) return rc;
  RAYT_CUDA_TRY(rayt::sort_i32_device(data, n, scratch, bytes, s));
  return rayt::check_device_error(s);
}

int rayt_scan_i32(int32_t* data, int n, void* stream) {
  if (n < 0 || (n > 0 && !data)) return fail(RAYT_E_ARG, "rayt_scan_i32: bad arguments");
  if (n >= (1 << 30)) return fail(RAYT_E_LIMIT, "rayt_scan_i32: n must be below 2^30");
  if (n == 0) return RAYT_OK;
  std::lock_guard<std::mutex> lock(rayt::prims_mutex());
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  void* scratch = nullptr;
  const size_t bytes = rayt::scan_scratch_bytes(n);
  int rc = rayt::get_scratch(bytes, &scratch, s);
  if (rc != RAYT_OK) return rc;
  RAYT_CUDA_TRY(rayt::scan_i32_device(data, n, scratch, bytes, s));
  return rayt::check_device_error(s);
}

int rayt_testing_set_lookback_epoch(uint32_t calls) {
  if (calls >= (1u << 27)) return fail(RAYT_E_ARG, "rayt_testing_set_lookback_epoch: epoch out of range");
  std::lock_guard<std::mutex> lock(rayt::prims_mutex());
  int dev = 0;
  RAYT_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(RAYT_E_ARG, "device ordinal out of range");
  RAYT_CUDA_TRY(rayt::set_lookback_epoch(calls, nullptr));
  RAYT_CUDA_TRY(cudaDeviceSynchronize());
  rayt::g_epoch_calls[dev] = calls;
  return RAYT_OK;
}

int rayt_selftest_bounded_wait(double limit_s, void* stream) {
  if (!(limit_s > 0) || limit_s > 10) return fail(RAYT_E_ARG, "rayt_selftest_bounded_wait: limit out of range (0, 10] s");
  std::lock_guard<std::mutex> lock(rayt::prims_mutex());
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  RAYT_CUDA_TRY(rayt::bounded_wait_probe(limit_s, s));
  const int rc = rayt::check_device_error(s);
  if (rc == RAYT_E_TIMEOUT) return RAYT_OK;  // the wait gave up as it must
  return rc != RAYT_OK ? rc : fail(RAYT_E_STATE, "bounded wait did not give up");
}

int rayt_feedback_unique(const int32_t* words, int n, int nib, int32_t* unique, int* unique_count, void* stream) {
  if (n < 0 || !unique_count || (n > 0 && (!words || !unique)) || nib < 0)
    return fail(RAYT_E_ARG, "rayt_feedback_unique: bad arguments");
  if (n >= (1 << 30)) return fail(RAYT_E_LIMIT, "rayt_feedback_unique: n must be below 2^30");
  if (n == 0) {
    *unique_count = 0;
    return RAYT_OK;
  }
  std::lock_guard<std::mutex> lock(rayt::prims_mutex());
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  void* scratch = nullptr;
  const size_t bytes = rayt::feedback_scratch_bytes(n) + 256;
  int rc = rayt::get_scratch(bytes, &scratch, s);
  if (rc != RAYT_OK) return rc;
  int* counts = reinterpret_cast<int*>(static_cast<uint8_t*>(scratch) + (bytes - 256));
  int dev = 0;
  RAYT_CUDA_TRY(cudaGetDevice(&dev));
  int* host = nullptr;
  if ((rc = rayt::lookback_epoch_step(s)) != RAYT_OK) return rc;
  rc = rayt::unique_launch(dev, words, n, nib, unique, scratch, bytes - 256, counts, s, &host);
  if (rc != RAYT_OK) return rc;
  RAYT_CUDA_TRY(cudaStreamSynchronize(s));
  if (host[1]) {
    const int zero = 0;
    cudaMemcpy(rayt::device_error_flag(), &zero, 4, cudaMemcpyHostToDevice);
    return fail(RAYT_E_TIMEOUT, "a bounded device wait gave up (look-back did not complete)");
  }
  *unique_count = host[0];
  return RAYT_OK;
}

}  // extern "C"
