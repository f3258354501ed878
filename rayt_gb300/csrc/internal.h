// Internal declarations shared by the host C++ and the CUDA translation units.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <mutex>
#include <string>
#include <vector>
#include "../../include/rayt_gb300.h"

namespace rayt {

// ---- errors -----------------------------------------------------------------
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);
#define RAYT_CUDA_TRY(expr)                                   \
  do {                                                        \
    cudaError_t e_ = (expr);                                  \
    if (e_ != cudaSuccess) return ::rayt::cuda_fail(e_, #expr); \
  } while (0)

constexpr int32_t kNoHit = 0x7fffffff;
constexpr uint32_t kRootParent = (1u << 24) - 1;

// ---- traversal ----------------------------------------------------------------
// Views' images (and recorded feedback words) share one buffer; view v starts
// at pixel pix_base (a multiple of 64).  A ray is identified by its pixel's
// index in that buffer, below 2^30.
constexpr int kMaxViews = 512;
constexpr int kViewsPerLaunch = 64;   // view descriptors travel in the launch parameters
constexpr int kMaxClients = 64;       // served mode: client framebuffers per server

// One view of a tracing launch.
struct ViewDesc {
  float m[16];             // view_proj_inv, row-major
  int width, height;
  int tiles_x;             // columns of 32-pixel tiles
  int tile_base;           // first tile of this view in the launch's tile space
  float lod;               // lod_voxel_size
  int pix_base;            // first pixel of the view in the shared image buffer
  float origin[4];         // InitTracingFrame's ray origin (m[2], m[6], m[10], 0) / m[14], per view
  const float* coords;     // PixelCoords(width, height) in device memory
};

// InitTracingFrame's normalised pixel coordinates, which depend only on the
// view's size: centres (x + 0.5) / W * 2 - 1 for x in [0, W), corners
// x / W * 2 - 1 for x in [0, W], then the same for y.  Computed once on the
// host with IEEE float arithmetic (the same operations and rounding as the
// kernel would do per ray), so looking them up changes no bit.
size_t pixel_coords_count(int w, int h);
void pixel_coords(int w, int h, float* out);
// The per-view origin the same way: (m[2], m[6], m[10], 0) / m[14].
void view_origin(const float* m, float* origin);

struct TraceParams {
  // cache (the reference's cache format)
  const uint32_t* links;
  const uint32_t* far_ptrs;
  const char4* normals;    // may be null
  const uchar4* colors;    // may be null
  uint32_t root;           // node index of the root (cache node indices are unsigned 32-bit)
  int nodes_in_block;
  uint32_t node_limit;     // nodes in the cache (max_blocks * nodes_in_block)
  uint32_t far_limit;      // far pointers in the cache (max_blocks * 8)
  float bg[4];             // background colour (0, 216/255, 1, 1)
  // outputs of every view
  uchar4* image;           // RGBA8, row 0 of each view at the bottom
  uchar4* host_image;      // optional: the same pixels also written here (page-locked host memory)
  int32_t* words_dense;    // optional per-pixel feedback words (recording)
  // first pass: the views of this launch and their tiles (32 rays each)
  int n_views;
  int total_tiles;
  int tile_w_log2;         // a warp's 32 first-pass rays cover (1 << tile_w_log2) x (32 >> tile_w_log2) pixels
  // faulted rays carried between passes: record i of the input list, and the
  // output list the rays that fault in this pass are appended to
  const float4* in_origin;
  const float4* in_dir;
  const int* in_parent;
  const uint32_t* in_ray;
  const int* n_in;
  float4* out_origin;      // xyz origin, w LOD bias
  float4* out_dir;         // xyz direction, w LOD coefficient
  int* out_parent;
  uint32_t* out_ray;
  int* n_out;
  // optional depth output (all four set, or all null): per pixel the distance
  // along the ray to what it shows and the cache node that shaded it; records
  // carry the distance a faulted ray advanced so far
  float* depth;
  int32_t* hit_node;
  const float* in_adv;
  float* out_adv;
  // feedback
  uint32_t* fault_bits;    // one bit per tree block
  int fault_bit_limit;     // number of tree blocks (bits in fault_bits)
  uint32_t* hit_bits;      // bit 2*cache_block + dup
  int* n_words;            // number of non-NO_HIT words this pass
  unsigned long long* counters;  // optional: rays, link fetches, far fetches, iterations, hits, faults
  // served mode (zero in the per-frame path).  Client slot i owns the pixels
  // [client_base[i], client_base[i + 1]) of the image buffer.
  int restart;             // faulted rays are recorded with their camera origin and traced afresh
  int n_clients;
  int client_base[kMaxClients + 1];
  unsigned long long finish_mask;  // continuation rays of these slots are finished, not traced
  int* client_faults;      // per slot: rays that faulted in this pass
  // persistent kernels
  int* work;               // work counter, zero before the launch
  int refill;              // idle lanes that let a warp take new rays (< 32)
  int step_budget;         // iterations a warp runs between refill checks
  ViewDesc views[kViewsPerLaunch];
};

// Faulted-ray records carried from one pass to the next (device arrays).
struct RayList {
  float4* origin = nullptr;  // xyz advanced to the fault, w LOD bias
  float4* dir = nullptr;     // xyz direction, w LOD coefficient
  int* parent = nullptr;     // node the ray faulted under
  uint32_t* ray = nullptr;   // pixel index in the image buffer
  float* adv = nullptr;      // distance advanced over earlier passes (depth output only)
};

// first: rays come from the views' cameras (refill = 32: one thread per ray
// over rays = total_tiles * 32 threads; refill < 32: the persistent
// work-stealing kernel over `grid` CTAs, 0 = as many as are resident).
// Otherwise the faulted rays of the input list, by a persistent kernel whose
// warps take 32 rays at a time (the count is read on the device).
cudaError_t launch_trace(const TraceParams& p, bool first, bool count, int rays, int grid, cudaStream_t s);
// The same launch as a kernel node of a CUDA graph (args: room for one pointer;
// p must stay valid until the node is added or updated).
cudaError_t trace_node_params(const TraceParams* p, bool first, bool count, int rays, int grid, void** args,
                              cudaKernelNodeParams* kp);
// Resident CTAs of the persistent traversal kernel on the current device.
int trace_persistent_grid(bool first, bool count);
cudaError_t launch_finish(const TraceParams& p, int max_rays, cudaStream_t s);
cudaError_t launch_fill_i32(int* p, int32_t v, size_t n, cudaStream_t s);
// The reference's debug depth view (raytracer.cl) of views[0] into image.
cudaError_t launch_depth_view(const TraceParams& p, cudaStream_t s);

// Feedback bitmaps -> the reference's sorted unique array.
struct UniqueFromBitsParams {
  const uint32_t* fault_bits;
  int fault_words;
  const uint32_t* hit_bits;
  int hit_words;
  const int* n_words;
  int total_pixels;
  int32_t* unique_out;   // room for fault bits + hit bits + 1
  const int* n_rays;     // rays the pass appended to its output list
  int* counts_out;       // [0] unique count (incl. NO_HIT), [1] fault count, [2] *n_rays
};
cudaError_t launch_unique_from_bits(const UniqueFromBitsParams& p, cudaStream_t s);
cudaError_t unique_node_params(const UniqueFromBitsParams* q, void** args, cudaKernelNodeParams* kp);

// ---- radix sort / scan / unique -------------------------------------------------
struct SortScratch {
  // sizes computed by sort_scratch_bytes
  size_t bytes;
};
size_t feedback_scratch_bytes(int n);
// Compaction (drop NO_HIT, NodeToBlock), radix sort, unique.  counts_dev[0]
// receives the unique count (incl. NO_HIT); everything stays on device.
cudaError_t feedback_unique_device(const int32_t* words, int n, int nib, int32_t* unique_out,
                                   int* counts_dev, void* scratch, size_t scratch_bytes, cudaStream_t s);
size_t sort_scratch_bytes(int n);
cudaError_t sort_i32_device(int32_t* data, int n, void* scratch, size_t scratch_bytes, cudaStream_t s);
size_t scan_scratch_bytes(int n);
cudaError_t scan_i32_device(int32_t* data, int n, void* scratch, size_t scratch_bytes, cudaStream_t s);
// Device error flag set by bounded waits that gave up (decoupled look-back).
int* device_error_flag();
// The sort/unique look-back words carry the tag epoch * 8 + pass, where the
// device-side epoch (27 bits) advances once per sort or unique call.  Sets
// that epoch (stream-ordered on s).
cudaError_t set_lookback_epoch(uint32_t epoch, cudaStream_t s);

// ---- stand-alone primitives (prims.cpp) -------------------------------------------
// Serialises every sort/scan/unique entry point on all devices: they share
// the device error flag and the look-back epoch, and each one holds the lock
// until its stream has finished its work.
std::mutex& prims_mutex();
// Called (with prims_mutex held) before each sort or unique call on the
// current device: counts epochs, and before the epoch would repeat a tag
// still present in a look-back table (after 2^27 - 1 calls), clears every
// look-back table of the device on s and restarts the epoch at 0.
int lookback_epoch_step(cudaStream_t s);
// Registers a scratch area holding look-back tables on the current device
// besides the library's growable scratch (the allocation-free entry point's
// static array), so lookback_epoch_step clears it too.
void register_lookback_area(void* p, size_t bytes);
// Runs one wait on a word nothing publishes, with a limit of limit_s seconds
// (restored to 1 s after); the wait must give up and set the error flag.
cudaError_t bounded_wait_probe(double limit_s, cudaStream_t s);

// ---- block upload --------------------------------------------------------------
constexpr int kMaxChannels = 8;
struct UploadParams {
  const uint8_t* stage;        // block contents, `stride` bytes apart
  size_t stride;               // content bytes rounded up to 16 (keeps every block aligned)
  const int* slots;            // destination cache slot per staged block
  int blocks;
  int nodes_in_block;
  int channels;
  int chan_bytes[kMaxChannels];
  uint8_t* chan[kMaxChannels]; // channel 0 = node links
  // With `file` set, the contents are read where they lie in the mapped block
  // file instead of from `stage`: block b's content starts at
  // file + file_first + file_stride * block_ids[b], at any alignment.
  const uint8_t* file;
  uint64_t file_first;         // header bytes + the 76-byte block header
  uint64_t file_stride;
  const int* block_ids;
  int parts;                   // CTAs per block (mapped reads; set by launch_upload)
};
struct Patch {
  uint32_t index;  // node-link index (below 2^32) or far-pointer index
  uint32_t value;
  uint32_t far;    // 1: far-pointer buffer, 0: node-link buffer
};
cudaError_t launch_upload(const UploadParams& p, cudaStream_t s);
cudaError_t launch_patches(const Patch* patches, int n, uint32_t* links, uint32_t* far_ptrs, cudaStream_t s);

// ---- glibc-compatible rand() stream -------------------------------------------
// The additive feedback generator behind glibc's rand()/srand() (TYPE_3:
// r[i] = r[i-3] + r[i-31], 16807 LCG seeding, 310 discarded outputs), as
// published in descriptions of the glibc random() algorithm.
class LibcRand {
 public:
  explicit LibcRand(uint32_t seed = 1) { Seed(seed); }
  void Seed(uint32_t seed);
  int Next();
 private:
  int32_t r_[34];
  int i_ = 0;
};

}  // namespace rayt
