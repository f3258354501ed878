// Frame driver: the reference's GPURayTracer::RenderFrame
// (rayt/GPU_renderer/gpu-ray-tracer.cpp:66-227) and the host half of its
// RayTracingFeedbackExtractor (rayt/GPU_renderer/ray-tracing-feedback-extractor.cpp:100-185).
//
// A renderer holds one view (the reference's GPURayTracer) or several views of
// any sizes that share one cache session per frame (batched form).  Per pass:
// one traversal launch over all views (first pass: every pixel from its
// view's camera, later passes: only rays that faulted; more than 64 views take
// one first-pass launch per 64), one launch that turns the feedback bitmaps
// into the reference's sorted unique array (written straight into host-mapped
// pinned memory), one stream synchronisation, then the host runs the
// reference's decode (all faults, plus a window of at most 4000 hits that
// starts at rand() % hits) and its cache transaction.  Block uploads go onto
// the same stream, so the next pass sees them without another wait.  The loop
// ends exactly where the reference's does: no faults, cache filled during the
// session, or (after the second pass) the time limit / pass cap.
#include <algorithm>
#include <climits>
#include <chrono>
#include <cstring>
#include <memory>

#include "cache.h"
#include "feedback.h"
#include "internal.h"

namespace rayt {

class Renderer {
 public:
  ~Renderer();
  int Init(Cache* cache, int n_views, const int* widths, const int* heights);
  int Frame(const float* m);
  int CountFetches(const float* m, int64_t* counts);
  int TimePass(const float* m, int reps, float* ms);
  int Autotune(const float* m, int reps, int* best);
  int ReadImage(int view, void* host, size_t bytes);
  int PassWords(int pass, int32_t* host, size_t count) const;
  int SetDepthOutput(bool on);
  int SetHostImage(void* host, size_t bytes);
  int DepthBuffers(int view, float** depth, int32_t** nodes) const;
  int ReadDepth(int view, float* depth, int32_t* nodes, size_t count);

  double time_limit = 1.0;  // the reference's default (gpu-ray-tracer.cpp:30-31)
  float lod = 1.5f;         // lod_voxel_size set by the caller
  float lod_used = 1.5f;    // the one frames render with (differs under LOD pressure)
  // LOD under cache pressure (the reference's todo "Decrease LOD when cache is
  // too small", msvs/rayt/todo.txt:5): after a frame whose session filled the
  // cache, the next frame's voxel size grows by `grow` (at most `max`); after a
  // frame that did not, it shrinks back by `shrink` (at least `lod`).
  bool lod_pressure = false;
  float lod_max = 16.0f, lod_grow = 1.5f, lod_shrink = 1.25f;
  int max_passes = 0;
  bool record = false;
  LibcRand rand;
  rayt_frame_stats stats{};
  // traversal launch shape
  int tile_w_log2 = 2;   // 4x8 pixel tiles (fastest on the 1080p flythrough)
  int refill = 32;       // 32: one thread per ray; below: the persistent kernel (slower on every
                         // measured frame, kept for the autotuner)
  int ctas_per_sm = 0;   // persistent kernel: 0 = as many as fit
  int step_budget = 16;  // persistent kernel: iterations between refill checks
  bool use_graphs = true;  // replay each pass's device work from a CUDA graph
  int n_views() const { return (int)views_.size(); }
  uchar4* image(int v) const { return d_images_ + views_[v].pix_base; }
  cudaStream_t stream() const { return s_; }

 private:
  static constexpr int kBlockInts = 16;  // pass block: {words, rays out, pad, pad, work counter per launch group}
  Cache* cache_ = nullptr;
  int total_pixels_ = 0, padded_pixels_ = 0;
  cudaStream_t s_ = nullptr;
  std::vector<ViewDesc> views_;     // sizes, tile layout and matrices of the current frame
  std::vector<int> group_tiles_;    // first-pass tiles per launch group of kViewsPerLaunch views
  uchar4* d_images_ = nullptr;      // every view's image at its pix_base
  int32_t* d_dense_ = nullptr;      // recorded feedback words, same layout
  float* d_coords_ = nullptr;       // every view's pixel_coords()
  bool depth_out_ = false;          // depth output on: the two buffers below and the lists' adv arrays
  float* d_depth_ = nullptr;        // per pixel (same layout as the images): distance to what it shows
  int32_t* d_hit_ = nullptr;        // per pixel: the cache node that shaded it (-1 miss, -2 error)
  RayList lists_[2];
  // [pass block 0][fault bits][hit bits][pass block 1]: pass k clears its own
  // block and the bitmaps with one memset and reads the other block's ray
  // count as its input.
  int* d_state_ = nullptr;
  int fault_words_ = 0, hit_words_ = 0;
  unsigned long long* d_fetch_ = nullptr;
  int32_t* h_unique_ = nullptr;      // mapped pinned
  int32_t* d_unique_ = nullptr;
  int* h_counts_ = nullptr;          // mapped pinned: unique count, fault count, rays faulted
  int* d_counts_ = nullptr;
  int32_t* h_dense_ = nullptr;       // pinned, for recording
  uint8_t* d_flush_ = nullptr;       // L2 flush buffer for TimePass
  // Host delivery of the image (one view): the caller's page-locked buffer,
  // its device address, a copy stream, and events "first pass done" (on the
  // renderer's stream) and "its copy done" (on the copy stream).
  uchar4* host_img_ = nullptr;
  uchar4* host_img_dev_ = nullptr;
  cudaStream_t copy_s_ = nullptr;
  cudaEvent_t copy_ev_[2] = {};
  cudaEvent_t ev_[8] = {};
  std::vector<std::vector<int32_t>> pass_words_;
  FeedbackDecoder fb_;

  int* block(int k) const { return k ? d_state_ + kBlockInts + fault_words_ + hit_words_ : d_state_; }
  int SetViews(const float* m);
  TraceParams Params(int it) const;
  int Grid(bool first, bool count) const;
  int Prepare(int it);
  int Trace(int it, bool count, int rays);
  UniqueFromBitsParams UniqueParams(int it) const;
  int RunPass(int it, int rays, int* launches);
  int PassGraph(int kind, int it, int rays);
  int groups() const { return (int)group_tiles_.size(); }

  // One pass's device work (clear feedback state, traversal, unique) as a
  // graph: kind 0 = first pass, 1 and 2 = later passes writing list 1 and 0.
  // The first pass's traversal nodes get the frame's view matrices before
  // every replay; later passes replay unchanged.
  struct Graph {
    cudaGraph_t graph = nullptr;  // kept: node handles refer to it
    cudaGraphExec_t exec = nullptr;
    std::vector<cudaGraphNode_t> trace_nodes;
    TraceParams key;  // the parameters (without views) it was built with
    int ctas = 0;     // and the persistent kernel's CTAs per SM
    unsigned blocks = 0;  // later passes: the traversal node's grid now
  };
  Graph graphs_[3];
  void DropGraphs();
};

void Renderer::DropGraphs() {
  for (auto& g : graphs_) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    if (g.graph) cudaGraphDestroy(g.graph);
    g.exec = nullptr;
    g.graph = nullptr;
    g.trace_nodes.clear();
  }
}

Renderer::~Renderer() {
  if (s_) cudaStreamSynchronize(s_);
  if (copy_s_) {
    cudaStreamSynchronize(copy_s_);
    cudaStreamDestroy(copy_s_);
  }
  for (auto& e : copy_ev_)
    if (e) cudaEventDestroy(e);
  DropGraphs();
  cudaFree(d_images_);
  cudaFree(d_coords_);
  for (auto& l : lists_) {
    cudaFree(l.origin);
    cudaFree(l.dir);
    cudaFree(l.parent);
    cudaFree(l.ray);
    cudaFree(l.adv);
  }
  cudaFree(d_depth_);
  cudaFree(d_hit_);
  cudaFree(d_dense_);
  cudaFree(d_state_);
  cudaFree(d_fetch_);
  cudaFree(d_flush_);
  cudaFreeHost(h_unique_);
  cudaFreeHost(h_counts_);
  cudaFreeHost(h_dense_);
  for (auto& e : ev_)
    if (e) cudaEventDestroy(e);
  Cache::Release(cache_);
}

int Renderer::Init(Cache* cache, int n_views, const int* widths, const int* heights) {
  if (n_views < 1 || n_views > kMaxViews) return fail(RAYT_E_ARG, "view count out of range (1..512)");
  cache->Retain();  // the cache (its stream and buffers) outlives this renderer
  cache_ = cache;
  s_ = cache->stream();
  views_.assign(n_views, ViewDesc{});
  int64_t pixels = 0, padded = 0;
  for (int v = 0; v < n_views; ++v) {
    const int w = widths[v], h = heights[v];
    if (w <= 0 || h <= 0 || (int64_t)w * h > (1 << 28)) return fail(RAYT_E_ARG, "view size out of range (at most 2^28 pixels)");
    views_[v].width = w;
    views_[v].height = h;
    views_[v].pix_base = (int)padded;
    pixels += (int64_t)w * h;
    padded += ((int64_t)w * h + 63) & ~(int64_t)63;
    if (padded >= (1 << 30)) return fail(RAYT_E_ARG, "total pixels of all views out of range (2^30)");
  }
  total_pixels_ = (int)pixels;
  padded_pixels_ = (int)padded;
  group_tiles_.assign((n_views + kViewsPerLaunch - 1) / kViewsPerLaunch, 0);
  const size_t n = pixels;
  if (cudaMalloc(&d_images_, (size_t)padded * 4) != cudaSuccess || cudaMalloc(&d_dense_, (size_t)padded * 4) != cudaSuccess ||
      cudaMalloc(&d_fetch_, 8 * 8) != cudaSuccess)
    return fail(RAYT_E_OOM, "renderer device allocation failed");
  for (auto& l : lists_)
    if (cudaMalloc(&l.origin, n * 16) != cudaSuccess || cudaMalloc(&l.dir, n * 16) != cudaSuccess ||
        cudaMalloc(&l.parent, n * 4) != cudaSuccess || cudaMalloc(&l.ray, n * 4) != cudaSuccess)
      return fail(RAYT_E_OOM, "ray list allocation failed");
  // one bit per block of the file; one bit per (cache block, duplicate flag)
  fault_words_ = (int)((cache->tree_blocks() + 31) / 32);
  hit_words_ = (int)(((uint64_t)cache->max_blocks() * 2 + 31) / 32);
  const size_t bit_words = (size_t)fault_words_ + hit_words_;
  if (cudaMalloc(&d_state_, (bit_words + 2 * kBlockInts) * 4) != cudaSuccess)
    return fail(RAYT_E_OOM, "feedback bitmap allocation failed");
  if (cudaHostAlloc(&h_unique_, (bit_words * 32 + 1) * 4, cudaHostAllocMapped) != cudaSuccess ||
      cudaHostAlloc(&h_counts_, 4 * 4, cudaHostAllocMapped) != cudaSuccess)
    return fail(RAYT_E_OOM, "pinned host allocation failed");
  RAYT_CUDA_TRY(cudaHostGetDevicePointer((void**)&d_unique_, h_unique_, 0));
  RAYT_CUDA_TRY(cudaHostGetDevicePointer((void**)&d_counts_, h_counts_, 0));
  for (auto& e : ev_) RAYT_CUDA_TRY(cudaEventCreate(&e));
  // the views' normalised pixel coordinates (they depend only on the sizes)
  std::vector<size_t> coord_at(n_views);
  std::vector<float> coords;
  for (int v = 0; v < n_views; ++v) {
    coord_at[v] = coords.size();
    coords.resize(coords.size() + pixel_coords_count(views_[v].width, views_[v].height));
    pixel_coords(views_[v].width, views_[v].height, coords.data() + coord_at[v]);
  }
  if (cudaMalloc(&d_coords_, coords.size() * sizeof(float)) != cudaSuccess)
    return fail(RAYT_E_OOM, "pixel coordinate table allocation failed");
  RAYT_CUDA_TRY(cudaMemcpy(d_coords_, coords.data(), coords.size() * sizeof(float), cudaMemcpyHostToDevice));
  for (int v = 0; v < n_views; ++v) views_[v].coords = d_coords_ + coord_at[v];
  RAYT_CUDA_TRY(cudaMemsetAsync(d_images_, 0, (size_t)padded * 4, s_));
  RAYT_CUDA_TRY(cudaMemsetAsync(d_state_, 0, (bit_words + 2 * kBlockInts) * 4, s_));
  RAYT_CUDA_TRY(cudaStreamSynchronize(s_));
  return RAYT_OK;
}

// Per-frame view descriptors: matrices, LOD and the tile layout of each
// launch group (they travel in the launch parameters).
int Renderer::SetViews(const float* m) {
  if (tile_w_log2 < 0 || tile_w_log2 > 5) return fail(RAYT_E_ARG, "tile width out of range");
  const int tw = 1 << tile_w_log2, th = 32 >> tile_w_log2;
  for (int g = 0; g < groups(); ++g) {
    int64_t tiles = 0;
    const int end = std::min(n_views(), (g + 1) * kViewsPerLaunch);
    for (int v = g * kViewsPerLaunch; v < end; ++v) {
      ViewDesc& d = views_[v];
      std::memcpy(d.m, m + 16 * v, sizeof(d.m));
      view_origin(d.m, d.origin);
      d.lod = lod_used;
      d.tiles_x = (d.width + tw - 1) / tw;
      d.tile_base = (int)std::min<int64_t>(tiles, INT32_MAX);
      tiles += (int64_t)d.tiles_x * ((d.height + th - 1) / th);
    }
    // the kernel counts first-pass rays (32 per tile) in int, with room for a
    // counter to run past the end by one grab per warp
    if (tiles * 32 > (int64_t)INT32_MAX - (1 << 24))
      return fail(RAYT_E_ARG, "too many pixel tiles for this tile shape; use a tile shape closer to the views' aspect");
    group_tiles_[g] = (int)tiles;
  }
  return RAYT_OK;
}

TraceParams Renderer::Params(int it) const {
  const int k = it & 1;
  TraceParams p;
  std::memset(&p, 0, sizeof(p));
  p.links = cache_->links();
  p.far_ptrs = cache_->far_ptrs();
  p.normals = static_cast<const char4*>(cache_->channel("normals", 4));
  p.colors = static_cast<const uchar4*>(cache_->channel("colors", 4));
  p.root = cache_->root_node();
  p.nodes_in_block = cache_->nodes_in_block();
  p.node_limit = (uint32_t)cache_->max_blocks() * (uint32_t)cache_->nodes_in_block();
  p.far_limit = (uint32_t)cache_->max_blocks() * 8u;
  p.bg[0] = 0.0f;
  p.bg[1] = (float)(216 / 255.);  // the reference's background (gpu-ray-tracer.cpp:190)
  p.bg[2] = 1.0f;
  p.bg[3] = 1.0f;
  p.image = d_images_;
  // the first pass's pixels reach the host image by one copy; later passes
  // write theirs there too
  p.host_image = it > 0 ? host_img_dev_ : nullptr;
  p.words_dense = record ? d_dense_ : nullptr;
  p.tile_w_log2 = tile_w_log2;
  const RayList& in = lists_[1 - k];
  const RayList& out = lists_[k];
  p.in_origin = in.origin;
  p.in_dir = in.dir;
  p.in_parent = in.parent;
  p.in_ray = in.ray;
  p.n_in = block(1 - k) + 1;
  p.out_origin = out.origin;
  p.out_dir = out.dir;
  p.out_parent = out.parent;
  p.out_ray = out.ray;
  p.n_out = block(k) + 1;
  if (depth_out_) {
    p.depth = d_depth_;
    p.hit_node = d_hit_;
    p.in_adv = in.adv;
    p.out_adv = out.adv;
  }
  p.fault_bits = reinterpret_cast<uint32_t*>(d_state_ + kBlockInts);
  p.fault_bit_limit = (int)cache_->tree_blocks();
  p.hit_bits = reinterpret_cast<uint32_t*>(d_state_ + kBlockInts + fault_words_);
  p.n_words = block(k);
  p.work = block(k) + 4;
  p.refill = refill;
  p.step_budget = step_budget;
  return p;
}

int Renderer::Grid(bool first, bool count) const {
  const int full = trace_persistent_grid(first, count);
  if (ctas_per_sm <= 0) return full;
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return std::min(full, sms * ctas_per_sm);
}


// Clears pass `it`'s block and the feedback bitmaps (one contiguous range).
int Renderer::Prepare(int it) {
  const size_t words = kBlockInts + (size_t)fault_words_ + hit_words_;
  RAYT_CUDA_TRY(cudaMemsetAsync((it & 1) ? d_state_ + kBlockInts : d_state_, 0, words * 4, s_));
  if (record) RAYT_CUDA_TRY(launch_fill_i32(d_dense_, kNoHit, (size_t)padded_pixels_, s_));
  return RAYT_OK;
}

// Pass `it`: the first pass launches once per group of kViewsPerLaunch views;
// later passes once over the `rays` faulted rays of the previous pass.
int Renderer::Trace(int it, bool count, int rays) {
  TraceParams p = Params(it);
  if (count) p.counters = d_fetch_;
  const int grid = refill < 32 ? Grid(it == 0, count) : 0;
  if (it > 0) {
    RAYT_CUDA_TRY(launch_trace(p, false, count, rays, grid, s_));
    return RAYT_OK;
  }
  for (int g = 0; g < groups(); ++g) {
    const int first = g * kViewsPerLaunch, end = std::min(n_views(), first + kViewsPerLaunch);
    p.n_views = end - first;
    std::memcpy(p.views, views_.data() + first, (size_t)p.n_views * sizeof(ViewDesc));
    p.total_tiles = group_tiles_[g];
    p.work = block(0) + 4 + g;
    RAYT_CUDA_TRY(launch_trace(p, true, count, group_tiles_[g] * 32, grid, s_));
  }
  return RAYT_OK;
}

UniqueFromBitsParams Renderer::UniqueParams(int it) const {
  UniqueFromBitsParams q{};
  q.fault_bits = reinterpret_cast<const uint32_t*>(d_state_ + kBlockInts);
  q.fault_words = fault_words_;
  q.hit_bits = reinterpret_cast<const uint32_t*>(d_state_ + kBlockInts + fault_words_);
  q.hit_words = hit_words_;
  q.n_words = block(it & 1);
  q.n_rays = block(it & 1) + 1;
  q.total_pixels = total_pixels_;
  q.unique_out = d_unique_;
  q.counts_out = d_counts_;
  return q;
}

// Builds (when missing or when the pass parameters changed) and updates the
// graph of pass kind `kind`, then launches it.  Events 1 (after traversal)
// and 2 (after unique) are recorded inside the graph.
int Renderer::PassGraph(int kind, int it, int rays) {
  Graph& g = graphs_[kind];
  TraceParams key = Params(it);
  if (g.exec && (std::memcmp(&key, &g.key, sizeof(key)) != 0 || g.ctas != ctas_per_sm)) {
    cudaGraphExecDestroy(g.exec);
    cudaGraphDestroy(g.graph);
    g.exec = nullptr;
    g.graph = nullptr;
    g.trace_nodes.clear();
  }
  const bool first = kind == 0;
  // per launch group (first pass) or one (later passes): parameters with views
  std::vector<TraceParams> tp(first ? groups() : 1, key);
  if (first) {
    for (int grp = 0; grp < groups(); ++grp) {
      TraceParams& p = tp[grp];
      const int v0 = grp * kViewsPerLaunch, v1 = std::min(n_views(), v0 + kViewsPerLaunch);
      p.n_views = v1 - v0;
      std::memcpy(p.views, views_.data() + v0, (size_t)p.n_views * sizeof(ViewDesc));
      p.total_tiles = group_tiles_[grp];
      p.work = block(0) + 4 + grp;
    }
  }
  const int grid = refill < 32 ? Grid(first, false) : 0;
  void* args[1];
  cudaKernelNodeParams kp;
  if (!g.exec) {
    cudaGraph_t graph;
    RAYT_CUDA_TRY(cudaGraphCreate(&graph, 0));
    cudaGraphNode_t prev = nullptr, node = nullptr;
    cudaMemsetParams mp{};
    mp.dst = (it & 1) ? d_state_ + kBlockInts : d_state_;
    mp.value = 0;
    mp.elementSize = 4;
    mp.width = kBlockInts + (size_t)fault_words_ + hit_words_;
    mp.height = 1;
    cudaError_t e = cudaGraphAddMemsetNode(&node, graph, nullptr, 0, &mp);
    prev = node;
    for (size_t i = 0; e == cudaSuccess && i < tp.size(); ++i) {
      trace_node_params(&tp[i], first, false, first ? group_tiles_[i] * 32 : rays, grid, args, &kp);
      g.blocks = kp.gridDim.x;
      e = cudaGraphAddKernelNode(&node, graph, &prev, 1, &kp);
      g.trace_nodes.push_back(node);
      prev = node;
    }
    if (e == cudaSuccess) e = cudaGraphAddEventRecordNode(&node, graph, &prev, 1, ev_[1]);
    prev = node;
    const UniqueFromBitsParams q = UniqueParams(it);
    if (e == cudaSuccess) {
      unique_node_params(&q, args, &kp);
      e = cudaGraphAddKernelNode(&node, graph, &prev, 1, &kp);
      prev = node;
    }
    if (e == cudaSuccess) e = cudaGraphAddEventRecordNode(&node, graph, &prev, 1, ev_[2]);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&g.exec, graph, 0);
    if (e != cudaSuccess) {
      cudaGraphDestroy(graph);
      g.exec = nullptr;
      g.trace_nodes.clear();
      return cuda_fail(e, "pass graph construction");
    }
    g.graph = graph;
    g.key = key;
    g.ctas = ctas_per_sm;
  } else if (first) {
    for (size_t i = 0; i < tp.size(); ++i) {
      trace_node_params(&tp[i], true, false, group_tiles_[i] * 32, grid, args, &kp);
      RAYT_CUDA_TRY(cudaGraphExecKernelNodeSetParams(g.exec, g.trace_nodes[i], &kp));
    }
  } else {
    // a later pass's grid follows its ray count
    trace_node_params(&tp[0], false, false, rays, grid, args, &kp);
    if (kp.gridDim.x != g.blocks) {
      RAYT_CUDA_TRY(cudaGraphExecKernelNodeSetParams(g.exec, g.trace_nodes[0], &kp));
      g.blocks = kp.gridDim.x;
    }
  }
  RAYT_CUDA_TRY(cudaGraphLaunch(g.exec, s_));
  return RAYT_OK;
}

// The device work of pass `it` over `rays` rays (traversal and feedback
// unique, with events 0..2 around them); adds the kernels it launched.
int Renderer::RunPass(int it, int rays, int* launches) {
  RAYT_CUDA_TRY(cudaEventRecord(ev_[0], s_));
  if (use_graphs && !record) {
    int rc = PassGraph(it == 0 ? 0 : ((it & 1) ? 1 : 2), it, rays);
    if (rc != RAYT_OK) return rc;
    *launches += (it == 0 ? groups() : 1) + 1;
    return RAYT_OK;
  }
  int rc = Prepare(it);
  if (rc != RAYT_OK) return rc;
  if (it == 0 || rays > 0) {
    if ((rc = Trace(it, false, rays)) != RAYT_OK) return rc;
    *launches += it == 0 ? groups() : 1;
  }
  RAYT_CUDA_TRY(cudaEventRecord(ev_[1], s_));
  RAYT_CUDA_TRY(launch_unique_from_bits(UniqueParams(it), s_));
  *launches += 1 + (record ? 1 : 0);
  RAYT_CUDA_TRY(cudaEventRecord(ev_[2], s_));
  return RAYT_OK;
}

int Renderer::Frame(const float* m) {
  const auto t0 = std::chrono::steady_clock::now();
  stats = rayt_frame_stats{};
  pass_words_.clear();
  const int64_t uploaded0 = cache_->stats().uploaded_blocks;
  const int64_t launches0 = cache_->launches();
  const int64_t h2d0 = cache_->stats().bytes_h2d;
  int launches = 0;
  int64_t d2h = 0;
  if (record && (uint64_t)cache_->max_blocks() * cache_->nodes_in_block() >= (1ull << 30))
    return fail(RAYT_E_LIMIT, "recorded feedback words need a cache of fewer than 2^30 nodes");
  int rc = SetViews(m);
  if (rc != RAYT_OK) return rc;
  rc = cache_->StartSession();
  if (rc != RAYT_OK) return rc;
  const int total = total_pixels_;
  int active_prev = total;  // rays traced by the first pass
  float ms_trace = 0, ms_fb = 0, ms_up = 0;
  using clock = std::chrono::steady_clock;
  auto ms_since = [](clock::time_point a) { return std::chrono::duration<double, std::milli>(clock::now() - a).count(); };
  int it;
  bool copy_pending = false;  // the first pass's pixels on their way to the host image
  for (it = 0;; ++it) {
    if (it > 0 && copy_pending) {  // later passes write host pixels only after the copy
      RAYT_CUDA_TRY(cudaStreamWaitEvent(s_, copy_ev_[1], 0));
      copy_pending = false;
    }
    if ((rc = RunPass(it, active_prev, &launches)) != RAYT_OK) break;
    if (it == 0 && host_img_) {
      // the copy runs while the host decodes the feedback and streams blocks
      const size_t bytes = (size_t)views_[0].width * views_[0].height * 4;
      RAYT_CUDA_TRY(cudaEventRecord(copy_ev_[0], s_));
      RAYT_CUDA_TRY(cudaStreamWaitEvent(copy_s_, copy_ev_[0], 0));
      RAYT_CUDA_TRY(cudaMemcpyAsync(host_img_, d_images_, bytes, cudaMemcpyDeviceToHost, copy_s_));
      RAYT_CUDA_TRY(cudaEventRecord(copy_ev_[1], copy_s_));
      copy_pending = true;
      d2h += (int64_t)bytes;
    }
    if (record) {
      if (!h_dense_) RAYT_CUDA_TRY(cudaHostAlloc(&h_dense_, (size_t)padded_pixels_ * 4, cudaHostAllocDefault));
      RAYT_CUDA_TRY(cudaMemcpyAsync(h_dense_, d_dense_, (size_t)padded_pixels_ * 4, cudaMemcpyDeviceToHost, s_));
    }
    const auto tw = clock::now();
    RAYT_CUDA_TRY(cudaStreamSynchronize(s_));
    stats.host_ms_wait += ms_since(tw);
    float a = 0, b = 0;
    cudaEventElapsedTime(&a, ev_[0], ev_[1]);
    cudaEventElapsedTime(&b, ev_[1], ev_[2]);
    ms_trace += a;
    ms_fb += b;
    stats.rays_traced += active_prev;
    if (record) {  // views in order, without the padding between them
      pass_words_.emplace_back();
      for (const ViewDesc& v : views_)
        pass_words_.back().insert(pass_words_.back().end(), h_dense_ + v.pix_base,
                                  h_dense_ + v.pix_base + (size_t)v.width * v.height);
    }
    const int active_now = h_counts_[2];
    d2h += 3 * 4 + (int64_t)h_counts_[0] * 4;  // counts, unique array (mapped reads)

    // the reference always gives the frame one round of loading, then stops
    // on its wall-clock limit (gpu-ray-tracer.cpp:123-125)
    const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (it > 0 && el > time_limit) { active_prev = active_now; break; }
    if (max_passes > 0 && it > 0 && it + 1 >= max_passes) { active_prev = active_now; break; }

    const auto td = clock::now();
    fb_.Decode(h_unique_, h_counts_[0], rand);
    if ((rc = cache_->StartTransaction((int)fb_.faults.size())) != RAYT_OK) break;
    cache_->MarkUsedBatch(fb_.hits, fb_.dup_hits);
    for (int f : fb_.faults) {
      if (cache_->TransactionFilled()) break;
      if ((rc = cache_->RequestBlock(f)) != RAYT_OK) break;
    }
    stats.faults += (int)fb_.faults.size();
    stats.host_ms_decode += ms_since(td);
    const auto tl = clock::now();
    const int erc = cache_->EndTransaction();
    stats.host_ms_load += ms_since(tl);
    if (rc == RAYT_OK) rc = erc;
    if (rc != RAYT_OK) break;
    active_prev = active_now;
    if (fb_.faults.empty() || cache_->SessionFilled()) break;
  }
  stats.passes = it + 1;
  stats.session_filled = cache_->in_session() && cache_->SessionFilled() ? 1 : 0;
  stats.lod_voxel_size = lod_used;
  if (lod_pressure) {
    if (stats.session_filled) lod_used = std::min(lod_max, lod_used * lod_grow);
    else if (lod_used > lod) lod_used = std::max(lod, lod_used / lod_shrink);
  }
  if (cache_->in_transaction()) cache_->EndTransaction();
  const int src = cache_->EndSession();
  if ((rc != RAYT_OK || src != RAYT_OK) && copy_pending) cudaStreamSynchronize(copy_s_);
  if (rc != RAYT_OK) return rc;
  if (src != RAYT_OK) return src;
  // FinishTracingFrame for the rays still faulted, against the cache as it is now
  const TraceParams p = Params(it);
  TraceParams f = p;
  f.in_origin = p.out_origin;
  f.in_dir = p.out_dir;
  f.in_parent = p.out_parent;
  f.in_ray = p.out_ray;
  f.in_adv = p.out_adv;
  f.n_in = p.n_out;
  f.host_image = host_img_dev_;
  if (copy_pending) RAYT_CUDA_TRY(cudaStreamWaitEvent(s_, copy_ev_[1], 0));  // also ends with the copy
  RAYT_CUDA_TRY(launch_finish(f, active_prev, s_));
  if (active_prev > 0) ++launches;
  const auto tw = clock::now();
  RAYT_CUDA_TRY(cudaStreamSynchronize(s_));
  stats.host_ms_wait += ms_since(tw);
  ms_up += cache_->TakeUploadMs();  // every batch the frame's transactions flushed
  stats.gpu_ms_trace = ms_trace;
  stats.gpu_ms_feedback = ms_fb;
  stats.gpu_ms_upload = ms_up;
  stats.uploaded_blocks = (int)(cache_->stats().uploaded_blocks - uploaded0);
  stats.frame_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  stats.kernel_launches = launches + (int)(cache_->launches() - launches0);
  stats.bytes_h2d = cache_->stats().bytes_h2d - h2d0;
  stats.bytes_d2h = d2h;
  return RAYT_OK;
}

int Renderer::CountFetches(const float* m, int64_t* counts) {
  int rc = SetViews(m);
  if (rc == RAYT_OK) rc = Prepare(0);
  if (rc != RAYT_OK) return rc;
  RAYT_CUDA_TRY(cudaMemsetAsync(d_fetch_, 0, 8 * 8, s_));
  if ((rc = Trace(0, true, 0)) != RAYT_OK) return rc;
  unsigned long long h[8];
  RAYT_CUDA_TRY(cudaMemcpyAsync(h, d_fetch_, sizeof(h), cudaMemcpyDeviceToHost, s_));
  RAYT_CUDA_TRY(cudaStreamSynchronize(s_));
  for (int k = 0; k < 6; ++k) counts[k] = (int64_t)h[k];
  return RAYT_OK;
}

// Back-to-back first passes; L2 is flushed (a 256 MiB write) before each and
// only the traversal launch is inside the timed events.
int Renderer::TimePass(const float* m, int reps, float* ms) {
  const size_t flush = 256u << 20;
  if (!d_flush_ && cudaMalloc(&d_flush_, flush) != cudaSuccess) return fail(RAYT_E_OOM, "flush buffer allocation failed");
  int rc = SetViews(m);
  if (rc != RAYT_OK) return rc;
  float total = 0;
  for (int r = 0; r < reps; ++r) {
    RAYT_CUDA_TRY(cudaMemsetAsync(d_flush_, r & 255, flush, s_));
    if ((rc = Prepare(0)) != RAYT_OK) return rc;
    RAYT_CUDA_TRY(cudaEventRecord(ev_[5], s_));
    if ((rc = Trace(0, false, 0)) != RAYT_OK) return rc;
    RAYT_CUDA_TRY(cudaEventRecord(ev_[6], s_));
    RAYT_CUDA_TRY(cudaEventSynchronize(ev_[6]));
    float a = 0;
    RAYT_CUDA_TRY(cudaEventElapsedTime(&a, ev_[5], ev_[6]));
    total += a;
  }
  *ms = reps > 0 ? total / reps : 0.0f;
  return RAYT_OK;
}

// Picks the traversal launch shape (tile shape, refill threshold and step
// budget, CTAs per SM) with the shortest first pass over these views, timed
// like TimePass.  The result is the renderer's shape from then on; best =
// {tile_w_log2, refill, ctas_per_sm, step_budget}.
int Renderer::Autotune(const float* m, int reps, int* best) {
  struct Refill { int refill, budget; };
  static const int kTiles[] = {2, 3, 4, 5};
  static const Refill kRefill[] = {{32, 0}, {24, 16}, {16, 16}, {16, 32}, {8, 32}};
  static const int kCtas[] = {0, 8, 6, 4};
  const int save[4] = {tile_w_log2, refill, ctas_per_sm, step_budget};
  float best_ms = 1e30f;
  int b[4] = {save[0], save[1], save[2], save[3]};
  for (int t : kTiles)
    for (const Refill& r : kRefill)
      for (int c : kCtas) {
        if (r.refill == 32 && c != 0) continue;  // CTAs per SM only shape the persistent kernel
        tile_w_log2 = t;
        refill = r.refill;
        step_budget = r.budget;
        ctas_per_sm = c;
        float ms = 0;
        int rc = TimePass(m, reps, &ms);
        if (rc != RAYT_OK) {
          tile_w_log2 = save[0], refill = save[1], ctas_per_sm = save[2], step_budget = save[3];
          return rc;
        }
        if (ms < best_ms) best_ms = ms, b[0] = t, b[1] = r.refill, b[2] = c, b[3] = r.budget;
      }
  tile_w_log2 = b[0];
  refill = b[1];
  ctas_per_sm = b[2];
  step_budget = b[3];
  if (best)
    for (int k = 0; k < 4; ++k) best[k] = b[k];
  return RAYT_OK;
}

// Host delivery: every frame's image also lands in `host` by the time the
// frame returns.  The buffer must be page-locked (cudaHostAlloc or
// cudaHostRegister): the copy engine and the traversal kernels write it
// directly.
int Renderer::SetHostImage(void* host, size_t bytes) {
  if (!host) {
    if (copy_s_) RAYT_CUDA_TRY(cudaStreamSynchronize(copy_s_));
    host_img_ = host_img_dev_ = nullptr;
    return RAYT_OK;
  }
  if (n_views() != 1) return fail(RAYT_E_ARG, "host image delivery needs a one-view renderer");
  if (bytes < (size_t)views_[0].width * views_[0].height * 4) return fail(RAYT_E_ARG, "host image buffer too small");
  if (reinterpret_cast<uintptr_t>(host) & 3u) return fail(RAYT_E_ARG, "host image must be 4-byte aligned (RGBA8 pixels)");
  // page-locked memory only (the runtime reports it as host memory; on a
  // system where the device also reaches pageable memory, a copy into that
  // would hold the calling thread until the copy ends)
  cudaPointerAttributes a{};
  void* dev = nullptr;
  if (cudaPointerGetAttributes(&a, host) == cudaSuccess && a.type == cudaMemoryTypeHost) {
    dev = a.devicePointer;
    if (!dev && cudaHostGetDevicePointer(&dev, host, 0) != cudaSuccess) dev = nullptr;
  }
  cudaGetLastError();
  if (!dev) return fail(RAYT_E_ARG, "host image must be page-locked memory (cudaHostAlloc or cudaHostRegister)");
  if (!copy_s_) {
    RAYT_CUDA_TRY(cudaStreamCreateWithFlags(&copy_s_, cudaStreamNonBlocking));
    for (auto& e : copy_ev_) RAYT_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  RAYT_CUDA_TRY(cudaStreamSynchronize(s_));  // no frame writes the old buffer any more
  RAYT_CUDA_TRY(cudaStreamSynchronize(copy_s_));
  host_img_ = static_cast<uchar4*>(host);
  host_img_dev_ = static_cast<uchar4*>(dev);
  return RAYT_OK;
}

int Renderer::ReadImage(int view, void* host, size_t bytes) {
  if (view < 0 || view >= n_views()) return fail(RAYT_E_ARG, "view index out of range");
  const size_t n = (size_t)views_[view].width * views_[view].height * 4;
  if (bytes < n) return fail(RAYT_E_ARG, "image buffer too small");
  RAYT_CUDA_TRY(cudaMemcpyAsync(host, image(view), n, cudaMemcpyDeviceToHost, s_));
  RAYT_CUDA_TRY(cudaStreamSynchronize(s_));
  return RAYT_OK;
}

int Renderer::PassWords(int pass, int32_t* host, size_t count) const {
  if (pass < 0 || pass >= (int)pass_words_.size()) return fail(RAYT_E_ARG, "no recorded pass with that index");
  if (count < pass_words_[pass].size()) return fail(RAYT_E_ARG, "word buffer too small");
  std::memcpy(host, pass_words_[pass].data(), pass_words_[pass].size() * 4);
  return RAYT_OK;
}

// Depth output buffers (allocated on first use, kept while the renderer
// lives): per-pixel distance and shading node, and the distance each faulted
// ray has advanced, carried on its record between passes.
int Renderer::SetDepthOutput(bool on) {
  if (on && !d_depth_) {
    const size_t n = (size_t)total_pixels_;
    if (cudaMalloc(&d_depth_, (size_t)padded_pixels_ * 4) != cudaSuccess ||
        cudaMalloc(&d_hit_, (size_t)padded_pixels_ * 4) != cudaSuccess ||
        cudaMalloc(&lists_[0].adv, n * 4) != cudaSuccess || cudaMalloc(&lists_[1].adv, n * 4) != cudaSuccess)
      return fail(RAYT_E_OOM, "depth output allocation failed");
    RAYT_CUDA_TRY(cudaMemsetAsync(d_depth_, 0, (size_t)padded_pixels_ * 4, s_));
    RAYT_CUDA_TRY(launch_fill_i32(d_hit_, -1, (size_t)padded_pixels_, s_));
  }
  depth_out_ = on;
  return RAYT_OK;
}

int Renderer::DepthBuffers(int view, float** depth, int32_t** nodes) const {
  if (view < 0 || view >= n_views()) return fail(RAYT_E_ARG, "view index out of range");
  if (!d_depth_) return fail(RAYT_E_STATE, "depth output was never turned on");
  if (depth) *depth = d_depth_ + views_[view].pix_base;
  if (nodes) *nodes = d_hit_ + views_[view].pix_base;
  return RAYT_OK;
}

int Renderer::ReadDepth(int view, float* depth, int32_t* nodes, size_t count) {
  float* dd = nullptr;
  int32_t* dn = nullptr;
  int rc = DepthBuffers(view, &dd, &dn);
  if (rc != RAYT_OK) return rc;
  const size_t n = (size_t)views_[view].width * views_[view].height;
  if (count < n) return fail(RAYT_E_ARG, "depth buffer too small");
  if (depth) RAYT_CUDA_TRY(cudaMemcpyAsync(depth, dd, n * 4, cudaMemcpyDeviceToHost, s_));
  if (nodes) RAYT_CUDA_TRY(cudaMemcpyAsync(nodes, dn, n * 4, cudaMemcpyDeviceToHost, s_));
  RAYT_CUDA_TRY(cudaStreamSynchronize(s_));
  return RAYT_OK;
}

}  // namespace rayt

using rayt::fail;
namespace {
rayt::Renderer* R(rayt_renderer* r) { return reinterpret_cast<rayt::Renderer*>(r); }
}  // namespace

extern "C" {

int rayt_renderer_create(rayt_cache* cache, int width, int height, rayt_renderer** out) {
  if (!cache || !out) return fail(RAYT_E_ARG, "rayt_renderer_create: null argument");
  rayt::Renderer* r = new rayt::Renderer();
  int rc = r->Init(reinterpret_cast<rayt::Cache*>(cache), 1, &width, &height);
  if (rc != RAYT_OK) {
    delete r;
    return rc;
  }
  *out = reinterpret_cast<rayt_renderer*>(r);
  return RAYT_OK;
}
int rayt_renderer_create_views(rayt_cache* cache, int n_views, const int* widths, const int* heights,
                               rayt_renderer** out) {
  if (!cache || !out || !widths || !heights) return fail(RAYT_E_ARG, "rayt_renderer_create_views: null argument");
  rayt::Renderer* r = new rayt::Renderer();
  int rc = r->Init(reinterpret_cast<rayt::Cache*>(cache), n_views, widths, heights);
  if (rc != RAYT_OK) {
    delete r;
    return rc;
  }
  *out = reinterpret_cast<rayt_renderer*>(r);
  return RAYT_OK;
}
void rayt_renderer_destroy(rayt_renderer* r) { delete R(r); }
int rayt_renderer_set_frame_time_limit(rayt_renderer* r, double s) {
  if (!r || !(s >= 0)) return fail(RAYT_E_ARG, "bad frame time limit");
  R(r)->time_limit = s;
  return RAYT_OK;
}
int rayt_renderer_set_lod_voxel_size(rayt_renderer* r, float v) {
  if (!r || !(v >= 0)) return fail(RAYT_E_ARG, "bad LOD voxel size");
  R(r)->lod = v;
  R(r)->lod_used = v;
  return RAYT_OK;
}
int rayt_renderer_set_lod_pressure(rayt_renderer* r, int on, float max_lod_voxel_size, float grow, float shrink) {
  if (!r || !(grow >= 1) || !(shrink >= 1) || !(max_lod_voxel_size >= 0)) return fail(RAYT_E_ARG, "bad LOD pressure settings");
  rayt::Renderer* q = R(r);
  q->lod_pressure = on != 0;
  q->lod_max = max_lod_voxel_size;
  q->lod_grow = grow;
  q->lod_shrink = shrink;
  if (!q->lod_pressure) q->lod_used = q->lod;
  return RAYT_OK;
}
int rayt_renderer_set_max_passes(rayt_renderer* r, int n) {
  if (!r || n < 0) return fail(RAYT_E_ARG, "bad pass cap");
  R(r)->max_passes = n;
  return RAYT_OK;
}
int rayt_renderer_seed(rayt_renderer* r, uint32_t seed) {
  if (!r) return fail(RAYT_E_ARG, "null renderer");
  R(r)->rand.Seed(seed);
  return RAYT_OK;
}
int rayt_renderer_use_graphs(rayt_renderer* r, int on) {
  if (!r) return fail(RAYT_E_ARG, "null renderer");
  R(r)->use_graphs = on != 0;
  return RAYT_OK;
}
int rayt_renderer_record_passes(rayt_renderer* r, int on) {
  if (!r) return fail(RAYT_E_ARG, "null renderer");
  R(r)->record = on != 0;
  return RAYT_OK;
}
int rayt_render_frame(rayt_renderer* r, const float m[16]) {
  if (!r || !m) return fail(RAYT_E_ARG, "rayt_render_frame: null argument");
  if (R(r)->n_views() != 1) return fail(RAYT_E_ARG, "rayt_render_frame: renderer has several views; use rayt_render_views");
  return R(r)->Frame(m);
}
int rayt_render_views(rayt_renderer* r, const float* m, int n_views) {
  if (!r || !m) return fail(RAYT_E_ARG, "rayt_render_views: null argument");
  if (n_views != R(r)->n_views()) return fail(RAYT_E_ARG, "rayt_render_views: matrix count differs from the renderer's views");
  return R(r)->Frame(m);
}
int rayt_renderer_view_count(const rayt_renderer* r) {
  if (!r) return fail(RAYT_E_ARG, "null renderer");
  return reinterpret_cast<const rayt::Renderer*>(r)->n_views();
}
int rayt_renderer_view_image(rayt_renderer* r, int view, void** dev) {
  if (!r || !dev) return fail(RAYT_E_ARG, "null argument");
  if (view < 0 || view >= R(r)->n_views()) return fail(RAYT_E_ARG, "view index out of range");
  *dev = R(r)->image(view);
  return RAYT_OK;
}
int rayt_renderer_read_view_image(rayt_renderer* r, int view, void* host, size_t bytes) {
  if (!r || !host) return fail(RAYT_E_ARG, "null argument");
  return R(r)->ReadImage(view, host, bytes);
}
int rayt_renderer_set_launch_shape(rayt_renderer* r, int tile_w_log2, int refill, int ctas_per_sm, int step_budget) {
  if (!r || tile_w_log2 < 0 || tile_w_log2 > 5 || refill < 1 || refill > 32 || ctas_per_sm < 0 ||
      step_budget < 0 || (refill < 32 && step_budget < 1))
    return fail(RAYT_E_ARG, "bad launch shape");
  R(r)->tile_w_log2 = tile_w_log2;
  R(r)->refill = refill;
  R(r)->ctas_per_sm = ctas_per_sm;
  R(r)->step_budget = step_budget;
  return RAYT_OK;
}
int rayt_renderer_get_launch_shape(const rayt_renderer* r, int shape[4]) {
  if (!r || !shape) return fail(RAYT_E_ARG, "null argument");
  const rayt::Renderer* q = reinterpret_cast<const rayt::Renderer*>(r);
  shape[0] = q->tile_w_log2;
  shape[1] = q->refill;
  shape[2] = q->ctas_per_sm;
  shape[3] = q->step_budget;
  return RAYT_OK;
}
int rayt_renderer_autotune(rayt_renderer* r, const float* m, int reps, int best[4]) {
  if (!r || !m || reps < 1) return fail(RAYT_E_ARG, "bad argument");
  return R(r)->Autotune(m, reps, best);
}
int rayt_renderer_stream(rayt_renderer* r, void** stream) {
  if (!r || !stream) return fail(RAYT_E_ARG, "null argument");
  *stream = R(r)->stream();
  return RAYT_OK;
}
int rayt_renderer_image(rayt_renderer* r, void** dev) {
  if (!r || !dev) return fail(RAYT_E_ARG, "null argument");
  *dev = R(r)->image(0);
  return RAYT_OK;
}
int rayt_renderer_read_image(rayt_renderer* r, void* host, size_t bytes) {
  if (!r || !host) return fail(RAYT_E_ARG, "null argument");
  return R(r)->ReadImage(0, host, bytes);
}
int rayt_renderer_pass_words(rayt_renderer* r, int pass, int32_t* host, size_t count) {
  if (!r || !host) return fail(RAYT_E_ARG, "null argument");
  return R(r)->PassWords(pass, host, count);
}
int rayt_renderer_set_host_image(rayt_renderer* r, void* host_rgba, size_t bytes) {
  return r ? R(r)->SetHostImage(host_rgba, bytes) : fail(RAYT_E_ARG, "null renderer");
}
int rayt_renderer_set_depth_output(rayt_renderer* r, int on) {
  if (!r) return fail(RAYT_E_ARG, "null renderer");
  return R(r)->SetDepthOutput(on != 0);
}
int rayt_renderer_depth(rayt_renderer* r, int view, void** device_depth, void** device_hit_nodes) {
  if (!r || (!device_depth && !device_hit_nodes)) return fail(RAYT_E_ARG, "null argument");
  float* d = nullptr;
  int32_t* n = nullptr;
  const int rc = R(r)->DepthBuffers(view, &d, &n);
  if (rc != RAYT_OK) return rc;
  if (device_depth) *device_depth = d;
  if (device_hit_nodes) *device_hit_nodes = n;
  return RAYT_OK;
}
int rayt_renderer_read_depth(rayt_renderer* r, int view, float* host_depth, int32_t* host_hit_nodes, size_t count) {
  if (!r || (!host_depth && !host_hit_nodes)) return fail(RAYT_E_ARG, "null argument");
  return R(r)->ReadDepth(view, host_depth, host_hit_nodes, count);
}
int rayt_renderer_stats(const rayt_renderer* r, rayt_frame_stats* out) {
  if (!r || !out) return fail(RAYT_E_ARG, "null argument");
  *out = reinterpret_cast<const rayt::Renderer*>(r)->stats;
  return RAYT_OK;
}
int rayt_cache_depth_view(rayt_cache* cache, const float view_proj_inv[16], float lod_voxel_size, int width,
                          int height, void* device_rgba, void* stream) {
  if (!cache || !view_proj_inv || !device_rgba) return fail(RAYT_E_ARG, "rayt_cache_depth_view: null argument");
  if (width <= 0 || height <= 0 || (int64_t)width * height >= (1ll << 31) || !(lod_voxel_size >= 0))
    return fail(RAYT_E_ARG, "rayt_cache_depth_view: bad size or LOD");
  rayt::Cache* c = reinterpret_cast<rayt::Cache*>(cache);
  rayt::TraceParams p;
  std::memset(&p, 0, sizeof(p));
  p.links = c->links();
  p.far_ptrs = c->far_ptrs();
  p.root = c->root_node();
  p.nodes_in_block = c->nodes_in_block();
  p.node_limit = (uint32_t)c->max_blocks() * (uint32_t)c->nodes_in_block();
  p.far_limit = (uint32_t)c->max_blocks() * 8u;
  p.image = static_cast<uchar4*>(device_rgba);
  p.n_views = 1;
  std::memcpy(p.views[0].m, view_proj_inv, sizeof(p.views[0].m));
  p.views[0].width = width;
  p.views[0].height = height;
  p.views[0].lod = lod_voxel_size;
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c->stream();
  RAYT_CUDA_TRY(rayt::launch_depth_view(p, s));
  RAYT_CUDA_TRY(cudaStreamSynchronize(s));
  return RAYT_OK;
}
int rayt_renderer_count_fetches(rayt_renderer* r, const float* m, int64_t counts[6]) {
  if (!r || !m || !counts) return fail(RAYT_E_ARG, "null argument");
  return R(r)->CountFetches(m, counts);
}
int rayt_renderer_time_pass(rayt_renderer* r, const float* m, int reps, float* ms) {
  if (!r || !m || !ms || reps < 1) return fail(RAYT_E_ARG, "bad argument");
  return R(r)->TimePass(m, reps, ms);
}

}  // extern "C"
