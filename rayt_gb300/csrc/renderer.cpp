// Frame driver: the reference's GPURayTracer::RenderFrame
// (rayt/GPU_renderer/gpu-ray-tracer.cpp:66-227) and the host half of its
// RayTracingFeedbackExtractor (rayt/GPU_renderer/ray-tracing-feedback-extractor.cpp:100-185).
//
// Per pass: one traversal launch (first pass: every pixel from the camera,
// later passes: only rays that faulted), one launch that turns the feedback
// bitmaps into the reference's sorted unique array (written straight into
// host-mapped pinned memory), one stream synchronisation, then the host runs
// the reference's decode (all faults, plus a window of at most 4000 hits that
// starts at rand() % hits) and its cache transaction.  Block uploads go onto
// the same stream, so the next pass sees them without another wait.  The loop
// ends exactly where the reference's does: no faults, cache filled during the
// session, or (after the second pass) the time limit / pass cap.
#include <chrono>
#include <cstring>
#include <memory>

#include "cache.h"
#include "internal.h"

namespace rayt {

class Renderer {
 public:
  ~Renderer();
  int Init(Cache* cache, int w, int h);
  int Frame(const float* m);
  int CountFetches(const float* m, int64_t* counts);
  int TimePass(const float* m, int reps, float* ms);
  int ReadImage(void* host, size_t bytes);
  int PassWords(int pass, int32_t* host, size_t count) const;

  double time_limit = 1.0;  // the reference's default (gpu-ray-tracer.cpp:30-31)
  float lod = 1.5f;
  int max_passes = 0;
  bool record = false;
  LibcRand rand;
  rayt_frame_stats stats{};
  uchar4* image() const { return d_image_; }
  cudaStream_t stream() const { return s_; }

 private:
  Cache* cache_ = nullptr;
  int w_ = 0, h_ = 0;
  int expected_faults_ = 1 << 16;  // ray-tracing-feedback-extractor.cpp:22-23
  int hits_to_extract_ = 4000;
  cudaStream_t s_ = nullptr;
  uchar4* d_image_ = nullptr;
  float4* d_origin_ = nullptr;
  float4* d_dir_ = nullptr;
  int* d_parent_ = nullptr;
  int* d_active_[2] = {nullptr, nullptr};
  int* d_dense_ = nullptr;
  uint32_t* d_bits_ = nullptr;
  int fault_words_ = 0, hit_words_ = 0;
  int* d_counters_ = nullptr;        // [0] words, [1],[2] active counts of the two lists
  int* h_pass_ = nullptr;            // pinned copy of d_counters_
  unsigned long long* d_fetch_ = nullptr;
  int32_t* h_unique_ = nullptr;      // mapped pinned
  int32_t* d_unique_ = nullptr;
  int* h_counts_ = nullptr;          // mapped pinned: unique count, fault count
  int* d_counts_ = nullptr;
  int32_t* h_dense_ = nullptr;       // pinned, for recording
  uint8_t* d_flush_ = nullptr;       // L2 flush buffer for TimePass
  cudaEvent_t ev_[8] = {};
  std::vector<std::vector<int32_t>> pass_words_;
  std::vector<int> faults_, hits_, dup_hits_;

  TraceParams Params(const float* m) const;
  void Decode(int count);
  int Prepare(int it);
};

Renderer::~Renderer() {
  if (s_) cudaStreamSynchronize(s_);
  cudaFree(d_image_);
  cudaFree(d_origin_);
  cudaFree(d_dir_);
  cudaFree(d_parent_);
  cudaFree(d_active_[0]);
  cudaFree(d_active_[1]);
  cudaFree(d_dense_);
  cudaFree(d_bits_);
  cudaFree(d_counters_);
  cudaFree(d_fetch_);
  cudaFree(d_flush_);
  cudaFreeHost(h_pass_);
  cudaFreeHost(h_unique_);
  cudaFreeHost(h_counts_);
  cudaFreeHost(h_dense_);
  for (auto& e : ev_)
    if (e) cudaEventDestroy(e);
}

int Renderer::Init(Cache* cache, int w, int h) {
  if (w <= 0 || h <= 0 || (int64_t)w * h >= (1ll << 30)) return fail(RAYT_E_ARG, "frame size out of range");
  cache_ = cache;
  w_ = w;
  h_ = h;
  s_ = cache->stream();
  const size_t n = (size_t)w * h;
  if (cudaMalloc(&d_image_, n * 4) != cudaSuccess || cudaMalloc(&d_origin_, n * 16) != cudaSuccess ||
      cudaMalloc(&d_dir_, n * 16) != cudaSuccess || cudaMalloc(&d_parent_, n * 4) != cudaSuccess ||
      cudaMalloc(&d_active_[0], n * 4) != cudaSuccess || cudaMalloc(&d_active_[1], n * 4) != cudaSuccess ||
      cudaMalloc(&d_dense_, n * 4) != cudaSuccess || cudaMalloc(&d_counters_, 16 * 4) != cudaSuccess ||
      cudaMalloc(&d_fetch_, 8 * 8) != cudaSuccess)
    return fail(RAYT_E_OOM, "renderer device allocation failed");
  // one bit per block of the file; one bit per (cache block, duplicate flag)
  fault_words_ = (int)((cache->tree_blocks() + 31) / 32);
  hit_words_ = (int)(((uint64_t)cache->max_blocks() * 2 + 31) / 32);
  const size_t bit_words = (size_t)fault_words_ + hit_words_;
  if (cudaMalloc(&d_bits_, bit_words * 4) != cudaSuccess) return fail(RAYT_E_OOM, "feedback bitmap allocation failed");
  if (cudaHostAlloc(&h_unique_, (bit_words * 32 + 1) * 4, cudaHostAllocMapped) != cudaSuccess ||
      cudaHostAlloc(&h_counts_, 4 * 4, cudaHostAllocMapped) != cudaSuccess ||
      cudaHostAlloc(&h_pass_, 16 * 4, cudaHostAllocDefault) != cudaSuccess)
    return fail(RAYT_E_OOM, "pinned host allocation failed");
  RAYT_CUDA_TRY(cudaHostGetDevicePointer((void**)&d_unique_, h_unique_, 0));
  RAYT_CUDA_TRY(cudaHostGetDevicePointer((void**)&d_counts_, h_counts_, 0));
  for (auto& e : ev_) RAYT_CUDA_TRY(cudaEventCreate(&e));
  RAYT_CUDA_TRY(cudaMemsetAsync(d_image_, 0, n * 4, s_));
  RAYT_CUDA_TRY(cudaStreamSynchronize(s_));
  return RAYT_OK;
}

TraceParams Renderer::Params(const float* m) const {
  TraceParams p{};
  p.links = cache_->links();
  p.far_ptrs = cache_->far_ptrs();
  p.normals = static_cast<const char4*>(cache_->channel("normals", 4));
  p.colors = static_cast<const uchar4*>(cache_->channel("colors", 4));
  p.root = cache_->root_node();
  p.nodes_in_block = cache_->nodes_in_block();
  p.node_limit = (uint32_t)cache_->max_blocks() * (uint32_t)cache_->nodes_in_block();
  p.far_limit = (uint32_t)cache_->max_blocks() * 8u;
  p.width = w_;
  p.height = h_;
  std::memcpy(p.m, m, sizeof(p.m));
  p.lod = lod;
  p.bg[0] = 0.0f;
  p.bg[1] = (float)(216 / 255.);  // the reference's background (gpu-ray-tracer.cpp:190)
  p.bg[2] = 1.0f;
  p.bg[3] = 1.0f;
  p.origin = d_origin_;
  p.dir = d_dir_;
  p.fault_parent = d_parent_;
  p.image = d_image_;
  p.fault_bits = d_bits_;
  p.fault_bit_limit = (int)cache_->tree_blocks();
  p.hit_bits = d_bits_ + fault_words_;
  p.n_words = d_counters_;
  return p;
}

// ProcessUnique + AdjustExpectedFaults (ray-tracing-feedback-extractor.cpp:108-185)
// over the unique array in mapped host memory.
void Renderer::Decode(int count) {
  faults_.clear();
  hits_.clear();
  dup_hits_.clear();
  const int32_t* u = h_unique_;
  auto add_hit = [this](int32_t v) {
    if (v & 1) dup_hits_.push_back((v >> 1) - 1);
    else hits_.push_back((v >> 1) - 1);
  };
  int stride = expected_faults_, size = 0;
  while (size < count && (size == 0 || u[size - 1] < 0)) {
    stride = std::min(stride, count - size);
    for (int i = size; i < size + stride; ++i) {
      if (u[i] < 0) faults_.push_back(-u[i] - 1);
      else if (u[i] != kNoHit) add_hit(u[i]);
    }
    size += stride;
    stride *= 2;
  }
  if (size < count) {
    const int len = count - size;
    const int start = rand.Next() % len;
    const int take = std::min(hits_to_extract_, len);
    int seg[2][2];
    int nseg = 0;
    if (start + take <= len) {
      seg[nseg][0] = start; seg[nseg][1] = take; ++nseg;
    } else {
      seg[nseg][0] = 0; seg[nseg][1] = start + take - len; ++nseg;
      seg[nseg][0] = start; seg[nseg][1] = len - start; ++nseg;
    }
    for (int k = 0; k < nseg; ++k)
      for (int i = 0; i < seg[k][1]; ++i) {
        const int32_t v = u[size + seg[k][0] + i];
        if (v != kNoHit) add_hit(v);
      }
  }
  if (expected_faults_ > 1 && (int)faults_.size() < expected_faults_) expected_faults_ /= 2;
  else if ((int)faults_.size() > expected_faults_) expected_faults_ *= 2;
}


// Clears the per-pass feedback state; pass `it` appends faulted rays to list it % 2.
int Renderer::Prepare(int it) {
  RAYT_CUDA_TRY(cudaMemsetAsync(d_bits_, 0, ((size_t)fault_words_ + hit_words_) * 4, s_));
  RAYT_CUDA_TRY(cudaMemsetAsync(d_counters_, 0, 4, s_));
  RAYT_CUDA_TRY(cudaMemsetAsync(d_counters_ + 1 + (it & 1), 0, 4, s_));
  if (record) RAYT_CUDA_TRY(launch_fill_i32(d_dense_, kNoHit, (size_t)w_ * h_, s_));
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
  int rc = cache_->StartSession();
  if (rc != RAYT_OK) return rc;
  const int total = w_ * h_;
  int active_prev = total;  // rays traced by the first pass
  float ms_trace = 0, ms_fb = 0, ms_up = 0;
  int it;
  for (it = 0;; ++it) {
    if ((rc = Prepare(it)) != RAYT_OK) break;
    TraceParams p = Params(m);
    p.active_in = d_active_[(it + 1) & 1];
    p.n_active_in = d_counters_ + 1 + ((it + 1) & 1);
    p.active_out = d_active_[it & 1];
    p.n_active_out = d_counters_ + 1 + (it & 1);
    p.words_dense = record ? d_dense_ : nullptr;
    RAYT_CUDA_TRY(cudaEventRecord(ev_[0], s_));
    RAYT_CUDA_TRY(launch_trace(p, it == 0, false, active_prev, s_));
    launches += (it == 0 || active_prev > 0) ? 1 : 0;
    RAYT_CUDA_TRY(cudaEventRecord(ev_[1], s_));
    UniqueFromBitsParams q{};
    q.fault_bits = d_bits_;
    q.fault_words = fault_words_;
    q.hit_bits = d_bits_ + fault_words_;
    q.hit_words = hit_words_;
    q.n_words = d_counters_;
    q.total_pixels = total;
    q.unique_out = d_unique_;
    q.counts_out = d_counts_;
    RAYT_CUDA_TRY(launch_unique_from_bits(q, s_));
    launches += 1 + (record ? 1 : 0);
    RAYT_CUDA_TRY(cudaEventRecord(ev_[2], s_));
    RAYT_CUDA_TRY(cudaMemcpyAsync(h_pass_, d_counters_, 3 * 4, cudaMemcpyDeviceToHost, s_));
    if (record) {
      if (!h_dense_) RAYT_CUDA_TRY(cudaHostAlloc(&h_dense_, (size_t)total * 4, cudaHostAllocDefault));
      RAYT_CUDA_TRY(cudaMemcpyAsync(h_dense_, d_dense_, (size_t)total * 4, cudaMemcpyDeviceToHost, s_));
    }
    RAYT_CUDA_TRY(cudaStreamSynchronize(s_));
    float a = 0, b = 0;
    cudaEventElapsedTime(&a, ev_[0], ev_[1]);
    cudaEventElapsedTime(&b, ev_[1], ev_[2]);
    ms_trace += a;
    ms_fb += b;
    stats.rays_traced += active_prev;
    if (record) pass_words_.emplace_back(h_dense_, h_dense_ + total);
    const int active_now = h_pass_[1 + (it & 1)];
    d2h += 3 * 4 + 2 * 4 + (int64_t)h_counts_[0] * 4;  // counters, counts, unique array

    // the reference always gives the frame one round of loading, then stops
    // on its wall-clock limit (gpu-ray-tracer.cpp:123-125)
    const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (it > 0 && el > time_limit) { active_prev = active_now; break; }
    if (max_passes > 0 && it > 0 && it + 1 >= max_passes) { active_prev = active_now; break; }

    Decode(h_counts_[0]);
    if ((rc = cache_->StartTransaction()) != RAYT_OK) break;
    for (int b2 : hits_) cache_->MarkBlockUsed(b2);
    for (int b2 : dup_hits_) cache_->MarkParentUsed(b2);
    for (int f : faults_) {
      if (cache_->TransactionFilled()) break;
      if ((rc = cache_->RequestBlock(f)) != RAYT_OK) break;
    }
    stats.faults += (int)faults_.size();
    RAYT_CUDA_TRY(cudaEventRecord(ev_[3], s_));
    const int erc = cache_->EndTransaction();
    RAYT_CUDA_TRY(cudaEventRecord(ev_[4], s_));
    if (rc == RAYT_OK) rc = erc;
    if (rc != RAYT_OK) break;
    active_prev = active_now;
    if (faults_.empty() || cache_->SessionFilled()) break;
  }
  stats.passes = it + 1;
  stats.session_filled = cache_->in_session() && cache_->SessionFilled() ? 1 : 0;
  if (cache_->in_transaction()) cache_->EndTransaction();
  const int src = cache_->EndSession();
  if (rc != RAYT_OK) return rc;
  if (src != RAYT_OK) return src;
  // FinishTracingFrame for the rays still faulted, against the cache as it is now
  TraceParams p = Params(m);
  p.active_in = d_active_[it & 1];
  p.n_active_in = d_counters_ + 1 + (it & 1);
  RAYT_CUDA_TRY(launch_finish(p, active_prev, s_));
  if (active_prev > 0) ++launches;
  RAYT_CUDA_TRY(cudaStreamSynchronize(s_));
  if (stats.passes > 1 || stats.faults) {
    float up = 0;
    if (cudaEventElapsedTime(&up, ev_[3], ev_[4]) == cudaSuccess) ms_up += up;
  }
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
  int rc = Prepare(0);
  if (rc != RAYT_OK) return rc;
  RAYT_CUDA_TRY(cudaMemsetAsync(d_fetch_, 0, 8 * 8, s_));
  TraceParams p = Params(m);
  p.active_out = d_active_[0];
  p.n_active_out = d_counters_ + 1;
  p.counters = d_fetch_;
  RAYT_CUDA_TRY(launch_trace(p, true, true, 0, s_));
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
  float total = 0;
  for (int r = 0; r < reps; ++r) {
    RAYT_CUDA_TRY(cudaMemsetAsync(d_flush_, r & 255, flush, s_));
    int rc = Prepare(0);
    if (rc != RAYT_OK) return rc;
    TraceParams p = Params(m);
    p.active_out = d_active_[0];
    p.n_active_out = d_counters_ + 1;
    RAYT_CUDA_TRY(cudaEventRecord(ev_[5], s_));
    RAYT_CUDA_TRY(launch_trace(p, true, false, 0, s_));
    RAYT_CUDA_TRY(cudaEventRecord(ev_[6], s_));
    RAYT_CUDA_TRY(cudaEventSynchronize(ev_[6]));
    float a = 0;
    RAYT_CUDA_TRY(cudaEventElapsedTime(&a, ev_[5], ev_[6]));
    total += a;
  }
  *ms = reps > 0 ? total / reps : 0.0f;
  return RAYT_OK;
}

int Renderer::ReadImage(void* host, size_t bytes) {
  if (bytes < (size_t)w_ * h_ * 4) return fail(RAYT_E_ARG, "image buffer too small");
  RAYT_CUDA_TRY(cudaMemcpyAsync(host, d_image_, (size_t)w_ * h_ * 4, cudaMemcpyDeviceToHost, s_));
  RAYT_CUDA_TRY(cudaStreamSynchronize(s_));
  return RAYT_OK;
}

int Renderer::PassWords(int pass, int32_t* host, size_t count) const {
  if (pass < 0 || pass >= (int)pass_words_.size()) return fail(RAYT_E_ARG, "no recorded pass with that index");
  if (count < pass_words_[pass].size()) return fail(RAYT_E_ARG, "word buffer too small");
  std::memcpy(host, pass_words_[pass].data(), pass_words_[pass].size() * 4);
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
  int rc = r->Init(reinterpret_cast<rayt::Cache*>(cache), width, height);
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
int rayt_renderer_record_passes(rayt_renderer* r, int on) {
  if (!r) return fail(RAYT_E_ARG, "null renderer");
  R(r)->record = on != 0;
  return RAYT_OK;
}
int rayt_render_frame(rayt_renderer* r, const float m[16]) {
  if (!r || !m) return fail(RAYT_E_ARG, "rayt_render_frame: null argument");
  return R(r)->Frame(m);
}
int rayt_renderer_stream(rayt_renderer* r, void** stream) {
  if (!r || !stream) return fail(RAYT_E_ARG, "null argument");
  *stream = R(r)->stream();
  return RAYT_OK;
}
int rayt_renderer_image(rayt_renderer* r, void** dev) {
  if (!r || !dev) return fail(RAYT_E_ARG, "null argument");
  *dev = R(r)->image();
  return RAYT_OK;
}
int rayt_renderer_read_image(rayt_renderer* r, void* host, size_t bytes) {
  if (!r || !host) return fail(RAYT_E_ARG, "null argument");
  return R(r)->ReadImage(host, bytes);
}
int rayt_renderer_pass_words(rayt_renderer* r, int pass, int32_t* host, size_t count) {
  if (!r || !host) return fail(RAYT_E_ARG, "null argument");
  return R(r)->PassWords(pass, host, count);
}
int rayt_renderer_stats(const rayt_renderer* r, rayt_frame_stats* out) {
  if (!r || !out) return fail(RAYT_E_ARG, "null argument");
  *out = reinterpret_cast<const rayt::Renderer*>(r)->stats;
  return RAYT_OK;
}
int rayt_renderer_count_fetches(rayt_renderer* r, const float m[16], int64_t counts[6]) {
  if (!r || !m || !counts) return fail(RAYT_E_ARG, "null argument");
  return R(r)->CountFetches(m, counts);
}
int rayt_renderer_time_pass(rayt_renderer* r, const float m[16], int reps, float* ms) {
  if (!r || !m || !ms || reps < 1) return fail(RAYT_E_ARG, "bad argument");
  return R(r)->TimePass(m, reps, ms);
}

}  // extern "C"
