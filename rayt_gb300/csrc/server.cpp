// Served form: frame requests of many clients rendered against one shared
// block cache, with continuous batching.  No counterpart in the reference,
// which renders one frame of one camera per RenderFrame
// (rayt/GPU_renderer/gpu-ray-tracer.cpp:66-227); the per-pass steps are that
// function's (traversal, feedback unique, decode, cache transaction).
//
// State on the device: one image buffer from which every client owns a
// framebuffer range (admission of clients by free framebuffer memory), the
// ray records of faulted rays between passes (admission of requests by free
// record capacity), per-client fault counters, the feedback bitmaps.
//
// A tick is one pass over everything in flight: requests admitted in this
// tick contribute their first-pass tiles, older requests their faulted rays,
// all in the same launches, so requests that arrive while others are on the
// GPU join at the next pass boundary.  One feedback unique serves the tick;
// its decode drives one cache transaction (shared LRU, block streaming).  A
// request ends when its rays stop faulting; at its pass cap (or when the
// cache filled during the tick) its faulted rays are shaded with their fault
// parent in the next tick instead.  Faulted rays restart from the camera
// (restart mode), so a request that ends without finishing rays has the
// image a fully resident cache gives, whichever requests shared its ticks.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>

#include "cache.h"
#include "feedback.h"
#include "internal.h"

namespace rayt {
namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

class Server {
 public:
  ~Server();
  int Init(Cache* cache, const rayt_server_config& cfg);
  int AddClient(int w, int h, int* id);
  int RemoveClient(int id);
  int Submit(int client, const float* m, uint64_t* request);
  int Step(int* finished);
  int Start();
  int Stop();
  int Wait(uint64_t request, double timeout_s, rayt_request_info* out);
  int ClientImage(int client, void** dev);
  int ReadClientImage(int client, void* host, size_t bytes);
  int HostImage(int client, const void** host);
  rayt_server_stats stats{};
  LibcRand rand;

 private:
  static constexpr int kBlockInts = 16;  // {words, rays out, pad, pad, work: first pass, continuation}
  struct Client {
    bool live = false;
    int w = 0, h = 0;
    int64_t base = 0;        // first pixel of its framebuffer
    int64_t pixels = 0;      // w * h rounded up to 64
    uint64_t in_flight = 0;  // request being rendered (0: none)
    uchar4* host = nullptr;  // pinned copy of the last finished frame (deliver_to_host)
    uchar4* stage = nullptr; // device copy of a finished frame on its way to `host`
    float* coords = nullptr; // pixel_coords(w, h) in device memory
  };
  struct Request {
    uint64_t id;
    int client;
    float m[16];
    double submit_s;
  };
  struct Flight {
    uint64_t id;
    int client;
    int passes = 0;
    bool fresh = true;       // first pass in the next tick
    bool finishing = false;  // next tick shades its faulted rays
    int64_t rays = 0;        // record capacity reserved
    float m[16];
    double submit_s, admit_s;
  };

  rayt_server_config cfg_{};
  Cache* cache_ = nullptr;
  cudaStream_t s_ = nullptr;
  uchar4* d_images_ = nullptr;
  int64_t image_pixels_ = 0;
  RayList lists_[2];
  int64_t list_cap_ = 0, reserved_ = 0;
  int* d_state_ = nullptr;  // [block 0][fault bits][hit bits][block 1][client faults]
  int fault_words_ = 0, hit_words_ = 0;
  int32_t* h_unique_ = nullptr;
  int32_t* d_unique_ = nullptr;
  int* h_counts_ = nullptr;  // mapped: unique count, fault count, rays faulted, client faults [kMaxClients]
  int* d_counts_ = nullptr;
  int* d_client_faults_ = nullptr;
  int tick_ = 0;
  int carried_ = 0;          // faulted rays carried into the next tick
  // deliver_to_host: finished frames are copied to their client's stage on
  // the GPU stream (the framebuffer is free for the client's next request
  // right after), and from there to the pinned host image on a copy stream
  // while the next ticks run; a host function on the copy stream records the
  // requests as done once their images are on the host.
  cudaStream_t copy_s_ = nullptr;
  cudaEvent_t staged_ev_ = nullptr, copied_ev_ = nullptr;
  bool copy_pending_ = false;  // copied_ev_ marks the last delivery
  struct Delivery {
    Server* server;
    std::vector<rayt_request_info> done;
  };
  static void CUDART_CB Delivered(void* delivery);
  FeedbackDecoder fb_;
  std::vector<Client> clients_;
  std::vector<Flight> flights_;

  std::mutex mu_;            // queue, done map, stats of waiters
  std::condition_variable cv_;
  std::deque<Request> queue_;
  std::unordered_map<uint64_t, rayt_request_info> done_;
  uint64_t next_id_ = 1;
  std::thread thread_;
  bool running_ = false, stop_ = false;
  int thread_rc_ = RAYT_OK;

  int* block(int k) const { return k ? d_state_ + kBlockInts + fault_words_ + hit_words_ : d_state_; }
  int Alloc(int64_t pixels, int64_t* base) const;
  TraceParams Params(int k) const;
  void Loop();
};

int Server::Init(Cache* cache, const rayt_server_config& cfg) {
  if (cfg.max_clients < 1 || cfg.max_clients > kMaxClients) return fail(RAYT_E_ARG, "max_clients out of range (1..64)");
  if (cfg.framebuffer_bytes < 256 || cfg.max_rays_in_flight < 1 || cfg.max_rays_in_flight >= (1ll << 30) ||
      cfg.max_passes < 1 || !(cfg.lod_voxel_size >= 0))
    return fail(RAYT_E_ARG, "bad server configuration");
  cfg_ = cfg;
  cache->Retain();  // the cache (its stream and buffers) outlives this server
  cache_ = cache;
  s_ = cache->stream();
  image_pixels_ = std::min<int64_t>(cfg.framebuffer_bytes / 4, 1ll << 30) & ~(int64_t)63;
  list_cap_ = cfg.max_rays_in_flight;
  clients_.resize(cfg.max_clients);
  if (cudaMalloc(&d_images_, image_pixels_ * 4) != cudaSuccess) return fail(RAYT_E_OOM, "framebuffer pool allocation failed");
  for (auto& l : lists_)
    if (cudaMalloc(&l.origin, list_cap_ * 16) != cudaSuccess || cudaMalloc(&l.dir, list_cap_ * 16) != cudaSuccess ||
        cudaMalloc(&l.parent, list_cap_ * 4) != cudaSuccess || cudaMalloc(&l.ray, list_cap_ * 4) != cudaSuccess)
      return fail(RAYT_E_OOM, "ray record allocation failed");
  fault_words_ = (int)((cache->tree_blocks() + 31) / 32);
  hit_words_ = (int)(((uint64_t)cache->max_blocks() * 2 + 31) / 32);
  const size_t words = 2 * kBlockInts + (size_t)fault_words_ + hit_words_ + kMaxClients;
  if (cudaMalloc(&d_state_, words * 4) != cudaSuccess) return fail(RAYT_E_OOM, "feedback state allocation failed");
  d_client_faults_ = d_state_ + 2 * kBlockInts + fault_words_ + hit_words_;
  const size_t bit_words = (size_t)fault_words_ + hit_words_;
  if (cudaHostAlloc(&h_unique_, (bit_words * 32 + 1) * 4, cudaHostAllocMapped) != cudaSuccess ||
      cudaHostAlloc(&h_counts_, (4 + kMaxClients) * 4, cudaHostAllocMapped) != cudaSuccess)
    return fail(RAYT_E_OOM, "pinned host allocation failed");
  RAYT_CUDA_TRY(cudaHostGetDevicePointer((void**)&d_unique_, h_unique_, 0));
  RAYT_CUDA_TRY(cudaHostGetDevicePointer((void**)&d_counts_, h_counts_, 0));
  RAYT_CUDA_TRY(cudaMemsetAsync(d_state_, 0, words * 4, s_));
  RAYT_CUDA_TRY(cudaMemsetAsync(d_images_, 0, image_pixels_ * 4, s_));
  if (cfg.deliver_to_host) {
    RAYT_CUDA_TRY(cudaStreamCreateWithFlags(&copy_s_, cudaStreamNonBlocking));
    RAYT_CUDA_TRY(cudaEventCreateWithFlags(&staged_ev_, cudaEventDisableTiming));
    RAYT_CUDA_TRY(cudaEventCreateWithFlags(&copied_ev_, cudaEventDisableTiming));
  }
  RAYT_CUDA_TRY(cudaStreamSynchronize(s_));
  return RAYT_OK;
}

Server::~Server() {
  Stop();
  if (s_) cudaStreamSynchronize(s_);
  if (copy_s_) {
    cudaStreamSynchronize(copy_s_);  // deliveries and their host functions end
    cudaStreamDestroy(copy_s_);
  }
  if (staged_ev_) cudaEventDestroy(staged_ev_);
  if (copied_ev_) cudaEventDestroy(copied_ev_);
  cudaFree(d_images_);
  for (auto& l : lists_) {
    cudaFree(l.origin);
    cudaFree(l.dir);
    cudaFree(l.parent);
    cudaFree(l.ray);
  }
  cudaFree(d_state_);
  cudaFreeHost(h_unique_);
  cudaFreeHost(h_counts_);
  for (auto& c : clients_) {
    if (c.host) cudaFreeHost(c.host);
    cudaFree(c.stage);
    cudaFree(c.coords);
  }
  Cache::Release(cache_);
}

void CUDART_CB Server::Delivered(void* delivery) {
  std::unique_ptr<Delivery> d(static_cast<Delivery*>(delivery));
  Server* s = d->server;
  const double t = now_s();
  std::lock_guard<std::mutex> lock(s->mu_);
  for (rayt_request_info& info : d->done) {
    info.done_s = std::max(info.done_s, t);
    s->done_[info.request] = info;
    ++s->stats.completed;
  }
  s->cv_.notify_all();
}

// First fit in the framebuffer pool (ranges ordered by base).
int Server::Alloc(int64_t pixels, int64_t* base) const {
  std::vector<std::pair<int64_t, int64_t>> used;
  for (const Client& c : clients_)
    if (c.live) used.emplace_back(c.base, c.base + c.pixels);
  std::sort(used.begin(), used.end());
  int64_t at = 0;
  for (auto& u : used) {
    if (u.first - at >= pixels) break;
    at = std::max(at, u.second);
  }
  if (at + pixels > image_pixels_) return RAYT_E_LIMIT;
  *base = at;
  return RAYT_OK;
}

int Server::AddClient(int w, int h, int* id) {
  if (w <= 0 || h <= 0 || (int64_t)w * h > (1 << 28)) return fail(RAYT_E_ARG, "client frame size out of range");
  if (running_) return fail(RAYT_E_ARG, "add clients while the scheduler thread is stopped");
  int slot = -1;
  for (int i = 0; i < (int)clients_.size(); ++i)
    if (!clients_[i].live) {
      slot = i;
      break;
    }
  if (slot < 0) return fail(RAYT_E_LIMIT, "no free client slot");
  const int64_t pixels = ((int64_t)w * h + 63) & ~(int64_t)63;
  int64_t base = 0;
  if (Alloc(pixels, &base) != RAYT_OK) return fail(RAYT_E_LIMIT, "not admitted: no free framebuffer memory");
  Client& c = clients_[slot];
  if (cfg_.deliver_to_host && !c.host &&
      cudaHostAlloc(&c.host, (size_t)w * h * 4, cudaHostAllocDefault) != cudaSuccess)
    return fail(RAYT_E_OOM, "pinned host image allocation failed");
  if (cfg_.deliver_to_host) {
    if (copy_s_) RAYT_CUDA_TRY(cudaStreamSynchronize(copy_s_));  // an earlier client's stage may still be read
    cudaFree(c.stage);
    c.stage = nullptr;
    if (cudaMalloc(&c.stage, (size_t)w * h * 4) != cudaSuccess) return fail(RAYT_E_OOM, "delivery stage allocation failed");
  }
  std::vector<float> coords(pixel_coords_count(w, h));
  pixel_coords(w, h, coords.data());
  cudaFree(c.coords);
  c.coords = nullptr;
  if (cudaMalloc(&c.coords, coords.size() * sizeof(float)) != cudaSuccess)
    return fail(RAYT_E_OOM, "pixel coordinate table allocation failed");
  RAYT_CUDA_TRY(cudaMemcpy(c.coords, coords.data(), coords.size() * sizeof(float), cudaMemcpyHostToDevice));
  c.live = true;
  c.w = w;
  c.h = h;
  c.base = base;
  c.pixels = pixels;
  c.in_flight = 0;
  *id = slot;
  return RAYT_OK;
}

int Server::RemoveClient(int id) {
  if (id < 0 || id >= (int)clients_.size() || !clients_[id].live) return fail(RAYT_E_ARG, "no such client");
  if (running_) return fail(RAYT_E_ARG, "remove clients while the scheduler thread is stopped");
  if (clients_[id].in_flight) return fail(RAYT_E_ARG, "client has a frame in flight");
  // its last delivery ends first (not under mu_: the delivery's host function takes it)
  if (copy_s_) RAYT_CUDA_TRY(cudaStreamSynchronize(copy_s_));
  std::lock_guard<std::mutex> lock(mu_);
  for (const Request& r : queue_)
    if (r.client == id) return fail(RAYT_E_ARG, "client has queued frames");
  clients_[id].live = false;
  if (clients_[id].host) cudaFreeHost(clients_[id].host);
  clients_[id].host = nullptr;
  cudaFree(clients_[id].stage);
  clients_[id].stage = nullptr;
  cudaFree(clients_[id].coords);
  clients_[id].coords = nullptr;
  return RAYT_OK;
}

int Server::Submit(int client, const float* m, uint64_t* request) {
  std::lock_guard<std::mutex> lock(mu_);
  if (client < 0 || client >= (int)clients_.size() || !clients_[client].live) return fail(RAYT_E_ARG, "no such client");
  Request r;
  r.id = next_id_++;
  r.client = client;
  std::memcpy(r.m, m, sizeof(r.m));
  r.submit_s = now_s();
  queue_.push_back(r);
  *request = r.id;
  ++stats.submitted;
  cv_.notify_all();
  return RAYT_OK;
}

TraceParams Server::Params(int k) const {
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
  p.bg[1] = (float)(216 / 255.);
  p.bg[2] = 1.0f;
  p.bg[3] = 1.0f;
  p.image = d_images_;
  p.tile_w_log2 = 2;
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
  p.fault_bits = reinterpret_cast<uint32_t*>(d_state_ + kBlockInts);
  p.fault_bit_limit = (int)cache_->tree_blocks();
  p.hit_bits = reinterpret_cast<uint32_t*>(d_state_ + kBlockInts + fault_words_);
  p.n_words = block(k);
  p.refill = 32;
  p.restart = 1;
  p.client_faults = d_client_faults_;
  // client slots by framebuffer base (free slots get an empty range at the end)
  std::vector<std::pair<int64_t, int>> order;
  for (int i = 0; i < (int)clients_.size(); ++i)
    if (clients_[i].live) order.emplace_back(clients_[i].base, i);
  std::sort(order.begin(), order.end());
  p.n_clients = (int)order.size();
  for (int i = 0; i < p.n_clients; ++i) p.client_base[i] = (int)order[i].first;
  p.client_base[p.n_clients] = (int)image_pixels_;
  return p;
}

// One tick: admit, one pass over everything in flight, feedback, transaction.
int Server::Step(int* finished) {
  if (finished) *finished = 0;
  {
    std::lock_guard<std::mutex> lock(mu_);
    // under the lock: every request admitted here was submitted before
    const double t_admit = now_s();
    for (auto it = queue_.begin(); it != queue_.end();) {
      Client& c = clients_[it->client];
      const int64_t rays = (int64_t)c.w * c.h;
      if (c.in_flight || reserved_ + rays > list_cap_) {
        ++it;
        continue;
      }
      Flight f;
      f.id = it->id;
      f.client = it->client;
      f.rays = rays;
      std::memcpy(f.m, it->m, sizeof(f.m));
      f.submit_s = it->submit_s;
      f.admit_s = t_admit;
      c.in_flight = f.id;
      reserved_ += rays;
      flights_.push_back(f);
      it = queue_.erase(it);
    }
  }
  if (flights_.empty()) return RAYT_OK;

  const int k = tick_ & 1;
  TraceParams p = Params(k);
  std::vector<int> slot_of_client(clients_.size(), -1);
  for (int i = 0; i < p.n_clients; ++i)
    for (int c = 0; c < (int)clients_.size(); ++c)
      if (clients_[c].live && clients_[c].base == p.client_base[i]) slot_of_client[c] = i;
  // clear this tick's block, the bitmaps and the client fault counters
  RAYT_CUDA_TRY(cudaMemsetAsync(k ? d_state_ + kBlockInts : d_state_, 0,
                                (kBlockInts + (size_t)fault_words_ + hit_words_) * 4, s_));
  RAYT_CUDA_TRY(cudaMemsetAsync(d_client_faults_, 0, kMaxClients * 4, s_));
  int64_t rays_tick = carried_;
  // first passes of newly admitted requests (one launch per 64 views)
  std::vector<ViewDesc> views;
  for (Flight& f : flights_)
    if (f.fresh) {
      const Client& c = clients_[f.client];
      ViewDesc v{};
      std::memcpy(v.m, f.m, sizeof(v.m));
      view_origin(v.m, v.origin);
      v.coords = c.coords;
      v.width = c.w;
      v.height = c.h;
      v.lod = cfg_.lod_voxel_size;
      v.pix_base = (int)c.base;
      views.push_back(v);
      rays_tick += (int64_t)c.w * c.h;
    }
  for (size_t g = 0; g < views.size(); g += kViewsPerLaunch) {
    TraceParams q = p;
    const int n = (int)std::min<size_t>(kViewsPerLaunch, views.size() - g);
    int64_t tiles = 0;
    for (int i = 0; i < n; ++i) {
      ViewDesc& v = views[g + i];
      v.tiles_x = (v.width + 3) / 4;
      v.tile_base = (int)tiles;
      tiles += (int64_t)v.tiles_x * ((v.height + 7) / 8);
      q.views[i] = v;
    }
    q.n_views = n;
    q.total_tiles = (int)tiles;
    q.work = block(k) + 4 + (int)(g / kViewsPerLaunch) % 8;
    RAYT_CUDA_TRY(launch_trace(q, true, false, (int)tiles * 32, 0, s_));
    ++stats.kernel_launches;
  }
  // faulted rays of older requests (finished instead for finishing ones)
  if (carried_ > 0) {
    TraceParams q = p;
    for (const Flight& f : flights_)
      if (!f.fresh && f.finishing) q.finish_mask |= 1ull << slot_of_client[f.client];
    q.work = block(k) + 12;
    RAYT_CUDA_TRY(launch_trace(q, false, false, carried_, 0, s_));
    ++stats.kernel_launches;
  }
  UniqueFromBitsParams u{};
  u.fault_bits = p.fault_bits;
  u.fault_words = fault_words_;
  u.hit_bits = p.hit_bits;
  u.hit_words = hit_words_;
  u.n_words = p.n_words;
  u.n_rays = p.n_out;
  u.total_pixels = (int)std::min<int64_t>(rays_tick, 1 << 30);
  u.unique_out = d_unique_;
  u.counts_out = d_counts_;
  RAYT_CUDA_TRY(launch_unique_from_bits(u, s_));
  ++stats.kernel_launches;
  RAYT_CUDA_TRY(cudaMemcpyAsync(h_counts_ + 4, d_client_faults_, kMaxClients * 4, cudaMemcpyDeviceToHost, s_));
  const double t_sync = now_s();
  RAYT_CUDA_TRY(cudaStreamSynchronize(s_));
  const double t_pass = now_s();
  stats.host_ms_wait += (t_pass - t_sync) * 1e3;
  stats.gpu_ms_upload += cache_->TakeUploadMs();  // the previous tick's block uploads
  stats.rays_traced += rays_tick;
  ++stats.ticks;
  carried_ = h_counts_[2];

  // which requests end with this tick
  std::vector<Flight> ended;
  std::vector<Flight> kept;
  for (Flight& f : flights_) {
    const int faults = h_counts_[4 + slot_of_client[f.client]];
    if (f.finishing) {  // its rays were shaded this tick
      ended.push_back(f);
      continue;
    }
    f.fresh = false;
    ++f.passes;
    if (faults == 0) ended.push_back(f);
    else {
      if (f.passes >= cfg_.max_passes) f.finishing = true;
      kept.push_back(f);
    }
  }

  // feedback decode and the cache transaction (shared LRU, block streaming)
  const int64_t uploaded0 = cache_->stats().uploaded_blocks;
  fb_.Decode(h_unique_, h_counts_[0], rand);
  int rc = cache_->StartSession();
  if (rc == RAYT_OK) rc = cache_->StartTransaction((int)fb_.faults.size());
  if (rc == RAYT_OK) {
    cache_->MarkUsedBatch(fb_.hits, fb_.dup_hits);
    for (int b : fb_.faults) {
      if (cache_->TransactionFilled()) break;
      if ((rc = cache_->RequestBlock(b)) != RAYT_OK) break;
    }
    const double t_lru = now_s();
    stats.host_ms_lru += (t_lru - t_pass) * 1e3;
    const int erc = cache_->EndTransaction();
    stats.host_ms_load += (now_s() - t_lru) * 1e3;
    if (rc == RAYT_OK) rc = erc;
  }
  stats.uploaded_blocks += cache_->stats().uploaded_blocks - uploaded0;
  const bool filled = cache_->in_session() && cache_->SessionFilled();
  if (cache_->in_transaction()) cache_->EndTransaction();
  if (cache_->in_session()) {
    const int src = cache_->EndSession();
    if (rc == RAYT_OK) rc = src;
  }
  if (rc != RAYT_OK) return rc;
  if (filled)  // the cache cannot hold this tick's blocks: stop the requests that still fault
    for (Flight& f : kept) f.finishing = true;
  stats.faults += (int64_t)fb_.faults.size();
  ++tick_;
  flights_.swap(kept);

  // deliver and record the requests that ended
  if (!ended.empty()) {
    std::unique_ptr<Delivery> delivery;
    if (cfg_.deliver_to_host) {
      // frames to their stages (after the previous delivery has read them),
      // then to the host on the copy stream; the framebuffers are free for the
      // clients' next requests in stream order
      delivery.reset(new Delivery{this, {}});
      if (copy_pending_) RAYT_CUDA_TRY(cudaStreamWaitEvent(s_, copied_ev_, 0));
      for (const Flight& f : ended) {
        const Client& c = clients_[f.client];
        RAYT_CUDA_TRY(cudaMemcpyAsync(c.stage, d_images_ + c.base, (size_t)c.w * c.h * 4, cudaMemcpyDeviceToDevice, s_));
      }
      RAYT_CUDA_TRY(cudaEventRecord(staged_ev_, s_));
      RAYT_CUDA_TRY(cudaStreamWaitEvent(copy_s_, staged_ev_, 0));
      for (const Flight& f : ended) {
        const Client& c = clients_[f.client];
        RAYT_CUDA_TRY(cudaMemcpyAsync(c.host, c.stage, (size_t)c.w * c.h * 4, cudaMemcpyDeviceToHost, copy_s_));
        stats.bytes_d2h += (int64_t)c.w * c.h * 4;
      }
      RAYT_CUDA_TRY(cudaEventRecord(copied_ev_, copy_s_));
      copy_pending_ = true;
    }
    const double t_done = now_s();
    std::lock_guard<std::mutex> lock(mu_);
    for (const Flight& f : ended) {
      rayt_request_info info{};
      info.request = f.id;
      info.client = f.client;
      info.passes = f.passes;
      info.truncated = f.finishing ? 1 : 0;
      info.submit_s = f.submit_s;
      info.admit_s = f.admit_s;
      info.done_s = std::max(t_pass, t_done);
      if (delivery) {
        delivery->done.push_back(info);  // done once the image is on the host
      } else {
        done_[f.id] = info;
        ++stats.completed;
      }
      clients_[f.client].in_flight = 0;
      reserved_ -= f.rays;
    }
    if (delivery) {
      RAYT_CUDA_TRY(cudaLaunchHostFunc(copy_s_, &Server::Delivered, delivery.get()));
      delivery.release();  // the host function owns it now
    } else {
      cv_.notify_all();
    }
  }
  if (finished) *finished = (int)ended.size();
  return RAYT_OK;
}

void Server::Loop() {
  for (;;) {
    {
      std::unique_lock<std::mutex> lock(mu_);
      cv_.wait(lock, [this] { return stop_ || !queue_.empty() || !flights_.empty(); });
      if (stop_) break;
    }
    const int rc = Step(nullptr);
    if (rc != RAYT_OK) {
      std::lock_guard<std::mutex> lock(mu_);
      thread_rc_ = rc;
      stop_ = true;
      cv_.notify_all();
      break;
    }
  }
}

int Server::Start() {
  if (running_) return RAYT_OK;
  stop_ = false;
  thread_rc_ = RAYT_OK;
  running_ = true;
  thread_ = std::thread([this] {
    int dev = 0;
    cudaGetDevice(&dev);
    Loop();
  });
  return RAYT_OK;
}

int Server::Stop() {
  if (!running_) return RAYT_OK;
  {
    std::lock_guard<std::mutex> lock(mu_);
    stop_ = true;
    cv_.notify_all();
  }
  thread_.join();
  running_ = false;
  return thread_rc_;
}

int Server::Wait(uint64_t request, double timeout_s, rayt_request_info* out) {
  const double deadline = now_s() + timeout_s;
  for (;;) {
    {
      std::unique_lock<std::mutex> lock(mu_);
      auto it = done_.find(request);
      if (it != done_.end()) {
        if (out) *out = it->second;
        done_.erase(it);
        return RAYT_OK;
      }
      if (request == 0 || request >= next_id_) return fail(RAYT_E_ARG, "unknown request");
      if (running_) {
        if (thread_rc_ != RAYT_OK) return thread_rc_;
        if (cv_.wait_until(lock, std::chrono::steady_clock::now() +
                                     std::chrono::duration<double>(std::max(0.0, deadline - now_s()))) ==
                std::cv_status::timeout &&
            done_.find(request) == done_.end())
          return fail(RAYT_E_TIMEOUT, "request not finished before the timeout");
        continue;
      }
    }
    if (now_s() > deadline) return fail(RAYT_E_TIMEOUT, "request not finished before the timeout");
    const bool idle = flights_.empty();
    const int rc = Step(nullptr);  // no scheduler thread: run ticks here
    if (rc != RAYT_OK) return rc;
    if (idle && copy_s_) RAYT_CUDA_TRY(cudaStreamSynchronize(copy_s_));  // a delivery still on its way
  }
}

int Server::ClientImage(int client, void** dev) {
  if (client < 0 || client >= (int)clients_.size() || !clients_[client].live) return fail(RAYT_E_ARG, "no such client");
  *dev = d_images_ + clients_[client].base;
  return RAYT_OK;
}

int Server::ReadClientImage(int client, void* host, size_t bytes) {
  if (client < 0 || client >= (int)clients_.size() || !clients_[client].live) return fail(RAYT_E_ARG, "no such client");
  const Client& c = clients_[client];
  if (bytes < (size_t)c.w * c.h * 4) return fail(RAYT_E_ARG, "image buffer too small");
  cudaStream_t s = nullptr;
  RAYT_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  cudaError_t e = cudaMemcpyAsync(host, d_images_ + c.base, (size_t)c.w * c.h * 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  RAYT_CUDA_TRY(e);
  return RAYT_OK;
}

int Server::HostImage(int client, const void** host) {
  if (client < 0 || client >= (int)clients_.size() || !clients_[client].live) return fail(RAYT_E_ARG, "no such client");
  if (!cfg_.deliver_to_host) return fail(RAYT_E_ARG, "server does not deliver frames to host memory");
  *host = clients_[client].host;
  return RAYT_OK;
}

}  // namespace rayt

using rayt::fail;
namespace {
rayt::Server* S(rayt_server* s) { return reinterpret_cast<rayt::Server*>(s); }
}  // namespace

extern "C" {

int rayt_server_create(rayt_cache* cache, const rayt_server_config* cfg, rayt_server** out) {
  if (!cache || !cfg || !out) return fail(RAYT_E_ARG, "rayt_server_create: null argument");
  rayt::Server* s = new rayt::Server();
  const int rc = s->Init(reinterpret_cast<rayt::Cache*>(cache), *cfg);
  if (rc != RAYT_OK) {
    delete s;
    return rc;
  }
  *out = reinterpret_cast<rayt_server*>(s);
  return RAYT_OK;
}
void rayt_server_destroy(rayt_server* s) { delete S(s); }
int rayt_server_add_client(rayt_server* s, int width, int height, int* client) {
  if (!s || !client) return fail(RAYT_E_ARG, "null argument");
  return S(s)->AddClient(width, height, client);
}
int rayt_server_remove_client(rayt_server* s, int client) {
  if (!s) return fail(RAYT_E_ARG, "null server");
  return S(s)->RemoveClient(client);
}
int rayt_server_seed(rayt_server* s, uint32_t seed) {
  if (!s) return fail(RAYT_E_ARG, "null server");
  S(s)->rand.Seed(seed);
  return RAYT_OK;
}
int rayt_server_submit(rayt_server* s, int client, const float view_proj_inv[16], uint64_t* request) {
  if (!s || !view_proj_inv || !request) return fail(RAYT_E_ARG, "null argument");
  return S(s)->Submit(client, view_proj_inv, request);
}
int rayt_server_step(rayt_server* s, int* finished) {
  if (!s) return fail(RAYT_E_ARG, "null server");
  return S(s)->Step(finished);
}
int rayt_server_start(rayt_server* s) { return s ? S(s)->Start() : fail(RAYT_E_ARG, "null server"); }
int rayt_server_stop(rayt_server* s) { return s ? S(s)->Stop() : fail(RAYT_E_ARG, "null server"); }
int rayt_server_wait(rayt_server* s, uint64_t request, double timeout_s, rayt_request_info* out) {
  if (!s) return fail(RAYT_E_ARG, "null server");
  return S(s)->Wait(request, timeout_s, out);
}
int rayt_server_client_image(rayt_server* s, int client, void** device_rgba) {
  if (!s || !device_rgba) return fail(RAYT_E_ARG, "null argument");
  return S(s)->ClientImage(client, device_rgba);
}
int rayt_server_read_client_image(rayt_server* s, int client, void* host_rgba, size_t bytes) {
  if (!s || !host_rgba) return fail(RAYT_E_ARG, "null argument");
  return S(s)->ReadClientImage(client, host_rgba, bytes);
}
int rayt_server_host_image(rayt_server* s, int client, const void** host_rgba) {
  if (!s || !host_rgba) return fail(RAYT_E_ARG, "null argument");
  return S(s)->HostImage(client, host_rgba);
}
int rayt_server_stats_get(const rayt_server* s, rayt_server_stats* out) {
  if (!s || !out) return fail(RAYT_E_ARG, "null argument");
  *out = reinterpret_cast<const rayt::Server*>(s)->stats;
  return RAYT_OK;
}

}  // extern "C"
