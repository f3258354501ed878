// Device block cache: the reference's GPUOctreeCacheManager + GPUOctreeCache +
// GPUOctreeData (rayt/GPU data/gpu-octree-cache-manager.cpp:13-212,
// gpu-octree-cache.cpp:11-313, gpu-octree-data.cpp:8-93).
//
// Policy and bookkeeping are the reference's, step for step, because they
// decide which slot every block lands in and therefore every node index the
// traversal reports:
//   * LRU order: least recently used first; MarkBlockAsUsed moves a block and
//     all its ancestors to the back; session/transaction markers sit in the
//     same list and count as "hit" once they reach the front
//     (gpu-octree-cache.cpp:58-76,236-241,295-313).
//   * UploadBlock: a free slot while there is one, otherwise protect the
//     parent and evict the LRU block, restoring up to 8 parent links to their
//     stored values (gpu-octree-cache.cpp:102-293).
// What differs is the mechanics: the LRU is an intrusive doubly linked list
// over slot ids with O(1) moves, block/parent lookups are flat arrays, and the
// device side of a batch of blocks is one scatter kernel that reads the blocks
// from the block file mapped into host memory (or from one pinned staging
// copy) and rewrites links on the device, and one patch kernel - instead of
// per-channel and per-pointer clEnqueueWriteBuffer calls.
#include "cache.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <mutex>
#include <thread>

namespace rayt {

// The distinct child blocks named by one block's fault links: an open-
// addressing set cleared in O(1) by a generation stamp, growing with the
// count (a block usually names a few dozen children, so the table stays in
// L1).  One per reading thread.
class ChildSet {
 public:
  void Clear() {
    n_ = 0;
    last_ = UINT32_MAX;
    if (++gen_ == 0) {  // stamps wrapped: forget every slot
      std::fill(stamp_.begin(), stamp_.end(), 0u);
      gen_ = 1;
    }
  }
  // True when v was not in the set (and is now).
  bool Insert(uint32_t v) {
    if (v == last_) return false;  // repeats are mostly adjacent links
    last_ = v;
    if (2 * (n_ + 1) > stamp_.size()) Grow();
    const uint32_t mask = (uint32_t)stamp_.size() - 1;
    for (uint32_t h = (v * 2654435761u) & mask;; h = (h + 1) & mask) {
      if (stamp_[h] != gen_) {
        stamp_[h] = gen_;
        key_[h] = v;
        ++n_;
        return true;
      }
      if (key_[h] == v) return false;
    }
  }

 private:
  std::vector<uint32_t> key_, stamp_;
  uint32_t gen_ = 1, n_ = 0, last_ = UINT32_MAX;
  void Grow() {
    const size_t size = stamp_.empty() ? 1024 : stamp_.size() * 4;
    std::vector<uint32_t> keys;
    for (size_t i = 0; i < stamp_.size(); ++i)
      if (stamp_[i] == gen_) keys.push_back(key_[i]);
    key_.assign(size, 0u);
    stamp_.assign(size, 0u);
    gen_ = 1;
    const uint32_t mask = (uint32_t)size - 1;
    for (uint32_t v : keys) {
      uint32_t h = (v * 2654435761u) & mask;
      while (stamp_[h] == gen_) h = (h + 1) & mask;
      stamp_[h] = gen_;
      key_[h] = v;
    }
  }
};

namespace {
ChildSet& child_set() {
  thread_local ChildSet s;
  return s;
}
}  // namespace

// Threads that read staged blocks from the file in parallel.  Run() returns
// only after every item is done and every worker has left the job, so the
// next Run() can reset the shared counters.  Wake() warns the pool that a job
// is coming: sleeping workers get up and spin (bounded) until it arrives, so
// the job does not pay for waking threads.
class Cache::ReadPool {
 public:
  explicit ReadPool(int threads) {
    for (int t = 0; t < threads; ++t) workers_.emplace_back([this] { Loop(); });
  }
  ~ReadPool() {
    {
      std::lock_guard<std::mutex> lock(mu_);
      quit_ = true;
    }
    cv_.notify_all();
    for (auto& w : workers_) w.join();
  }
  // Workers spin for up to `us` microseconds waiting for the next Run().
  void Wake(int us) {
    {
      std::lock_guard<std::mutex> lock(mu_);
      spin_until_ = Clock::now() + std::chrono::microseconds(us);
    }
    cv_.notify_all();
  }
  // Runs fn(0..n-1) on the pool and the calling thread.
  void Run(int n, std::function<void(int)> fn) {
    Start(n, std::move(fn));
    Wait();
  }
  // Hands fn(0..n-1) to the workers and returns at once; Wait() joins in and
  // returns when every item is done.  One job at a time.
  void Start(int n, std::function<void(int)> fn) {
    {
      std::lock_guard<std::mutex> lock(mu_);
      job_ = std::move(fn);
      fn_ = &job_;
      n_ = n;
      next_.store(0);
      done_ = 0;
      ++gen_;
      gen_seen_.store(gen_, std::memory_order_release);
    }
    cv_.notify_all();
  }
  void Wait() {
    if (!fn_) return;
    const int mine = Work(job_, n_) + helped_;
    helped_ = 0;
    std::unique_lock<std::mutex> lock(mu_);
    done_ += mine;
    done_cv_.wait(lock, [this] { return done_ == n_ && active_ == 0; });
    fn_ = nullptr;
  }
  // Between Start() and Wait(), on the thread that called Start(): runs the
  // job's next unclaimed item, if any (false when all are claimed).
  bool RunOne() {
    if (!fn_) return false;
    const int i = next_.fetch_add(1);
    if (i >= n_) return false;
    job_(i);
    ++helped_;
    return true;
  }

 private:
  using Clock = std::chrono::steady_clock;
  std::vector<std::thread> workers_;
  std::mutex mu_;
  std::condition_variable cv_, done_cv_;
  std::function<void(int)> job_;
  const std::function<void(int)>* fn_ = nullptr;  // &job_ while a job runs
  int n_ = 0, done_ = 0, active_ = 0;
  int helped_ = 0;  // items the starting thread ran through RunOne()
  uint64_t gen_ = 0;
  std::atomic<uint64_t> gen_seen_{0};  // gen_, readable without the lock
  Clock::time_point spin_until_{};
  std::atomic<int> next_{0};
  bool quit_ = false;

  int Work(const std::function<void(int)>& fn, int n) {
    int finished = 0;
    for (;;) {
      const int i = next_.fetch_add(1);
      if (i >= n) break;
      fn(i);
      ++finished;
    }
    return finished;
  }
  void Loop() {
    uint64_t seen = 0;
    for (;;) {
      const std::function<void(int)>* fn = nullptr;
      int n = 0;
      Clock::time_point spin{};
      {
        std::unique_lock<std::mutex> lock(mu_);
        cv_.wait(lock, [&] { return quit_ || (gen_ != seen && fn_) || spin_until_ > Clock::now(); });
        if (quit_) return;
        if (gen_ != seen && fn_) {
          seen = gen_;
          fn = fn_;
          n = n_;
          ++active_;
        } else {
          spin = spin_until_;
        }
      }
      if (!fn) {  // woken ahead of a job: wait for it without sleeping
        while (gen_seen_.load(std::memory_order_acquire) == seen && Clock::now() < spin) std::this_thread::yield();
        continue;
      }
      const int finished = Work(*fn, n);
      {
        std::lock_guard<std::mutex> lock(mu_);
        done_ += finished;
        --active_;
      }
      done_cv_.notify_all();
    }
  }
};

namespace {
inline uint32_t CacheLink(uint32_t mask, bool fault, bool dup, bool far_flag, uint32_t ptr) {
  return (ptr << 11) | ((far_flag ? 1u : 0u) << 10) | ((dup ? 1u : 0u) << 9) | ((fault ? 1u : 0u) << 8) | mask;
}
inline uint32_t NearValue(int64_t from, int64_t to) { return (uint32_t)((1 << 20) + (to - from)); }
constexpr int kStageBlocksMin = 16;
constexpr size_t kStageBytes = 32u << 20;  // per half
// Mapped blocks: positions per half.  A half is also the batch a transaction
// flushes while it places the next one, so that the device's reads of the
// file overlap the placement.
constexpr int kMappedStageBlocks = 512;
// A group of reads of at most this many links in all (8 blocks of 4096 nodes)
// runs on the calling thread: checking them (about 1.6 us per 4096 links on a
// Grace core) takes less than waking the pool's threads for them.
constexpr int64_t kInlineReadLinks = 32768;
}  // namespace

Cache::~Cache() {
  delete pool_;
  if (stream_) cudaStreamSynchronize(stream_);
  for (uint8_t* p : d_chan_) cudaFree(p);
  cudaFree(d_far_);
  cudaFree(d_stage_);  // d_slots_, d_blocks_, d_patches_ are the device views of the pinned arrays below
  cudaFreeHost(h_stage_);
  cudaFreeHost(h_slots_);
  cudaFreeHost(h_blocks_);
  cudaFreeHost(h_patches_);
  for (auto& e : stage_free_)
    if (e) cudaEventDestroy(e);
  for (auto& e : patch_free_)
    if (e) cudaEventDestroy(e);
  for (auto& e : flush_ev_) {
    cudaEventDestroy(e.first);
    cudaEventDestroy(e.second);
  }
  if (stream_) cudaStreamDestroy(stream_);
  Tree::Release(tree_);  // after every kernel that read its mapping has finished
}

int Cache::Init(Tree* tree, int max_blocks) {
  tree->Retain();
  tree_ = tree;
  nib_ = (int)tree->info.nodes_in_block;
  max_blocks_ = max_blocks > 0 ? max_blocks : (int)tree->info.blocks_count;
  const uint64_t nodes = (uint64_t)max_blocks_ * (uint64_t)nib_;
  // cache-format limits: far pointer slots (index*8+i) must fit in 21 bits;
  // node indices (far pointer values, the traversal's node arithmetic) are
  // unsigned 32-bit (the reference's per-pixel feedback word ((node+1)<<1)|dup
  // needs node < 2^30, which only recorded passes build)
  if (nodes >= (1ull << 32)) return fail(RAYT_E_LIMIT, "cache holds >= 2^32 nodes");
  if ((uint64_t)max_blocks_ * 8 >= (1ull << 21)) return fail(RAYT_E_LIMIT, "cache has >= 2^18 blocks (far pointer index overflows)");
  if (tree->chan_names.size() > (size_t)kMaxChannels) return fail(RAYT_E_LIMIT, "too many channels");
  RAYT_CUDA_TRY(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
  for (size_t c = 0; c < tree->chan_names.size(); ++c) {
    uint8_t* p = nullptr;
    const size_t bytes = (size_t)nodes * tree->chan_bytes[c];
    if (cudaMalloc(&p, bytes) != cudaSuccess) return fail(RAYT_E_OOM, "cache channel allocation failed");
    d_chan_.push_back(p);
    chan_bytes_.push_back(tree->chan_bytes[c]);
    RAYT_CUDA_TRY(cudaMemsetAsync(p, 0, bytes, stream_));
  }
  if (cudaMalloc(&d_far_, (size_t)max_blocks_ * 8 * 4) != cudaSuccess) return fail(RAYT_E_OOM, "far pointer allocation failed");
  RAYT_CUDA_TRY(cudaMemsetAsync(d_far_, 0, (size_t)max_blocks_ * 8 * 4, stream_));

  {
    const char* io = std::getenv("RAYT_BLOCK_IO");
    if (!(io && std::strcmp(io, "read") == 0)) file_host_ = tree->MapForDevice(&file_dev_);
    if (!file_dev_) file_host_ = nullptr;
    stats_.mapped = file_host_ ? 1 : 0;
  }
  area_ = ((size_t)tree->info.content_bytes + 80 + 15) & ~(size_t)15;
  // The per-position slot and block arrays and the patch records are small:
  // they live in mapped pinned memory that the upload and patch kernels read
  // directly (no copy per batch).
  auto mapped_alloc = [](void** host, void** dev, size_t bytes) {
    return cudaHostAlloc(host, bytes, cudaHostAllocMapped) == cudaSuccess &&
           cudaHostGetDevicePointer(dev, *host, 0) == cudaSuccess;
  };
  if (file_host_) {
    stage_cap_ = kMappedStageBlocks;
    if (!mapped_alloc(reinterpret_cast<void**>(&h_blocks_), reinterpret_cast<void**>(&d_blocks_),
                      sizeof(int) * stage_cap_ * 2))
      return fail(RAYT_E_OOM, "staging allocation failed");
  } else {
    stage_cap_ = (int)std::max<size_t>(kStageBlocksMin, kStageBytes / area_);
    if (cudaHostAlloc(&h_stage_, area_ * stage_cap_ * 2, cudaHostAllocDefault) != cudaSuccess ||
        cudaMalloc(&d_stage_, area_ * stage_cap_ * 2) != cudaSuccess)
      return fail(RAYT_E_OOM, "staging allocation failed");
  }
  if (!mapped_alloc(reinterpret_cast<void**>(&h_slots_), reinterpret_cast<void**>(&d_slots_),
                    sizeof(int) * stage_cap_ * 2))
    return fail(RAYT_E_OOM, "staging allocation failed");
  for (auto& e : stage_free_) RAYT_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  for (auto& e : patch_free_) RAYT_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  meta_.resize((size_t)stage_cap_ * 2);
  ready_.reset(new std::atomic<uint8_t>[(size_t)stage_cap_ * 2]);
  for (size_t k = 0; k < (size_t)stage_cap_ * 2; ++k) ready_[k].store(0, std::memory_order_relaxed);
  patch_cap_ = stage_cap_ * 32 + 64;
  if (!mapped_alloc(reinterpret_cast<void**>(&h_patches_), reinterpret_cast<void**>(&d_patches_),
                    sizeof(Patch) * patch_cap_ * 2))
    return fail(RAYT_E_OOM, "patch buffer allocation failed");
  {
    // Block checks on the mapped file are cheap (about 1.6 us for 4096
    // links), and the pool's workers spin from StartTransaction until the
    // reads arrive, where they compete with the decode and LRU marks on the
    // calling thread: for blocks of up to 4096 nodes 8 threads beat 16 by 6%
    // per c3 frame (4, 6 and 12 fell between).  Larger blocks (the served
    // workload's 16384 nodes) take 4x the check each and keep 16, as do reads
    // with pread into staging.
    const char* e = std::getenv("RAYT_IO_THREADS");
    const int hw = std::max(1, (int)std::thread::hardware_concurrency());
    const int want = file_host_ && nib_ <= 4096 ? 8 : 16;
    int threads = e && std::atoi(e) > 0 ? std::atoi(e) : std::min(hw, want);
    threads = std::max(1, std::min(threads, 16));
    pool_ = new ReadPool(threads - 1);  // the calling thread reads too
  }

  slots_.resize((size_t)max_blocks_);
  block_slot_.assign(tree->info.blocks_count, -1);
  parent_slot_.assign(tree->info.blocks_count, -1);
  validated_.assign(tree->info.blocks_count, 0);
  written_.assign((size_t)max_blocks_, 0);
  written_pos_.assign((size_t)max_blocks_, -1);
  patched_.assign((size_t)max_blocks_, 0);
  patch_head_.assign((size_t)max_blocks_, -1);
  const int ids = max_blocks_ + kMarkers + 1;
  prev_.assign(ids, -1);
  next_.assign(ids, -1);
  head_ = max_blocks_ + kMarkers;
  prev_[head_] = next_[head_] = head_;
  RAYT_CUDA_TRY(cudaStreamSynchronize(stream_));
  return RAYT_OK;
}

const void* Cache::channel(const std::string& name, int bytes) const {
  for (size_t c = 0; c < tree_->chan_names.size(); ++c)
    if (tree_->chan_names[c] == name && tree_->chan_bytes[c] == bytes) return d_chan_[c];
  return nullptr;
}

int Cache::Buffer(const char* name, void** ptr, size_t* bytes) {
  if (!name) return fail(RAYT_E_ARG, "null buffer name");
  if (std::string(name) == "far pointers") {
    if (ptr) *ptr = d_far_;
    if (bytes) *bytes = (size_t)max_blocks_ * 8 * 4;
    return RAYT_OK;
  }
  for (size_t c = 0; c < tree_->chan_names.size(); ++c)
    if (tree_->chan_names[c] == name) {
      if (ptr) *ptr = d_chan_[c];
      if (bytes) *bytes = (size_t)max_blocks_ * nib_ * chan_bytes_[c];
      return RAYT_OK;
    }
  return fail(RAYT_E_ARG, std::string("no cache channel named ") + name);
}

// ---- LRU list ----------------------------------------------------------------
void Cache::Unlink(int id) {
  next_[prev_[id]] = next_[id];
  prev_[next_[id]] = prev_[id];
  prev_[id] = next_[id] = -1;
}
void Cache::InsertBefore(int id, int before) {
  prev_[id] = prev_[before];
  next_[id] = before;
  next_[prev_[before]] = id;
  prev_[before] = id;
}
// MarkBlockAsUsed: the block and every ancestor, bottom up, to the MRU end.
void Cache::Touch(int slot) {
  for (int s = slot; s != (int)kRootParent; s = slots_[s].parent) {
    Unlink(s);
    InsertBefore(s, head_);
  }
  DequeueMarkers();
}
void Cache::DequeueMarkers() {
  while (next_[head_] != head_ && next_[head_] >= max_blocks_) {
    const int id = next_[head_];
    markers_[id - max_blocks_].hit = true;
    markers_[id - max_blocks_].live = false;
    Unlink(id);
  }
}
void Cache::InsertMarker(int k) {
  DropMarker(k);
  markers_[k].hit = false;
  markers_[k].live = true;
  InsertBefore(max_blocks_ + k, head_);
}
void Cache::DropMarker(int k) {
  if (markers_[k].live) Unlink(max_blocks_ + k);
  markers_[k].live = false;
}

// ---- uploads -------------------------------------------------------------------
void Cache::AddPatch(bool far_buffer, uint32_t index, uint32_t value) {
  const uint64_t where = ((uint64_t)(far_buffer ? 1 : 0) << 32) | index;
  const int at = patch_at_.Find(where);
  if (at >= 0) {
    patches_[at].value = value;  // last write to an address wins
    patch_dead_[at] = 0;         // (after any newer content of its slot)
  } else {
    const int pos = (int)patches_.size();
    patch_at_.Insert(where, pos);
    patches_.push_back(Patch{index, value, far_buffer ? 1u : 0u});
    patch_dead_.push_back(0);
    int next = -1;
    if (!far_buffer) {  // chain the slot's link patches of this batch
      const uint32_t s = index / (uint32_t)nib_;
      if (patched_[s] == epoch_) next = patch_head_[s];
      patched_[s] = epoch_;
      patch_head_[s] = pos;
    }
    patch_next_.push_back(next);
  }
  ++stats_.pointer_patches;
  if (far_buffer) ++stats_.far_pointer_writes;
}

// Uploads positions [batch_begin_, end) of the current half (slot -1 =
// staged but not placed: skipped by the kernel), then the batch's patches.
int Cache::FlushTo(int end) {
  if (end <= batch_begin_ && patches_.empty()) return RAYT_OK;
  const int h = half_;
  // device time of the batch: events around its copies and kernels (the
  // last 256 batches between two TakeUploadMs calls are counted)
  if (flush_used_ == kFlushEvents) flush_used_ = 0;
  if (flush_used_ == (int)flush_ev_.size()) {
    cudaEvent_t a = nullptr, b = nullptr;
    RAYT_CUDA_TRY(cudaEventCreate(&a));
    RAYT_CUDA_TRY(cudaEventCreate(&b));
    flush_ev_.emplace_back(a, b);
  }
  const std::pair<cudaEvent_t, cudaEvent_t> ev = flush_ev_[flush_used_++];
  RAYT_CUDA_TRY(cudaEventRecord(ev.first, stream_));
  if (end > batch_begin_) {
    const size_t first = (size_t)stage_cap_ * h + batch_begin_;
    const int n = end - batch_begin_;
    UploadParams up{};
    if (file_host_) {  // the kernel reads the blocks from the mapped file
      up.file = file_dev_;
      up.file_first = tree_->info.header_bytes + 76;
      up.file_stride = tree_->info.block_stride;
      up.block_ids = d_blocks_ + first;
    } else {
      uint8_t* hs = h_stage_ + area_ * first;
      uint8_t* ds = d_stage_ + area_ * first;
      RAYT_CUDA_TRY(cudaMemcpyAsync(ds, hs, area_ * n, cudaMemcpyHostToDevice, stream_));
      up.stage = ds + 80;
      up.stride = area_;
    }
    up.slots = d_slots_ + first;  // read by the kernel from pinned host memory
    up.blocks = n;
    up.nodes_in_block = nib_;
    up.channels = (int)d_chan_.size();
    for (int c = 0; c < up.channels; ++c) {
      up.chan_bytes[c] = chan_bytes_[c];
      up.chan[c] = d_chan_[c];
    }
    RAYT_CUDA_TRY(launch_upload(up, stream_));
    ++launches_;
    stats_.bytes_h2d += (int64_t)(file_host_ ? (size_t)tree_->info.content_bytes * n : area_ * n);
  }
  size_t live = 0;  // patches newer content of their slot did not overwrite, in order
  for (size_t i = 0; i < patches_.size(); ++i)
    if (!patch_dead_[i]) patches_[live++] = patches_[i];
  patches_.resize(live);
  size_t done = 0;
  while (done < patches_.size()) {
    const size_t n = std::min(patches_.size() - done, (size_t)patch_cap_);
    const int ph = patch_half_;
    Patch* hp = h_patches_ + (size_t)patch_cap_ * ph;
    Patch* dp = d_patches_ + (size_t)patch_cap_ * ph;
    // a pinned patch half is refilled only after the kernel that read it finished
    RAYT_CUDA_TRY(cudaEventSynchronize(patch_free_[ph]));
    std::memcpy(hp, patches_.data() + done, n * sizeof(Patch));
    RAYT_CUDA_TRY(launch_patches(dp, (int)n, reinterpret_cast<uint32_t*>(d_chan_[0]), d_far_, stream_));
    RAYT_CUDA_TRY(cudaEventRecord(patch_free_[ph], stream_));
    patch_half_ ^= 1;
    ++launches_;
    stats_.bytes_h2d += (int64_t)(n * sizeof(Patch));
    done += n;
  }
  patches_.clear();
  patch_dead_.clear();
  patch_next_.clear();
  patch_at_.Clear();
  batch_begin_ = std::max(batch_begin_, end);
  ++epoch_;
  RAYT_CUDA_TRY(cudaEventRecord(ev.second, stream_));
  return RAYT_OK;
}

// Sum of the device time of the batches flushed since the last call (their
// copies, upload and patch kernels); the caller has synchronised the stream.
float Cache::TakeUploadMs() {
  float total = 0;
  for (int i = 0; i < flush_used_; ++i) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, flush_ev_[i].first, flush_ev_[i].second) == cudaSuccess) total += ms;
  }
  flush_used_ = 0;
  return total;
}

// Flushes what is staged and continues in the other half once that half's
// last copies have finished.
int Cache::NextHalf() {
  int rc = FlushTo(staged_);
  if (rc != RAYT_OK) return rc;
  RAYT_CUDA_TRY(cudaEventRecord(stage_free_[half_], stream_));
  half_ ^= 1;
  staged_ = batch_begin_ = 0;
  RAYT_CUDA_TRY(cudaEventSynchronize(stage_free_[half_]));
  return RAYT_OK;
}

// UnloadLRUBlock (gpu-octree-cache.cpp:243-293)
int Cache::Unload() {
  const int s = next_[head_];
  if (s == head_ || s >= max_blocks_) {
    set_error("cache: LRU front is not a block");
    return -1;
  }
  Slot& info = slots_[s];
  const int p = info.parent;
  if (p == (int)kRootParent) {
    set_error("cache: the root block reached the LRU front");
    return -1;
  }
  for (int i = 0; i < info.roots_count; ++i) {
    uint32_t v = info.ptr_value[i];
    const uint32_t mask = v & 255u, fault = (v >> 8) & 1u, dup = (v >> 9) & 1u, ptr = v >> 11;
    if (mask && !fault) v = CacheLink(mask, false, dup != 0, false, NearValue(info.ptr_index[i], ptr));
    AddPatch(false, (uint32_t)((int64_t)p * nib_ + info.ptr_index[i]), v);
  }
  for (int c : info.children) parent_slot_[c] = -1;
  info.children.clear();
  Unlink(s);
  block_slot_[info.block] = -1;
  DequeueMarkers();
  return s;
}

// LoadBlock (stored-octree-loader.cpp:31-58) for staging position `pos` of
// the current half, with the checks and the fault-link scan UploadBlock needs:
// the block record is read into the position's staging area, or, with the
// file mapped, checked where it lies.  Safe to run on several threads for
// different positions.
int Cache::ReadOne(int pos, int block) {
  Staged& m = meta_[(size_t)stage_cap_ * half_ + pos];
  m.block = block;
  m.rc = RAYT_OK;
  m.faults.clear();
  const int64_t off = (int64_t)tree_->info.header_bytes + (int64_t)tree_->info.block_stride * (uint32_t)block;
  const uint8_t* raw;  // the 76-byte block header, then the content (any alignment when mapped)
  if (file_host_) {
    raw = file_host_ + off;
  } else {
    uint8_t* area = h_stage_ + area_ * ((size_t)stage_cap_ * half_ + pos);
    if (!tree_->Read(off, 76 + (size_t)tree_->info.content_bytes, area + 4)) {
      m.rc = RAYT_E_IO;
      m.err = "block read failed";
      return m.rc;
    }
    raw = area + 4;
  }
  rayt_block_header& hdr = m.hdr;
  std::memcpy(&hdr.block_index, raw, 4);
  std::memcpy(&hdr.parent_block_index, raw + 4, 4);
  std::memcpy(&hdr.roots_count, raw + 8, 4);
  for (int i = 0; i < 8; ++i) {
    std::memcpy(&hdr.roots[i].parent_pointer_index, raw + 12 + 8 * i, 2);
    std::memcpy(&hdr.roots[i].pointed_child_index, raw + 14 + 8 * i, 2);
    std::memcpy(&hdr.roots[i].parent_pointer_value, raw + 16 + 8 * i, 4);
  }
  auto bad = [&m](const char* why) {
    m.rc = RAYT_E_FORMAT;
    m.err = why;
    return m.rc;
  };
  if (hdr.roots_count < 1 || hdr.roots_count > 8) return bad("block has an invalid root count");
  const uint32_t blocks = tree_->info.blocks_count;
  if (hdr.parent_block_index != kRootParent) {
    for (uint32_t i = 0; i < hdr.roots_count; ++i) {
      const rayt_block_root& r = hdr.roots[i];
      const uint32_t pv = r.parent_pointer_value;
      if (r.parent_pointer_index >= nib_ || r.pointed_child_index >= nib_ ||
          (((pv >> 8) & 1u) && (pv & 255u) && (pv >> 11) >= blocks))
        return bad("block root record is out of range");
    }
  }
  const uint8_t* links = raw + 76;
  auto link = [links](int n) {
    uint32_t l;
    std::memcpy(&l, links + 4 * (size_t)n, 4);
    return l;
  };
  // Fault links name child blocks, most of them many times: keep each child
  // once, in order of first appearance (Place records a child under the first
  // link that names it, so later repeats change nothing there).
  ChildSet& seen = child_set();
  seen.Clear();
  auto children = [&](int from, int to) {  // fault links (fault bit and a non-empty mask)
    for (int k = from; k < to; ++k) {
      const uint32_t l = link(k);
      if ((l & 0x1FFu) > 0x100u && seen.Insert(l >> 11)) m.faults.push_back(l >> 11);
    }
  };
  if (validated_[block]) {  // links checked on an earlier load: only the fault children
    int n = 0;
    for (; n + 16 <= nib_; n += 16) {
      uint32_t any_fault = 0;
      for (int k = 0; k < 16; ++k) any_fault |= (uint32_t)((link(n + k) & 0x1FFu) > 0x100u);
      if (any_fault) children(n, n + 16);
    }
    children(n, nib_);
    return RAYT_OK;
  }
  // Every used link must stay in range: a child link's children inside the
  // block (ptr + children <= nodes in the block), a fault link's block below
  // the block count.  Checked branch-free in groups of 16 links (the group's
  // loop vectorises: 5.8 -> 4.2 us per 4096-link block on a Grace core); a
  // group holding a fault link is read again for the children.
  uint32_t child_bad = 0, fault_bad = 0;
  auto check = [&](uint32_t l, uint32_t& any_fault) {
    const uint32_t mask = l & 255u, ptr = l >> 11, fault = (l >> 8) & 1u;
    uint32_t c = mask - ((mask >> 1) & 0x55u);  // children: popcount of the 8-bit mask
    c = (c & 0x33u) + ((c >> 2) & 0x33u);
    c = (c + (c >> 4)) & 0x0Fu;
    const uint32_t used = mask != 0;
    child_bad |= used & (fault ^ 1u) & (uint32_t)(ptr + c > (uint32_t)nib_);
    fault_bad |= used & fault & (uint32_t)(ptr >= blocks);
    any_fault |= used & fault;
  };
  int n = 0;
  for (; n + 16 <= nib_; n += 16) {
    uint32_t any_fault = 0;
    for (int k = 0; k < 16; ++k) check(link(n + k), any_fault);
    if (any_fault) children(n, n + 16);
  }
  {
    uint32_t any_fault = 0;
    for (int k = n; k < nib_; ++k) check(link(k), any_fault);
    if (any_fault) children(n, nib_);
  }
  if (child_bad) return bad("child link points past the end of its block");
  if (fault_bad) return bad("fault link points past the last block");
  validated_[block] = 1;  // one byte per block: threads reading other blocks touch other bytes
  return RAYT_OK;
}

// Reads blocks[0..n) into positions [staged_, staged_ + n) in parallel.
int Cache::Prefetch(const int* blocks, int n) {
  StartRead(blocks, n);
  FinishRead();
  return RAYT_OK;
}

// Starts reading blocks[0..n) into positions [staged_, staged_ + n) on the
// pool and claims the positions; FinishRead() waits for them.  The caller
// may place earlier positions meanwhile (reads touch only their positions).
void Cache::StartRead(const int* blocks, int n) {
  const int first = staged_;
  const size_t base = (size_t)stage_cap_ * half_ + first;
  read_started_ = std::chrono::steady_clock::now();
  for (int i = 0; i < n; ++i) {
    h_slots_[base + i] = -1;
    if (h_blocks_) h_blocks_[base + i] = blocks[i];
    ready_[base + i].store(0, std::memory_order_relaxed);
  }
  auto read = [this, first, base, blocks](int i) {
    if (!cancel_reads_.load(std::memory_order_relaxed)) ReadOne(first + i, blocks[i]);
    ready_[base + i].store(1, std::memory_order_release);
  };
  if ((int64_t)n * nib_ <= kInlineReadLinks) {
    for (int i = 0; i < n; ++i) read(i);  // few: no pool
  } else {
    pool_->Start(n, read);
  }
  staged_ += n;
}
void Cache::FinishRead() {
  pool_->Wait();
  stats_.io_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - read_started_).count();
}

// UploadBlock (gpu-octree-cache.cpp:102-234) for the block staged at `pos`;
// with a queue, its fault children are appended in InitialFillCache's
// breadth-first order.
int Cache::Place(int pos, std::vector<int>* queue) {
  Staged& m = meta_[(size_t)stage_cap_ * half_ + pos];
  if (m.rc != RAYT_OK) return fail(m.rc, "cache: " + m.err);
  const int block = m.block;
  const rayt_block_header& hdr = m.hdr;
  stats_.bytes_read += (int64_t)tree_->info.content_bytes + 76;
  const bool is_root = hdr.parent_block_index == kRootParent;
  const int root_child = hdr.roots[0].pointed_child_index;
  if (!is_root && parent_slot_[block] < 0) return fail(RAYT_E_STATE, "cache: parent of a requested block is not resident");

  int s;
  if (first_free_ == max_blocks_) {
    if (!is_root) Touch(parent_slot_[block]);  // MarkParentAsUsed(block, global)
    s = Unload();
    if (s < 0) return RAYT_E_STATE;
  } else {
    s = first_free_++;
  }
  // This content overwrites the whole slot: an older content of the slot in
  // this batch is not uploaded, and the batch's earlier patches into the
  // slot's links are dropped (the sequential order would overwrite both).
  const size_t spos = (size_t)stage_cap_ * half_ + pos;
  if (written_[s] == epoch_) h_slots_[written_pos_[s]] = -1;
  if (patched_[s] == epoch_)
    for (int q = patch_head_[s]; q >= 0; q = patch_next_[q]) patch_dead_[q] = 1;
  written_[s] = epoch_;
  written_pos_[s] = (int)spos;
  h_slots_[spos] = s;

  Slot& info = slots_[s];
  for (uint32_t ptr : m.faults) {
    if (parent_slot_[ptr] < 0) {
      parent_slot_[ptr] = s;
      info.children.push_back((int)ptr);
    }
    if (queue) queue->push_back((int)ptr);
  }
  ++stats_.uploaded_blocks;

  if (!is_root) {
    const int ps = parent_slot_[block];
    info.parent = ps;
    info.roots_count = (int)hdr.roots_count;
    for (uint32_t i = 0; i < hdr.roots_count; ++i) {
      const rayt_block_root& r = hdr.roots[i];
      const uint32_t pv = r.parent_pointer_value;
      info.ptr_index[i] = r.parent_pointer_index;
      info.ptr_value[i] = r.parent_pointer_value;
      const int64_t absolute = (int64_t)s * nib_ + r.pointed_child_index;
      const int64_t ptr_at = (int64_t)ps * nib_ + r.parent_pointer_index;
      const bool far_flag = (ptr_at > absolute ? ptr_at - absolute : absolute - ptr_at) >= (1 << 20);
      uint32_t ptr;
      if (far_flag) {
        ptr = (uint32_t)s * 8 + i;
        AddPatch(true, ptr, (uint32_t)absolute);
      } else {
        ptr = NearValue(ptr_at, absolute);
      }
      // a root whose stored parent pointer is not a fault duplicates a node of
      // the parent block (gpu-octree-cache.cpp:207-208)
      AddPatch(false, (uint32_t)ptr_at, CacheLink(pv & 255u, false, ((pv >> 8) & 1u) == 0, far_flag, ptr));
    }
  } else {
    info.parent = (int)kRootParent;
    info.roots_count = 0;
  }
  block_slot_[block] = s;
  info.block = block;
  InsertBefore(s, next_[head_]);  // LRU front, then MarkBlockAsUsed
  Touch(s);
  if (is_root) root_node_ = (uint32_t)s * (uint32_t)nib_ + (uint32_t)root_child;
  return RAYT_OK;
}

// InitialFillCache (gpu-octree-cache-manager.cpp:60-108)
// The queue holds a block once per fault link that names it (often dozens of
// times); the reference skips an entry whose block is already in the cache
// when it pops it.  Here the next chunk takes the first occurrence of each
// block not yet loaded, reads the chunk in parallel and loads it in order -
// the same blocks in the same order.
int Cache::InitialFill() {
  std::vector<int> queue{(int)tree_->info.root_block_index};
  std::vector<uint8_t> taken(tree_->info.blocks_count, 0);
  std::vector<int> chunk;
  size_t head = 0;
  int rc = RAYT_OK;
  while (first_free_ < max_blocks_ && head < queue.size()) {
    if (staged_ == stage_cap_ && (rc = NextHalf()) != RAYT_OK) return rc;
    const int room = std::min(stage_cap_ - staged_, max_blocks_ - first_free_);
    chunk.clear();
    while (head < queue.size() && (int)chunk.size() < room) {
      const int b = queue[head++];
      if (taken[b] || block_slot_[b] >= 0) continue;
      taken[b] = 1;
      chunk.push_back(b);
    }
    if (chunk.empty()) break;
    const int first = staged_;
    if ((rc = Prefetch(chunk.data(), (int)chunk.size())) != RAYT_OK) return rc;
    for (int i = 0; i < (int)chunk.size() && first_free_ < max_blocks_; ++i)
      if ((rc = Place(first + i, &queue)) != RAYT_OK) return rc;
  }
  if ((rc = FlushTo(staged_)) != RAYT_OK) return rc;
  RAYT_CUDA_TRY(cudaStreamSynchronize(stream_));
  TakeUploadMs();  // frames report their own uploads, not the fill's
  return RAYT_OK;
}

int Cache::StartSession() {
  if (in_session_) return fail(RAYT_E_STATE, "session already started");
  in_session_ = true;
  InsertMarker(kSession);
  return RAYT_OK;
}
int Cache::StartTransaction(int expected_requests) {
  if (in_transaction_ || !in_session_) return fail(RAYT_E_STATE, "transaction needs an open session");
  in_transaction_ = true;
  InsertMarker(kTransaction);
  // the reads of EndTransaction follow the requests shortly (unless they are
  // few enough to run on this thread)
  if (expected_requests < 0 || (int64_t)expected_requests * nib_ > kInlineReadLinks) pool_->Wake(500);
  return RAYT_OK;
}
int Cache::MarkBlockUsed(int slot) {
  if (slot < 0 || slot >= first_free_) return fail(RAYT_E_ARG, "cache slot out of range");
  Touch(slot);
  return RAYT_OK;
}
int Cache::MarkParentUsed(int slot) {
  if (slot < 0 || slot >= first_free_) return fail(RAYT_E_ARG, "cache slot out of range");
  const int p = slots_[slot].parent;
  if (p == (int)kRootParent) DequeueMarkers();
  else Touch(p);
  return RAYT_OK;
}
// The feedback's marks of one pass: MarkBlockAsUsed for each hit block, then
// MarkParentAsUsed for each duplicate hit (ray-tracing-feedback-extractor.cpp
// order), with the list ending exactly as after the calls one by one.  One
// by one, every call moves its block and each ancestor up to the root block
// to the MRU end, so the list ends with the untouched slots in their old
// order followed by every touched slot in the order of its last move; and a
// marker reaches the front (and is taken off) once every slot before it has
// moved, which the last call's DequeueMarkers sees too, since nothing is
// inserted ahead of a marker.  The last move of a slot falls in the last call
// whose chain holds it, at its place in that chain (below its ancestors).
// Walking the calls from the last back, a chain stops at the first slot
// already seen (every ancestor of it was seen with it), so the batch walks
// each touched slot once instead of every chain to the root block (a pass
// marks up to 4000 blocks, most of them sharing their upper ancestors).
void Cache::MarkUsedBatch(const std::vector<int>& hits, const std::vector<int>& dup_hits) {
  touch_starts_.clear();
  for (int s : hits)
    if (s >= 0 && s < first_free_) touch_starts_.push_back(s);
  bool any = !touch_starts_.empty();
  for (int s : dup_hits) {
    if (s < 0 || s >= first_free_) continue;
    any = true;  // a root-level parent only dequeues markers
    if (slots_[s].parent != (int)kRootParent) touch_starts_.push_back(slots_[s].parent);
  }
  if (!any) return;
  if (touch_seen_.size() != (size_t)max_blocks_) touch_seen_.assign(max_blocks_, 0u);
  if (++touch_epoch_ == 0) {
    std::fill(touch_seen_.begin(), touch_seen_.end(), 0u);
    touch_epoch_ = 1;
  }
  touch_order_.clear();
  touch_groups_.clear();
  for (size_t i = touch_starts_.size(); i-- > 0;) {
    const int begin = (int)touch_order_.size();
    for (int s = touch_starts_[i]; s != (int)kRootParent && touch_seen_[s] != touch_epoch_; s = slots_[s].parent) {
      touch_seen_[s] = touch_epoch_;
      touch_order_.push_back(s);
    }
    if ((int)touch_order_.size() > begin) touch_groups_.emplace_back(begin, (int)touch_order_.size());
  }
  for (size_t g = touch_groups_.size(); g-- > 0;)
    for (int k = touch_groups_[g].first; k < touch_groups_[g].second; ++k) {
      Unlink(touch_order_[k]);
      InsertBefore(touch_order_[k], head_);
    }
  DequeueMarkers();
}

// RequestBlock (gpu-octree-cache-manager.cpp:138-148)
int Cache::RequestBlock(int block) {
  if (!in_transaction_) return fail(RAYT_E_STATE, "request outside a transaction");
  if (block < 0 || block >= (int)tree_->info.blocks_count) return fail(RAYT_E_ARG, "block index out of range");
  if (block_slot_[block] >= 0) return RAYT_OK;
  if (parent_slot_[block] < 0) return fail(RAYT_E_STATE, "requested block has no resident parent");
  pending_.push_back(block);
  Touch(parent_slot_[block]);
  return RAYT_OK;
}
// EndRequestTransaction (gpu-octree-cache-manager.cpp:150-194)
// The pending blocks are placed one by one in request order until the
// transaction fills the cache, exactly as the reference's loop does.  Reads
// have no side effects, so they run ahead: the pool reads the next chunk of
// kReadChunk blocks while this thread places the current one.
int Cache::EndTransaction() {
  if (!in_transaction_) return fail(RAYT_E_STATE, "no open transaction");
  int rc = RAYT_OK;
  size_t i = 0;  // next pending block to stage
  bool filled = TransactionFilled();
  using clock = std::chrono::steady_clock;
  auto secs = [](clock::time_point a) { return std::chrono::duration<double>(clock::now() - a).count(); };
  // One read job per staging half: the pool reads the half's blocks in
  // request order (each position flagged ready when its read is done) while
  // this thread places them in the same order as soon as each is ready,
  // helping with unclaimed reads while it waits.  No barrier between groups of
  // reads; reads not started when the transaction fills the cache are skipped.
  while (rc == RAYT_OK && !filled && i < pending_.size()) {
    if (staged_ == stage_cap_ && (rc = NextHalf()) != RAYT_OK) break;
    const int first = staged_;
    const int n = (int)std::min<size_t>((size_t)(stage_cap_ - staged_), pending_.size() - i);
    const size_t base = (size_t)stage_cap_ * half_ + first;
    StartRead(pending_.data() + i, n);
    i += (size_t)n;
    const auto t_loop = clock::now();
    double waited = 0;
    for (int k = 0; k < n; ++k) {
      if (!ready_[base + k].load(std::memory_order_acquire)) {
        const auto tw = clock::now();
        while (!ready_[base + k].load(std::memory_order_acquire))
          if (!pool_->RunOne()) std::this_thread::yield();
        waited += secs(tw);
      }
      if (TransactionFilled()) {
        filled = true;
        break;
      }
      if (block_slot_[meta_[base + k].block] >= 0) continue;
      if ((rc = Place(first + k, nullptr)) != RAYT_OK) break;
    }
    stats_.io_wait_seconds += waited;
    stats_.place_seconds += secs(t_loop) - waited;
    if (filled || rc != RAYT_OK) cancel_reads_.store(true, std::memory_order_relaxed);
    FinishRead();
    cancel_reads_.store(false, std::memory_order_relaxed);
  }
  pending_.clear();
  const auto tf = clock::now();
  const int frc = FlushTo(staged_);
  stats_.flush_seconds += secs(tf);
  in_transaction_ = false;
  DropMarker(kTransaction);
  return rc != RAYT_OK ? rc : frc;
}
int Cache::EndSession() {
  if (!in_session_ || in_transaction_) return fail(RAYT_E_STATE, "no open session (or a transaction is open)");
  in_session_ = false;
  DropMarker(kSession);
  return RAYT_OK;
}

}  // namespace rayt

// ---- C ABI -----------------------------------------------------------------------
using rayt::fail;
namespace {
rayt::Cache* C(rayt_cache* c) { return reinterpret_cast<rayt::Cache*>(c); }
const rayt::Cache* C(const rayt_cache* c) { return reinterpret_cast<const rayt::Cache*>(c); }
}  // namespace

extern "C" {

int rayt_cache_create(rayt_tree* tree, int max_blocks, rayt_cache** out) {
  if (!tree || !out) return fail(RAYT_E_ARG, "rayt_cache_create: null argument");
  rayt::Cache* c = new rayt::Cache();
  int rc = c->Init(reinterpret_cast<rayt::Tree*>(tree), max_blocks);
  if (rc != RAYT_OK) {
    delete c;
    return rc;
  }
  *out = reinterpret_cast<rayt_cache*>(c);
  return RAYT_OK;
}
void rayt_cache_destroy(rayt_cache* c) { rayt::Cache::Release(C(c)); }
int rayt_cache_initial_fill(rayt_cache* c) { return c ? C(c)->InitialFill() : fail(RAYT_E_ARG, "null cache"); }
int rayt_cache_root_node_index(const rayt_cache* c, int* out) {
  if (!c || !out) return fail(RAYT_E_ARG, "null argument");
  *out = (int)C(c)->root_node();  // the node index's 32 bits (unsigned beyond 2^31 - 1)
  return RAYT_OK;
}
int rayt_cache_blocks(const rayt_cache* c, int* loaded, int* max_blocks) {
  if (!c) return fail(RAYT_E_ARG, "null cache");
  if (loaded) *loaded = C(c)->loaded();
  if (max_blocks) *max_blocks = C(c)->max_blocks();
  return RAYT_OK;
}
int rayt_cache_device_buffer(rayt_cache* c, const char* name, void** ptr, size_t* bytes) {
  return c ? C(c)->Buffer(name, ptr, bytes) : fail(RAYT_E_ARG, "null cache");
}
int rayt_cache_read_buffer(rayt_cache* c, const char* name, void* host, size_t bytes) {
  if (!c || !host) return fail(RAYT_E_ARG, "null argument");
  void* d = nullptr;
  size_t have = 0;
  int rc = C(c)->Buffer(name, &d, &have);
  if (rc != RAYT_OK) return rc;
  if (bytes > have) return fail(RAYT_E_ARG, "read larger than the buffer");
  RAYT_CUDA_TRY(cudaStreamSynchronize(C(c)->stream()));
  RAYT_CUDA_TRY(cudaMemcpy(host, d, bytes, cudaMemcpyDeviceToHost));
  return RAYT_OK;
}
int rayt_cache_start_session(rayt_cache* c) { return c ? C(c)->StartSession() : fail(RAYT_E_ARG, "null cache"); }
int rayt_cache_start_transaction(rayt_cache* c) { return c ? C(c)->StartTransaction() : fail(RAYT_E_ARG, "null cache"); }
int rayt_cache_mark_block_used(rayt_cache* c, int slot) {
  if (!c) return fail(RAYT_E_ARG, "null cache");
  if (!C(c)->in_transaction()) return fail(RAYT_E_STATE, "mark outside a transaction");
  return C(c)->MarkBlockUsed(slot);
}
int rayt_cache_mark_parent_used(rayt_cache* c, int slot) {
  if (!c) return fail(RAYT_E_ARG, "null cache");
  if (!C(c)->in_transaction()) return fail(RAYT_E_STATE, "mark outside a transaction");
  return C(c)->MarkParentUsed(slot);
}
int rayt_testing_cache_mark_batch(rayt_cache* c, const int* hits, int n_hits, const int* dup_hits, int n_dup) {
  if (!c || n_hits < 0 || n_dup < 0 || (n_hits > 0 && !hits) || (n_dup > 0 && !dup_hits))
    return fail(RAYT_E_ARG, "rayt_testing_cache_mark_batch: bad argument");
  if (!C(c)->in_transaction()) return fail(RAYT_E_STATE, "mark outside a transaction");
  const std::vector<int> h(hits, hits + n_hits), d(dup_hits, dup_hits + n_dup);
  C(c)->MarkUsedBatch(h, d);
  return RAYT_OK;
}
int rayt_cache_request_block(rayt_cache* c, int block) { return c ? C(c)->RequestBlock(block) : fail(RAYT_E_ARG, "null cache"); }
int rayt_cache_transaction_filled(const rayt_cache* c, int* out) {
  if (!c || !out) return fail(RAYT_E_ARG, "null argument");
  if (!C(c)->in_transaction()) return fail(RAYT_E_STATE, "no open transaction");
  *out = C(c)->TransactionFilled() ? 1 : 0;
  return RAYT_OK;
}
int rayt_cache_session_filled(const rayt_cache* c, int* out) {
  if (!c || !out) return fail(RAYT_E_ARG, "null argument");
  if (!C(c)->in_session()) return fail(RAYT_E_STATE, "no open session");
  *out = C(c)->SessionFilled() ? 1 : 0;
  return RAYT_OK;
}
int rayt_cache_end_transaction(rayt_cache* c) { return c ? C(c)->EndTransaction() : fail(RAYT_E_ARG, "null cache"); }
int rayt_cache_end_session(rayt_cache* c) { return c ? C(c)->EndSession() : fail(RAYT_E_ARG, "null cache"); }
int rayt_cache_stats_get(const rayt_cache* c, rayt_cache_stats* out) {
  if (!c || !out) return fail(RAYT_E_ARG, "null argument");
  *out = C(c)->stats();
  return RAYT_OK;
}

}  // extern "C"
