// Device block cache with the reference's LRU policy (host bookkeeping,
// device buffers and batched uploads).  See cache.cpp.
#pragma once
#include <cuda_runtime.h>
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdint>
#include <memory>
#include <string>
#include <unordered_map>
#include <vector>
#include "internal.h"
#include "tree.h"

namespace rayt {

// Position of each patched address in a batch's patch list: open addressing
// over 64-bit keys, cleared in O(1) by a generation stamp (the batch's
// patches are few, so the table stays in L1; std::unordered_map allocated a
// node per insert).
class PatchIndex {
 public:
  void Clear() {
    n_ = 0;
    if (++gen_ == 0) {
      std::fill(stamp_.begin(), stamp_.end(), 0u);
      gen_ = 1;
    }
  }
  // The value stored for key, or -1; with insert, stores `value` for a new key.
  int Find(uint64_t key) const {
    if (stamp_.empty()) return -1;
    const size_t mask = stamp_.size() - 1;
    for (size_t h = Hash(key) & mask;; h = (h + 1) & mask) {
      if (stamp_[h] != gen_) return -1;
      if (key_[h] == key) return val_[h];
    }
  }
  void Insert(uint64_t key, int value) {  // key must not be present
    if (2 * (n_ + 1) > stamp_.size()) Grow();
    const size_t mask = stamp_.size() - 1;
    size_t h = Hash(key) & mask;
    while (stamp_[h] == gen_) h = (h + 1) & mask;
    stamp_[h] = gen_;
    key_[h] = key;
    val_[h] = value;
    ++n_;
  }

 private:
  std::vector<uint64_t> key_;
  std::vector<int> val_;
  std::vector<uint32_t> stamp_;
  uint32_t gen_ = 1;
  size_t n_ = 0;
  static size_t Hash(uint64_t k) { return (size_t)((k * 0x9E3779B97F4A7C15ull) >> 20); }
  void Grow() {
    std::vector<uint64_t> keys;
    std::vector<int> vals;
    for (size_t i = 0; i < stamp_.size(); ++i)
      if (stamp_[i] == gen_) keys.push_back(key_[i]), vals.push_back(val_[i]);
    const size_t size = stamp_.empty() ? 1024 : stamp_.size() * 4;
    key_.assign(size, 0);
    val_.assign(size, 0);
    stamp_.assign(size, 0u);
    gen_ = 1;
    n_ = 0;
    for (size_t i = 0; i < keys.size(); ++i) Insert(keys[i], vals[i]);
  }
};

class Cache {
 public:
  ~Cache();
  int Init(Tree* tree, int max_blocks);
  // Reference count: the creator holds one; every renderer and server on the
  // cache holds one, so whichever is released last frees it.
  void Retain() { refs_.fetch_add(1); }
  static void Release(Cache* c) {
    if (c && c->refs_.fetch_sub(1) == 1) delete c;
  }

  // GPUOctreeCacheManager protocol
  int InitialFill();
  int StartSession();
  // expected_requests: the blocks the caller is about to request, when it
  // knows (a transaction that small reads them on the calling thread, so the
  // read pool is not woken for it); -1 when it does not.
  int StartTransaction(int expected_requests = -1);
  int MarkBlockUsed(int slot);
  int MarkParentUsed(int slot);
  // MarkBlockUsed for every slot of hits, then MarkParentUsed for every slot
  // of dup_hits, in that order, applied as one batch with the same result
  // (slots out of range are skipped, as the one-by-one calls refuse them).
  void MarkUsedBatch(const std::vector<int>& hits, const std::vector<int>& dup_hits);
  int RequestBlock(int block);
  bool TransactionFilled() const { return markers_[kTransaction].hit; }
  bool SessionFilled() const { return markers_[kSession].hit; }
  int EndTransaction();
  int EndSession();

  uint32_t root_node() const { return root_node_; }
  int loaded() const { return first_free_; }
  int max_blocks() const { return max_blocks_; }
  int nodes_in_block() const { return nib_; }
  uint32_t tree_blocks() const { return tree_->info.blocks_count; }
  cudaStream_t stream() const { return stream_; }
  const uint32_t* links() const { return reinterpret_cast<const uint32_t*>(d_chan_[0]); }
  const uint32_t* far_ptrs() const { return d_far_; }
  const void* channel(const std::string& name, int bytes) const;
  int Buffer(const char* name, void** ptr, size_t* bytes);
  const rayt_cache_stats& stats() const { return stats_; }
  int64_t launches() const { return launches_; }
  int uploaded_since(int64_t mark) const { return (int)(stats_.uploaded_blocks - mark); }
  bool in_transaction() const { return in_transaction_; }
  bool in_session() const { return in_session_; }
  // Device time (ms) of the upload batches flushed since the last call: host
  // to device copies, upload and patch kernels.  Call after a stream sync.
  float TakeUploadMs();

 private:
  static constexpr int kSession = 0, kTransaction = 1, kMarkers = 2;
  struct Slot {
    int block = -1;
    int parent = (int)kRootParent;
    int roots_count = 0;
    uint16_t ptr_index[8];
    uint32_t ptr_value[8];
    std::vector<int> children;
  };
  struct Marker {
    bool hit = false;
    bool live = false;
  };

  std::atomic<int> refs_{1};
  Tree* tree_ = nullptr;
  int nib_ = 0, max_blocks_ = 0, first_free_ = 0;
  uint32_t root_node_ = 0;   // node index: below 2^32 (caches hold fewer than 2^32 nodes)
  cudaStream_t stream_ = nullptr;
  std::vector<uint8_t*> d_chan_;
  std::vector<int> chan_bytes_;
  uint32_t* d_far_ = nullptr;

  // LRU: doubly linked list over node ids [0, max_blocks) = slots,
  // max_blocks + k = marker k, head = max_blocks + kMarkers (sentinel).
  std::vector<int> prev_, next_;
  int head_ = 0;
  Marker markers_[kMarkers];
  std::vector<Slot> slots_;
  std::vector<int32_t> block_slot_;    // tree block -> cache slot, -1 absent
  std::vector<int32_t> parent_slot_;   // tree block -> slot of its parent, -1 absent
  std::vector<uint8_t> validated_;     // tree block -> its links passed the check once (the file is read-only)
  std::vector<int> pending_;
  bool in_session_ = false, in_transaction_ = false;

  // Block staging: two halves of stage_cap_ positions.  Positions
  // [batch_begin_, staged_) of the current half form the batch the next
  // flush uploads.  Two ways to bring a block's bytes to the device:
  // - mapped (the block file is mapped and registered with the device, see
  //   Tree::MapForDevice): a position holds only the block's index; the reading
  //   threads check the block where it lies in the page cache, and the upload
  //   kernel reads its content from there;
  // - read (the file cannot be mapped, or RAYT_BLOCK_IO=read): a position holds
  //   one block record read with a single pread into pinned host memory - the
  //   76-byte header at +4 and the content at +80, so the content is 16-byte
  //   aligned - and a batch goes to the device in one copy.
  const uint8_t* file_host_ = nullptr;  // mapped: the file in host memory
  const uint8_t* file_dev_ = nullptr;   // mapped: the same bytes for kernels
  int* h_blocks_ = nullptr;             // mapped: pinned, per position, the block index
  int* d_blocks_ = nullptr;
  struct Staged {
    int block = -1;
    int rc = RAYT_OK;
    std::string err;
    rayt_block_header hdr{};
    std::vector<uint32_t> faults;  // fault-link targets, in node order
  };
  uint8_t* h_stage_ = nullptr;
  uint8_t* d_stage_ = nullptr;
  size_t area_ = 0;              // bytes per staging position
  int stage_cap_ = 0, half_ = 0, staged_ = 0, batch_begin_ = 0;
  cudaEvent_t stage_free_[2] = {nullptr, nullptr};
  std::vector<Staged> meta_;     // per position, both halves
  // per position, both halves: 1 once its read finished (or was skipped)
  std::unique_ptr<std::atomic<uint8_t>[]> ready_;
  std::atomic<bool> cancel_reads_{false};  // reads not started yet are skipped
  int* h_slots_ = nullptr;       // pinned, per position (-1: staged but not placed)
  int* d_slots_ = nullptr;
  // A batch applies every block content, then every patch (the last value per
  // address).  A slot may take new content several times in one batch (evicted
  // and reused): the newest content supersedes the older staged ones (their
  // positions are skipped) and patches into the slot's links made before it
  // are dropped, so the batch leaves the slot as the reference's sequential
  // order would.
  std::vector<Patch> patches_;
  std::vector<uint8_t> patch_dead_;  // per patch: overwritten by newer content of its slot
  std::vector<int> patch_next_;      // per link patch: the slot's previous link patch in the batch, -1 none
  PatchIndex patch_at_;          // (far << 32 | index) -> position in patches_
  Patch* h_patches_ = nullptr;   // pinned, two halves
  Patch* d_patches_ = nullptr;
  int patch_cap_ = 0, patch_half_ = 0;
  cudaEvent_t patch_free_[2] = {nullptr, nullptr};
  std::vector<int> written_;     // per slot: batch epoch of its newest content
  std::vector<int> written_pos_; // per slot: staging index (both halves) of that content
  std::vector<int> patched_;     // per slot: batch epoch of its newest link patch
  std::vector<int> patch_head_;  // per slot: newest link patch of the batch
  int epoch_ = 1;
  class ReadPool;
  ReadPool* pool_ = nullptr;

  rayt_cache_stats stats_{};
  int64_t launches_ = 0;   // upload and patch kernels launched
  static constexpr int kFlushEvents = 256;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> flush_ev_;  // per flushed batch, reused
  int flush_used_ = 0;

  // MarkUsedBatch's scratch: chain starts in call order, the nodes whose last
  // move falls in each call (walk order), those calls' ranges, seen stamps
  std::vector<int> touch_starts_, touch_order_;
  std::vector<std::pair<int, int>> touch_groups_;
  std::vector<uint32_t> touch_seen_;
  uint32_t touch_epoch_ = 0;

  // list helpers
  void Unlink(int id);
  void InsertBefore(int id, int before);
  void Touch(int slot);
  void DequeueMarkers();
  void InsertMarker(int k);
  void DropMarker(int k);

  int ReadOne(int pos, int block);
  int Prefetch(const int* blocks, int n);
  void StartRead(const int* blocks, int n);
  void FinishRead();
  std::chrono::steady_clock::time_point read_started_;
  int Place(int pos, std::vector<int>* queue);
  int Unload();
  void AddPatch(bool far_buffer, uint32_t index, uint32_t value);
  int FlushTo(int end);
  int NextHalf();
};

}  // namespace rayt
