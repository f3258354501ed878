// Device block cache with the reference's LRU policy (host bookkeeping,
// device buffers and batched uploads).  See cache.cpp.
#pragma once
#include <cuda_runtime.h>
#include <chrono>
#include <cstdint>
#include <string>
#include <unordered_map>
#include <vector>
#include "internal.h"
#include "tree.h"

namespace rayt {

class Cache {
 public:
  ~Cache();
  int Init(Tree* tree, int max_blocks);

  // GPUOctreeCacheManager protocol
  int InitialFill();
  int StartSession();
  int StartTransaction();
  int MarkBlockUsed(int slot);
  int MarkParentUsed(int slot);
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

  // Block staging: two halves of stage_cap_ positions in pinned host memory
  // and in device memory.  A position holds one block record read with a
  // single pread: the 76-byte header at +4 and the content at +80, so the
  // content is 16-byte aligned.  Positions [batch_begin_, staged_) of the
  // current half form the batch the next flush uploads.
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
  int* h_slots_ = nullptr;       // pinned, per position (-1: staged but not placed)
  int* d_slots_ = nullptr;
  std::vector<Patch> patches_;
  std::unordered_map<uint64_t, int> patch_at_;  // (far << 32 | index) -> position in patches_
  Patch* h_patches_ = nullptr;   // pinned, two halves
  Patch* d_patches_ = nullptr;
  int patch_cap_ = 0, patch_half_ = 0;
  cudaEvent_t patch_free_[2] = {nullptr, nullptr};
  std::vector<int> touched_;     // batch epoch in which a slot was written or patched
  int epoch_ = 1;
  class ReadPool;
  ReadPool* pool_ = nullptr;

  rayt_cache_stats stats_{};
  int64_t launches_ = 0;   // upload and patch kernels launched

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
