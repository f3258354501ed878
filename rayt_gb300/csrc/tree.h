// Block file reader (host).  See tree.cpp.
#pragma once
#include <atomic>
#include <cstdint>
#include <mutex>
#include <string>
#include <vector>
#include "../../include/rayt_gb300.h"

namespace rayt {
struct Tree {
  int fd = -1;
  rayt_tree_info info{};
  std::vector<int> chan_bytes;
  std::vector<std::string> chan_names;
  int Open(const char* path);
  // header may be null; content (info.content_bytes) may be null
  int LoadBlock(uint32_t index, rayt_block_header* header, void* content) const;
  bool Read(int64_t off, size_t n, void* out) const;
  // The whole file mapped read-only into host memory and registered with the
  // device (page-locked, device-readable), made on first use and shared by
  // every cache on this tree: a block's bytes are then at map + offset on the
  // host and device_map + offset for kernels.  Null when the file cannot be
  // mapped or registered, or is shorter than its header says; readers then use
  // Read().
  const uint8_t* MapForDevice(const uint8_t** device_map);
  // The tree stays open while a cache uses it: rayt_tree_close and each cache
  // on the tree hold one reference (a cache's kernels may read the mapping).
  void Retain() { refs_.fetch_add(1); }
  static void Release(Tree* t) {
    if (t && t->refs_.fetch_sub(1) == 1) delete t;
  }
  ~Tree();

 private:
  std::atomic<int> refs_{1};
  std::mutex map_mu_;
  bool map_tried_ = false;
  uint8_t* map_ = nullptr;
  size_t map_len_ = 0;
  bool registered_ = false;
  const uint8_t* device_map_ = nullptr;
};
}  // namespace rayt
