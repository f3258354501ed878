// Block file reader (host).  See tree.cpp.
#pragma once
#include <cstdint>
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
  ~Tree();
};
}  // namespace rayt
