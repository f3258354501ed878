// Block-file builder: packs a scene source into the reference's stored-octree
// block file (format: rayt/doc/storage data format.txt:1-33).
//
// The packing follows the reference builder's steps exactly
// (rayt/CPU data/stored-octree-builder-impl.h:53-521), because block numbering,
// node order inside a block and the duplicated block roots all show up in the
// file bytes:
//   * Expand(): breadth-first growth of one block until 8 more nodes would not
//     fit (BuildRecursive, impl.h:393-456),
//   * Settle(): depth-first pass over a full block that builds child blocks
//     for its frontier nodes and bubbles small subtrees up behind duplicated
//     roots (ProcessBlockNodes, impl.h:297-389),
//   * Pack(): greedy grouping of leftover subtrees into leaf blocks
//     (GroupIntoBlocks, impl.h:216-252) and Commit() (CommitBlock, impl.h:166-201).
// The data structures are this file's own: node groups come from a free-list
// pool, channel payloads live inline in the node, and blocks are written with
// pwrite.
#pragma once
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>
#include <fcntl.h>
#include <unistd.h>

namespace rayt_build {

constexpr uint32_t kRootParent = (1u << 24) - 1;
constexpr int kBlockHeaderBytes = 76;
constexpr int kMaxPayload = 32;  // bytes of non-link channel data per node

inline uint32_t PackStoredLink(uint32_t mask, bool fault, bool dup, uint32_t ptr) {
  if (ptr >= (1u << 21)) throw std::runtime_error("block file: pointer does not fit in 21 bits");
  return (ptr << 11) | ((dup ? 1u : 0u) << 9) | ((fault ? 1u : 0u) << 8) | mask;
}

struct Channel {
  int bytes;
  std::string name;
};

// Writes the header and block records at their fixed offsets.
class BlockFileWriter {
 public:
  BlockFileWriter(const std::string& path, int nodes_in_block, const std::vector<Channel>& channels)
      : nib_(nodes_in_block), channels_(channels) {
    fd_ = ::open(path.c_str(), O_CREAT | O_TRUNC | O_WRONLY, 0644);
    if (fd_ < 0) throw std::runtime_error("cannot create block file " + path);
    header_bytes_ = 20 + 8 + 10;  // fixed part + "node links" record
    payload_ = 0;
    for (const Channel& c : channels_) {
      header_bytes_ += 8 + (int)c.name.size();
      payload_ += c.bytes;
    }
    record_bytes_ = kBlockHeaderBytes + nib_ * (payload_ + 4);
  }
  ~BlockFileWriter() {
    if (fd_ >= 0) ::close(fd_);
  }
  int record_bytes() const { return record_bytes_; }
  int header_bytes() const { return header_bytes_; }

  void WriteRecord(uint32_t index, const std::vector<uint8_t>& rec) {
    Put(rec.data(), rec.size(), (int64_t)header_bytes_ + (int64_t)record_bytes_ * index);
  }
  void WriteHeader(uint32_t blocks, uint32_t root_block) {
    std::vector<uint8_t> h;
    auto u32 = [&h](uint32_t v) { for (int i = 0; i < 4; ++i) h.push_back((uint8_t)(v >> (8 * i))); };
    u32((uint32_t)nib_);
    u32(blocks);
    u32(root_block);
    u32((uint32_t)record_bytes_);
    u32((uint32_t)channels_.size() + 1);
    u32(4);
    u32(10);
    for (char ch : std::string("node links")) h.push_back((uint8_t)ch);
    for (const Channel& c : channels_) {
      u32((uint32_t)c.bytes);
      u32((uint32_t)c.name.size());
      for (char ch : c.name) h.push_back((uint8_t)ch);
    }
    Put(h.data(), h.size(), 0);
  }

 private:
  int fd_ = -1;
  int nib_;
  std::vector<Channel> channels_;
  int header_bytes_, payload_, record_bytes_;
  void Put(const uint8_t* p, size_t n, int64_t off) {
    while (n > 0) {
      ssize_t w = ::pwrite(fd_, p, n, off);
      if (w <= 0) throw std::runtime_error("block file write failed");
      p += w;
      n -= (size_t)w;
      off += w;
    }
  }
};

template <class Source>
class BlockBuilder {
  using Tnode = decltype(std::declval<Source&>().GetRoot());

  struct Group;
  struct Node {
    Tnode data;
    int mask = -1;             // children mask, -1 until the source was asked
    Group* kids = nullptr;     // children packed in the same block, if any
    int fault_block = -1;      // block holding the children otherwise
    bool dup = false;          // copy of a node stored in the parent block
    bool has_payload = false;
    uint8_t payload[kMaxPayload];
    uint32_t Link() const {
      if (!mask) return PackStoredLink(0, false, false, 0);
      return PackStoredLink((uint32_t)mask, !kids, dup, kids ? (uint32_t)kids->first : (uint32_t)fault_block);
    }
  };
  struct Group {           // the (up to 8) children of one node, stored consecutively
    int first = -1;        // index of nodes[0] inside its block, -1 = unplaced
    std::vector<Node> nodes;
  };
  struct Subtree {
    Group* owner = nullptr;   // what to release once the subtree is written
    Group* root = nullptr;    // first group of the subtree in its block
    Group* parent = nullptr;  // group (in the parent block) holding the link to root
    int slot = 0;             // index of that link inside parent->nodes
    int count = 0;            // nodes in the subtree
  };
  struct Settled {
    bool movable = false;           // root_subtree present
    Subtree root;
    std::vector<Subtree> leftover;  // remaining_subtrees
  };

 public:
  BlockBuilder(const std::string& path, int nodes_in_block, const std::vector<Channel>& channels, Source* src)
      : writer_(path, nodes_in_block, channels), nib_(nodes_in_block), channels_(channels), src_(src) {
    payload_ = 0;
    for (const Channel& c : channels_) payload_ += c.bytes;
    if (payload_ > kMaxPayload) throw std::runtime_error("builder: node payload too large");
    if (nodes_in_block < 9 || nodes_in_block > 65536) throw std::runtime_error("builder: nodes_in_block out of range");
    record_.assign((size_t)writer_.record_bytes(), 0);
  }

  // Builds the whole tree and writes the file; returns the block count.
  uint32_t Build() {
    Group* root = NewGroup();
    root->nodes.emplace_back();
    root->nodes.back().data = src_->GetRoot();
    int index = blocks_++;
    Subtree s;
    if (Expand(root, nullptr, 0, index, kRootParent, &s)) {
      --blocks_;
      Commit({s}, blocks_++, kRootParent);
    }
    writer_.WriteHeader((uint32_t)blocks_, 0);
    if (live_groups_ != 0) throw std::runtime_error("builder: group accounting mismatch");
    return (uint32_t)blocks_;
  }
  uint64_t nodes() const { return nodes_; }

 private:
  BlockFileWriter writer_;
  int nib_;
  std::vector<Channel> channels_;
  Source* src_;
  int payload_;
  int blocks_ = 0;
  uint64_t nodes_ = 0;
  int64_t live_groups_ = 0;
  std::vector<Group*> free_;
  // record buffer reused across blocks; root records past roots_count are
  // written as zeros (the reference leaves whatever its reused header held, so
  // those bytes carry no meaning and file comparisons mask them)
  std::vector<uint8_t> record_;
  uint32_t roots_[8][3] = {};  // parent_pointer_index, pointed_child_index, parent_pointer_value

  Group* NewGroup() {
    ++live_groups_;
    if (!free_.empty()) {
      Group* g = free_.back();
      free_.pop_back();
      g->first = -1;
      g->nodes.clear();
      return g;
    }
    return new Group();
  }
  void Release(Group* g) {
    for (Node& n : g->nodes)
      if (n.kids) Release(n.kids);
    --live_groups_;
    free_.push_back(g);
  }
  Group* CloneGroup(const Group* g) {
    Group* c = NewGroup();
    c->first = g->first;
    c->nodes = g->nodes;
    return c;
  }

  void Number(Group* g, int& next) {
    g->first = next;
    next += (int)g->nodes.size();
    for (Node& n : g->nodes)
      if (n.kids) Number(n.kids, next);
  }

  void Fill(Node& n, Group* kids_override = nullptr) {
    Group* kids = kids_override ? kids_override : n.kids;
    std::vector<std::pair<int, Tnode*>> ptrs;
    if (n.mask) {
      int p = 0;
      for (int j = 0; j < 8; ++j)
        if (n.mask & (1 << j)) ptrs.push_back(std::make_pair(j, &kids->nodes[p++].data));
    }
    src_->GetNodeData(n.data, ptrs, n.payload);
    n.has_payload = true;
    ++nodes_;
  }
  void FillAll(Group* g) {
    for (Node& n : g->nodes) {
      if (n.mask) FillAll(n.kids);
      Fill(n);
    }
  }

  void SetFault(Node& n, int block) {
    if (n.mask && !n.kids) n.fault_block = block;
    if (n.kids)
      for (Node& k : n.kids->nodes) SetFault(k, block);
  }

  Group* Children(Node& n) {
    std::vector<std::pair<int, Tnode>> kids = src_->GetChildren(n.data);
    n.mask = 0;
    if (kids.empty()) return nullptr;
    Group* g = NewGroup();
    for (auto& k : kids) {
      n.mask |= 1 << k.first;
      g->nodes.emplace_back();
      g->nodes.back().data = k.second;
    }
    return g;
  }

  // Returns true (with *out) when the subtree fit with room to spare and was
  // not written; false when a full block `index` (and maybe one leaf block)
  // was committed.
  bool Expand(Group* root, Group* parent, int slot, int index, uint32_t parent_block, Subtree* out) {
    Subtree res;
    res.owner = res.root = root;
    res.parent = parent;
    res.slot = slot;
    res.count = (int)root->nodes.size();
    std::vector<Group*> queue{root};
    size_t head = 0;
    bool full = false;
    while (head < queue.size() && !full) {
      Group* cur = queue[head++];
      for (Node& n : cur->nodes) {
        if (res.count + 8 > nib_) {
          full = true;
          break;
        }
        n.kids = Children(n);
        if (n.kids) {
          queue.push_back(n.kids);
          res.count += (int)n.kids->nodes.size();
        }
      }
    }
    if (!full) {
      FillAll(root);
      if (parent) Fill(parent->nodes[slot], root);
      *out = res;
      return true;
    }
    int next = 0;
    Number(root, next);
    Settled s = Settle(root, index, nullptr, 0);
    if (parent) Fill(parent->nodes[slot], root);
    if (!s.leftover.empty()) Commit(s.leftover, blocks_++, (uint32_t)index);
    Commit({res}, index, parent_block);
    return false;
  }

  Settled Settle(Group* g, int block, Group* parent, int slot) {
    bool all_movable = true;
    const int nn = (int)g->nodes.size();
    std::vector<Subtree> movable(nn);
    std::vector<Group*> spare;                 // movable copies nobody will hold
    std::vector<std::vector<Subtree>> pending;  // subtree groups awaiting a block
    int count = nn;
    for (int i = 0; i < nn; ++i) {
      Node& n = g->nodes[i];
      movable[i].root = nullptr;
      if (n.mask == -1) {
        Group* kids = Children(n);
        if (kids) {
          int child_index = blocks_++;
          Subtree r;
          if (!Expand(kids, g, i, child_index, (uint32_t)block, &r)) {
            n.fault_block = child_index;
            all_movable = false;
          } else {
            --blocks_;
            movable[i] = r;
            pending.push_back({r});
            count += r.count;
          }
        }
      }
      if (n.mask == 0) {
        Fill(n);
        movable[i].root = nullptr;
        movable[i].count = 0;
      } else if (n.kids) {
        Settled s = Settle(n.kids, block, g, i);
        Fill(n);
        if (!s.movable) {
          all_movable = false;
        } else {
          movable[i] = s.root;
          count += s.root.count;
          if (s.leftover.empty()) spare.push_back(s.root.owner);
        }
        if (!s.leftover.empty()) pending.push_back(s.leftover);
      }
    }

    Settled res;
    if (all_movable && count < nib_ && parent) {
      Subtree copy;
      copy.slot = slot;
      copy.parent = parent;
      copy.count = count;
      copy.root = copy.owner = CloneGroup(g);
      copy.root->first = -1;
      for (int i = 0; i < (int)copy.root->nodes.size(); ++i) {
        Node& n = copy.root->nodes[i];
        n.dup = true;
        if (n.mask) n.kids = movable[i].root;
      }
      res.movable = true;
      res.root = copy;
      if (pending.size() == 1) {
        res.leftover = pending[0];
        res.leftover[0].owner = copy.root;
      } else if (pending.size() > 1) {
        res.leftover.push_back(copy);
      }
    } else {
      for (Group* sp : spare) Release(sp);
      Pack(pending, (uint32_t)block, &res.leftover);
    }
    return res;
  }

  static int Nodes(const std::vector<Subtree>& v) {
    int r = 0;
    for (const Subtree& s : v) r += s.count;
    return r;
  }

  void Pack(std::vector<std::vector<Subtree>> groups, uint32_t parent_block, std::vector<Subtree>* rest) {
    int total_nodes = 0, total_trees = 0;
    for (auto& gr : groups) {
      total_nodes += Nodes(gr);
      total_trees += (int)gr.size();
    }
    if (total_nodes < nib_ && total_trees < 8) {
      for (auto& gr : groups) rest->insert(rest->end(), gr.begin(), gr.end());
      return;
    }
    std::sort(groups.begin(), groups.end(),
              [](const std::vector<Subtree>& a, const std::vector<Subtree>& b) { return Nodes(a) < Nodes(b); });
    while (total_nodes >= nib_ || total_trees >= 8) {
      int gn = 0, gt = 0;
      std::vector<Subtree> block;
      for (int i = (int)groups.size() - 1; i >= 0; --i) {
        int nodes = Nodes(groups[i]);
        int trees = (int)groups[i].size();
        if (gn + nodes <= nib_ && gt + trees <= 8) {
          gn += nodes;
          gt += trees;
          block.insert(block.end(), groups[i].begin(), groups[i].end());
          groups.erase(groups.begin() + i);
        }
      }
      Commit(block, blocks_++, parent_block);
      total_nodes -= gn;
      total_trees -= gt;
    }
    for (auto& gr : groups) rest->insert(rest->end(), gr.begin(), gr.end());
  }

  void Store(Group* g) {
    uint8_t* content = record_.data() + kBlockHeaderBytes;
    for (int i = 0; i < (int)g->nodes.size(); ++i) {
      Node& n = g->nodes[i];
      if (!n.has_payload) throw std::runtime_error("builder: node without data");
      int at = g->first + i;
      uint32_t link = n.Link();
      std::memcpy(content + (size_t)at * 4, &link, 4);
      int off = 0;
      for (const Channel& c : channels_) {
        std::memcpy(content + (size_t)(off + 4) * nib_ + (size_t)c.bytes * at, n.payload + off, (size_t)c.bytes);
        off += c.bytes;
      }
      if (n.kids) Store(n.kids);
    }
  }

  void Commit(const std::vector<Subtree>& trees, int index, uint32_t parent_block) {
    std::memset(record_.data() + kBlockHeaderBytes, 0, record_.size() - kBlockHeaderBytes);
    std::memset(roots_, 0, sizeof(roots_));
    int placed = 0;  // nodes of the earlier subtrees of this block
    for (size_t si = 0; si < trees.size(); ++si) {
      const Subtree& t = trees[si];
      if (t.root->first == -1) {
        int next = placed;
        Number(t.root, next);
      }
      if (t.parent) SetFault(t.parent->nodes[t.slot], index);
      placed += t.count;
      roots_[si][1] = (uint32_t)t.root->first;
      if (t.parent) {
        roots_[si][0] = (uint32_t)(t.parent->first + t.slot);
        roots_[si][2] = t.parent->nodes[t.slot].Link();
      } else {
        roots_[si][0] = roots_[si][2] = 0;
      }
      Store(t.root);
      Release(t.owner);
    }
    if (placed > nib_) throw std::runtime_error("builder: block overflow");
    uint8_t* h = record_.data();
    auto u32 = [&h](int off, uint32_t v) { std::memcpy(h + off, &v, 4); };
    auto u16 = [&h](int off, uint32_t v) { uint16_t s = (uint16_t)v; std::memcpy(h + off, &s, 2); };
    u32(0, (uint32_t)index);
    u32(4, parent_block);
    u32(8, (uint32_t)trees.size());
    for (int i = 0; i < 8; ++i) {
      u16(12 + 8 * i, roots_[i][0]);
      u16(12 + 8 * i + 2, roots_[i][1]);
      u32(12 + 8 * i + 4, roots_[i][2]);
    }
    writer_.WriteRecord((uint32_t)index, record_);
  }
};

}  // namespace rayt_build
