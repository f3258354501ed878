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
//
// Parallel build, same bytes: every child-block subtree of a frontier node
// takes a contiguous range of block indices, and its blocks depend only on its
// own nodes.  So the frontier subtrees of the root block are built on worker
// threads with block indices local to the subtree (records kept in memory),
// while the main thread replays the root block's Settle() in the reference's
// order; when it reaches a frontier node it takes that subtree's outcome,
// gives it its global base index, adds the base to every block reference in
// the subtree's records (block index, parent index, fault links, root parent
// values) and writes them.  Workers run at most a bounded window ahead of the
// main thread, which bounds the records held in memory.
#pragma once
#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <functional>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
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

  void WriteRecord(uint32_t index, const uint8_t* rec) {
    Put(rec, (size_t)record_bytes_, (int64_t)header_bytes_ + (int64_t)record_bytes_ * index);
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
    bool frontier = false;     // root-block frontier node built by a worker
    bool has_payload = false;
    uint8_t payload[kMaxPayload];
    uint32_t Link() const {
      if (!mask) return PackStoredLink(0, false, false, 0);
      return PackStoredLink((uint32_t)mask, !kids, dup, kids ? (uint32_t)kids->first : (uint32_t)fault_block);
    }
  };
  // At most 8 nodes, stored inline (no allocation per group).
  struct NodeList {
    Node v[8];
    int n = 0;
    size_t size() const { return (size_t)n; }
    bool empty() const { return n == 0; }
    Node& operator[](size_t i) { return v[i]; }
    const Node& operator[](size_t i) const { return v[i]; }
    Node* begin() { return v; }
    Node* end() { return v + n; }
    const Node* begin() const { return v; }
    const Node* end() const { return v + n; }
    Node* data() { return v; }
    Node& emplace_back() { v[n] = Node(); return v[n++]; }
    Node& back() { return v[n - 1]; }
    void clear() { n = 0; }
  };
  struct Group {           // the (up to 8) children of one node, stored consecutively
    int first = -1;        // index of nodes[0] inside its block, -1 = unplaced
    NodeList nodes;
  };
  // Released groups are kept per thread for reuse.
  struct GroupPool {
    std::vector<Group*> free;
    ~GroupPool() {
      for (Group* g : free) delete g;
    }
  };
  static GroupPool& Pool() {
    static thread_local GroupPool pool;
    return pool;
  }
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
  // What a worker found under one frontier node of the root block.
  struct Outcome {
    bool ready = false;
    bool has_kids = false;
    bool full = false;              // a full child block (and its descendants) was written
    int blocks = 0;                 // blocks of the subtree (local indices 0..blocks-1)
    Subtree r;                      // the subtree handed back when it was not full
    std::vector<std::pair<uint32_t, std::vector<uint8_t>>> records;
    std::string error;
  };

  // The packing state of one thread: either the main packer writing the file
  // or a worker collecting records of one subtree with local block indices.
  class Packer {
   public:
    Packer(BlockBuilder* b, bool to_memory) : b_(b), to_memory_(to_memory) {
      record_.assign((size_t)b->record_bytes_, 0);
    }
    int blocks = 0;
    uint64_t nodes = 0;
    int64_t groups = 0;  // groups taken minus groups released by this packer
    std::vector<std::pair<uint32_t, std::vector<uint8_t>>> records;  // worker sink
    // main packer of a parallel build: the worker outcome of each frontier
    // node of the root block, handed over in visiting order
    std::function<Outcome*(Node&)> frontier_hook;

    Group* Children(Node& n) {
      int slots[8];
      Tnode kids[8];
      const int k = b_->src_->ChildrenInto(n.data, slots, kids);
      n.mask = 0;
      if (k == 0) return nullptr;
      Group* g = NewGroup();
      for (int i = 0; i < k; ++i) {
        n.mask |= 1 << slots[i];
        g->nodes.emplace_back().data = kids[i];
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
      if (!GrowBlock(root, &res.count)) {
        FillAll(root);
        if (parent) Fill(parent->nodes[slot], root);
        *out = res;
        return true;
      }
      int next = 0;
      Number(root, next);
      Settled s = Settle(root, index, nullptr, 0);
      if (parent) Fill(parent->nodes[slot], root);
      if (!s.leftover.empty()) Commit(s.leftover, blocks++, (uint32_t)index);
      Commit({res}, index, parent_block);
      return false;
    }

    // Breadth-first growth; true when the block is full.
    bool GrowBlock(Group* root, int* count) {
      std::vector<Group*> queue{root};
      size_t head = 0;
      while (head < queue.size()) {
        Group* cur = queue[head++];
        for (Node& n : cur->nodes) {
          if (*count + 8 > b_->nib_) return true;
          n.kids = Children(n);
          if (n.kids) {
            queue.push_back(n.kids);
            *count += (int)n.kids->nodes.size();
          }
        }
      }
      return false;
    }

    static void Number(Group* g, int& next) {
      g->first = next;
      next += (int)g->nodes.size();
      for (Node& n : g->nodes)
        if (n.kids) Number(n.kids, next);
    }

    void Fill(Node& n, Group* kids_override = nullptr) {
      Group* kids = kids_override ? kids_override : n.kids;
      const Tnode* ptrs[8];
      int k = 0;
      if (n.mask)
        for (int j = 0; j < 8; ++j)
          if (n.mask & (1 << j)) { ptrs[k] = &kids->nodes[k].data; ++k; }
      b_->src_->NodeDataInto(n.data, ptrs, k, n.payload);
      n.has_payload = true;
      ++nodes;
    }
    void FillAll(Group* g) {
      for (Node& n : g->nodes) {
        if (n.mask) FillAll(n.kids);
        Fill(n);
      }
    }

    static void SetFault(Node& n, int block) {
      if (n.mask && !n.kids) n.fault_block = block;
      if (n.kids)
        for (Node& k : n.kids->nodes) SetFault(k, block);
    }

    Settled Settle(Group* g, int block, Group* parent, int slot) {
      bool all_movable = true;
      const int nn = (int)g->nodes.size();
      std::vector<Subtree> movable(nn);
      std::vector<Group*> spare;                  // movable copies nobody will hold
      std::vector<std::vector<Subtree>> pending;  // subtree groups awaiting a block
      int count = nn;
      for (int i = 0; i < nn; ++i) {
        Node& n = g->nodes[i];
        movable[i].root = nullptr;
        // (a worker may be filling in a frontier node: read its fields only
        // after the hook has handed its outcome over)
        if (n.frontier || n.mask == -1) {
          if (frontier_hook && n.frontier) {
            // a worker built this subtree: place it at the next indices
            Outcome* o = frontier_hook(n);
            if (o->has_kids) {
              const int child_index = blocks++;
              if (o->full) {
                n.fault_block = child_index;
                all_movable = false;
                b_->WriteRelocated(o, child_index);
                blocks = child_index + o->blocks;
              } else {
                --blocks;
                movable[i] = o->r;
                pending.push_back({o->r});
                count += o->r.count;
              }
            }
          } else {
            Group* kids = Children(n);
            if (kids) {
              const int child_index = blocks++;
              Subtree r;
              if (!Expand(kids, g, i, child_index, (uint32_t)block, &r)) {
                n.fault_block = child_index;
                all_movable = false;
              } else {
                --blocks;
                movable[i] = r;
                pending.push_back({r});
                count += r.count;
              }
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
      if (all_movable && count < b_->nib_ && parent) {
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
      const int nib = b_->nib_;
      if (total_nodes < nib && total_trees < 8) {
        for (auto& gr : groups) rest->insert(rest->end(), gr.begin(), gr.end());
        return;
      }
      std::sort(groups.begin(), groups.end(),
                [](const std::vector<Subtree>& a, const std::vector<Subtree>& b) { return Nodes(a) < Nodes(b); });
      while (total_nodes >= nib || total_trees >= 8) {
        int gn = 0, gt = 0;
        std::vector<Subtree> block;
        for (int i = (int)groups.size() - 1; i >= 0; --i) {
          const int nodes_i = Nodes(groups[i]);
          const int trees = (int)groups[i].size();
          if (gn + nodes_i <= nib && gt + trees <= 8) {
            gn += nodes_i;
            gt += trees;
            block.insert(block.end(), groups[i].begin(), groups[i].end());
            groups.erase(groups.begin() + i);
          }
        }
        Commit(block, blocks++, parent_block);
        total_nodes -= gn;
        total_trees -= gt;
      }
      for (auto& gr : groups) rest->insert(rest->end(), gr.begin(), gr.end());
    }

    void Store(Group* g) {
      const int nib = b_->nib_;
      uint8_t* content = record_.data() + kBlockHeaderBytes;
      for (int i = 0; i < (int)g->nodes.size(); ++i) {
        Node& n = g->nodes[i];
        if (!n.has_payload) throw std::runtime_error("builder: node without data");
        const int at = g->first + i;
        const uint32_t link = n.Link();
        std::memcpy(content + (size_t)at * 4, &link, 4);
        int off = 0;
        for (const Channel& c : b_->channels_) {
          std::memcpy(content + (size_t)(off + 4) * nib + (size_t)c.bytes * at, n.payload + off, (size_t)c.bytes);
          off += c.bytes;
        }
        if (n.kids) Store(n.kids);
      }
    }

    // Root records past roots_count are written as zeros (the reference
    // leaves whatever its reused header held there; nothing reads them).
    void Commit(const std::vector<Subtree>& trees, int index, uint32_t parent_block) {
      std::memset(record_.data(), 0, record_.size());
      uint32_t roots[8][3] = {};  // parent_pointer_index, pointed_child_index, parent_pointer_value
      int placed = 0;             // nodes of the earlier subtrees of this block
      for (size_t si = 0; si < trees.size(); ++si) {
        const Subtree& t = trees[si];
        if (t.root->first == -1) {
          int next = placed;
          Number(t.root, next);
        }
        if (t.parent) SetFault(t.parent->nodes[t.slot], index);
        placed += t.count;
        roots[si][1] = (uint32_t)t.root->first;
        if (t.parent) {
          roots[si][0] = (uint32_t)(t.parent->first + t.slot);
          roots[si][2] = t.parent->nodes[t.slot].Link();
        }
        Store(t.root);
        Release(t.owner);
      }
      if (placed > b_->nib_) throw std::runtime_error("builder: block overflow");
      uint8_t* h = record_.data();
      auto u32 = [&h](int off, uint32_t v) { std::memcpy(h + off, &v, 4); };
      auto u16 = [&h](int off, uint32_t v) { uint16_t s = (uint16_t)v; std::memcpy(h + off, &s, 2); };
      u32(0, (uint32_t)index);
      u32(4, parent_block);
      u32(8, (uint32_t)trees.size());
      for (int i = 0; i < 8; ++i) {
        u16(12 + 8 * i, roots[i][0]);
        u16(12 + 8 * i + 2, roots[i][1]);
        u32(12 + 8 * i + 4, roots[i][2]);
      }
      if (to_memory_) records.emplace_back((uint32_t)index, record_);
      else b_->writer_.WriteRecord((uint32_t)index, record_.data());
    }

    Group* NewGroup() {
      ++groups;
      GroupPool& pool = Pool();
      if (pool.free.empty()) return new Group();
      Group* g = pool.free.back();
      pool.free.pop_back();
      g->first = -1;
      g->nodes.clear();
      return g;
    }
    void Release(Group* g) {
      for (Node& n : g->nodes)
        if (n.kids) Release(n.kids);
      --groups;
      Pool().free.push_back(g);
    }
    Group* CloneGroup(const Group* g) {
      Group* c = NewGroup();
      c->first = g->first;
      c->nodes = g->nodes;
      return c;
    }

   private:
    BlockBuilder* b_;
    bool to_memory_;
    std::vector<uint8_t> record_;
  };

 public:
  BlockBuilder(const std::string& path, int nodes_in_block, const std::vector<Channel>& channels, Source* src,
               int threads = 1)
      : writer_(path, nodes_in_block, channels), nib_(nodes_in_block), channels_(channels), src_(src),
        threads_(std::max(1, threads)) {
    for (const Channel& c : channels_) payload_ += c.bytes;
    if (payload_ > kMaxPayload) throw std::runtime_error("builder: node payload too large");
    if (nodes_in_block < 9 || nodes_in_block > 65536) throw std::runtime_error("builder: nodes_in_block out of range");
    record_bytes_ = writer_.record_bytes();
  }

  // Builds the whole tree and writes the file; returns the block count.
  uint32_t Build() {
    Packer main(this, false);
    Group* root = main.NewGroup();
    root->nodes.emplace_back();
    root->nodes.back().data = src_->GetRoot();
    const int index = main.blocks++;
    if (threads_ <= 1) {
      Subtree s;
      if (main.Expand(root, nullptr, 0, index, kRootParent, &s)) {
        --main.blocks;
        main.Commit({s}, main.blocks++, kRootParent);
      }
    } else {
      BuildParallel(main, root, index);
    }
    nodes_ = main.nodes + worker_nodes_.load();
    writer_.WriteHeader((uint32_t)main.blocks, 0);
    if (main.groups + live_groups_.load() != 0) throw std::runtime_error("builder: group accounting mismatch");
    return (uint32_t)main.blocks;
  }
  uint64_t nodes() const { return nodes_; }

 private:
  BlockFileWriter writer_;
  int nib_;
  std::vector<Channel> channels_;
  Source* src_;
  int threads_;
  int payload_ = 0;
  int record_bytes_ = 0;
  uint64_t nodes_ = 0;
  std::atomic<uint64_t> worker_nodes_{0};
  std::atomic<int64_t> live_groups_{0};


  static uint32_t Rebase(uint32_t link, uint32_t base) {
    if ((link & 255u) && (link & (1u << 8)))
      return PackStoredLink(link & 255u, true, ((link >> 9) & 1u) != 0, (link >> 11) + base);
    return link;
  }

  // Adds `base` to every block reference of a subtree built with local block
  // indices and writes its records.  The subtree's top block (local 0) keeps
  // its parent index, which lies outside the subtree.
  void WriteRelocated(Outcome* o, int base) {
    const uint32_t b = (uint32_t)base;
    for (auto& rec : o->records) {
      uint8_t* h = rec.second.data();
      uint32_t v;
      std::memcpy(&v, h, 4);
      v += b;
      std::memcpy(h, &v, 4);
      if (rec.first != 0) {
        std::memcpy(&v, h + 4, 4);
        v += b;
        std::memcpy(h + 4, &v, 4);
      }
      uint32_t roots;
      std::memcpy(&roots, h + 8, 4);
      for (uint32_t i = 0; i < roots && i < 8; ++i) {
        std::memcpy(&v, h + 16 + 8 * i, 4);
        v = Rebase(v, b);
        std::memcpy(h + 16 + 8 * i, &v, 4);
      }
      uint8_t* links = h + kBlockHeaderBytes;
      for (int n = 0; n < nib_; ++n) {
        std::memcpy(&v, links + 4 * n, 4);
        v = Rebase(v, b);
        std::memcpy(links + 4 * n, &v, 4);
      }
      writer_.WriteRecord(rec.first + b, h);
    }
    o->records.clear();
    o->records.shrink_to_fit();
  }

  // Frontier nodes of the root block in the order Settle() visits them, each
  // with the group holding it.
  static void CollectFrontier(Group* g, std::vector<std::pair<Node*, Group*>>* out) {
    for (Node& n : g->nodes) {
      if (n.mask == -1) {
        n.frontier = true;
        out->push_back(std::make_pair(&n, g));
      } else if (n.kids) {
        CollectFrontier(n.kids, out);
      }
    }
  }

  void BuildParallel(Packer& main, Group* root, int index) {
    Subtree res;
    res.owner = res.root = root;
    res.count = (int)root->nodes.size();
    if (!main.GrowBlock(root, &res.count)) {  // the whole tree fits in one block
      main.FillAll(root);
      --main.blocks;
      main.Commit({res}, main.blocks++, kRootParent);
      return;
    }
    int next = 0;
    Packer::Number(root, next);
    std::vector<std::pair<Node*, Group*>> frontier;
    CollectFrontier(root, &frontier);
    const size_t nf = frontier.size();
    std::vector<std::unique_ptr<Outcome>> outcomes(nf);
    for (auto& o : outcomes) o.reset(new Outcome());
    std::mutex mu;
    std::condition_variable cv;
    size_t consumed = 0, next_task = 0;
    const size_t window = (size_t)threads_ * 64;
    bool stop = false;
    auto worker = [&]() {
      for (;;) {
        size_t k;
        {
          std::unique_lock<std::mutex> lock(mu);
          cv.wait(lock, [&] { return stop || next_task >= nf || next_task < consumed + window; });
          if (stop || next_task >= nf) return;
          k = next_task++;
        }
        Outcome* o = outcomes[k].get();
        try {
          Packer w(this, true);
          Node& n = *frontier[k].first;
          Group* g = frontier[k].second;
          Group* kids = w.Children(n);
          if (kids) {
            o->has_kids = true;
            const int local = w.blocks++;  // local index 0
            Subtree r;
            if (!w.Expand(kids, g, (int)(&n - g->nodes.begin()), local, (uint32_t)index, &r)) {
              o->full = true;
              o->blocks = w.blocks;
              o->records = std::move(w.records);
            } else {
              o->r = r;
            }
          }
          worker_nodes_.fetch_add(w.nodes);
          live_groups_.fetch_add(w.groups);
        } catch (const std::exception& e) {
          o->error = e.what();
        }
        {
          std::lock_guard<std::mutex> lock(mu);
          o->ready = true;
        }
        cv.notify_all();
      }
    };
    std::vector<std::thread> pool;
    for (int t = 0; t < threads_; ++t) pool.emplace_back(worker);
    size_t taken = 0;
    main.frontier_hook = [&](Node& n) -> Outcome* {
      if (taken >= nf || frontier[taken].first != &n) throw std::runtime_error("builder: frontier order mismatch");
      Outcome* o = outcomes[taken].get();
      {
        std::unique_lock<std::mutex> lock(mu);
        cv.wait(lock, [&] { return o->ready; });
        ++taken;
        consumed = taken;
      }
      cv.notify_all();
      if (!o->error.empty()) throw std::runtime_error(o->error);
      return o;
    };
    auto finish = [&]() {
      {
        std::lock_guard<std::mutex> lock(mu);
        stop = true;
      }
      cv.notify_all();
      for (auto& th : pool) th.join();
      main.frontier_hook = nullptr;
    };
    try {
      Settled s = main.Settle(root, index, nullptr, 0);
      if (!s.leftover.empty()) main.Commit(s.leftover, main.blocks++, (uint32_t)index);
      main.Commit({res}, index, kRootParent);
    } catch (...) {
      finish();
      throw;
    }
    finish();
  }
};

}  // namespace rayt_build
