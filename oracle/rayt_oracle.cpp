// ORACLE - test infrastructure only.  A plain CPU restatement of the reference
// per-frame path, used as the parity checker by tests/, by
// __graft_entry__.smoke(), and as the timed CPU baseline in bench.py.  The
// product library never links, loads or calls this file.
//
// Pinned against the reference itself: tests/golden/ holds outputs of the
// reference's own host code and .cl kernels run on the CPU (script:
// tests/golden/make_golden.py), and tests/test_oracle_golden.py checks this
// restatement against every one of them.
//
// What is restated (reference file:line in each function's comment):
//   block file reader        rayt/CPU data/stored-octree-loader.cpp:31-98
//   cache manager + LRU      rayt/GPU data/gpu-octree-cache-manager.cpp:60-212,
//                            rayt/GPU data/gpu-octree-cache.cpp:58-313
//   ray setup                rayt/GPU_renderer/kernels/init_tracing_frame.cl:3-45
//   ray cast                 rayt/GPU_renderer/kernels/raycast.cl:33-256
//   tracing pass             rayt/GPU_renderer/kernels/raytracing_pass.cl:4-61
//   shading                  rayt/GPU_renderer/kernels/shading.cl:4-33
//   finish                   rayt/GPU_renderer/kernels/finish_tracing_frame.cl:3-24
//   feedback unique          rayt/GPU_renderer/kernels/feedback_compression.cl:4-34,
//                            rayt/GPU algorithms/kernels/merge_sort.cl:2-73, scan.cl:2-12
//   feedback decode          rayt/GPU_renderer/ray-tracing-feedback-extractor.cpp:108-185
//   frame loop               rayt/GPU_renderer/gpu-ray-tracer.cpp:66-227
// Built with -ffp-contract=off; float built-ins follow the pinned definitions
// (dot left to right, normalize = v / sqrt(dot(v, v)), component-wise divides).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <list>
#include <map>
#include <memory>
#include <queue>
#include <string>
#include <vector>
#include <fcntl.h>
#include <unistd.h>

namespace {

constexpr int32_t kNoHit = 0x7fffffff;
constexpr uint32_t kRootParent = (1u << 24) - 1;
constexpr int kSMax = 23;
constexpr float kEps = 0.00000011920928955078125f;

thread_local std::string g_error;

// ---------------------------------------------------------------------------
// Block file (stored-octree-loader.cpp:31-98).
struct BlockRoot {
  uint16_t parent_pointer_index, pointed_child_index;
  uint32_t parent_pointer_value;
};
struct Block {
  uint32_t index, parent, roots_count;
  BlockRoot roots[8];
  std::vector<uint8_t> content;
};

struct TreeFile {
  int fd = -1;
  uint32_t nib = 0, blocks = 0, root_block = 0, stride = 0;
  int64_t header_bytes = 0;
  std::vector<std::pair<int, std::string>> channels;
  int content_bytes = 0;
  ~TreeFile() { if (fd >= 0) close(fd); }
  bool Read(int64_t off, size_t n, void* out) {
    uint8_t* p = (uint8_t*)out;
    while (n) {
      ssize_t r = pread(fd, p, n, off);
      if (r <= 0) return false;
      p += r; n -= (size_t)r; off += r;
    }
    return true;
  }
  bool Open(const char* path) {
    fd = open(path, O_RDONLY);
    if (fd < 0) { g_error = "cannot open"; return false; }
    uint32_t h[5];
    if (!Read(0, 20, h)) return false;
    nib = h[0]; blocks = h[1]; root_block = h[2]; stride = h[3];
    int64_t pos = 20;
    content_bytes = 0;
    for (uint32_t i = 0; i < h[4]; ++i) {
      uint32_t c[2];
      if (!Read(pos, 8, c)) return false;
      pos += 8;
      std::string name(c[1], '\0');
      if (!Read(pos, c[1], &name[0])) return false;
      pos += c[1];
      channels.emplace_back((int)c[0], name);
      content_bytes += (int)c[0];
    }
    content_bytes *= (int)nib;
    header_bytes = pos;
    return true;
  }
  bool Load(uint32_t index, Block* b) {
    uint8_t hdr[76];
    int64_t off = header_bytes + (int64_t)stride * index;
    if (!Read(off, 76, hdr)) return false;
    std::memcpy(&b->index, hdr, 4);
    std::memcpy(&b->parent, hdr + 4, 4);
    std::memcpy(&b->roots_count, hdr + 8, 4);
    for (int i = 0; i < 8; ++i) {
      std::memcpy(&b->roots[i].parent_pointer_index, hdr + 12 + 8 * i, 2);
      std::memcpy(&b->roots[i].pointed_child_index, hdr + 14 + 8 * i, 2);
      std::memcpy(&b->roots[i].parent_pointer_value, hdr + 16 + 8 * i, 4);
    }
    b->content.resize((size_t)content_bytes);
    return Read(off + 76, (size_t)content_bytes, b->content.data());
  }
};

inline uint32_t CacheLink(uint32_t mask, bool fault, bool dup, bool far_, uint32_t ptr) {
  return (ptr << 11) | ((far_ ? 1u : 0u) << 10) | ((dup ? 1u : 0u) << 9) | ((fault ? 1u : 0u) << 8) | mask;
}
inline uint32_t NearValue(int64_t from, int64_t to) { return (uint32_t)((1 << 20) + (to - from)); }

// ---------------------------------------------------------------------------
// Cache with LRU (gpu-octree-cache.cpp:58-313, gpu-octree-cache-manager.cpp).
// The "device" buffers are host arrays here.
struct Marker {
  bool hit = false;
  std::list<int64_t>::iterator it;
};

struct Cache {
  TreeFile* tree;
  int nib, max_blocks, first_free = 0, root_node = 0;
  std::vector<std::vector<uint8_t>> chan;   // per channel: max_blocks * nib * bytes
  std::vector<int> chan_bytes;
  std::vector<uint32_t> far;                // max_blocks * 8
  struct Slot {
    int block = -1;
    int parent = (int)kRootParent;
    int roots_count = 0;
    uint16_t ptr_index[8];
    uint32_t ptr_value[8];
    std::list<int64_t>::iterator lru;
    std::vector<int> children;
  };
  std::vector<Slot> slots;
  std::map<int, int> block_slot, parent_slot;
  // LRU entries: >= 0 is a slot, < 0 is -(marker id)-1
  std::list<int64_t> lru;
  std::map<int64_t, Marker*> markers;
  int64_t next_marker = 0;
  Marker *session = nullptr, *transaction = nullptr;
  std::vector<int> pending;
  // counters
  long long uploaded = 0, patches = 0, far_patches = 0;

  uint32_t* links() { return reinterpret_cast<uint32_t*>(chan[0].data()); }

  void DequeueMarkers() {
    while (!lru.empty() && lru.front() < 0) {
      markers[lru.front()]->hit = true;
      lru.pop_front();
    }
  }
  void Touch(int slot) {  // MarkBlockAsUsed: the block and every ancestor to MRU
    for (int s = slot; s != (int)kRootParent; s = slots[s].parent) {
      lru.erase(slots[s].lru);
      slots[s].lru = lru.insert(lru.end(), s);
    }
    DequeueMarkers();
  }
  Marker* NewMarker() {
    Marker* m = new Marker();
    int64_t id = -(++next_marker);
    markers[id] = m;
    m->it = lru.insert(lru.end(), id);
    return m;
  }
  void DropMarker(Marker*& m) {
    if (!m) return;
    if (!m->hit) lru.erase(m->it);
    for (auto it = markers.begin(); it != markers.end(); ++it)
      if (it->second == m) { markers.erase(it); break; }
    delete m;
    m = nullptr;
  }

  int Unload() {  // UnloadLRUBlock
    int s = (int)lru.front();
    Slot& info = slots[s];
    int p = info.parent;
    for (int i = 0; i < info.roots_count; ++i) {
      uint32_t v = info.ptr_value[i];
      uint32_t mask = v & 255, fault = (v >> 8) & 1, dup = (v >> 9) & 1, ptr = v >> 11;
      if (mask && !fault) v = CacheLink(mask, false, dup, false, NearValue(info.ptr_index[i], ptr));
      links()[(int64_t)p * nib + info.ptr_index[i]] = v;
      ++patches;
    }
    for (int c : info.children) parent_slot.erase(c);
    info.children.clear();
    lru.pop_front();
    block_slot.erase(info.block);
    DequeueMarkers();
    return s;
  }

  void Upload(Block& b) {  // UploadBlock
    int s;
    if (first_free == max_blocks) {
      if (b.parent != kRootParent) Touch(parent_slot.at((int)b.index));  // MarkParentAsUsed(global)
      s = Unload();
    } else {
      s = first_free++;
    }
    Slot& info = slots[s];
    uint32_t* src = reinterpret_cast<uint32_t*>(b.content.data());
    for (int n = 0; n < nib; ++n) {
      uint32_t l = src[n], mask = l & 255, fault = (l >> 8) & 1, dup = (l >> 9) & 1, ptr = l >> 11;
      if (!mask) continue;
      if (!fault) {
        src[n] = CacheLink(mask, false, dup, false, NearValue(n, ptr));
      } else if (!parent_slot.count((int)ptr)) {
        parent_slot[(int)ptr] = s;
        info.children.push_back((int)ptr);
      }
    }
    const uint8_t* p = b.content.data();
    for (size_t c = 0; c < chan.size(); ++c) {
      size_t bytes = (size_t)nib * chan_bytes[c];
      std::memcpy(chan[c].data() + (size_t)s * bytes, p, bytes);
      p += bytes;
    }
    ++uploaded;
    if (b.parent != kRootParent) {
      int ps = parent_slot.at((int)b.index);
      info.parent = ps;
      info.roots_count = (int)b.roots_count;
      for (uint32_t i = 0; i < b.roots_count; ++i) {
        const BlockRoot& r = b.roots[i];
        info.ptr_index[i] = r.parent_pointer_index;
        info.ptr_value[i] = r.parent_pointer_value;
        int64_t absolute = (int64_t)s * nib + r.pointed_child_index;
        int64_t ptr_at = (int64_t)ps * nib + r.parent_pointer_index;
        bool far_ = std::llabs(ptr_at - absolute) >= (1 << 20);
        uint32_t ptr;
        if (far_) {
          ptr = (uint32_t)s * 8 + i;
          far[ptr] = (uint32_t)absolute;
          ++far_patches;
        } else {
          ptr = NearValue(ptr_at, absolute);
        }
        uint32_t pv = r.parent_pointer_value;
        links()[ptr_at] = CacheLink(pv & 255, false, !((pv >> 8) & 1), far_, ptr);
        ++patches;
      }
    } else {
      info.parent = (int)kRootParent;
    }
    block_slot[(int)b.index] = s;
    info.block = (int)b.index;
    info.lru = lru.insert(lru.begin(), s);
    Touch(s);
  }

  bool LoadAndUpload(int index) {
    Block b;
    if (!tree->Load((uint32_t)index, &b)) { g_error = "load failed"; return false; }
    bool root = b.parent == kRootParent;
    int root_child = b.roots[0].pointed_child_index;
    Upload(b);
    if (root) root_node = block_slot[index] * nib + root_child;
    return true;
  }

  bool InitialFill() {  // gpu-octree-cache-manager.cpp:60-108
    std::queue<int> q;
    q.push((int)tree->root_block);
    while (first_free < max_blocks && !q.empty()) {
      int index = q.front();
      q.pop();
      if (block_slot.count(index)) continue;
      Block b;
      if (!tree->Load((uint32_t)index, &b)) { g_error = "load failed"; return false; }
      const uint32_t* l = reinterpret_cast<const uint32_t*>(b.content.data());
      for (int i = 0; i < nib; ++i)
        if ((l[i] & 255) && ((l[i] >> 8) & 1)) q.push((int)(l[i] >> 11));
      bool root = b.parent == kRootParent;
      int root_child = b.roots[0].pointed_child_index;
      Upload(b);
      if (root) root_node = block_slot[index] * nib + root_child;
    }
    return true;
  }

  void StartSession() { DropMarker(session); session = NewMarker(); }
  void StartTransaction() { DropMarker(transaction); transaction = NewMarker(); }
  void MarkUsed(int slot) { Touch(slot); }
  void MarkParentUsed(int slot) {
    int p = slots[slot].parent;
    if (p != (int)kRootParent) Touch(p); else DequeueMarkers();
  }
  void Request(int block) {
    if (block_slot.count(block)) return;
    pending.push_back(block);
    Touch(parent_slot.at(block));
  }
  bool TransactionFilled() const { return transaction->hit; }
  bool SessionFilled() const { return session->hit; }
  bool EndTransaction() {
    bool ok = true;
    for (size_t i = 0; i < pending.size(); ++i) {
      if (TransactionFilled()) break;
      if (!LoadAndUpload(pending[i])) { ok = false; break; }
    }
    pending.clear();
    DropMarker(transaction);
    return ok;
  }
  void EndSession() { DropMarker(session); }
};

// ---------------------------------------------------------------------------
// Kernels (the .cl files) as scalar C++.
struct V4 { float x, y, z, w; };
inline V4 v4(float x, float y, float z, float w) { return V4{x, y, z, w}; }
inline float Dot(V4 a, V4 b) { float r = a.x * b.x; r = r + a.y * b.y; r = r + a.z * b.z; r = r + a.w * b.w; return r; }
inline V4 Sub(V4 a, V4 b) { return v4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
inline V4 Div(V4 a, float s) { return v4(a.x / s, a.y / s, a.z / s, a.w / s); }
inline float Len(V4 a) { return std::sqrt(Dot(a, a)); }

// init_tracing_frame.cl:3-9
inline V4 MulPoint(const float* m, V4 p) {
  V4 h = v4(p.x, p.y, p.z, 1);
  float d = Dot(h, v4(m[12], m[13], m[14], m[15]));
  return Div(v4(Dot(h, v4(m[0], m[1], m[2], m[3])), Dot(h, v4(m[4], m[5], m[6], m[7])),
                Dot(h, v4(m[8], m[9], m[10], m[11])), 0.0f), d);
}

struct RayState {
  V4 origin;  // w: LOD size bias
  V4 dir;     // w: LOD size coefficient
  int fault_parent;
  uint8_t color[4];
  uint8_t mult[4];
  // Depth output (no reference counterpart): the distance the ray advanced
  // over faulted passes (the t of each fault, summed in float in pass order),
  // and the pixel's final depth and shading node.
  float adv;
  float depth;
  int node;
};
constexpr uint32_t kDepthNaN = 0x7fffffffu, kDepthInf = 0x7f800000u;
inline float FloatBits(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }

// init_tracing_frame.cl:11-45
void InitRay(RayState& s, int x, int y, int W, int H, const float* m, float lod) {
  V4 tmp = v4((x + 0.5f) / W * 2 - 1, (y + 0.5f) / H * 2 - 1, -1, 0);
  V4 origin = Div(v4(m[2], m[6], m[10], 0.0f), m[14]);
  tmp.z = 0;
  V4 dir = Sub(MulPoint(m, tmp), origin);
  dir = Div(dir, Len(dir));
  V4 p1 = MulPoint(m, v4((float)x / W * 2 - 1, (float)y / H * 2 - 1, 0, 0));
  V4 p2 = MulPoint(m, v4((float)(x + 1) / W * 2 - 1, (float)(y + 1) / H * 2 - 1, 0, 0));
  float coef = lod * Len(Sub(p1, p2)) / Len(Sub(origin, p1));
  s.origin = v4(origin.x, origin.y, origin.z, 0);
  s.dir = v4(dir.x, dir.y, dir.z, coef);
  s.fault_parent = -1;
  std::memset(s.color, 0, 4);
  std::memset(s.mult, 255, 4);
  s.adv = 0.0f;
  s.depth = FloatBits(kDepthInf);
  s.node = -1;
}

struct CastResult {
  float t;
  int node, fault_block, dup, error;
  int fetches, far_fetches, iterations;
};

inline int AsInt(float f) { int r; std::memcpy(&r, &f, 4); return r; }
inline uint32_t AsUint(float f) { uint32_t r; std::memcpy(&r, &f, 4); return r; }
inline float AsFloat(uint32_t u) { float r; std::memcpy(&r, &u, 4); return r; }

// raycast.cl:33-256 (ESVO descent in [1,2]^3 with block-cache faults)
// Three guards make the reference's undefined accesses explicit (all
// unreachable on a well-formed cache and a tree of at most 23 levels): a pop
// that lands past the root ends the loop before reading stack[scale >= 23]; a
// node or far index outside the cache ends the ray with the iteration-limit
// error; a node at scale 0 ends the ray like a leaf (its children would lie
// below float resolution, and the reference would index its stack at -1).
void Cast(const uint32_t* links, const uint32_t* far, int root, V4 p, V4 d, float coef, float bias, CastResult* r,
          uint32_t node_limit, uint32_t far_limit) {
  p.x = p.x + 1; p.y = p.y + 1; p.z = p.z + 1;
  r->fault_block = -1; r->error = 0; r->dup = 0; r->fetches = 0; r->far_fetches = 0;
  uint32_t stack_parent[kSMax + 1];
  float stack_tmax[kSMax + 1];
  if (std::fabs(d.x) < kEps) d.x = std::copysign(kEps, d.x);
  if (std::fabs(d.y) < kEps) d.y = std::copysign(kEps, d.y);
  if (std::fabs(d.z) < kEps) d.z = std::copysign(kEps, d.z);
  float tx_coef = 1.0f / -std::fabs(d.x), ty_coef = 1.0f / -std::fabs(d.y), tz_coef = 1.0f / -std::fabs(d.z);
  float tx_bias = tx_coef * p.x, ty_bias = ty_coef * p.y, tz_bias = tz_coef * p.z;
  int octant = 0;
  if (d.x > 0.0f) octant ^= 1, tx_bias = 3.0f * tx_coef - tx_bias;
  if (d.y > 0.0f) octant ^= 2, ty_bias = 3.0f * ty_coef - ty_bias;
  if (d.z > 0.0f) octant ^= 4, tz_bias = 3.0f * tz_coef - tz_bias;
  float t_min = std::fmax(std::fmax(2.0f * tx_coef - tx_bias, 2.0f * ty_coef - ty_bias), 2.0f * tz_coef - tz_bias);
  float t_max = std::fmin(std::fmin(tx_coef - tx_bias, ty_coef - ty_bias), tz_coef - tz_bias);
  float h = t_max;
  t_min = std::fmax(t_min, 0.0f);
  uint32_t parent = (uint32_t)root, desc = 0;
  int idx = 0;
  float px = 1.0f, py = 1.0f, pz = 1.0f;
  int scale = kSMax - 1;
  float scale_exp2 = 0.5f;
  if (1.5f * tx_coef - tx_bias > t_min) idx ^= 1, px = 1.5f;
  if (1.5f * ty_coef - ty_bias > t_min) idx ^= 2, py = 1.5f;
  if (1.5f * tz_coef - tz_bias > t_min) idx ^= 4, pz = 1.5f;
  int iter = 0;
  while (scale < kSMax) {
    if (++iter > 300) {
      r->error = 1; r->t = t_min; r->node = (int)parent; r->iterations = iter;
      return;
    }
    if (desc == 0) {
      if (parent >= node_limit) { r->error = 1; r->t = t_min; r->node = 0; r->iterations = iter; return; }
      desc = links[parent];
      ++r->fetches;
    }
    float tx_corner = px * tx_coef - tx_bias, ty_corner = py * ty_coef - ty_bias, tz_corner = pz * tz_coef - tz_bias;
    float tc_max = std::fmin(std::fmin(tx_corner, ty_corner), tz_corner);
    int shift = idx ^ octant;
    uint32_t bit = 1u << shift;
    if ((desc & bit) != 0 && t_min <= t_max) {
      if ((desc & (1u << 8)) != 0) {
        r->node = (int)parent; r->t = t_min; r->fault_block = (int)(desc >> 11); r->iterations = iter;
        return;
      }
      uint32_t ofs;
      if (desc & (1u << 10)) {
        if ((desc >> 11) >= far_limit) { r->error = 1; r->t = t_min; r->node = (int)parent; r->iterations = iter; return; }
        ofs = far[desc >> 11];
        ++r->far_fetches;
      } else {
        ofs = (desc >> 11) + parent - (1u << 20);
      }
      ofs += (uint32_t)__builtin_popcount(desc & (bit - 1) & 255u);
      if (ofs >= node_limit) { r->error = 1; r->t = t_min; r->node = (int)parent; r->iterations = iter; return; }
      desc = links[ofs];
      ++r->fetches;
      if (!(desc & 255) || scale == 0 || tc_max * coef + bias >= scale_exp2) {
        r->t = t_min; r->node = (int)ofs; r->dup = (int)((desc >> 9) & 1); r->iterations = iter;
        return;
      }
      float half = scale_exp2 * 0.5f;
      float tx_center = half * tx_coef + tx_corner, ty_center = half * ty_coef + ty_corner, tz_center = half * tz_coef + tz_corner;
      if (tc_max < h) { stack_parent[scale] = parent; stack_tmax[scale] = t_max; }
      h = tc_max;
      parent = ofs;
      idx = 0;
      --scale;
      scale_exp2 = half;
      if (tx_center > t_min) idx ^= 1, px = px + scale_exp2;
      if (ty_center > t_min) idx ^= 2, py = py + scale_exp2;
      if (tz_center > t_min) idx ^= 4, pz = pz + scale_exp2;
      t_max = tc_max;
      // desc keeps the link just read: it is the new parent's descriptor
      continue;
    }
    int step = 0;
    if (tx_corner <= tc_max) step ^= 1, px = px - scale_exp2;
    if (ty_corner <= tc_max) step ^= 2, py = py - scale_exp2;
    if (tz_corner <= tc_max) step ^= 4, pz = pz - scale_exp2;
    t_min = tc_max;
    idx ^= step;
    if ((idx & step) != 0) {
      uint32_t diff = 0;
      if (step & 1) diff |= (uint32_t)(AsInt(px) ^ AsInt(px + scale_exp2));
      if (step & 2) diff |= (uint32_t)(AsInt(py) ^ AsInt(py + scale_exp2));
      if (step & 4) diff |= (uint32_t)(AsInt(pz) ^ AsInt(pz + scale_exp2));
      scale = (AsInt((float)diff) >> 23) - 127;
      if (scale >= kSMax) break;
      scale_exp2 = AsFloat((uint32_t)((scale - kSMax + 127) << 23));
      parent = stack_parent[scale];
      t_max = stack_tmax[scale];
      uint32_t shx = AsUint(px) >> scale, shy = AsUint(py) >> scale, shz = AsUint(pz) >> scale;
      px = AsFloat(shx << scale); py = AsFloat(shy << scale); pz = AsFloat(shz << scale);
      idx = (int)((shx & 1) | ((shy & 1) << 1) | ((shz & 1) << 2));
      h = 0.0f;
      desc = 0;
    }
  }
  r->t = 1e30f; r->node = -1; r->iterations = iter;
}

// raytracer.cl:18-71 (RaytraceKernel, the reference's debug depth view): one
// pass from the near plane over the cache as it is, no feedback; red for a
// fault or error, black for a miss, else grey = 255 * (1 - log-depth in
// [0.01, 5]).  The grey conversion clamps to [0, 255] (the reference's
// conversion is undefined outside that range).
void DepthView(const uint32_t* links, const uint32_t* far, int root, uint32_t node_limit, uint32_t far_limit,
               const float* m, float lod, int W, int H, uint8_t* out) {
#pragma omp parallel for schedule(dynamic, 256)
  for (long long i = 0; i < (long long)W * H; ++i) {
    const int x = (int)(i % W), y = (int)(i / W);
    V4 tmp = v4((x + 0.5f) / W * 2 - 1, (y + 0.5f) / H * 2 - 1, -1, 0);
    const V4 origin = MulPoint(m, tmp);
    tmp.z = 0;
    V4 dir = Sub(MulPoint(m, tmp), origin);
    dir = Div(dir, Len(dir));
    tmp = v4((float)x / W * 2 - 1, (float)y / H * 2 - 1, -1, 0);
    const V4 p1n = MulPoint(m, tmp);
    tmp.z = 0;
    const V4 p1f = MulPoint(m, tmp);
    tmp = v4((float)(x + 1) / W * 2 - 1, (float)(y + 1) / H * 2 - 1, -1, 0);
    const V4 p2n = MulPoint(m, tmp);
    tmp.z = 0;
    const V4 p2f = MulPoint(m, tmp);
    const float bias = lod * Len(Sub(p1n, p2n));
    const float coef = (bias < 1e-10f) ? 0 : (lod * (Len(Sub(p1f, p2f)) - Len(Sub(p1n, p2n))) / Len(Sub(p1n, p1f)));
    CastResult r{};
    Cast(links, far, root, origin, dir, coef, bias, &r, node_limit, far_limit);
    uint8_t* o = out + i * 4;
    if (r.error || r.fault_block != -1) {
      o[0] = 255, o[1] = 0, o[2] = 0, o[3] = 255;
    } else if (r.node == -1) {
      o[0] = 0, o[1] = 0, o[2] = 0, o[3] = 255;
    } else {
      const float near_ = 0.01f, far_ = 5;
      float d = (std::log(r.t) - std::log(near_)) / (std::log(far_) - std::log(near_));
      d = (1 - d) * 255;
      d = std::min(255.0f, std::max(0.0f, d));
      const uint8_t g = (uint8_t)d;
      o[0] = g, o[1] = g, o[2] = g, o[3] = 255;
    }
  }
}

// shading.cl:4-33
void Shade(int node, RayState& s, const int8_t* normals, const uint8_t* colors) {
  static const V4 L1 = [] { V4 v = v4(2, -2, 3, 0); V4 n = Div(v, Len(v)); return v4(n.x * .6f, n.y * .6f, n.z * .6f, n.w * .6f); }();
  static const V4 L2 = [] { V4 v = v4(-3, -3, -2, 0); V4 n = Div(v, Len(v)); return v4(n.x * .5f, n.y * .5f, n.z * .5f, n.w * .5f); }();
  static const V4 L3 = [] { V4 v = v4(1, 2.5f, -1, 0); V4 n = Div(v, Len(v)); return v4(n.x * .3f, n.y * .3f, n.z * .3f, n.w * .3f); }();
  const int8_t* cn = normals + 4 * (int64_t)node;
  V4 n = v4((float)cn[0] / 127.f, (float)cn[1] / 127.f, (float)cn[2] / 127.f, 0.0f / 127.f);
  V4 neg = v4(-n.x, -n.y, -n.z, -n.w);
  float a1 = std::max(0.f, Dot(neg, L1)), a2 = std::max(0.f, Dot(neg, L2)), a3 = std::max(0.f, Dot(neg, L3));
  // ambient + a1*col1 + a2*col2 + a3*col3 with white light colours (w component 0)
  float lx = ((.1f + a1 * 1.f) + a2 * 1.f) + a3 * 1.f;
  float lw = ((0.f + a1 * 0.f) + a2 * 0.f) + a3 * 0.f;
  const uint8_t* cc = colors + 4 * (int64_t)node;
  float c[4] = {(float)cc[0] * lx, (float)cc[1] * lx, (float)cc[2] * lx, 255.0f * lw};
  for (int k = 0; k < 3; ++k) {
    float v = c[k] > 255.0f ? 255.0f : c[k];  // min(255, v) with the OpenCL definition
    s.color[k] = (uint8_t)v;
  }
  s.color[3] = 255;
  std::memset(s.mult, 0, 4);
}

inline bool Done(const RayState& s) { return !s.mult[0] && !s.mult[1] && !s.mult[2] && !s.mult[3]; }

struct PassCounters { long long rays = 0, fetches = 0, far_fetches = 0, iterations = 0, hits = 0; };

// raytracing_pass.cl:4-61 for one pixel; returns the feedback word
int32_t TracePixel(RayState& s, const Cache& c, const uint32_t* links, const int8_t* normals,
                   const uint8_t* colors, CastResult* res) {
  if (Done(s)) return kNoHit;
  Cast(links, c.far.data(), c.root_node, s.origin, s.dir, s.dir.w, s.origin.w, res,
       (uint32_t)c.max_blocks * (uint32_t)c.nib, (uint32_t)c.max_blocks * 8u);
  if (res->error) {
    s.color[0] = 255; s.color[1] = 0; s.color[2] = 0; s.color[3] = 255;
    std::memset(s.mult, 0, 4);
    s.depth = FloatBits(kDepthNaN);
    s.node = -2;
    return kNoHit;
  }
  if (res->fault_block != -1) {
    s.origin.x = s.origin.x + s.dir.x * res->t;
    s.origin.y = s.origin.y + s.dir.y * res->t;
    s.origin.z = s.origin.z + s.dir.z * res->t;
    s.origin.w = s.origin.w + s.dir.w * res->t;
    s.fault_parent = res->node;
    s.adv = s.adv + res->t;
    return -res->fault_block - 1;
  }
  if (res->node == -1) {
    std::memset(s.mult, 0, 4);
    s.depth = FloatBits(kDepthInf);
    s.node = -1;
    return kNoHit;
  }
  if (normals && colors) Shade(res->node, s, normals, colors);
  else std::memset(s.mult, 0, 4);
  s.depth = s.adv + res->t;
  s.node = res->node;
  return (int32_t)(((uint32_t)(res->node + 1) << 1) | (uint32_t)res->dup);
}

// finish_tracing_frame.cl:3-24
void FinishPixel(RayState& s, const int8_t* normals, const uint8_t* colors, uint8_t* out) {
  if (!Done(s)) {  // still faulted: the parent's colour at the distance where the ray stopped
    s.depth = s.adv;
    s.node = s.fault_parent;
  }
  if (!Done(s) && normals && colors) Shade(s.fault_parent, s, normals, colors);
  const float bg[4] = {0.0f, (float)(216 / 255.), 1.0f, 1.0f};
  for (int k = 0; k < 4; ++k) {
    float t = (float)s.color[k] + bg[k] * (255.f - (float)s.color[3]) + .5f;
    float v = std::max(0.f, std::min(255.f, t));
    out[k] = (uint8_t)v;
  }
}

// ---------------------------------------------------------------------------
// Feedback: NodeToBlock -> merge sort -> flag -> scan -> compress
// (feedback_compression.cl, merge_sort.cl, scan.cl), restated as the same
// rank-by-binary-search merge passes and the same Hillis-Steele scan.
void NodeToBlock(int32_t* d, int n, int nib) {
  for (int i = 0; i < n; ++i) {
    int32_t v = d[i];
    if (v > 0 && v != kNoHit) d[i] = ((((v >> 1) - 1) / nib + 1) << 1) | (v & 1);
  }
}

// merge_sort.cl:47-73 - one pass merging sibling runs of `len` by ranking each
// element in its sibling run (ties broken by index, so the merge is stable).
void MergePass(const int32_t* in, int32_t* out, int n, int len) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) {
    int key = in[i];
    int ii = i & (len - 1);
    int sib = (i - ii) ^ len;
    int pos;
    if (sib >= n || in[sib] > key || (in[sib] == key && sib > i)) {
      pos = -1;
    } else {
      pos = 0;
      for (int inc = len >> 1; inc > 0; inc >>= 1) {
        int j = sib + pos + inc;
        bool smaller = j < n && (in[j] < key || (in[j] == key && j < i));
        pos += smaller ? inc : 0;
      }
    }
    out[(ii + pos + 1) | (i & ~((len << 1) - 1))] = key;
  }
}

// GPUSort::Sort (gpu-sort.cpp:16-49): runs of the work-group size are sorted
// first (LocalMergeSortKernel is the same rank merge inside a group, which the
// passes of length 1..128 reproduce), then global passes double the run length.
void MergeSort(int32_t* data, int n) {
  std::vector<int32_t> tmp((size_t)n);
  int32_t* in = data;
  int32_t* out = tmp.data();
  for (int len = 1; len < n; len *= 2) {
    MergePass(in, out, n, len);
    std::swap(in, out);
  }
  if (in != data) std::memcpy(data, in, (size_t)n * 4);
}

// GPUScan::Scan (gpu-scan.cpp:15-43): inclusive Hillis-Steele, wrapping int32.
void Scan(int32_t* data, int n) {
  std::vector<int32_t> tmp((size_t)n);
  int32_t* in = data;
  int32_t* out = tmp.data();
  for (int len = 1; len < n; len *= 2) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
      uint32_t v = (uint32_t)in[i];
      if (i - len >= 0) v += (uint32_t)in[i - len];
      out[i] = (int32_t)v;
    }
    std::swap(in, out);
  }
  if (in != data) std::memcpy(data, in, (size_t)n * 4);
}

// GetUnique (ray-tracing-feedback-extractor.cpp:44-98); words are modified
// (block-converted and sorted) like the reference's buffer.  Returns the
// unique count including a trailing NO_HIT when present.
int Unique(int32_t* words, int n, int nib, int32_t* out) {
  if (nib > 0) NodeToBlock(words, n, nib);
  MergeSort(words, n);
  std::vector<int32_t> idx((size_t)n);
  for (int i = 0; i < n; ++i) idx[i] = (i != 0 && words[i - 1] != words[i]) ? 1 : 0;
  Scan(idx.data(), n);
  for (int i = 0; i < n; ++i) {
    if (i == 0) out[0] = words[0];
    else if (words[i - 1] != words[i]) out[idx[i]] = words[i];
  }
  return n ? idx[n - 1] + 1 : 0;
}

struct Feedback {
  int expected_faults = 1 << 16;
  int hits_to_extract = 4000;
  std::vector<int> faults, hits, dup_hits;
  void AddHit(int v) {
    if (v & 1) dup_hits.push_back((v >> 1) - 1);
    else hits.push_back((v >> 1) - 1);
  }
  // ProcessUnique + AdjustExpectedFaults (:108-185)
  void Decode(const int32_t* u, int count) {
    faults.clear(); hits.clear(); dup_hits.clear();
    int stride = expected_faults, size = 0;
    while (size < count && (size == 0 || u[size - 1] < 0)) {
      stride = std::min(stride, count - size);
      for (int i = size; i < size + stride; ++i) {
        if (u[i] < 0) faults.push_back(-u[i] - 1);
        else if (u[i] != kNoHit) AddHit(u[i]);
      }
      size += stride;
      stride *= 2;
    }
    if (size < count) {
      int len = count - size;
      int start = rand() % len;
      int take = std::min(hits_to_extract, len);
      std::vector<std::pair<int, int>> segs;
      if (start + take <= len) segs.emplace_back(start, take);
      else { segs.emplace_back(0, start + take - len); segs.emplace_back(start, len - start); }
      for (auto& sg : segs)
        for (int i = 0; i < sg.second; ++i) {
          int v = u[size + sg.first + i];
          if (v != kNoHit) AddHit(v);
        }
    }
    if (expected_faults > 1 && (int)faults.size() < expected_faults) expected_faults /= 2;
    else if ((int)faults.size() > expected_faults) expected_faults *= 2;
  }
};

// Views: the reference renders one (w, h) view per frame.  Several views of
// one frame (the batched form, which has no reference counterpart) are traced
// pass by pass together: their words are concatenated in view order, so the
// feedback of a pass is one unique array over all views and NO_HIT is present
// unless every ray of every view produced a word.
struct Renderer {
  Cache* cache;
  int w, h;                        // the first view
  std::vector<int> vw, vh;
  std::vector<size_t> voff;        // first pixel of each view
  size_t total = 0;
  float lod = 1.5f;
  double time_limit = 1.0;
  int max_passes = 0;
  bool record = false;
  std::vector<RayState> st;
  std::vector<int32_t> words, sorted, uniq;
  std::vector<uint8_t> image;
  Feedback fb;
  std::vector<std::vector<int32_t>> pass_words;
  PassCounters counters;
  int passes = 0;
  long long faults_total = 0;

  const int8_t* Normals() const {
    for (size_t c = 0; c < cache->tree->channels.size(); ++c)
      if (cache->tree->channels[c].first == 4 && cache->tree->channels[c].second == "normals")
        return reinterpret_cast<const int8_t*>(cache->chan[c].data());
    return nullptr;
  }
  const uint8_t* Colors() const {
    for (size_t c = 0; c < cache->tree->channels.size(); ++c)
      if (cache->tree->channels[c].first == 4 && cache->tree->channels[c].second == "colors")
        return cache->chan[c].data();
    return nullptr;
  }

  void Pass() {
    const uint32_t* links = cache->links();
    const int8_t* nrm = Normals();
    const uint8_t* col = Colors();
    long long fetches = 0, fars = 0, iters = 0, rays = 0, hits = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : fetches, fars, iters, rays, hits)
    for (long long i = 0; i < (long long)total; ++i) {
      CastResult r{};
      bool live = !Done(st[i]);
      words[i] = TracePixel(st[i], *cache, links, nrm, col, &r);
      if (live) {
        ++rays;
        fetches += r.fetches; fars += r.far_fetches; iters += r.iterations;
        if (words[i] > 0 && words[i] != kNoHit) ++hits;
      }
    }
    counters.rays += rays; counters.fetches += fetches; counters.far_fetches += fars;
    counters.iterations += iters; counters.hits += hits;
  }

  // GPURayTracer::RenderFrame (gpu-ray-tracer.cpp:66-227)
  void SetViews(int n, const int* ws, const int* hs) {
    vw.assign(ws, ws + n);
    vh.assign(hs, hs + n);
    voff.clear();
    total = 0;
    for (int v = 0; v < n; ++v) {
      voff.push_back(total);
      total += (size_t)ws[v] * hs[v];
    }
    w = ws[0];
    h = hs[0];
  }

  // InitTracingFrame for every view; m holds one matrix per view
  void InitViews(const float* m) {
    st.resize(total);
    words.resize(total);
    for (size_t v = 0; v < vw.size(); ++v)
      for (int y = 0; y < vh[v]; ++y)
        for (int x = 0; x < vw[v]; ++x)
          InitRay(st[voff[v] + (size_t)y * vw[v] + x], x, y, vw[v], vh[v], m + 16 * v, lod);
  }

  bool Frame(const float* m) {
    auto t0 = std::chrono::steady_clock::now();
    uniq.resize(total);
    image.resize(total * 4);
    pass_words.clear();
    InitViews(m);
    cache->StartSession();
    bool ok = true;
    int it;
    for (it = 0;; ++it) {
      Pass();
      if (record) pass_words.push_back(words);
      double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      if (it > 0 && el > time_limit) break;
      if (max_passes > 0 && it + 1 >= max_passes && it > 0) break;
      sorted = words;
      int count = Unique(sorted.data(), (int)total, cache->nib, uniq.data());
      fb.Decode(uniq.data(), count);
      cache->StartTransaction();
      for (int b : fb.hits) cache->MarkUsed(b);
      for (int b : fb.dup_hits) cache->MarkParentUsed(b);
      for (int f : fb.faults) {
        if (cache->TransactionFilled()) break;
        cache->Request(f);
      }
      faults_total += (long long)fb.faults.size();
      if (!cache->EndTransaction()) { ok = false; break; }
      if (fb.faults.empty() || cache->SessionFilled()) break;
    }
    passes = it + 1;
    cache->EndSession();
    const int8_t* nrm = Normals();
    const uint8_t* col = Colors();
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)total; ++i) FinishPixel(st[i], nrm, col, &image[(size_t)i * 4]);
    return ok;
  }
};

}  // namespace

// ---------------------------------------------------------------------------
extern "C" {

const char* oracle_last_error() { return g_error.c_str(); }

void* oracle_tree_open(const char* path) {
  TreeFile* t = new TreeFile();
  if (!t->Open(path)) { delete t; return nullptr; }
  return t;
}
void oracle_tree_close(void* t) { delete static_cast<TreeFile*>(t); }
int oracle_tree_blocks(void* t) { return (int)static_cast<TreeFile*>(t)->blocks; }
int oracle_tree_nib(void* t) { return (int)static_cast<TreeFile*>(t)->nib; }

void* oracle_cache_create(void* tree, int max_blocks) {
  TreeFile* t = static_cast<TreeFile*>(tree);
  Cache* c = new Cache();
  c->tree = t;
  c->nib = (int)t->nib;
  c->max_blocks = max_blocks > 0 ? max_blocks : (int)t->blocks;
  for (auto& ch : t->channels) {
    c->chan_bytes.push_back(ch.first);
    c->chan.emplace_back((size_t)c->max_blocks * c->nib * ch.first, 0);
  }
  c->far.assign((size_t)c->max_blocks * 8, 0);
  c->slots.resize((size_t)c->max_blocks);
  return c;
}
void oracle_cache_destroy(void* c) { delete static_cast<Cache*>(c); }
int oracle_cache_initial_fill(void* c) { return static_cast<Cache*>(c)->InitialFill() ? 0 : -1; }
int oracle_cache_root(void* c) { return static_cast<Cache*>(c)->root_node; }
int oracle_cache_loaded(void* c) { return static_cast<Cache*>(c)->first_free; }
int oracle_cache_max_blocks(void* c) { return static_cast<Cache*>(c)->max_blocks; }
// channel index or -1 for far pointers
int oracle_cache_read(void* cp, int channel, void* out, long long bytes) {
  Cache* c = static_cast<Cache*>(cp);
  if (channel < 0) {
    if (bytes > (long long)c->far.size() * 4) return -1;
    std::memcpy(out, c->far.data(), (size_t)bytes);
    return 0;
  }
  if (channel >= (int)c->chan.size() || bytes > (long long)c->chan[channel].size()) return -1;
  std::memcpy(out, c->chan[channel].data(), (size_t)bytes);
  return 0;
}
void oracle_cache_counters(void* cp, long long* out3) {
  Cache* c = static_cast<Cache*>(cp);
  out3[0] = c->uploaded; out3[1] = c->patches; out3[2] = c->far_patches;
}

void* oracle_renderer_create(void* cache, int w, int h, float lod, double time_limit, int max_passes) {
  Renderer* r = new Renderer();
  r->cache = static_cast<Cache*>(cache);
  r->SetViews(1, &w, &h);
  r->lod = lod; r->time_limit = time_limit; r->max_passes = max_passes;
  return r;
}
void* oracle_renderer_create_views(void* cache, int n, const int* ws, const int* hs, float lod, double time_limit,
                                   int max_passes) {
  Renderer* r = new Renderer();
  r->cache = static_cast<Cache*>(cache);
  r->SetViews(n, ws, hs);
  r->lod = lod; r->time_limit = time_limit; r->max_passes = max_passes;
  return r;
}
int oracle_frame_view_image(void* rp, int view, unsigned char* out) {
  Renderer* r = static_cast<Renderer*>(rp);
  if (view < 0 || view >= (int)r->vw.size()) return -1;
  std::memcpy(out, r->image.data() + r->voff[view] * 4, (size_t)r->vw[view] * r->vh[view] * 4);
  return 0;
}
void oracle_renderer_destroy(void* r) { delete static_cast<Renderer*>(r); }
void oracle_renderer_record(void* r, int on) { static_cast<Renderer*>(r)->record = on != 0; }
int oracle_render_frame(void* rp, const float* view_proj_inv) {
  Renderer* r = static_cast<Renderer*>(rp);
  return r->Frame(view_proj_inv) ? r->passes : -1;
}
int oracle_frame_image(void* rp, unsigned char* out) {
  Renderer* r = static_cast<Renderer*>(rp);
  std::memcpy(out, r->image.data(), r->image.size());
  return 0;
}
// Depth output of the last frame: per pixel (views concatenated in order) the
// distance to what it shows and the cache node that shaded it.
int oracle_frame_depth(void* rp, float* depth, int* nodes) {
  Renderer* r = static_cast<Renderer*>(rp);
  for (size_t i = 0; i < r->total; ++i) {
    if (depth) depth[i] = r->st[i].depth;
    if (nodes) nodes[i] = r->st[i].node;
  }
  return 0;
}
int oracle_frame_pass_words(void* rp, int pass, int* out) {
  Renderer* r = static_cast<Renderer*>(rp);
  if (pass < 0 || pass >= (int)r->pass_words.size()) return -1;
  std::memcpy(out, r->pass_words[pass].data(), r->pass_words[pass].size() * 4);
  return 0;
}
// rays, node-link fetches, far-pointer fetches, iterations, hits, faults (since create)
void oracle_renderer_counters(void* rp, long long* out6) {
  Renderer* r = static_cast<Renderer*>(rp);
  out6[0] = r->counters.rays; out6[1] = r->counters.fetches; out6[2] = r->counters.far_fetches;
  out6[3] = r->counters.iterations; out6[4] = r->counters.hits; out6[5] = r->faults_total;
}

// One tracing pass from a fresh camera over the resident cache, no feedback:
// writes per-pixel words and RGBA (done pixels final, others unfinished).
int oracle_trace_once(void* rp, const float* m, int* words_out, unsigned char* rgba_out) {
  Renderer* r = static_cast<Renderer*>(rp);
  r->InitViews(m);
  r->Pass();
  if (words_out) std::memcpy(words_out, r->words.data(), r->words.size() * 4);
  if (rgba_out) {
    const int8_t* nrm = r->Normals();
    const uint8_t* col = r->Colors();
    for (long long i = 0; i < (long long)r->total; ++i) {
      RayState s = r->st[i];
      FinishPixel(s, nrm, col, rgba_out + (size_t)i * 4);
    }
  }
  return 0;
}

int oracle_depth_view(void* cp, const float* m, float lod, int w, int h, unsigned char* out) {
  Cache* c = static_cast<Cache*>(cp);
  DepthView(c->links(), c->far.data(), c->root_node, (uint32_t)c->max_blocks * (uint32_t)c->nib,
            (uint32_t)c->max_blocks * 8u, m, lod, w, h, out);
  return 0;
}

void oracle_sort(int* data, int n) { MergeSort(data, n); }
void oracle_scan(int* data, int n) { Scan(data, n); }
int oracle_feedback_unique(int* words, int n, int nib, int* out) { return Unique(words, n, nib, out); }

}  // extern "C"
