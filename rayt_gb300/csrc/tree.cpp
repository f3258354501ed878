// Block-file access, scene building and camera math (host C++).
//
//  * rayt_tree_*: the reference's StoredOctreeLoader
//    (rayt/CPU data/stored-octree-loader.cpp:9-98) over pread(2); the header
//    layout is rayt/doc/storage data format.txt:1-33.  For the block cache the
//    file can also be mapped and registered with the device once, so that
//    streamed blocks are read by the upload kernel where they lie in the page
//    cache instead of being copied into staging buffers first.
//  * rayt_build_*: BuildOctree (rayt/CPU data/stored-octree-builder.h:40-41)
//    through block_builder.h with the sources of scene_source.h.
//  * rayt_camera_view_proj_inv: Camera::ViewProjectionMatrix().Inverse()
//    (rayt/scene/camera.cpp:23-28, rayt/util/mat.cpp:20-194): the same float
//    view-projection (horizontal FOV, infinite far plane, y up) inverted by
//    the reference's float cofactor method, so the 16 floats are its own.
#include <algorithm>
#include <cerrno>
#include <cstdlib>
#include <thread>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>
#include <cuda_runtime.h>
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include "block_builder.h"
#include "internal.h"
#include "scene_source.h"
#include "tree.h"

namespace rayt {

bool Tree::Read(int64_t off, size_t n, void* out) const {
  uint8_t* p = static_cast<uint8_t*>(out);
  while (n > 0) {
    ssize_t r = ::pread(fd, p, n, off);
    if (r < 0 && errno == EINTR) continue;
    if (r <= 0) return false;
    p += r;
    n -= (size_t)r;
    off += r;
  }
  return true;
}

int Tree::Open(const char* path) {
  fd = ::open(path, O_RDONLY);
  if (fd < 0) return fail(RAYT_E_IO, std::string("cannot open block file ") + path);
  uint32_t h[5];
  if (!Read(0, sizeof(h), h)) return fail(RAYT_E_FORMAT, "block file header is truncated");
  info.nodes_in_block = h[0];
  info.blocks_count = h[1];
  info.root_block_index = h[2];
  info.block_stride = h[3];
  info.channels_count = h[4];
  if (h[0] == 0 || h[0] > 65536 || h[4] == 0 || h[4] > 64 || h[1] == 0 || h[2] >= h[1])
    return fail(RAYT_E_FORMAT, "block file header has invalid sizes");
  int64_t pos = 20;
  uint64_t sum = 0;
  for (uint32_t i = 0; i < h[4]; ++i) {
    uint32_t c[2];
    if (!Read(pos, 8, c)) return fail(RAYT_E_FORMAT, "channel table is truncated");
    pos += 8;
    if (c[0] == 0 || c[0] > 64 || c[1] > 4096) return fail(RAYT_E_FORMAT, "channel record is invalid");
    std::string name(c[1], '\0');
    if (c[1] && !Read(pos, c[1], &name[0])) return fail(RAYT_E_FORMAT, "channel name is truncated");
    pos += c[1];
    chan_bytes.push_back((int)c[0]);
    chan_names.push_back(name);
    sum += c[0];
  }
  if (chan_names[0] != "node links" || chan_bytes[0] != 4)
    return fail(RAYT_E_FORMAT, "first channel must be \"node links\" with 4 bytes per node");
  const uint64_t content = sum * h[0];
  if (content + 76 > h[3]) return fail(RAYT_E_FORMAT, "block stride is smaller than a block record");
  info.content_bytes = (uint32_t)content;
  info.header_bytes = (uint64_t)pos;
  return RAYT_OK;
}

int Tree::LoadBlock(uint32_t index, rayt_block_header* hdr, void* content) const {
  if (index >= info.blocks_count) return fail(RAYT_E_ARG, "block index out of range");
  const int64_t off = (int64_t)info.header_bytes + (int64_t)info.block_stride * index;
  uint8_t raw[76];
  if (!Read(off, 76, raw)) return fail(RAYT_E_IO, "block header read failed");
  if (hdr) {
    std::memcpy(&hdr->block_index, raw, 4);
    std::memcpy(&hdr->parent_block_index, raw + 4, 4);
    std::memcpy(&hdr->roots_count, raw + 8, 4);
    for (int i = 0; i < 8; ++i) {
      std::memcpy(&hdr->roots[i].parent_pointer_index, raw + 12 + 8 * i, 2);
      std::memcpy(&hdr->roots[i].pointed_child_index, raw + 14 + 8 * i, 2);
      std::memcpy(&hdr->roots[i].parent_pointer_value, raw + 16 + 8 * i, 4);
    }
    if (hdr->roots_count < 1 || hdr->roots_count > 8) return fail(RAYT_E_FORMAT, "block has an invalid root count");
  }
  if (content && !Read(off + 76, info.content_bytes, content)) return fail(RAYT_E_IO, "block content read failed");
  return RAYT_OK;
}

const uint8_t* Tree::MapForDevice(const uint8_t** device_map) {
  std::lock_guard<std::mutex> lock(map_mu_);
  if (!map_tried_) {
    map_tried_ = true;
    struct stat st {};
    const uint64_t need = info.header_bytes + (uint64_t)info.block_stride * (info.blocks_count - 1) + 76 +
                          info.content_bytes;  // the last block's record ends here
    if (fd >= 0 && ::fstat(fd, &st) == 0 && (uint64_t)st.st_size >= need) {
      const size_t page = (size_t)::sysconf(_SC_PAGESIZE);
      const size_t len = ((size_t)st.st_size + page - 1) / page * page;
      void* p = ::mmap(nullptr, len, PROT_READ, MAP_SHARED, fd, 0);
      if (p != MAP_FAILED) {
        map_ = static_cast<uint8_t*>(p);
        map_len_ = len;
        void* d = nullptr;
        if (cudaHostRegister(map_, map_len_, cudaHostRegisterMapped | cudaHostRegisterPortable) == cudaSuccess) {
          registered_ = true;
          if (cudaHostGetDevicePointer(&d, map_, 0) == cudaSuccess) device_map_ = static_cast<const uint8_t*>(d);
        }
        cudaGetLastError();  // a refused registration leaves its error behind
        if (!device_map_) {
          if (registered_) cudaHostUnregister(map_);
          registered_ = false;
          ::munmap(map_, map_len_);
          map_ = nullptr;
        }
      }
    }
  }
  *device_map = device_map_;
  return map_;
}

Tree::~Tree() {
  if (map_) {
    if (registered_) cudaHostUnregister(map_);
    ::munmap(map_, map_len_);
  }
  if (fd >= 0) ::close(fd);
}

// ---- camera (mat.cpp) -------------------------------------------------------------
namespace {
struct M4 {
  float m[16];
};
M4 Mul(const M4& a, const M4& b) {
  M4 r;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      float t = 0;
      for (int k = 0; k < 4; ++k) t += a.m[(i << 2) + k] * b.m[(k << 2) + j];
      r.m[(i << 2) + j] = t;
    }
  return r;
}
M4 Identity() {
  M4 r{};
  r.m[0] = r.m[5] = r.m[10] = r.m[15] = 1;
  return r;
}
const float kDegToRad = 3.1415926535897932384626433832795f / 180.0f;
M4 RotX(float a) {
  float c = (float)std::cos((double)(a * kDegToRad)), s = (float)std::sin((double)(a * kDegToRad));
  M4 r = Identity();
  r.m[5] = c; r.m[6] = -s; r.m[9] = s; r.m[10] = c;
  return r;
}
M4 RotY(float a) {
  float c = (float)std::cos((double)(a * kDegToRad)), s = (float)std::sin((double)(a * kDegToRad));
  M4 r = Identity();
  r.m[0] = c; r.m[2] = s; r.m[8] = -s; r.m[10] = c;
  return r;
}
M4 RotZ(float a) {
  float c = (float)std::cos((double)(a * kDegToRad)), s = (float)std::sin((double)(a * kDegToRad));
  M4 r = Identity();
  r.m[0] = c; r.m[1] = -s; r.m[4] = s; r.m[5] = c;
  return r;
}
M4 Transposed(const M4& a) {
  M4 r;
  for (int i = 0; i < 4; ++i) {
    r.m[i] = a.m[(i << 2) + 0];
    r.m[i + 4] = a.m[(i << 2) + 1];
    r.m[i + 8] = a.m[(i << 2) + 2];
    r.m[i + 12] = a.m[(i << 2) + 3];
  }
  return r;
}
// fmat4::Inverse (rayt/util/mat.cpp:20-107): the cofactor method of Intel's
// published SSE 4x4-inverse note, in float with the reference's operation
// order, so the 16 floats match the reference bit for bit.  With s the
// transpose of the matrix, each cofactor is (three pair-products x s) minus
// (three pair-products x s), each sum taken left to right; the pair products
// of the first eight cofactors come from s's rows 2-3, those of the last eight
// from rows 0-1.
struct Cofactor {
  uint8_t plus[3][2], minus[3][2];  // {pair product, s index}
};
constexpr uint8_t kPairsLo[12][2] = {{10, 15}, {11, 14}, {9, 15}, {11, 13}, {9, 14}, {10, 13},
                                     {8, 15},  {11, 12}, {8, 14}, {10, 12}, {8, 13}, {9, 12}};
constexpr uint8_t kPairsHi[12][2] = {{2, 7}, {3, 6}, {1, 7}, {3, 5}, {1, 6}, {2, 5},
                                     {0, 7}, {3, 4}, {0, 6}, {2, 4}, {0, 5}, {1, 4}};
constexpr Cofactor kCofactors[16] = {
    {{{0, 5}, {3, 6}, {4, 7}}, {{1, 5}, {2, 6}, {5, 7}}},
    {{{1, 4}, {6, 6}, {9, 7}}, {{0, 4}, {7, 6}, {8, 7}}},
    {{{2, 4}, {7, 5}, {10, 7}}, {{3, 4}, {6, 5}, {11, 7}}},
    {{{5, 4}, {8, 5}, {11, 6}}, {{4, 4}, {9, 5}, {10, 6}}},
    {{{1, 1}, {2, 2}, {5, 3}}, {{0, 1}, {3, 2}, {4, 3}}},
    {{{0, 0}, {7, 2}, {8, 3}}, {{1, 0}, {6, 2}, {9, 3}}},
    {{{3, 0}, {6, 1}, {11, 3}}, {{2, 0}, {7, 1}, {10, 3}}},
    {{{4, 0}, {9, 1}, {10, 2}}, {{5, 0}, {8, 1}, {11, 2}}},
    {{{0, 13}, {3, 14}, {4, 15}}, {{1, 13}, {2, 14}, {5, 15}}},
    {{{1, 12}, {6, 14}, {9, 15}}, {{0, 12}, {7, 14}, {8, 15}}},
    {{{2, 12}, {7, 13}, {10, 15}}, {{3, 12}, {6, 13}, {11, 15}}},
    {{{5, 12}, {8, 13}, {11, 14}}, {{4, 12}, {9, 13}, {10, 14}}},
    {{{2, 10}, {5, 11}, {1, 9}}, {{4, 11}, {0, 9}, {3, 10}}},
    {{{8, 11}, {0, 8}, {7, 10}}, {{6, 10}, {9, 11}, {1, 8}}},
    {{{6, 9}, {11, 11}, {3, 8}}, {{10, 11}, {2, 8}, {7, 9}}},
    {{{10, 10}, {4, 8}, {9, 9}}, {{8, 9}, {11, 10}, {5, 8}}},
};
M4 Inverse(const M4& a) {
  const M4 s = Transposed(a);
  float lo[12], hi[12];
  for (int k = 0; k < 12; ++k) {
    lo[k] = s.m[kPairsLo[k][0]] * s.m[kPairsLo[k][1]];
    hi[k] = s.m[kPairsHi[k][0]] * s.m[kPairsHi[k][1]];
  }
  M4 r;
  for (int j = 0; j < 16; ++j) {
    const float* pr = j < 8 ? lo : hi;
    const Cofactor& c = kCofactors[j];
    float v = pr[c.plus[0][0]] * s.m[c.plus[0][1]] + pr[c.plus[1][0]] * s.m[c.plus[1][1]] +
              pr[c.plus[2][0]] * s.m[c.plus[2][1]];
    v -= pr[c.minus[0][0]] * s.m[c.minus[0][1]] + pr[c.minus[1][0]] * s.m[c.minus[1][1]] +
         pr[c.minus[2][0]] * s.m[c.minus[2][1]];
    r.m[j] = v;
  }
  float det = s.m[0] * r.m[0] + s.m[1] * r.m[1] + s.m[2] * r.m[2] + s.m[3] * r.m[3];
  det = 1.0f / det;
  for (int j = 0; j < 16; ++j) r.m[j] *= det;
  return r;
}
}  // namespace

// Builder threads: RAYT_BUILD_THREADS if set, else every hardware thread.  The
// file is the same for any thread count.
int build_threads() {
  const char* e = std::getenv("RAYT_BUILD_THREADS");
  if (e && std::atoi(e) > 0) return std::atoi(e);
  const unsigned hw = std::thread::hardware_concurrency();
  return hw ? (int)hw : 1;
}

}  // namespace rayt

using rayt::fail;

extern "C" {

int rayt_tree_open(const char* path, rayt_tree** out) {
  if (!path || !out) return fail(RAYT_E_ARG, "rayt_tree_open: null argument");
  std::unique_ptr<rayt::Tree> t(new rayt::Tree());
  int rc = t->Open(path);
  if (rc != RAYT_OK) return rc;
  *out = reinterpret_cast<rayt_tree*>(t.release());
  return RAYT_OK;
}

void rayt_tree_close(rayt_tree* tree) { rayt::Tree::Release(reinterpret_cast<rayt::Tree*>(tree)); }

int rayt_tree_info_get(const rayt_tree* tree, rayt_tree_info* out) {
  if (!tree || !out) return fail(RAYT_E_ARG, "rayt_tree_info_get: null argument");
  *out = reinterpret_cast<const rayt::Tree*>(tree)->info;
  return RAYT_OK;
}

int rayt_tree_channel(const rayt_tree* tree, int index, int* bytes_in_node, char* name, int cap) {
  if (!tree) return fail(RAYT_E_ARG, "rayt_tree_channel: null tree");
  const rayt::Tree* t = reinterpret_cast<const rayt::Tree*>(tree);
  if (index < 0 || index >= (int)t->chan_names.size()) return fail(RAYT_E_ARG, "channel index out of range");
  if (bytes_in_node) *bytes_in_node = t->chan_bytes[index];
  if (name && cap > 0) {
    std::strncpy(name, t->chan_names[index].c_str(), (size_t)cap - 1);
    name[cap - 1] = 0;
  }
  return RAYT_OK;
}

int rayt_tree_load_block(rayt_tree* tree, uint32_t index, rayt_block_header* header, void* content,
                         size_t content_bytes) {
  if (!tree) return fail(RAYT_E_ARG, "rayt_tree_load_block: null tree");
  const rayt::Tree* t = reinterpret_cast<const rayt::Tree*>(tree);
  if (content && content_bytes < t->info.content_bytes) return fail(RAYT_E_ARG, "content buffer too small");
  return t->LoadBlock(index, header, content);
}

int rayt_build_sphere_test(const char* path, float cx, float cy, float cz, float radius, int depth,
                           int nodes_in_block, uint32_t* blocks_out) {
  if (!path || depth < 0 || depth > 20) return fail(RAYT_E_ARG, "rayt_build_sphere_test: bad arguments");
  try {
    rayt_scene::SphereTestSource src(cx, cy, cz, radius, depth);
    std::vector<rayt_build::Channel> ch{{4, "node index"}, {1, "node index % 211"}};
    rayt_build::BlockBuilder<rayt_scene::SphereTestSource> b(path, nodes_in_block, ch, &src, rayt::build_threads());
    uint32_t n = b.Build();
    if (blocks_out) *blocks_out = n;
  } catch (const std::exception& e) {
    return fail(RAYT_E_IO, e.what());
  }
  return RAYT_OK;
}

int rayt_build_terrain(const char* path, const rayt_terrain_params* prm, int nodes_in_block, uint32_t* blocks_out,
                       uint64_t* nodes_out) {
  if (!path || !prm || prm->depth < 1 || prm->depth > 15 || prm->octaves < 1 || prm->base_cells < 1 ||
      prm->spheres < 0 || prm->min_radius < 1 || prm->max_radius < prm->min_radius)
    return fail(RAYT_E_ARG, "rayt_build_terrain: bad arguments");
  try {
    rayt_scene::TerrainParams p;
    p.depth = prm->depth;
    p.seed = prm->seed;
    p.base_cells = prm->base_cells;
    p.octaves = prm->octaves;
    p.spheres = prm->spheres;
    p.sphere_seed = prm->sphere_seed;
    p.min_radius = prm->min_radius;
    p.max_radius = prm->max_radius;
    rayt_scene::TerrainSource src(p);
    std::vector<rayt_build::Channel> ch{{4, "normals"}, {4, "colors"}};
    rayt_build::BlockBuilder<rayt_scene::TerrainSource> b(path, nodes_in_block, ch, &src, rayt::build_threads());
    uint32_t n = b.Build();
    if (blocks_out) *blocks_out = n;
    if (nodes_out) *nodes_out = b.nodes();
  } catch (const std::exception& e) {
    return fail(RAYT_E_IO, e.what());
  }
  return RAYT_OK;
}

int rayt_camera_view_proj_inv(const rayt_camera* c, float out[16]) {
  if (!c || !out) return fail(RAYT_E_ARG, "rayt_camera_view_proj_inv: null argument");
  using namespace rayt;
  // PerspectiveProjectionMatrix(fov, aspect, near, 0) (mat.cpp:180-194)
  M4 proj{};
  const float f = (float)(1.0f / std::tan((double)(c->field_of_view * (kDegToRad / 2))));
  proj.m[0] = f;
  proj.m[5] = f * c->aspect_ratio;
  proj.m[14] = -1;
  proj.m[10] = -1;
  proj.m[11] = -2 * c->near_clip_plane;
  // RotationMatrix(-yaw, pitch, -roll) = RotY * RotX * RotZ (mat.cpp:176-178)
  M4 rot = Mul(Mul(RotY(-c->yaw), RotX(c->pitch)), RotZ(-c->roll));
  M4 tr = Identity();
  tr.m[3] = -c->position[0];
  tr.m[7] = -c->position[1];
  tr.m[11] = -c->position[2];
  M4 vp = Mul(Mul(proj, Transposed(rot)), tr);
  M4 inv = Inverse(vp);
  std::memcpy(out, inv.m, sizeof(inv.m));
  return RAYT_OK;
}

}  // extern "C"
