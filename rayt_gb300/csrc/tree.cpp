// Block-file access, scene building and camera math (host C++).
//
//  * rayt_tree_*: the reference's StoredOctreeLoader
//    (rayt/CPU data/stored-octree-loader.cpp:9-98) over pread(2); the header
//    layout is rayt/doc/storage data format.txt:1-33.
//  * rayt_build_*: BuildOctree (rayt/CPU data/stored-octree-builder.h:40-41)
//    through block_builder.h with the sources of scene_source.h.
//  * rayt_camera_view_proj_inv: Camera::ViewProjectionMatrix().Inverse()
//    (rayt/scene/camera.cpp:23-28, rayt/util/mat.cpp:108-194): the same
//    view-projection (horizontal FOV, infinite far plane, y up) inverted in
//    double precision; see Inverse() below for why it is not bit-identical.
#include <algorithm>
#include <cerrno>
#include <cstdlib>
#include <thread>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>
#include <fcntl.h>
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

Tree::~Tree() {
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
// Inverse by Gauss-Jordan elimination with partial pivoting, in double
// precision, rounded to float at the end.  (The reference inverts in float by
// cofactors; the two can differ in the last bits, which is why parity runs
// pass the reference's own 16 floats to rayt_render_frame.)
M4 Inverse(const M4& a) {
  double w[4][8];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 8; ++j) w[i][j] = j < 4 ? (double)a.m[i * 4 + j] : (j - 4 == i ? 1.0 : 0.0);
  for (int col = 0; col < 4; ++col) {
    int piv = col;
    for (int r = col + 1; r < 4; ++r)
      if (std::fabs(w[r][col]) > std::fabs(w[piv][col])) piv = r;
    if (piv != col)
      for (int j = 0; j < 8; ++j) std::swap(w[piv][j], w[col][j]);
    const double inv = 1.0 / w[col][col];
    for (int j = 0; j < 8; ++j) w[col][j] *= inv;
    for (int r = 0; r < 4; ++r) {
      if (r == col) continue;
      const double f = w[r][col];
      if (f == 0.0) continue;
      for (int j = 0; j < 8; ++j) w[r][j] -= f * w[col][j];
    }
  }
  M4 r;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) r.m[i * 4 + j] = (float)w[i][4 + j];
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

void rayt_tree_close(rayt_tree* tree) { delete reinterpret_cast<rayt::Tree*>(tree); }

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
