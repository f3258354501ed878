// Seeded scene generators that feed the block-file builder.
//
// Each source has the three calls of the reference's builder data-source
// interface (rayt/CPU data/stored-octree-builder.h:21-35): GetRoot once,
// GetChildren once per node (child slot 0-7: bit 0 = +x, bit 1 = +y, bit 2 = +z
// half of the cube), then GetNodeData once per node with its children.
//
//  * SphereTestSource - the reference's analytic sphere-shell known-answer tree
//    (rayt/scene sources/stored-octree-test.cpp:235-313): channels
//    "node index" (uint32 path id, root 1, child id*8+slot) and
//    "node index % 211" (1 byte).
//  * TerrainSource - the benchmark scenes: an fBm value-noise heightfield
//    (6 octaves, lacunarity 2, gain 0.5) with height along world y (the
//    reference's camera has y up, rayt/scene/camera.h:7), optionally unioned
//    with seeded voxelised sphere shells.  Channels "normals" (char4, x127, w=0)
//    and "colors" (uchar4, A=255) with internal nodes averaging their children,
//    the conventions of rayt/scene sources/import-obj-scene.cpp:516-526,611-627.
//
// Everything is integer or IEEE float/double arithmetic with no fused
// multiply-add (built with -ffp-contract=off), so a scene is bit-identical on
// every host.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <utility>
#include <vector>

namespace rayt_scene {

// ---------------------------------------------------------------------------
// Reference sphere known-answer source.
struct SphereTestNode {
  int depth;
  float minp[3], maxp[3];
  int32_t node_id;
};

class SphereTestSource {
 public:
  SphereTestSource(float cx, float cy, float cz, float radius, int max_depth)
      : max_depth_(max_depth) {
    c_[0] = cx; c_[1] = cy; c_[2] = cz;
    r2_ = radius * radius;
  }
  static int channel_bytes() { return 5; }

  SphereTestNode GetRoot() { return SphereTestNode{0, {0, 0, 0}, {1, 1, 1}, 1}; }

  // Children of `node` in slot order into slots[]/kids[] (room for 8).
  int ChildrenInto(const SphereTestNode& node, int* slots, SphereTestNode* kids) const {
    if (node.depth == max_depth_) return 0;
    int k = 0;
    for (int ch = 0; ch < 8; ++ch) {
      SphereTestNode n;
      for (int a = 0; a < 3; ++a) {
        float mid = (node.minp[a] + node.maxp[a]) * 0.5f;
        n.minp[a] = (ch >> a) & 1 ? mid : node.minp[a];
        n.maxp[a] = (ch >> a) & 1 ? node.maxp[a] : mid;
      }
      if (!Straddles(n.minp, n.maxp)) continue;
      n.depth = node.depth + 1;
      n.node_id = (int32_t)((uint32_t)node.node_id * 8u + (uint32_t)ch);
      slots[k] = ch;
      kids[k++] = n;
    }
    return k;
  }
  void NodeDataInto(SphereTestNode& node, const SphereTestNode* const*, int, void* out) const {
    unsigned char* d = static_cast<unsigned char*>(out);
    uint32_t id = (uint32_t)node.node_id;
    std::memcpy(d, &id, 4);
    d[4] = (unsigned char)(signed char)(node.node_id % 211);
  }

  std::vector<std::pair<int, SphereTestNode>> GetChildren(SphereTestNode& node) {
    int slots[8];
    SphereTestNode kids[8];
    const int k = ChildrenInto(node, slots, kids);
    std::vector<std::pair<int, SphereTestNode>> res;
    for (int i = 0; i < k; ++i) res.push_back(std::make_pair(slots[i], kids[i]));
    return res;
  }
  void GetNodeData(SphereTestNode& node, const std::vector<std::pair<int, SphereTestNode*>>&, void* out) {
    NodeDataInto(node, nullptr, 0, out);
  }

 private:
  float c_[3];
  float r2_;
  int max_depth_;

  float Dist2(float x, float y, float z) const {
    float dx = x - c_[0], dy = y - c_[1], dz = z - c_[2];
    float s = dx * dx;
    s = s + dy * dy;
    s = s + dz * dz;
    return s;
  }
  // A child cube is kept when it contains the centre strictly inside, or when
  // its corners are neither all inside nor all outside the sphere.
  bool Straddles(const float* mn, const float* mx) const {
    bool inside_box = c_[0] > mn[0] && c_[1] > mn[1] && c_[2] > mn[2] &&
                      c_[0] < mx[0] && c_[1] < mx[1] && c_[2] < mx[2];
    if (inside_box) return true;
    bool was_in = false, was_out = false;
    for (int i = 0; i < 8; ++i) {
      float x = i & 1 ? mx[0] : mn[0];
      float y = i & 2 ? mx[1] : mn[1];
      float z = i & 4 ? mx[2] : mn[2];
      if (Dist2(x, y, z) < r2_) {
        was_in = true;
        if (was_out) break;
      } else {
        was_out = true;
        if (was_in) break;
      }
    }
    return was_in && was_out;
  }
};

// ---------------------------------------------------------------------------
// Heightfield (+ spheres) benchmark source.

struct TerrainParams {
  int depth = 10;          // the grid is 2^depth voxels per axis
  uint32_t seed = 1;       // heightfield seed
  int base_cells = 4;      // value-noise lattice cells across the scene at octave 0
  int octaves = 6;
  double lacunarity = 2.0;
  double gain = 0.5;
  double base_height = 0.1;   // heights span [base, base + amplitude) of the cube
  double amplitude = 0.4;
  int spheres = 0;         // number of sphere shells (0 = heightfield only)
  uint32_t sphere_seed = 2;
  int min_radius = 8;      // sphere radii, in voxels, log-uniform in [min, max]
  int max_radius = 256;
};

struct TerrainNode {
  int depth;
  int x, y, z;   // integer cube coordinates at this depth
  float normal[3];
  float color[3];
};

class TerrainSource {
 public:
  explicit TerrainSource(const TerrainParams& p) : p_(p) {
    n_ = 1 << p.depth;
    BuildHeights();
    BuildSpheres();
  }
  static int channel_bytes() { return 8; }
  int grid() const { return n_; }
  int sphere_count() const { return (int)spheres_.size(); }

  TerrainNode GetRoot() {
    TerrainNode r{};
    return r;
  }

  // Children of `node` in slot order into slots[]/kids[] (room for 8).
  int ChildrenInto(const TerrainNode& node, int* slots, TerrainNode* kids) const {
    if (node.depth == p_.depth) return 0;
    int k = 0;
    for (int ch = 0; ch < 8; ++ch) {
      TerrainNode c{};
      c.depth = node.depth + 1;
      c.x = node.x * 2 + (ch & 1);
      c.y = node.y * 2 + ((ch >> 1) & 1);
      c.z = node.z * 2 + ((ch >> 2) & 1);
      if (!Occupied(c)) continue;
      slots[k] = ch;
      kids[k++] = c;
    }
    return k;
  }

  std::vector<std::pair<int, TerrainNode>> GetChildren(TerrainNode& node) {
    int slots[8];
    TerrainNode kids[8];
    const int k = ChildrenInto(node, slots, kids);
    std::vector<std::pair<int, TerrainNode>> res;
    for (int i = 0; i < k; ++i) res.push_back(std::make_pair(slots[i], kids[i]));
    return res;
  }
  void GetNodeData(TerrainNode& node, const std::vector<std::pair<int, TerrainNode*>>& children, void* out) {
    const TerrainNode* kids[8];
    for (size_t i = 0; i < children.size() && i < 8; ++i) kids[i] = children[i].second;
    NodeDataInto(node, kids, (int)children.size(), out);
  }

  // Node data from the children (in slot order); kids may be null when n == 0.
  void NodeDataInto(TerrainNode& node, const TerrainNode* const* kids, int n, void* out) const {
    float nx = 0, ny = 0, nz = 0;
    if (n == 0) {
      LeafData(node);
    } else {
      float cr = 0, cg = 0, cb = 0;
      for (int i = 0; i < n; ++i) {
        const TerrainNode* c = kids[i];
        nx = nx + c->normal[0]; ny = ny + c->normal[1]; nz = nz + c->normal[2];
        cr = cr + c->color[0]; cg = cg + c->color[1]; cb = cb + c->color[2];
      }
      float inv = 1.0f / (float)n;
      node.color[0] = cr * inv; node.color[1] = cg * inv; node.color[2] = cb * inv;
      node.normal[0] = nx; node.normal[1] = ny; node.normal[2] = nz;
    }
    // Normalise; a degenerate sum becomes +z (import-obj-scene.cpp:630-633).
    nx = node.normal[0]; ny = node.normal[1]; nz = node.normal[2];
    float l2 = nx * nx;
    l2 = l2 + ny * ny;
    l2 = l2 + nz * nz;
    if (l2 < 1e-5f) {
      node.normal[0] = 0; node.normal[1] = 0; node.normal[2] = 1;
    } else {
      float inv = 1.0f / std::sqrt(l2);
      node.normal[0] = nx * inv; node.normal[1] = ny * inv; node.normal[2] = nz * inv;
    }
    unsigned char* d = static_cast<unsigned char*>(out);
    d[0] = (unsigned char)(signed char)(node.normal[0] * 127);
    d[1] = (unsigned char)(signed char)(node.normal[1] * 127);
    d[2] = (unsigned char)(signed char)(node.normal[2] * 127);
    d[3] = 0;
    for (int k = 0; k < 3; ++k) {
      float v = node.color[k] * 255;
      v = v < 0.0f ? 0.0f : (v > 255.0f ? 255.0f : v);
      d[4 + k] = (unsigned char)v;
    }
    d[7] = 255;
  }

  // Column surface height (voxel index of the top voxel) - exposed for tests.
  int Height(int x, int z) const { return hi_[(size_t)z * n_ + x]; }

 private:
  struct Sphere {
    int64_t cx2, cy2, cz2;   // doubled centre coordinates (centres sit at voxel centres)
    int64_t r2x4;            // (2r)^2
    int r;
    float color[3];
  };

  TerrainParams p_;
  int n_;
  std::vector<uint16_t> hi_, lo_;
  // mip pyramids over square footprints: level L holds min(lo)/max(hi) over
  // 2^L x 2^L columns
  std::vector<std::vector<uint16_t>> minlo_, maxhi_;
  std::vector<Sphere> spheres_;
  int cell_shift_ = 0;     // spatial hash: cells of 2^cell_shift voxels per axis
  int cells_ = 1;
  std::vector<std::vector<int>> cell_spheres_;

  static uint32_t Mix(uint32_t h) {
    h ^= h >> 16; h *= 0x7feb352du;
    h ^= h >> 15; h *= 0x846ca68bu;
    h ^= h >> 16;
    return h;
  }
  static double Lattice(int ix, int iz, uint32_t seed) {
    uint32_t h = Mix((uint32_t)ix * 0x9E3779B1u ^ Mix((uint32_t)iz * 0x85EBCA77u ^ Mix(seed)));
    return (double)(h >> 8) * (1.0 / 16777216.0);
  }
  static double Smooth(double t) { return t * t * (3.0 - 2.0 * t); }
  static double ValueNoise(double px, double pz, uint32_t seed) {
    double fx = std::floor(px), fz = std::floor(pz);
    int ix = (int)fx, iz = (int)fz;
    double tx = Smooth(px - fx), tz = Smooth(pz - fz);
    double a = Lattice(ix, iz, seed), b = Lattice(ix + 1, iz, seed);
    double c = Lattice(ix, iz + 1, seed), d = Lattice(ix + 1, iz + 1, seed);
    double ab = a + (b - a) * tx;
    double cd = c + (d - c) * tx;
    return ab + (cd - ab) * tz;
  }
  double Fbm(double u, double v) const {
    double sum = 0, norm = 0, amp = 1, freq = p_.base_cells;
    for (int o = 0; o < p_.octaves; ++o) {
      sum = sum + amp * ValueNoise(u * freq, v * freq, p_.seed * 131u + (uint32_t)o);
      norm = norm + amp;
      amp = amp * p_.gain;
      freq = freq * p_.lacunarity;
    }
    return sum / norm;
  }

  void BuildHeights() {
    const size_t cols = (size_t)n_ * n_;
    hi_.resize(cols);
    lo_.resize(cols);
    for (int z = 0; z < n_; ++z) {
      for (int x = 0; x < n_; ++x) {
        double h = p_.base_height + p_.amplitude * Fbm((x + 0.5) / n_, (z + 0.5) / n_);
        int v = (int)std::floor(h * n_);
        if (v < 0) v = 0;
        if (v > n_ - 1) v = n_ - 1;
        hi_[(size_t)z * n_ + x] = (uint16_t)v;
      }
    }
    // A column is filled from the lowest 4-neighbour top up to its own top, so
    // the surface has no holes.
    for (int z = 0; z < n_; ++z) {
      for (int x = 0; x < n_; ++x) {
        int h = hi_[(size_t)z * n_ + x], l = h;
        if (x > 0) l = std::min(l, (int)hi_[(size_t)z * n_ + x - 1]);
        if (x + 1 < n_) l = std::min(l, (int)hi_[(size_t)z * n_ + x + 1]);
        if (z > 0) l = std::min(l, (int)hi_[(size_t)(z - 1) * n_ + x]);
        if (z + 1 < n_) l = std::min(l, (int)hi_[(size_t)(z + 1) * n_ + x]);
        lo_[(size_t)z * n_ + x] = (uint16_t)l;
      }
    }
    minlo_.assign(1, lo_);
    maxhi_.assign(1, hi_);
    for (int lvl = 1, w = n_ / 2; w >= 1; ++lvl, w /= 2) {
      const auto& pl = minlo_[lvl - 1];
      const auto& ph = maxhi_[lvl - 1];
      std::vector<uint16_t> ml((size_t)w * w), mh((size_t)w * w);
      for (int z = 0; z < w; ++z)
        for (int x = 0; x < w; ++x) {
          size_t i00 = (size_t)(2 * z) * (2 * w) + 2 * x, i01 = i00 + 1;
          size_t i10 = i00 + 2 * w, i11 = i10 + 1;
          ml[(size_t)z * w + x] = std::min(std::min(pl[i00], pl[i01]), std::min(pl[i10], pl[i11]));
          mh[(size_t)z * w + x] = std::max(std::max(ph[i00], ph[i01]), std::max(ph[i10], ph[i11]));
        }
      minlo_.push_back(std::move(ml));
      maxhi_.push_back(std::move(mh));
    }
  }

  void BuildSpheres() {
    if (p_.spheres <= 0) return;
    uint32_t s = Mix(p_.sphere_seed * 0x632BE5ABu + 1);
    auto next = [&s]() { s = Mix(s + 0x9E3779B9u); return s; };
    auto unit = [&next]() { return (double)(next() >> 8) * (1.0 / 16777216.0); };
    const double lr = std::log((double)p_.max_radius / p_.min_radius);
    for (int i = 0; i < p_.spheres; ++i) {
      Sphere sp;
      int r = (int)std::floor(p_.min_radius * std::exp(lr * unit()));
      if (r < p_.min_radius) r = p_.min_radius;
      if (r > p_.max_radius) r = p_.max_radius;
      int x = (int)(unit() * n_), z = (int)(unit() * n_);
      if (x >= n_) x = n_ - 1;
      if (z >= n_) z = n_ - 1;
      // rest the sphere on (or float it just above) the terrain under its centre
      int y = Height(x, z) + (int)(r * (0.3 + 1.2 * unit()));
      if (y > n_ - 1) y = n_ - 1;
      sp.cx2 = 2 * (int64_t)x + 1;
      sp.cy2 = 2 * (int64_t)y + 1;
      sp.cz2 = 2 * (int64_t)z + 1;
      sp.r = r;
      sp.r2x4 = 4 * (int64_t)r * r;
      sp.color[0] = (float)(0.35 + 0.6 * unit());
      sp.color[1] = (float)(0.2 + 0.6 * unit());
      sp.color[2] = (float)(0.2 + 0.75 * unit());
      spheres_.push_back(sp);
    }
    // coarse spatial hash of sphere bounding boxes (16 cells per axis at most)
    cell_shift_ = p_.depth > 4 ? p_.depth - 4 : 0;
    cells_ = n_ >> cell_shift_;
    cell_spheres_.assign((size_t)cells_ * cells_ * cells_, std::vector<int>());
    for (int i = 0; i < (int)spheres_.size(); ++i) {
      const Sphere& sp = spheres_[i];
      int lo[3], hi[3];
      int64_t c2[3] = {sp.cx2, sp.cy2, sp.cz2};
      for (int a = 0; a < 3; ++a) {
        int64_t mn = (c2[a] - 2 * sp.r) / 2 - 1, mx = (c2[a] + 2 * sp.r) / 2 + 1;
        if (mn < 0) mn = 0;
        if (mx > n_ - 1) mx = n_ - 1;
        lo[a] = (int)(mn >> cell_shift_);
        hi[a] = (int)(mx >> cell_shift_);
      }
      for (int cz = lo[2]; cz <= hi[2]; ++cz)
        for (int cy = lo[1]; cy <= hi[1]; ++cy)
          for (int cx = lo[0]; cx <= hi[0]; ++cx)
            cell_spheres_[((size_t)cz * cells_ + cy) * cells_ + cx].push_back(i);
    }
  }

  // Does the voxel range of node c intersect the heightfield surface?
  bool TerrainHit(int depth, int x, int y, int z) const {
    int lvl = p_.depth - depth;
    int y0 = y << lvl, y1 = ((y + 1) << lvl) - 1;
    size_t w = (size_t)(n_ >> lvl);
    int mlo = minlo_[lvl][(size_t)z * w + x];
    int mhi = maxhi_[lvl][(size_t)z * w + x];
    return mlo <= y1 && mhi >= y0;
  }

  // Does the closed cube (in voxel units) straddle sphere sp?  Exact: the
  // lattice points of the cube hold some point strictly inside and some point
  // on or outside the sphere.
  static bool SphereHit(const Sphere& sp, int64_t x0, int64_t y0, int64_t z0, int64_t size) {
    int64_t lo[3] = {2 * x0, 2 * y0, 2 * z0};
    int64_t c2[3] = {sp.cx2, sp.cy2, sp.cz2};
    int64_t dmin = 0, dmax = 0;
    for (int a = 0; a < 3; ++a) {
      int64_t hi = lo[a] + 2 * size;
      // nearest lattice point (even doubled coordinate) to the centre, in range
      int64_t n = c2[a] - 1;  // centre is odd: both neighbours are equally close
      if (n < lo[a]) n = lo[a];
      if (n > hi) n = hi;
      int64_t dn = n - c2[a];
      dmin += dn * dn;
      int64_t d0 = lo[a] - c2[a], d1 = hi - c2[a];
      dmax += std::max(d0 * d0, d1 * d1);
    }
    return dmin < sp.r2x4 && dmax >= sp.r2x4;
  }

  const std::vector<int>* CellList(int depth, int x, int y, int z) const {
    int lvl = p_.depth - depth;
    if (lvl > cell_shift_) return nullptr;  // bigger than a cell: test all spheres
    int sh = cell_shift_ - lvl;
    return &cell_spheres_[((size_t)(z >> sh) * cells_ + (y >> sh)) * cells_ + (x >> sh)];
  }

  int FirstSphere(int depth, int x, int y, int z) const {
    if (spheres_.empty()) return -1;
    int lvl = p_.depth - depth;
    int64_t size = (int64_t)1 << lvl;
    const std::vector<int>* list = CellList(depth, x, y, z);
    if (list) {
      for (int i : *list)
        if (SphereHit(spheres_[i], (int64_t)x << lvl, (int64_t)y << lvl, (int64_t)z << lvl, size))
          return i;
      return -1;
    }
    for (int i = 0; i < (int)spheres_.size(); ++i)
      if (SphereHit(spheres_[i], (int64_t)x << lvl, (int64_t)y << lvl, (int64_t)z << lvl, size))
        return i;
    return -1;
  }

  bool Occupied(const TerrainNode& c) const {
    return TerrainHit(c.depth, c.x, c.y, c.z) || FirstSphere(c.depth, c.x, c.y, c.z) >= 0;
  }

  void LeafData(TerrainNode& node) const {
    int s = FirstSphere(node.depth, node.x, node.y, node.z);
    if (s >= 0) {
      const Sphere& sp = spheres_[s];
      float dx = (float)(2 * node.x + 1 - sp.cx2);
      float dy = (float)(2 * node.y + 1 - sp.cy2);
      float dz = (float)(2 * node.z + 1 - sp.cz2);
      node.normal[0] = dx; node.normal[1] = dy; node.normal[2] = dz;
      for (int k = 0; k < 3; ++k) node.color[k] = sp.color[k];
      return;
    }
    int x = node.x, z = node.z;
    int xm = x > 0 ? x - 1 : x, xp = x + 1 < n_ ? x + 1 : x;
    int zm = z > 0 ? z - 1 : z, zp = z + 1 < n_ ? z + 1 : z;
    float gx = (float)(Height(xp, z) - Height(xm, z)) / (float)(xp - xm);
    float gz = (float)(Height(x, zp) - Height(x, zm)) / (float)(zp - zm);
    node.normal[0] = -gx; node.normal[1] = 1.0f; node.normal[2] = -gz;
    // height ramp over the heightfield's range: green valleys, brown slopes,
    // white peaks
    float t = ((float)node.y / (float)n_ - (float)p_.base_height) / (float)p_.amplitude;
    static const float ramp[4][4] = {{0.00f, 0.20f, 0.45f, 0.15f},
                                     {0.40f, 0.30f, 0.55f, 0.20f},
                                     {0.62f, 0.50f, 0.40f, 0.30f},
                                     {0.78f, 0.95f, 0.95f, 0.97f}};
    int k = 0;
    while (k < 2 && t > ramp[k + 1][0]) ++k;
    float u = (t - ramp[k][0]) / (ramp[k + 1][0] - ramp[k][0]);
    if (u < 0) u = 0;
    if (u > 1) u = 1;
    for (int c = 0; c < 3; ++c)
      node.color[c] = ramp[k][c + 1] + (ramp[k + 1][c + 1] - ramp[k][c + 1]) * u;
  }
};

}  // namespace rayt_scene
