// Tracing passes, the hot path: traversal of the rays of one or many views
// against the block cache, plus the reference's debug depth view.
//
// Per ray this fuses what the reference runs as separate full-frame kernels
// with a 48-byte TracingState round trip through memory:
//   ray setup       InitTracingFrame   (rayt/GPU_renderer/kernels/init_tracing_frame.cl:11-45)
//   traversal       CastRay            (rayt/GPU_renderer/kernels/raycast.cl:33-256)
//   pass logic      RaytracingPass     (rayt/GPU_renderer/kernels/raytracing_pass.cl:4-61)
//   shading         ProcessHit         (rayt/GPU_renderer/kernels/shading.cl:4-33)
//   final colour    FinishTracingFrame (rayt/GPU_renderer/kernels/finish_tracing_frame.cl:3-24)
//   block words     NodeToBlockKernel  (rayt/GPU_renderer/kernels/feedback_compression.cl:4-13)
//
// Kernels:
//   trace_kernel             first pass, one thread per ray over the 32-pixel
//                            tiles of all views of the launch (4x8 by default;
//                            lane i of a tile = pixel (i % tile_w, i / tile_w))
//   trace_queue_kernel       later passes: persistent warps take 32 rays at a
//                            time of the compacted list of rays that faulted
//   trace_persistent_kernel  first pass with work stealing: warps stop their
//                            rays every step_budget iterations and refill idle
//                            lanes (an autotuner candidate; slower on the
//                            measured workloads, see the design notes)
//   finish_kernel            FinishTracingFrame for rays still faulted
//   depth_view_kernel        raytracer.cl, the reference's debug depth view
//   unique_from_bits_kernel  the feedback bitmaps as the reference's sorted
//                            unique array
// A ray that ends (hit, miss, iteration limit) writes its final RGBA8 pixel;
// a ray that faults on a missing block is appended with its state (advanced
// origin, direction, parent node, pixel) to the next pass's list.  Feedback
// goes into two bitmaps (fault blocks; hit cache blocks with the duplicate
// flag).
//
// FP32 arithmetic follows the reference's operation order exactly; the file is
// compiled with --fmad=false and IEEE division/sqrt so no operation is fused or
// approximated, which keeps hit node IDs identical to the CPU oracle.
#include <algorithm>

#include "internal.h"

namespace rayt {
namespace {

constexpr int kSMax = 23;
constexpr float kEps = 0.00000011920928955078125f;  // exp2(-S_MAX)
constexpr int kIterLimit = 300;
constexpr int kBlockThreads = 128;
constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ float dot4(float ax, float ay, float az, float aw, float bx, float by, float bz, float bw) {
  float r = ax * bx;
  r = r + ay * by;
  r = r + az * bz;
  r = r + aw * bw;
  return r;
}

// 0 / d as an IEEE division gives it: a zero with d's sign, NaN for a zero
// or NaN d.
__device__ __forceinline__ float zero_over(float d) {
  return (d == 0.0f || d != d) ? __int_as_float(0x7fffffff) : copysignf(0.0f, d);
}

// mul(float16, float3) of init_tracing_frame.cl:3-9
__device__ __forceinline__ void mul_point(const float* m, float x, float y, float z, float* o) {
  float d = dot4(x, y, z, 1.0f, m[12], m[13], m[14], m[15]);
  o[0] = __fdiv_rn(dot4(x, y, z, 1.0f, m[0], m[1], m[2], m[3]), d);
  o[1] = __fdiv_rn(dot4(x, y, z, 1.0f, m[4], m[5], m[6], m[7]), d);
  o[2] = __fdiv_rn(dot4(x, y, z, 1.0f, m[8], m[9], m[10], m[11]), d);
  o[3] = zero_over(d);
}

// InitTracingFrame for pixel (x, y) of view v.  The view's origin and its
// normalised pixel coordinates come precomputed (the same IEEE operations,
// done once per view and per column/row instead of per ray).
__device__ __forceinline__ void init_ray(const ViewDesc& v, int x, int y, float4& o, float4& d) {
  const float* m = v.m;
  const int W = v.width, H = v.height;
  const float* cx = v.coords;          // (x + 0.5) / W * 2 - 1
  const float* ax = cx + W;            // x / W * 2 - 1, x in [0, W]
  const float* cy = ax + W + 1;        // (y + 0.5) / H * 2 - 1
  const float* ay = cy + H;            // y / H * 2 - 1, y in [0, H]
  const float ox = v.origin[0], oy = v.origin[1], oz = v.origin[2], ow = v.origin[3];
  float q[4];
  mul_point(m, __ldg(cx + x), __ldg(cy + y), 0.0f, q);
  float dx = q[0] - ox, dy = q[1] - oy, dz = q[2] - oz, dw = q[3] - ow;
  float len = __fsqrt_rn(dot4(dx, dy, dz, dw, dx, dy, dz, dw));
  dx = __fdiv_rn(dx, len);
  dy = __fdiv_rn(dy, len);
  dz = __fdiv_rn(dz, len);
  float p1[4], p2[4];
  mul_point(m, __ldg(ax + x), __ldg(ay + y), 0.0f, p1);
  mul_point(m, __ldg(ax + x + 1), __ldg(ay + y + 1), 0.0f, p2);
  float bx = p1[0] - p2[0], by = p1[1] - p2[1], bz = p1[2] - p2[2], bw = p1[3] - p2[3];
  float ex = ox - p1[0], ey = oy - p1[1], ez = oz - p1[2], ew = ow - p1[3];
  float dist12 = __fsqrt_rn(dot4(bx, by, bz, bw, bx, by, bz, bw));
  float dist01 = __fsqrt_rn(dot4(ex, ey, ez, ew, ex, ey, ez, ew));
  float coef = __fdiv_rn(v.lod * dist12, dist01);
  o = make_float4(ox, oy, oz, 0.0f);
  d = make_float4(dx, dy, dz, coef);
}

// CastRay (raycast.cl:33-256) split into cast_begin() (everything before its
// while loop) and cast_run() (the loop, for a bounded number of iterations),
// so a warp can stop its rays at a common point and hand idle lanes new rays.
// The state is the reference's loop state; the outcome is encoded in it
// (see Outcome) instead of extra result registers.
struct Cast {
  float tx_coef, ty_coef, tz_coef, tx_bias, ty_bias, tz_bias;
  float t_min, t_max, h, px, py, pz, scale_exp2, coef, bias;
  uint32_t parent, desc;
  int idx, scale, octant, iter;
};

// How cast_run left a ray.  kHit: node = parent, duplicate flag = bit 9 of
// desc.  kFault: node = parent, t = t_min, block = desc >> 11.
enum Outcome : int { kRunning = 0, kHit = 1, kFault = 2, kMiss = 3, kError = 4 };

__device__ __forceinline__ void cast_begin(Cast& c, uint32_t root, float4 o, float4 d) {
  float px0 = o.x + 1.0f, py0 = o.y + 1.0f, pz0 = o.z + 1.0f;
  float dx = d.x, dy = d.y, dz = d.z;
  c.coef = d.w;
  c.bias = o.w;
  if (fabsf(dx) < kEps) dx = copysignf(kEps, dx);
  if (fabsf(dy) < kEps) dy = copysignf(kEps, dy);
  if (fabsf(dz) < kEps) dz = copysignf(kEps, dz);
  c.tx_coef = __fdiv_rn(1.0f, -fabsf(dx));
  c.ty_coef = __fdiv_rn(1.0f, -fabsf(dy));
  c.tz_coef = __fdiv_rn(1.0f, -fabsf(dz));
  c.tx_bias = c.tx_coef * px0;
  c.ty_bias = c.ty_coef * py0;
  c.tz_bias = c.tz_coef * pz0;
  c.octant = 0;
  if (dx > 0.0f) c.octant ^= 1, c.tx_bias = 3.0f * c.tx_coef - c.tx_bias;
  if (dy > 0.0f) c.octant ^= 2, c.ty_bias = 3.0f * c.ty_coef - c.ty_bias;
  if (dz > 0.0f) c.octant ^= 4, c.tz_bias = 3.0f * c.tz_coef - c.tz_bias;
  c.t_min = fmaxf(fmaxf(2.0f * c.tx_coef - c.tx_bias, 2.0f * c.ty_coef - c.ty_bias), 2.0f * c.tz_coef - c.tz_bias);
  c.t_max = fminf(fminf(c.tx_coef - c.tx_bias, c.ty_coef - c.ty_bias), c.tz_coef - c.tz_bias);
  c.h = c.t_max;
  c.t_min = fmaxf(c.t_min, 0.0f);
  c.parent = root;
  c.desc = 0;
  c.idx = 0;
  c.px = 1.0f;
  c.py = 1.0f;
  c.pz = 1.0f;
  c.scale = kSMax - 1;
  c.scale_exp2 = 0.5f;
  if (1.5f * c.tx_coef - c.tx_bias > c.t_min) c.idx ^= 1, c.px = 1.5f;
  if (1.5f * c.ty_coef - c.ty_bias > c.t_min) c.idx ^= 2, c.py = 1.5f;
  if (1.5f * c.tz_coef - c.tz_bias > c.t_min) c.idx ^= 4, c.pz = 1.5f;
  c.iter = 0;
}

// How a ray ended.  error: iteration limit or a corrupt cache; fault_block
// != -1: the children of `node` are not loaded (t = where the ray stopped);
// node == -1: miss; else a hit on `node` with the duplicate flag `dup`.
struct RayEnd {
  float t;
  int node, fault_block, dup, error;
  int iter;
};

// CastRay as one function over local state, for rays that run to their end
// in one go (the one-thread-per-ray kernel).  The arithmetic and stack rules
// are cast_begin + cast_run's; kept as a single loop with the reference's
// shape because that form compiles to about 5% fewer warp instructions on
// sm_103a than the resumable one.
template <bool kCount>
__device__ __forceinline__ RayEnd cast_ray(const TraceParams& p, float4 o, float4 d, uint32_t& fetches,
                                           uint32_t& far_fetches) {
  RayEnd r;
  r.fault_block = -1;
  r.error = 0;
  r.dup = 0;
  const float px0 = o.x + 1.0f, py0 = o.y + 1.0f, pz0 = o.z + 1.0f;
  float dx = d.x, dy = d.y, dz = d.z;
  const float coef = d.w, bias = o.w;
  // (parent, t_max, the parent's descriptor): a pop needs no reload of the
  // descriptor, which no pass changes (1.7% off the first pass)
  uint4 stack[kSMax + 1];
  if (fabsf(dx) < kEps) dx = copysignf(kEps, dx);
  if (fabsf(dy) < kEps) dy = copysignf(kEps, dy);
  if (fabsf(dz) < kEps) dz = copysignf(kEps, dz);
  const float tx_coef = __fdiv_rn(1.0f, -fabsf(dx));
  const float ty_coef = __fdiv_rn(1.0f, -fabsf(dy));
  const float tz_coef = __fdiv_rn(1.0f, -fabsf(dz));
  float tx_bias = tx_coef * px0, ty_bias = ty_coef * py0, tz_bias = tz_coef * pz0;
  int octant = 0;
  if (dx > 0.0f) octant ^= 1, tx_bias = 3.0f * tx_coef - tx_bias;
  if (dy > 0.0f) octant ^= 2, ty_bias = 3.0f * ty_coef - ty_bias;
  if (dz > 0.0f) octant ^= 4, tz_bias = 3.0f * tz_coef - tz_bias;
  float t_min = fmaxf(fmaxf(2.0f * tx_coef - tx_bias, 2.0f * ty_coef - ty_bias), 2.0f * tz_coef - tz_bias);
  float t_max = fminf(fminf(tx_coef - tx_bias, ty_coef - ty_bias), tz_coef - tz_bias);
  float h = t_max;
  t_min = fmaxf(t_min, 0.0f);
  uint32_t parent = (uint32_t)p.root, desc = 0;
  int idx = 0;
  float px = 1.0f, py = 1.0f, pz = 1.0f;
  int scale = kSMax - 1;
  float scale_exp2 = 0.5f;
  if (1.5f * tx_coef - tx_bias > t_min) idx ^= 1, px = 1.5f;
  if (1.5f * ty_coef - ty_bias > t_min) idx ^= 2, py = 1.5f;
  if (1.5f * tz_coef - tz_bias > t_min) idx ^= 4, pz = 1.5f;
  int iter = 0;
  // Every parent is the root or a child index clamped below node_limit, so
  // only the root needs a check (a root outside the cache ends the ray as an
  // error, like the iteration limit).
  if (p.root >= p.node_limit) {
    r.error = 1;
    r.node = -1;
    r.t = 0.0f;
    r.iter = 0;
    return r;
  }
  // The parent's descriptor is in hand where the reference's loop will need
  // it: fetched here for the root, and taken from the stack entry at each pop
  // (raycast.cl fetches it at the top of the next iteration, which always
  // follows a pop; same value, one fewer test per iteration).  The counting
  // form keeps the reference's fetch points so its counts equal the oracle's.
  if (!kCount) desc = __ldg(p.links + parent);
  while (scale < kSMax) {
    if (++iter > kIterLimit) {
      r.error = 1;
      break;
    }
    if (kCount && desc == 0) {
      desc = __ldg(p.links + parent);
      ++fetches;
    }
    const float tx_corner = px * tx_coef - tx_bias;
    const float ty_corner = py * ty_coef - ty_bias;
    const float tz_corner = pz * tz_coef - tz_bias;
    const float tc_max = fminf(fminf(tx_corner, ty_corner), tz_corner);
    const uint32_t bit = 1u << (idx ^ octant);
    if ((desc & bit) != 0 && t_min <= t_max) {
      if (desc & (1u << 8)) {  // children not loaded: fault
        r.node = (int)parent;
        r.t = t_min;
        r.fault_block = (int)(desc >> 11);
        break;
      }
      // Both indices below are clamped into their buffers instead of tested
      // (a test ends the ray as an error, a branch out of the loop that costs
      // 9% of the first pass).  On a cache this library filled neither clamp
      // ever acts: child links are checked to stay inside their block before
      // upload, and far pointers are written by the cache itself.
      const uint32_t pdesc = desc;
      uint32_t ofs;
      if (desc & (1u << 10)) {
        ofs = __ldg(p.far_ptrs + min(desc >> 11, p.far_limit - 1u));
        if (kCount) ++far_fetches;
      } else {
        ofs = (desc >> 11) + parent - (1u << 20);
      }
      ofs = min(ofs + __popc(desc & (bit - 1) & 255u), p.node_limit - 1u);
      desc = __ldg(p.links + ofs);
      if (kCount) ++fetches;
      if (!(desc & 255u) || scale == 0 || tc_max * coef + bias >= scale_exp2) {
        r.t = t_min;
        r.node = (int)ofs;
        r.dup = (int)((desc >> 9) & 1u);
        break;
      }
      const float half = scale_exp2 * 0.5f;
      const float tx_center = half * tx_coef + tx_corner;
      const float ty_center = half * ty_coef + ty_corner;
      const float tz_center = half * tz_coef + tz_corner;
      if (tc_max < h) stack[scale] = make_uint4(parent, __float_as_uint(t_max), pdesc, 0u);
      h = tc_max;
      parent = ofs;
      idx = 0;
      --scale;
      scale_exp2 = half;
      if (tx_center > t_min) idx ^= 1, px = px + scale_exp2;
      if (ty_center > t_min) idx ^= 2, py = py + scale_exp2;
      if (tz_center > t_min) idx ^= 4, pz = pz + scale_exp2;
      t_max = tc_max;
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
      if (step & 1) diff |= (uint32_t)(__float_as_int(px) ^ __float_as_int(px + scale_exp2));
      if (step & 2) diff |= (uint32_t)(__float_as_int(py) ^ __float_as_int(py + scale_exp2));
      if (step & 4) diff |= (uint32_t)(__float_as_int(pz) ^ __float_as_int(pz + scale_exp2));
      scale = (__float_as_int((float)diff) >> 23) - 127;
      if (scale >= kSMax) break;
      scale_exp2 = __int_as_float((scale - kSMax + 127) << 23);
      const uint4 e = stack[scale];
      parent = e.x;
      t_max = __uint_as_float(e.y);
      desc = kCount ? 0u : e.z;  // the parent's descriptor, needed next iteration
      const uint32_t shx = __float_as_uint(px) >> scale;
      const uint32_t shy = __float_as_uint(py) >> scale;
      const uint32_t shz = __float_as_uint(pz) >> scale;
      px = __uint_as_float(shx << scale);
      py = __uint_as_float(shy << scale);
      pz = __uint_as_float(shz << scale);
      idx = (int)((shx & 1u) | ((shy & 1u) << 1) | ((shz & 1u) << 2));
      h = 0.0f;
    }
  }
  if (scale >= kSMax && !r.error && r.fault_block == -1) r.node = -1;  // left the octree: miss
  r.iter = iter;
  return r;
}

// CastRay's loop until the ray ends or (kBudget) its iteration count reaches
// `stop` <= kIterLimit (kRunning: the ray continues from there on the next
// call).  The loop runs on local copies of the state, written back once at
// the end, and leaves through one exit.
// A node at scale 0 ends the ray like a leaf: its children would lie below
// float resolution and below the stack, which only a tree deeper than 23
// levels reaches (the reference reads and writes past its stack there).  So
// every stack index stays in [0, 22].
template <bool kCount, bool kBudget>
__device__ __forceinline__ int cast_run(Cast& c, int stop, uint2* stack, const TraceParams& p, uint32_t& fetches,
                                        uint32_t& far_fetches) {
  const float tx_coef = c.tx_coef, ty_coef = c.ty_coef, tz_coef = c.tz_coef;
  const float tx_bias = c.tx_bias, ty_bias = c.ty_bias, tz_bias = c.tz_bias;
  const float coef = c.coef, bias = c.bias;
  const int octant = c.octant;
  float t_min = c.t_min, t_max = c.t_max, h = c.h, px = c.px, py = c.py, pz = c.pz, scale_exp2 = c.scale_exp2;
  uint32_t parent = c.parent, desc = c.desc;
  int idx = c.idx, scale = c.scale, iter = c.iter;
  int outcome = kMiss;
  while (scale < kSMax) {
    if (++iter > (kBudget ? stop : kIterLimit)) {
      if (!kBudget || iter > kIterLimit) {
        outcome = kError;
      } else {
        --iter;
        outcome = kRunning;
      }
      break;
    }
    if (desc == 0) {
      if (parent >= p.node_limit) {  // only reachable from a corrupt cache
        outcome = kError;
        break;
      }
      desc = __ldg(p.links + parent);
      if (kCount) ++fetches;
    }
    const float tx_corner = px * tx_coef - tx_bias;
    const float ty_corner = py * ty_coef - ty_bias;
    const float tz_corner = pz * tz_coef - tz_bias;
    const float tc_max = fminf(fminf(tx_corner, ty_corner), tz_corner);
    const uint32_t bit = 1u << (idx ^ octant);
    if ((desc & bit) != 0 && t_min <= t_max) {
      if (desc & (1u << 8)) {  // children not loaded
        outcome = kFault;
        break;
      }
      uint32_t ofs;  // indices clamped into their buffers, as in cast_ray
      if (desc & (1u << 10)) {
        ofs = __ldg(p.far_ptrs + min(desc >> 11, p.far_limit - 1u));
        if (kCount) ++far_fetches;
      } else {
        ofs = (desc >> 11) + parent - (1u << 20);
      }
      ofs = min(ofs + __popc(desc & (bit - 1) & 255u), p.node_limit - 1u);
      desc = __ldg(p.links + ofs);
      if (kCount) ++fetches;
      if (!(desc & 255u) || scale == 0 || tc_max * coef + bias >= scale_exp2) {
        parent = ofs;
        outcome = kHit;
        break;
      }
      const float half = scale_exp2 * 0.5f;
      const float tx_center = half * tx_coef + tx_corner;
      const float ty_center = half * ty_coef + ty_corner;
      const float tz_center = half * tz_coef + tz_corner;
      if (tc_max < h) stack[scale] = make_uint2(parent, __float_as_uint(t_max));
      h = tc_max;
      parent = ofs;
      idx = 0;
      --scale;
      scale_exp2 = half;
      if (tx_center > t_min) idx ^= 1, px = px + scale_exp2;
      if (ty_center > t_min) idx ^= 2, py = py + scale_exp2;
      if (tz_center > t_min) idx ^= 4, pz = pz + scale_exp2;
      t_max = tc_max;
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
      if (step & 1) diff |= (uint32_t)(__float_as_int(px) ^ __float_as_int(px + scale_exp2));
      if (step & 2) diff |= (uint32_t)(__float_as_int(py) ^ __float_as_int(py + scale_exp2));
      if (step & 4) diff |= (uint32_t)(__float_as_int(pz) ^ __float_as_int(pz + scale_exp2));
      // (float)diff is exact (diff < 2^23), so its exponent is the top bit
      scale = (__float_as_int((float)diff) >> 23) - 127;
      // popping past the root ends the loop (the reference reads one more
      // stack entry first, whose value it never uses)
      if (scale >= kSMax) break;
      scale_exp2 = __int_as_float((scale - kSMax + 127) << 23);
      const uint2 e = stack[scale];
      parent = e.x;
      t_max = __uint_as_float(e.y);
      const uint32_t shx = __float_as_uint(px) >> scale;
      const uint32_t shy = __float_as_uint(py) >> scale;
      const uint32_t shz = __float_as_uint(pz) >> scale;
      px = __uint_as_float(shx << scale);
      py = __uint_as_float(shy << scale);
      pz = __uint_as_float(shz << scale);
      idx = (int)((shx & 1u) | ((shy & 1u) << 1) | ((shz & 1u) << 2));
      h = 0.0f;
      desc = 0;
    }
  }
  c.t_min = t_min;
  c.t_max = t_max;
  c.h = h;
  c.px = px;
  c.py = py;
  c.pz = pz;
  c.scale_exp2 = scale_exp2;
  c.parent = parent;
  c.desc = desc;
  c.idx = idx;
  c.scale = scale;
  c.iter = iter;
  return outcome;
}

// x / 127 correctly rounded for an integer x in [-128, 127] (a char normal
// component): the product with the rounded reciprocal, then one FMA-exact
// residual correction.  Equal to the IEEE quotient for all 256 inputs (a CPU
// test checks every one); a fifth of a full-range division's instructions.
__device__ __forceinline__ float div127(float x) {
  const float r = 1.0f / 127.0f;
  const float q0 = x * r;
  const float e = fmaf(-q0, 127.0f, x);
  return fmaf(e, r, q0);
}

// ProcessHit: fixed ambient + three directional lights; returns RGBA8 (A=255).
__device__ __forceinline__ uchar4 shade(const TraceParams& p, uint32_t node) {
  const char4 cn = p.normals[node];
  // the reference's w component is 0 / 127 = +0
  const float nx = div127((float)cn.x), ny = div127((float)cn.y), nz = div127((float)cn.z), nw = 0.0f;
  // The light directions (shading.cl:7-32): normalize(v) * w for v, w =
  // (2,-2,3), .6; (-3,-3,-2), .5; (1,2.5,-1), .3, each as the reference
  // computes it per call in IEEE float (dot left to right, correctly rounded
  // sqrt and divisions, then the product).  Constants, so no ray pays for 3
  // square roots and 9 divisions; a CPU test recomputes them.
  const float l[3][3] = {{0x1.2a071ep-2f, -0x1.2a071ep-2f, 0x1.bf0aacp-2f},
                         {-0x1.4779eep-2f, -0x1.4779eep-2f, -0x1.b4a294p-3f},
                         {0x1.abd032p-4f, 0x1.0b6220p-2f, -0x1.abd032p-4f}};
  float a[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float dd = dot4(-nx, -ny, -nz, -nw, l[k][0], l[k][1], l[k][2], 0.0f);
    a[k] = 0.f < dd ? dd : 0.f;
  }
  const float light = ((.1f + a[0] * 1.f) + a[1] * 1.f) + a[2] * 1.f;
  const uchar4 cc = p.colors[node];
  float c0 = (float)cc.x * light, c1 = (float)cc.y * light, c2 = (float)cc.z * light;
  c0 = c0 < 255.f ? c0 : 255.f;
  c1 = c1 < 255.f ? c1 : 255.f;
  c2 = c2 < 255.f ? c2 : 255.f;
  return make_uchar4((unsigned char)c0, (unsigned char)c1, (unsigned char)c2, 255);
}

// FinishTracingFrame's blend of the accumulated colour over the background.
__device__ __forceinline__ uchar4 finish(const TraceParams& p, uchar4 c) {
  const float w = 255.f - (float)c.w;
  float t[4] = {(float)c.x + p.bg[0] * w + .5f, (float)c.y + p.bg[1] * w + .5f,
                (float)c.z + p.bg[2] * w + .5f, (float)c.w + p.bg[3] * w + .5f};
  unsigned char o[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    float v = t[k] < 255.f ? t[k] : 255.f;
    v = 0.f < v ? v : 0.f;
    o[k] = (unsigned char)v;
  }
  return make_uchar4(o[0], o[1], o[2], o[3]);
}

// Appends `pred` lanes of the active warp to a global list: returns this
// lane's slot (or -1).
__device__ __forceinline__ int warp_append(int* counter, bool pred) {
  const unsigned active = __activemask();
  const unsigned mask = __ballot_sync(active, pred);
  if (!mask) return -1;
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(mask) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(counter, __popc(mask));
  base = __shfl_sync(active, base, leader);
  return pred ? base + __popc(mask & ((1u << lane) - 1)) : -1;
}

// Sets bit `bit` (>= 0) of a bitmap, one atomic per distinct word in the warp.
__device__ __forceinline__ void warp_set_bit(uint32_t* bits, int bit) {
  const unsigned active = __activemask();
  const int word = bit >= 0 ? (bit >> 5) : -1;
  const unsigned peers = __match_any_sync(active, word);
  if (word < 0) return;
  const unsigned m = 1u << (bit & 31);
  unsigned acc = 0;
  unsigned rest = peers;
  while (rest) {
    const int src = __ffs(rest) - 1;
    acc |= __shfl_sync(peers, m, src);
    rest &= rest - 1;
  }
  const int lane = threadIdx.x & 31;
  if (lane == __ffs(peers) - 1) {
    if ((__ldcg(bits + word) & acc) != acc) atomicOr(bits + word, acc);
  }
}

// View of the launch holding tile `tile` (tile_base is ascending).
__device__ __forceinline__ int view_of_tile(const TraceParams& p, int tile) {
  int lo = 0, hi = p.n_views - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (p.views[mid].tile_base <= tile) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Served mode: the client slot owning pixel `ray` (client_base ascending).
__device__ __forceinline__ int slot_of(const TraceParams& p, uint32_t ray) {
  int lo = 0, hi = p.n_clients - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if ((uint32_t)p.client_base[mid] <= ray) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Pixel (x, y) and view of first-pass ray r (tile r / 32, lane r % 32);
// false for the lanes of a partial tile that fall outside the view.
__device__ __forceinline__ bool first_pass_pixel(const TraceParams& p, int r, int& v, int& x, int& y) {
  const int tile = (int)(r >> 5), k = (int)(r & 31);
  v = view_of_tile(p, tile);
  const ViewDesc& vd = p.views[v];
  const int t = tile - vd.tile_base;
  x = ((t % vd.tiles_x) << p.tile_w_log2) + (k & ((1 << p.tile_w_log2) - 1));
  y = (t / vd.tiles_x) * (32 >> p.tile_w_log2) + (k >> p.tile_w_log2);
  return x < vd.width && y < vd.height;
}

// kBudget: warps stop their rays every step_budget iterations and refill idle
// lanes once `refill` of them are idle; otherwise a warp takes new rays once
// all 32 ended.
// Ray r of the launch (first pass: tile r / 32 of the views; later passes:
// record r of the input list): its pixel, origin, direction and (depth
// output) the distance it advanced in earlier passes; false for the lanes of
// a partial tile that fall outside their view.
template <bool kFirst>
__device__ __forceinline__ bool ray_at(const TraceParams& p, int r, uint32_t& ray, float4& o, float4& d,
                                       float& adv) {
  adv = 0.0f;
  if (kFirst) {
    int v, x, y;
    if (!first_pass_pixel(p, r, v, x, y)) return false;
    const ViewDesc& vd = p.views[v];
    init_ray(vd, x, y, o, d);
    ray = (uint32_t)(vd.pix_base + y * vd.width + x);
  } else {
    o = p.in_origin[r];
    d = p.in_dir[r];
    ray = p.in_ray[r];
    if (p.in_adv) adv = p.in_adv[r];
  }
  return true;
}

// Depth output of a pixel whose ray ended: the distance along the ray to what
// the pixel shows (earlier passes' advances plus this pass's t, in float, in
// pass order) and the cache node that shaded it.  Miss: +inf and -1; error
// (iteration limit, corrupt cache): NaN and -2.
__device__ __forceinline__ void write_depth(const TraceParams& p, uint32_t ray, float depth, int node) {
  p.depth[ray] = depth;
  p.hit_node[ray] = node;
}
constexpr uint32_t kDepthNaN = 0x7fffffffu;
constexpr uint32_t kDepthInf = 0x7f800000u;

// A final pixel: into the image, and into the caller's host image when the
// renderer delivers one (later passes and the finish; the first pass's pixels
// reach it by one copy).
__device__ __forceinline__ void put_pixel(const TraceParams& p, uint32_t ray, uchar4 px) {
  p.image[ray] = px;
  if (p.host_image) p.host_image[ray] = px;
}

// RaytracingPass's handling of an ended ray (raytracing_pass.cl:20-58) plus
// FinishTracingFrame for rays that end here: the final pixel, the next pass's
// record of a faulted ray, the feedback bitmaps and counters.  Called by the
// lanes whose rays ended, together.
template <bool kCount>
__device__ __forceinline__ void end_ray(const TraceParams& p, const RayEnd& e, uint32_t ray, float4 o, const float4 d,
                                        float adv, uint32_t fetches, uint32_t far_fetches) {
  const int lane = threadIdx.x & 31;
  const bool faulted = !e.error && e.fault_block != -1;
  const bool hit = !e.error && e.fault_block == -1 && e.node != -1;
  const int node = e.node, dup = e.dup, fault_block = e.fault_block;
  int32_t word = kNoHit;
  if (e.error) {
    put_pixel(p, ray, finish(p, make_uchar4(255, 0, 0, 255)));
    if (p.depth) write_depth(p, ray, __uint_as_float(kDepthNaN), -2);
  } else if (faulted) {
    word = -fault_block - 1;
  } else if (!hit) {
    put_pixel(p, ray, finish(p, make_uchar4(0, 0, 0, 0)));
    if (p.depth) write_depth(p, ray, __uint_as_float(kDepthInf), -1);
  } else {
    const uchar4 col = (p.normals && p.colors) ? shade(p, (uint32_t)node) : make_uchar4(0, 0, 0, 0);
    put_pixel(p, ray, finish(p, col));
    word = (int32_t)(((uint32_t)(node + 1) << 1) | (uint32_t)dup);
    if (p.depth) write_depth(p, ray, adv + e.t, node);
  }
  if (p.words_dense) p.words_dense[ray] = word;
  const int slot = warp_append(p.n_out, faulted);
  if (faulted) {
    if (!p.restart) {  // origin moved to the fault (raytracing_pass.cl:37-41)
      o.x = o.x + d.x * e.t;
      o.y = o.y + d.y * e.t;
      o.z = o.z + d.z * e.t;
      o.w = o.w + d.w * e.t;
    }
    if (p.client_faults) atomicAdd(p.client_faults + slot_of(p, ray), 1);
    p.out_origin[slot] = o;
    p.out_dir[slot] = d;
    p.out_parent[slot] = node;
    p.out_ray[slot] = ray;
    if (p.out_adv) p.out_adv[slot] = p.restart ? adv : adv + e.t;
  }
  warp_set_bit(p.fault_bits, faulted && fault_block < p.fault_bit_limit ? fault_block : -1);
  warp_set_bit(p.hit_bits, hit ? (int)(2 * ((uint32_t)node / (uint32_t)p.nodes_in_block)) + dup : -1);
  {
    const unsigned active = __activemask();
    const unsigned m = __ballot_sync(active, word != kNoHit);
    if (m && lane == __ffs(m) - 1) atomicAdd(p.n_words, __popc(m));
  }
  if (kCount) {
    const unsigned v[6] = {1u, fetches, far_fetches, (unsigned)e.iter, hit ? 1u : 0u, faulted ? 1u : 0u};
    const unsigned active = __activemask();
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const unsigned sum = __reduce_add_sync(active, v[k]);
      if (lane == __ffs(active) - 1) atomicAdd(p.counters + k, (unsigned long long)sum);
    }
  }
}

// One ray per thread over a grid that covers the launch's rays (a warp = one
// 32-ray tile); the hardware hands CTAs to SMs as earlier ones retire.
template <bool kFirst, bool kCount>
__global__ void __launch_bounds__(kBlockThreads) trace_kernel(const __grid_constant__ TraceParams p) {
  const int total = kFirst ? p.total_tiles * 32 : *p.n_in;
  const int r = blockIdx.x * kBlockThreads + threadIdx.x;
  if (r >= total) return;
  uint32_t ray;
  float4 o, d;
  float adv;
  if (!ray_at<kFirst>(p, r, ray, o, d, adv)) return;
  uint32_t fetches = 0, far_fetches = 0;
  const RayEnd e = cast_ray<kCount>(p, o, d, fetches, far_fetches);
  end_ray<kCount>(p, e, ray, o, d, adv, fetches, far_fetches);
}

// Persistent form: one CTA per SM slot; every warp takes rays from the
// launch's work counter.  A warp runs its rays for step_budget iterations at a
// time and, once at least `refill` of its lanes sit idle (refill = 32: all of
// them), hands those lanes the next rays, so lanes do not idle through the
// warp's longest ray.  Once the counter is exhausted the rays run to the end.
template <bool kFirst, bool kCount>
__global__ void __launch_bounds__(kBlockThreads) trace_persistent_kernel(const __grid_constant__ TraceParams p) {
  __shared__ float4 s_origin[kBlockThreads], s_dir[kBlockThreads];
  const int lane = threadIdx.x & 31;
  const int total = kFirst ? p.total_tiles * 32 : *p.n_in;  // below 2^31: at most 2^30 pixels
  uint2 stack[kSMax + 1];
  Cast c;
  int outcome = kRunning;
  uint32_t ray = 0;
  float adv = 0.0f;
  bool have = false, exhausted = false;
  uint32_t fetches = 0, far_fetches = 0;

  for (;;) {
    const unsigned idle = __ballot_sync(kFull, !have);
    if (!exhausted && __popc(idle) >= p.refill) {
      const int want = __popc(idle);
      const int leader = __ffs(idle) - 1;
      int base = 0;
      if (lane == leader) base = atomicAdd(p.work, want);
      base = __shfl_sync(kFull, base, leader);
      if (base + want >= total) exhausted = true;
      if (!have) {
        const int r = base + __popc(idle & ((1u << lane) - 1));
        float4 o, d;
        if (r < total && ray_at<kFirst>(p, r, ray, o, d, adv)) {
          s_origin[threadIdx.x] = o;  // kept for the ray's fault record
          s_dir[threadIdx.x] = d;
          cast_begin(c, p.root, o, d);
          have = true;
          fetches = far_fetches = 0;
        }
      }
    }
    if (!__ballot_sync(kFull, have)) {
      if (exhausted) break;
      continue;
    }
    if (have && outcome == kRunning) {
      const int stop = exhausted ? kIterLimit : min(c.iter + p.step_budget, kIterLimit);
      outcome = cast_run<kCount, true>(c, stop, stack, p, fetches, far_fetches);
    }
    if (outcome != kRunning) {
      RayEnd e;
      e.t = c.t_min;
      e.node = outcome == kMiss ? -1 : (int)c.parent;
      e.fault_block = outcome == kFault ? (int)(c.desc >> 11) : -1;
      e.dup = (int)((c.desc >> 9) & 1u);
      e.error = outcome == kError;
      e.iter = c.iter;
      end_ray<kCount>(p, e, ray, s_origin[threadIdx.x], s_dir[threadIdx.x], adv, fetches, far_fetches);
      have = false;
      outcome = kRunning;
    }
  }
}

// Persistent form without lane refills, for the passes after the first: each
// warp takes 32 rays at a time from the work counter and runs them to their
// end.  Its grid does not depend on the ray count (read on the device), so the
// pass can be replayed from a CUDA graph unchanged.
template <bool kFirst, bool kCount>
__global__ void __launch_bounds__(kBlockThreads) trace_queue_kernel(const __grid_constant__ TraceParams p) {
  const int lane = threadIdx.x & 31;
  const int total = kFirst ? p.total_tiles * 32 : *p.n_in;
  for (;;) {
    int base = 0;
    if (lane == 0) base = atomicAdd(p.work, 32);
    base = __shfl_sync(kFull, base, 0);
    if (base >= total) break;
    const int r = base + lane;
    uint32_t ray;
    float4 o, d;
    float adv;
    if (r < total && ray_at<kFirst>(p, r, ray, o, d, adv)) {
      if (!kFirst && p.finish_mask && ((p.finish_mask >> slot_of(p, ray)) & 1ull)) {
        // served mode: the request stops here; FinishTracingFrame's shading
        // with the fault's parent node
        const uchar4 col = (p.normals && p.colors) ? shade(p, (uint32_t)p.in_parent[r]) : make_uchar4(0, 0, 0, 0);
        put_pixel(p, ray, finish(p, col));
        if (p.depth) write_depth(p, ray, adv, p.in_parent[r]);
      } else {
        uint32_t fetches = 0, far_fetches = 0;
        const RayEnd e = cast_ray<kCount>(p, o, d, fetches, far_fetches);
        end_ray<kCount>(p, e, ray, o, d, adv, fetches, far_fetches);
      }
    }
  }
}

// FinishTracingFrame for rays still faulted at the end of the frame: shade
// with the fault's parent node as the cache holds it now.  Depth output: the
// distance at which the ray stopped and that parent node.
__global__ void __launch_bounds__(kBlockThreads) finish_kernel(const __grid_constant__ TraceParams p) {
  const int i = blockIdx.x * kBlockThreads + threadIdx.x;
  if (i >= *p.n_in) return;
  const uchar4 col = (p.normals && p.colors) ? shade(p, (uint32_t)p.in_parent[i]) : make_uchar4(0, 0, 0, 0);
  put_pixel(p, p.in_ray[i], finish(p, col));
  if (p.depth) write_depth(p, p.in_ray[i], p.in_adv[i], p.in_parent[i]);
}

// raytracer.cl:18-71 (RaytraceKernel, the reference's debug depth view) for
// view 0 of the parameters: rays from the near plane, one pass over the cache
// as it is, no feedback.  Red for a fault or an error, black for a miss, else
// grey = 255 * (1 - log-depth in [0.01, 5]) clamped to [0, 255] (the
// reference's float-to-uchar conversion is undefined outside that range).
__global__ void __launch_bounds__(kBlockThreads) depth_view_kernel(const __grid_constant__ TraceParams p) {
  const ViewDesc& v = p.views[0];
  const int W = v.width, H = v.height;
  const int i = blockIdx.x * kBlockThreads + threadIdx.x;
  if (i >= W * H) return;
  const int x = i % W, y = i / W;
  const float cx = __fdiv_rn(x + 0.5f, (float)W) * 2 - 1, cy = __fdiv_rn(y + 0.5f, (float)H) * 2 - 1;
  float o[4], q[4], p1n[4], p1f[4], p2n[4], p2f[4];
  mul_point(v.m, cx, cy, -1.0f, o);
  mul_point(v.m, cx, cy, 0.0f, q);
  float dx = q[0] - o[0], dy = q[1] - o[1], dz = q[2] - o[2], dw = q[3] - o[3];
  const float len = __fsqrt_rn(dot4(dx, dy, dz, dw, dx, dy, dz, dw));
  dx = __fdiv_rn(dx, len);
  dy = __fdiv_rn(dy, len);
  dz = __fdiv_rn(dz, len);
  const float ax = __fdiv_rn((float)x, (float)W) * 2 - 1, ay = __fdiv_rn((float)y, (float)H) * 2 - 1;
  const float bx = __fdiv_rn((float)(x + 1), (float)W) * 2 - 1, by = __fdiv_rn((float)(y + 1), (float)H) * 2 - 1;
  mul_point(v.m, ax, ay, -1.0f, p1n);
  mul_point(v.m, ax, ay, 0.0f, p1f);
  mul_point(v.m, bx, by, -1.0f, p2n);
  mul_point(v.m, bx, by, 0.0f, p2f);
  auto dist = [](const float* a, const float* b) {
    const float ex = a[0] - b[0], ey = a[1] - b[1], ez = a[2] - b[2], ew = a[3] - b[3];
    return __fsqrt_rn(dot4(ex, ey, ez, ew, ex, ey, ez, ew));
  };
  const float bias = v.lod * dist(p1n, p2n);
  const float coef = bias < 1e-10f ? 0.0f : __fdiv_rn(v.lod * (dist(p1f, p2f) - dist(p1n, p2n)), dist(p1n, p1f));
  uint32_t fetches = 0, far_fetches = 0;
  const RayEnd e = cast_ray<false>(p, make_float4(o[0], o[1], o[2], bias), make_float4(dx, dy, dz, coef), fetches,
                                   far_fetches);
  uchar4 c;
  if (e.error || e.fault_block != -1) {
    c = make_uchar4(255, 0, 0, 255);
  } else if (e.node == -1) {
    c = make_uchar4(0, 0, 0, 255);
  } else {
    const float near_ = 0.01f, far_ = 5.0f;
    float d = __fdiv_rn(logf(e.t) - logf(near_), logf(far_) - logf(near_));
    d = (1 - d) * 255;
    d = fminf(255.0f, fmaxf(0.0f, d));
    const unsigned char g = (unsigned char)d;
    c = make_uchar4(g, g, g, 255);
  }
  p.image[i] = c;
}

__global__ void fill_kernel(int* p, int32_t v, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) p[i] = v;
}

// Bitmaps -> [faults by descending block][hits ascending][NO_HIT], the order
// of the reference's sorted unique array.  One CTA; each thread owns a run of
// bitmap words in output order.
constexpr int kUniqThreads = 1024;
__global__ void __launch_bounds__(kUniqThreads) unique_from_bits_kernel(const UniqueFromBitsParams q) {
  __shared__ int warp_sums[32];
  __shared__ int fsum;
  const int total = q.fault_words + q.hit_words;
  const int per = (total + kUniqThreads - 1) / kUniqThreads;
  const int begin = min(total, (int)threadIdx.x * per), end = min(total, begin + per);
  auto word_at = [&](int k) -> uint32_t {
    return k < q.fault_words ? q.fault_bits[q.fault_words - 1 - k] : q.hit_bits[k - q.fault_words];
  };
  int cnt = 0, fcnt = 0;
  for (int k = begin; k < end; ++k) {
    const int n = __popc(word_at(k));
    cnt += n;
    if (k < q.fault_words) fcnt += n;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = cnt;
  for (int off = 1; off < 32; off <<= 1) {
    int v = __shfl_up_sync(kFull, incl, off);
    if (lane >= off) incl += v;
  }
  if (lane == 31) warp_sums[warp] = incl;
  if (threadIdx.x == 0) fsum = 0;
  __syncthreads();
  if (warp == 0) {
    int v = warp_sums[lane];
    int s = v;
    for (int off = 1; off < 32; off <<= 1) {
      int u = __shfl_up_sync(kFull, s, off);
      if (lane >= off) s += u;
    }
    warp_sums[lane] = s - v;  // exclusive
  }
  __syncthreads();
  int pos = warp_sums[warp] + incl - cnt;
  for (int k = begin; k < end; ++k) {
    uint32_t w = word_at(k);
    if (k < q.fault_words) {
      const int wi = q.fault_words - 1 - k;
      while (w) {  // descending bits
        const int b = 31 - __clz(w);
        w &= ~(1u << b);
        q.unique_out[pos++] = -(wi * 32 + b) - 1;
      }
    } else {
      const int wi = k - q.fault_words;
      while (w) {  // ascending bits: value = bit index + 2
        const int b = __ffs(w) - 1;
        w &= w - 1;
        q.unique_out[pos++] = wi * 32 + b + 2;
      }
    }
  }
  int f = fcnt;
  for (int off = 16; off > 0; off >>= 1) f += __shfl_down_sync(kFull, f, off);
  if (lane == 0) atomicAdd(&fsum, f);
  __syncthreads();
  if (threadIdx.x == kUniqThreads - 1) {
    int n = pos;  // the last thread's end position = total set bits
    if (*q.n_words < q.total_pixels) q.unique_out[n++] = kNoHit;
    q.counts_out[0] = n;
    q.counts_out[1] = fsum;
    q.counts_out[2] = q.n_rays ? *q.n_rays : 0;
  }
}

template <typename Kernel>
int resident_grid(Kernel kernel) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBlockThreads, 0);
  return sms * (per_sm > 0 ? per_sm : 1);
}

template <bool kFirst, bool kCount>
int persistent_grid() {
  static const int grid = resident_grid(trace_persistent_kernel<kFirst, kCount>);
  return grid;
}

template <bool kCount>
int queue_grid() {
  static const int grid = resident_grid(trace_queue_kernel<false, kCount>);
  return grid;
}

// The traversal launch for pass kind (first, count): function and grid.
template <bool kFirst, bool kCount>
void trace_launch_shape(const TraceParams& p, int rays, int grid, void** func, dim3* blocks) {
  if (!kFirst) {
    // persistent warps over the faulted rays; when the caller knows their
    // count, no more CTAs than they fill (a later pass often traces a few
    // hundred rays, and every idle warp of a full grid still launches and
    // claims from the one work counter)
    *func = reinterpret_cast<void*>(trace_queue_kernel<false, kCount>);
    const int full = queue_grid<kCount>();
    *blocks = dim3(rays > 0 ? std::min(full, (rays + kBlockThreads - 1) / kBlockThreads) : full);
  } else if (p.refill < 32) {
    *func = reinterpret_cast<void*>(trace_persistent_kernel<true, kCount>);
    *blocks = dim3(grid > 0 ? grid : persistent_grid<true, kCount>());
  } else {
    *func = reinterpret_cast<void*>(trace_kernel<true, kCount>);
    *blocks = dim3((rays + kBlockThreads - 1) / kBlockThreads);
  }
}

}  // namespace

int trace_persistent_grid(bool first, bool count) {
  if (first) return count ? persistent_grid<true, true>() : persistent_grid<true, false>();
  return count ? persistent_grid<false, true>() : persistent_grid<false, false>();
}

cudaError_t trace_node_params(const TraceParams* p, bool first, bool count, int rays, int grid, void** args,
                              cudaKernelNodeParams* kp) {
  void* func = nullptr;
  dim3 blocks;
  if (first) {
    if (count) trace_launch_shape<true, true>(*p, rays, grid, &func, &blocks);
    else trace_launch_shape<true, false>(*p, rays, grid, &func, &blocks);
  } else {
    if (count) trace_launch_shape<false, true>(*p, rays, grid, &func, &blocks);
    else trace_launch_shape<false, false>(*p, rays, grid, &func, &blocks);
  }
  args[0] = const_cast<TraceParams*>(p);
  *kp = cudaKernelNodeParams{};
  kp->func = func;
  kp->gridDim = blocks;
  kp->blockDim = dim3(kBlockThreads);
  kp->sharedMemBytes = 0;
  kp->kernelParams = args;
  kp->extra = nullptr;
  return cudaSuccess;
}

cudaError_t launch_trace(const TraceParams& p, bool first, bool count, int rays, int grid, cudaStream_t s) {
  void* args[1];
  cudaKernelNodeParams kp;
  trace_node_params(&p, first, count, rays, grid, args, &kp);
  if (kp.gridDim.x == 0) return cudaSuccess;
  return cudaLaunchKernel(kp.func, kp.gridDim, kp.blockDim, kp.kernelParams, 0, s);
}

cudaError_t unique_node_params(const UniqueFromBitsParams* q, void** args, cudaKernelNodeParams* kp) {
  args[0] = const_cast<UniqueFromBitsParams*>(q);
  *kp = cudaKernelNodeParams{};
  kp->func = reinterpret_cast<void*>(unique_from_bits_kernel);
  kp->gridDim = dim3(1);
  kp->blockDim = dim3(kUniqThreads);
  kp->kernelParams = args;
  return cudaSuccess;
}

cudaError_t launch_finish(const TraceParams& p, int max_rays, cudaStream_t s) {
  if (max_rays <= 0) return cudaSuccess;
  finish_kernel<<<(max_rays + kBlockThreads - 1) / kBlockThreads, kBlockThreads, 0, s>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_depth_view(const TraceParams& p, cudaStream_t s) {
  const long long n = (long long)p.views[0].width * p.views[0].height;
  if (n <= 0) return cudaSuccess;
  depth_view_kernel<<<(unsigned)((n + kBlockThreads - 1) / kBlockThreads), kBlockThreads, 0, s>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_fill_i32(int* ptr, int32_t v, size_t n, cudaStream_t s) {
  if (!n) return cudaSuccess;
  int grid = (int)((n + 255) / 256);
  if (grid > 4096) grid = 4096;
  fill_kernel<<<grid, 256, 0, s>>>(ptr, v, n);
  return cudaGetLastError();
}

cudaError_t launch_unique_from_bits(const UniqueFromBitsParams& q, cudaStream_t s) {
  unique_from_bits_kernel<<<1, kUniqThreads, 0, s>>>(q);
  return cudaGetLastError();
}

}  // namespace rayt
