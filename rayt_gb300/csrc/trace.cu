// Tracing pass, the hot path: one thread per primary ray.
//
// Per ray this fuses what the reference runs as separate full-frame kernels
// with a 48-byte TracingState round trip through memory:
//   ray setup       InitTracingFrame   (rayt/GPU_renderer/kernels/init_tracing_frame.cl:11-45)
//   traversal       CastRay            (rayt/GPU_renderer/kernels/raycast.cl:33-256)
//   pass logic      RaytracingPass     (rayt/GPU_renderer/kernels/raytracing_pass.cl:4-61)
//   shading         ProcessHit         (rayt/GPU_renderer/kernels/shading.cl:4-33)
//   final colour    FinishTracingFrame (rayt/GPU_renderer/kernels/finish_tracing_frame.cl:3-24)
//   block words     NodeToBlockKernel  (rayt/GPU_renderer/kernels/feedback_compression.cl:4-13)
// A ray that finishes (hit, miss, iteration limit) writes its final RGBA8
// pixel at once; only a ray that faults on a missing block stores its state
// (advanced origin, direction, parent node) and joins the next pass's active
// list, so later passes launch over faulted rays only.  Feedback goes straight
// into two bitmaps (fault blocks, hit blocks) instead of a per-pixel word array.
//
// FP32 arithmetic follows the reference's operation order exactly; the file is
// compiled with --fmad=false and IEEE division/sqrt so no operation is fused or
// approximated, which keeps hit node IDs identical to the CPU oracle.
#include "internal.h"

namespace rayt {
namespace {

constexpr int kSMax = 23;
constexpr float kEps = 0.00000011920928955078125f;  // exp2(-S_MAX)
constexpr int kIterLimit = 300;
constexpr int kTileW = 8, kTileH = 4;  // one warp = 8x4 pixels
constexpr int kBlockThreads = 128;

struct Cast {
  float t;
  int node;
  int fault_block;
  int dup;
  int error;
};

__device__ __forceinline__ float dot4(float ax, float ay, float az, float aw, float bx, float by, float bz, float bw) {
  float r = ax * bx;
  r = r + ay * by;
  r = r + az * bz;
  r = r + aw * bw;
  return r;
}

// mul(float16, float3) of init_tracing_frame.cl:3-9
__device__ __forceinline__ void mul_point(const float* m, float x, float y, float z, float* o) {
  float d = dot4(x, y, z, 1.0f, m[12], m[13], m[14], m[15]);
  o[0] = __fdiv_rn(dot4(x, y, z, 1.0f, m[0], m[1], m[2], m[3]), d);
  o[1] = __fdiv_rn(dot4(x, y, z, 1.0f, m[4], m[5], m[6], m[7]), d);
  o[2] = __fdiv_rn(dot4(x, y, z, 1.0f, m[8], m[9], m[10], m[11]), d);
  o[3] = __fdiv_rn(0.0f, d);
}

// InitTracingFrame for pixel (x, y).
__device__ __forceinline__ void init_ray(const TraceParams& p, int x, int y, float4& o, float4& d) {
  const float* m = p.m;
  const int W = p.width, H = p.height;
  float ox = __fdiv_rn(m[2], m[14]), oy = __fdiv_rn(m[6], m[14]), oz = __fdiv_rn(m[10], m[14]);
  float ow = __fdiv_rn(0.0f, m[14]);
  float q[4];
  mul_point(m, __fdiv_rn(x + 0.5f, (float)W) * 2 - 1, __fdiv_rn(y + 0.5f, (float)H) * 2 - 1, 0.0f, q);
  float dx = q[0] - ox, dy = q[1] - oy, dz = q[2] - oz, dw = q[3] - ow;
  float len = __fsqrt_rn(dot4(dx, dy, dz, dw, dx, dy, dz, dw));
  dx = __fdiv_rn(dx, len);
  dy = __fdiv_rn(dy, len);
  dz = __fdiv_rn(dz, len);
  float p1[4], p2[4];
  mul_point(m, __fdiv_rn((float)x, (float)W) * 2 - 1, __fdiv_rn((float)y, (float)H) * 2 - 1, 0.0f, p1);
  mul_point(m, __fdiv_rn((float)(x + 1), (float)W) * 2 - 1, __fdiv_rn((float)(y + 1), (float)H) * 2 - 1, 0.0f, p2);
  float ax = p1[0] - p2[0], ay = p1[1] - p2[1], az = p1[2] - p2[2], aw = p1[3] - p2[3];
  float bx = ox - p1[0], by = oy - p1[1], bz = oz - p1[2], bw = ow - p1[3];
  float dist12 = __fsqrt_rn(dot4(ax, ay, az, aw, ax, ay, az, aw));
  float dist01 = __fsqrt_rn(dot4(bx, by, bz, bw, bx, by, bz, bw));
  float coef = __fdiv_rn(p.lod * dist12, dist01);
  o = make_float4(ox, oy, oz, 0.0f);
  d = make_float4(dx, dy, dz, coef);
}

__device__ __forceinline__ uint32_t ld_link(const uint32_t* links, uint32_t i) { return __ldg(links + i); }

// CastRay: ESVO descent in [1,2]^3 over cache-format links; stops at a leaf,
// at the LOD size, on a missing child block (fault), or after 300 iterations.
template <bool kCount>
__device__ __forceinline__ Cast cast_ray(const TraceParams& p, float4 o, float4 d, uint32_t* fetches,
                                         uint32_t* far_fetches, uint32_t* iters) {
  Cast r;
  r.fault_block = -1;
  r.error = 0;
  r.dup = 0;
  float px0 = o.x + 1.0f, py0 = o.y + 1.0f, pz0 = o.z + 1.0f;
  float dx = d.x, dy = d.y, dz = d.z;
  const float coef = d.w, bias = o.w;
  uint2 stack[kSMax + 1];

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

  uint32_t parent = (uint32_t)p.root;
  uint32_t desc = 0;
  int idx = 0;
  float px = 1.0f, py = 1.0f, pz = 1.0f;
  int scale = kSMax - 1;
  float scale_exp2 = 0.5f;
  if (1.5f * tx_coef - tx_bias > t_min) idx ^= 1, px = 1.5f;
  if (1.5f * ty_coef - ty_bias > t_min) idx ^= 2, py = 1.5f;
  if (1.5f * tz_coef - tz_bias > t_min) idx ^= 4, pz = 1.5f;

  int iter = 0;
  while (scale < kSMax) {
    if (++iter > kIterLimit) {
      r.error = 1;
      r.t = t_min;
      r.node = (int)parent;
      break;
    }
    if (desc == 0) {
      if (parent >= p.node_limit) {  // only reachable from a corrupt cache
        r.error = 1;
        r.t = t_min;
        r.node = 0;
        break;
      }
      desc = ld_link(p.links, parent);
      if (kCount) ++*fetches;
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
      uint32_t ofs;
      if (desc & (1u << 10)) {
        if ((desc >> 11) >= p.far_limit) {
          r.error = 1;
          r.t = t_min;
          r.node = (int)parent;
          break;
        }
        ofs = __ldg(p.far_ptrs + (desc >> 11));
        if (kCount) ++*far_fetches;
      } else {
        ofs = (desc >> 11) + parent - (1u << 20);
      }
      ofs += __popc(desc & (bit - 1) & 255u);
      if (ofs >= p.node_limit) {
        r.error = 1;
        r.t = t_min;
        r.node = (int)parent;
        break;
      }
      desc = ld_link(p.links, ofs);
      if (kCount) ++*fetches;
      if (!(desc & 255u) || tc_max * coef + bias >= scale_exp2) {
        r.t = t_min;
        r.node = (int)ofs;
        r.dup = (int)((desc >> 9) & 1u);
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
      // popping past the root: the loop ends here (the reference reads one
      // more stack entry first, whose value it never uses)
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
  if (scale >= kSMax && !r.error && r.fault_block == -1) {
    r.t = 1e30f;
    r.node = -1;
  }
  if (kCount) *iters = (uint32_t)iter;
  return r;
}

// ProcessHit: fixed ambient + three directional lights; returns RGBA8 (A=255).
__device__ __forceinline__ uchar4 shade(const TraceParams& p, int node) {
  // normalize((2,-2,3,0))*.6, normalize((-3,-3,-2,0))*.5, normalize((1,2.5,-1,0))*.3
  float l[3][3];
  const float src[3][4] = {{2.f, -2.f, 3.f, .6f}, {-3.f, -3.f, -2.f, .5f}, {1.f, 2.5f, -1.f, .3f}};
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float len = __fsqrt_rn(dot4(src[k][0], src[k][1], src[k][2], 0.f, src[k][0], src[k][1], src[k][2], 0.f));
#pragma unroll
    for (int c = 0; c < 3; ++c) l[k][c] = __fdiv_rn(src[k][c], len) * src[k][3];
  }
  const char4 cn = p.normals[node];
  const float nx = __fdiv_rn((float)cn.x, 127.f), ny = __fdiv_rn((float)cn.y, 127.f),
              nz = __fdiv_rn((float)cn.z, 127.f), nw = __fdiv_rn(0.0f, 127.f);
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
  unsigned m = 1u << (bit & 31);
  // OR together the bits of all lanes that share the word
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

template <bool kFirst, bool kCount>
__global__ void __launch_bounds__(kBlockThreads) trace_kernel(const __grid_constant__ TraceParams p) {
  int pixel, x = 0, y = 0;
  float4 o, d;
  if (kFirst) {
    // CTA = 4 x 8 warps; each warp covers an 8 x 4 pixel tile
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tiles_x = (p.width + kTileW - 1) / kTileW;
    const int tile = blockIdx.x * (kBlockThreads / 32) + warp;
    x = (tile % tiles_x) * kTileW + (lane & (kTileW - 1));
    y = (tile / tiles_x) * kTileH + (lane / kTileW);
    if (x >= p.width || y >= p.height) return;
    pixel = y * p.width + x;
    init_ray(p, x, y, o, d);
  } else {
    const int i = blockIdx.x * kBlockThreads + threadIdx.x;
    if (i >= *p.n_active_in) return;
    pixel = p.active_in[i];
    o = p.origin[pixel];
    d = p.dir[pixel];
  }

  uint32_t fetches = 0, far_fetches = 0, iters = 0;
  const Cast c = cast_ray<kCount>(p, o, d, &fetches, &far_fetches, &iters);

  int32_t word = kNoHit;
  bool faulted = false;
  if (c.error) {
    p.image[pixel] = finish(p, make_uchar4(255, 0, 0, 255));
  } else if (c.fault_block != -1) {
    faulted = true;
    o.x = o.x + d.x * c.t;
    o.y = o.y + d.y * c.t;
    o.z = o.z + d.z * c.t;
    o.w = o.w + d.w * c.t;
    p.origin[pixel] = o;
    if (kFirst) p.dir[pixel] = d;
    p.fault_parent[pixel] = c.node;
    word = -c.fault_block - 1;
  } else if (c.node == -1) {
    p.image[pixel] = finish(p, make_uchar4(0, 0, 0, 0));
  } else {
    const uchar4 col = (p.normals && p.colors) ? shade(p, c.node) : make_uchar4(0, 0, 0, 0);
    p.image[pixel] = finish(p, col);
    word = (int32_t)(((uint32_t)(c.node + 1) << 1) | (uint32_t)c.dup);
  }
  if (p.words_dense) p.words_dense[pixel] = word;

  // next pass's active list
  const int slot = warp_append(p.n_active_out, faulted);
  if (faulted) p.active_out[slot] = pixel;
  // feedback bitmaps (NodeToBlock applied: hits are per cache block)
  const bool is_hit = word != kNoHit && word > 0;
  warp_set_bit(p.fault_bits, faulted && c.fault_block < p.fault_bit_limit ? c.fault_block : -1);
  warp_set_bit(p.hit_bits, is_hit ? 2 * (c.node / p.nodes_in_block) + c.dup : -1);
  {
    const unsigned active = __activemask();
    const unsigned m = __ballot_sync(active, word != kNoHit);
    if (m && (threadIdx.x & 31) == __ffs(m) - 1) atomicAdd(p.n_words, __popc(m));
  }
  if (kCount) {
    const unsigned v[6] = {1u, fetches, far_fetches, iters, is_hit ? 1u : 0u, faulted ? 1u : 0u};
    const unsigned active = __activemask();
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const unsigned s = __reduce_add_sync(active, v[k]);
      if ((threadIdx.x & 31) == __ffs(active) - 1) atomicAdd(p.counters + k, (unsigned long long)s);
    }
  }
}

// FinishTracingFrame for rays still faulted at the end of the frame: shade
// with the fault's parent node as the cache holds it now.
__global__ void __launch_bounds__(kBlockThreads) finish_kernel(const __grid_constant__ TraceParams p) {
  const int i = blockIdx.x * kBlockThreads + threadIdx.x;
  if (i >= *p.n_active_in) return;
  const int pixel = p.active_in[i];
  const uchar4 col = (p.normals && p.colors) ? shade(p, p.fault_parent[pixel]) : make_uchar4(0, 0, 0, 0);
  p.image[pixel] = finish(p, col);
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
  const int total = q.fault_words + q.hit_words;
  const int per = (total + kUniqThreads - 1) / kUniqThreads;
  const int begin = min(total, (int)threadIdx.x * per), end = min(total, begin + per);
  auto word_at = [&](int k) -> uint32_t {
    return k < q.fault_words ? q.fault_bits[q.fault_words - 1 - k] : q.hit_bits[k - q.fault_words];
  };
  int cnt = 0, fcnt = 0;
  for (int k = begin; k < end; ++k) {
    const int c = __popc(word_at(k));
    cnt += c;
    if (k < q.fault_words) fcnt += c;
  }
  // block exclusive scan of cnt (and a reduction of fcnt)
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = cnt;
  for (int off = 1; off < 32; off <<= 1) {
    int v = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off) incl += v;
  }
  if (lane == 31) warp_sums[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int v = warp_sums[lane];
    int s = v;
    for (int off = 1; off < 32; off <<= 1) {
      int u = __shfl_up_sync(0xffffffffu, s, off);
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
  // totals
  int f = fcnt;
  for (int off = 16; off > 0; off >>= 1) f += __shfl_down_sync(0xffffffffu, f, off);
  __shared__ int fsum;
  if (threadIdx.x == 0) fsum = 0;
  __syncthreads();
  if (lane == 0) atomicAdd(&fsum, f);
  __syncthreads();
  if (threadIdx.x == kUniqThreads - 1) {
    int n = pos;  // last thread's end position = total set bits
    if (*q.n_words < q.total_pixels) q.unique_out[n++] = kNoHit;
    q.counts_out[0] = n;
    q.counts_out[1] = fsum;
  }
}

}  // namespace

cudaError_t launch_trace(const TraceParams& p, bool first, bool count, int max_active, cudaStream_t s) {
  if (first) {
    const int tiles = ((p.width + kTileW - 1) / kTileW) * ((p.height + kTileH - 1) / kTileH);
    const int grid = (tiles + (kBlockThreads / 32) - 1) / (kBlockThreads / 32);
    if (count) trace_kernel<true, true><<<grid, kBlockThreads, 0, s>>>(p);
    else trace_kernel<true, false><<<grid, kBlockThreads, 0, s>>>(p);
  } else {
    if (max_active <= 0) return cudaSuccess;
    const int grid = (max_active + kBlockThreads - 1) / kBlockThreads;
    if (count) trace_kernel<false, true><<<grid, kBlockThreads, 0, s>>>(p);
    else trace_kernel<false, false><<<grid, kBlockThreads, 0, s>>>(p);
  }
  return cudaGetLastError();
}

cudaError_t launch_finish(const TraceParams& p, int max_active, cudaStream_t s) {
  if (max_active <= 0) return cudaSuccess;
  finish_kernel<<<(max_active + kBlockThreads - 1) / kBlockThreads, kBlockThreads, 0, s>>>(p);
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
