// Feedback primitives: stream compaction, LSD radix sort and unique of int32
// feedback words, and an inclusive scan.
//
// The reference does this with a work-group merge sort plus log2(N/wg) global
// merge passes (rayt/GPU algorithms/kernels/merge_sort.cl:2-73), an
// adjacent-difference flag, a Hillis-Steele scan of log2(N) full passes
// (rayt/GPU algorithms/kernels/scan.cl:2-12) and a scatter
// (rayt/GPU_renderer/kernels/feedback_compression.cl:4-34).  Here:
//   compact_kernel   drops NO_HIT words, applies NodeToBlock, maps each word
//                    to an unsigned key (x ^ 0x80000000 keeps signed order) and
//                    builds all four 8-bit digit histograms in the same read,
//   digit_kernel     one stable counting pass per digit: tiles of 4096 keys,
//                    warp match_any ranking, per-digit decoupled look-back for
//                    the tile's global offsets, scatter staged through shared
//                    memory so each digit run is written contiguously,
//   unique_kernel    run starts counted per tile with a look-back prefix.
// Tile ids are taken from an atomic counter, so a tile only waits on tiles
// already claimed by running CTAs; every wait is bounded and sets an error
// flag instead of hanging.
#include "internal.h"

namespace rayt {
namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kItems = 16;
constexpr int kTile = kThreads * kItems;  // 4096 keys
constexpr int kBuckets = 256;
constexpr int kPasses = 4;
constexpr uint32_t kFlagAgg = 1u << 30, kFlagPrefix = 2u << 30, kValueMask = (1u << 30) - 1;
constexpr long long kSpinLimit = 1ll << 26;

__device__ int g_error_flag;

__device__ __forceinline__ uint32_t ld_volatile(const uint32_t* p) { return *(const volatile uint32_t*)p; }
__device__ __forceinline__ void st_volatile(uint32_t* p, uint32_t v) { *(volatile uint32_t*)p = v; }
__device__ __forceinline__ unsigned long long ld_volatile64(const unsigned long long* p) {
  return *(const volatile unsigned long long*)p;
}

// Sum of the values published by tiles before `tile` for one lane of a
// look-back table with `stride` entries per tile.
__device__ uint32_t look_back(const uint32_t* status, int tile, int stride, int lane) {
  uint32_t excl = 0;
  for (int j = tile - 1; j >= 0; --j) {
    uint32_t s;
    long long spins = 0;
    while (((s = ld_volatile(status + (size_t)j * stride + lane)) & ~kValueMask) == 0) {
      if (++spins > kSpinLimit) {
        atomicExch(&g_error_flag, 1);
        return excl;
      }
    }
    excl += s & kValueMask;
    if (s & kFlagPrefix) break;
  }
  return excl;
}

struct SortScratchLayout {
  uint32_t* keys_a;
  uint32_t* keys_b;
  uint32_t* hist;      // kPasses * kBuckets counts, then turned into offsets
  uint32_t* status;    // tiles * kBuckets look-back words
  int* tile_counter;   // kPasses + 2 counters
  int* count;          // [0] compacted keys, [1] unique count
  size_t bytes;
};

SortScratchLayout layout(void* base, int n) {
  const size_t tiles = ((size_t)n + kTile - 1) / kTile + 1;
  auto up = [](size_t v) { return (v + 255) & ~(size_t)255; };
  SortScratchLayout l{};
  size_t off = 0;
  uint8_t* b = static_cast<uint8_t*>(base);
  l.keys_a = reinterpret_cast<uint32_t*>(b + off); off += up((size_t)n * 4 + 16);
  l.keys_b = reinterpret_cast<uint32_t*>(b + off); off += up((size_t)n * 4 + 16);
  l.hist = reinterpret_cast<uint32_t*>(b + off); off += up(kPasses * kBuckets * 4);
  l.status = reinterpret_cast<uint32_t*>(b + off); off += up(tiles * kBuckets * 4);
  l.tile_counter = reinterpret_cast<int*>(b + off); off += up(16 * 4);
  l.count = reinterpret_cast<int*>(b + off); off += up(4 * 4);
  l.bytes = off;
  return l;
}

// ---- compaction + histograms -------------------------------------------------
template <bool kCompact>
__global__ void __launch_bounds__(kThreads) compact_kernel(const int32_t* words, int n, int nib, uint32_t* keys,
                                                           int* count, uint32_t* hist) {
  __shared__ uint32_t sh[kPasses][kBuckets];
  for (int i = threadIdx.x; i < kPasses * kBuckets; i += kThreads) (&sh[0][0])[i] = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  for (int base = blockIdx.x * kTile; base < n; base += gridDim.x * kTile) {
#pragma unroll 4
    for (int it = 0; it < kItems; ++it) {
      const int i = base + it * kThreads + threadIdx.x;
      int32_t w = i < n ? words[i] : kNoHit;
      bool keep = i < n;
      if (kCompact) {
        keep = keep && w != kNoHit;
        if (keep && w > 0 && nib > 0) w = ((((w >> 1) - 1) / nib + 1) << 1) | (w & 1);
      }
      const uint32_t key = (uint32_t)w ^ 0x80000000u;
      int slot = i;
      if (kCompact) {
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        int b = 0;
        if (m && lane == __ffs(m) - 1) b = atomicAdd(count, __popc(m));
        b = __shfl_sync(0xffffffffu, b, __ffs(m ? m : 1u) - 1);
        slot = b + __popc(m & ((1u << lane) - 1));
      }
      if (keep) {
        keys[slot] = key;
#pragma unroll
        for (int p = 0; p < kPasses; ++p) atomicAdd(&sh[p][(key >> (8 * p)) & 255u], 1u);
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kPasses * kBuckets; i += kThreads) {
    const uint32_t v = (&sh[0][0])[i];
    if (v) atomicAdd(hist + i, v);
  }
}

// hist counts -> exclusive offsets, one pass per warp-group of 256 threads
__global__ void hist_offsets_kernel(uint32_t* hist) {
  __shared__ uint32_t s[kBuckets];
  for (int p = 0; p < kPasses; ++p) {
    s[threadIdx.x] = hist[p * kBuckets + threadIdx.x];
    __syncthreads();
    if (threadIdx.x == 0) {
      uint32_t run = 0;
      for (int d = 0; d < kBuckets; ++d) {
        const uint32_t v = s[d];
        s[d] = run;
        run += v;
      }
    }
    __syncthreads();
    hist[p * kBuckets + threadIdx.x] = s[threadIdx.x];
    __syncthreads();
  }
}

// ---- one stable counting pass over 8 bits ------------------------------------
__global__ void __launch_bounds__(kThreads) digit_kernel(const uint32_t* in, uint32_t* out, const int* count,
                                                         int shift, const uint32_t* digit_base, uint32_t* status,
                                                         int* tile_counter, bool last, int32_t* final_out) {
  __shared__ uint32_t s_keys[kTile];
  __shared__ uint32_t s_warp[kWarps][kBuckets];
  __shared__ uint32_t s_tile_start[kBuckets];   // tile-local start of each digit run
  __shared__ uint32_t s_global[kBuckets];       // global position of each digit run
  __shared__ int s_tile;
  if (threadIdx.x == 0) s_tile = atomicAdd(tile_counter, 1);
  for (int i = threadIdx.x; i < kWarps * kBuckets; i += kThreads) (&s_warp[0][0])[i] = 0;
  __syncthreads();
  const int tile = s_tile;
  const int m = *count;
  const int base = tile * kTile;
  if (base >= m) return;
  const int valid = min(kTile, m - base);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  // warp `warp` ranks keys [warp*512, warp*512+512) of the tile, 32 per round
  uint32_t keys[kItems];
  uint32_t ranks[kItems];
#pragma unroll
  for (int r = 0; r < kItems; ++r) {
    const int li = warp * (kItems * 32) + r * 32 + lane;
    const bool ok = li < valid;
    keys[r] = ok ? in[base + li] : 0u;
    const uint32_t d = ok ? (keys[r] >> shift) & 255u : 0x100u + (uint32_t)lane;  // invalid keys match nobody
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const uint32_t before = ok ? s_warp[warp][d] : 0u;
    ranks[r] = before + __popc(peers & ((1u << lane) - 1));
    __syncwarp();
    if (ok && lane == __ffs(peers) - 1) s_warp[warp][d] = before + __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // per digit: exclusive prefix over warps, tile total, look-back
  {
    const int d = threadIdx.x;
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) {
      const uint32_t v = s_warp[w][d];
      s_warp[w][d] = run;
      run += v;
    }
    uint32_t* st = status + (size_t)tile * kBuckets + d;
    if (tile == 0) {
      st_volatile(st, kFlagPrefix | run);
      s_global[d] = digit_base[d];
    } else {
      st_volatile(st, kFlagAgg | run);
      const uint32_t excl = look_back(status, tile, kBuckets, d);
      st_volatile(st, kFlagPrefix | ((excl + run) & kValueMask));
      s_global[d] = digit_base[d] + excl;
    }
    s_tile_start[d] = run;  // temporarily the count; scanned below
  }
  __syncthreads();
  if (threadIdx.x < 32) {  // exclusive scan of 256 counts by one warp
    uint32_t v[8], sum = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) { v[k] = s_tile_start[lane * 8 + k]; sum += v[k]; }
    uint32_t incl = sum;
    for (int off = 1; off < 32; off <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, incl, off);
      if (lane >= off) incl += t;
    }
    uint32_t run = incl - sum;
#pragma unroll
    for (int k = 0; k < 8; ++k) { s_tile_start[lane * 8 + k] = run; run += v[k]; }
  }
  __syncthreads();
  // stage keys in tile-local sorted order
#pragma unroll
  for (int r = 0; r < kItems; ++r) {
    const int li = warp * (kItems * 32) + r * 32 + lane;
    if (li < valid) {
      const uint32_t d = (keys[r] >> shift) & 255u;
      s_keys[s_tile_start[d] + s_warp[warp][d] + ranks[r]] = keys[r];
    }
  }
  __syncthreads();
  // contiguous write-out of each digit run
  for (int i = threadIdx.x; i < valid; i += kThreads) {
    const uint32_t k = s_keys[i];
    const uint32_t d = (k >> shift) & 255u;
    const uint32_t pos = s_global[d] + (uint32_t)i - s_tile_start[d];
    if (pos >= (uint32_t)m) continue;  // only after a look-back gave up (error flag set)
    if (last && final_out) final_out[pos] = (int32_t)(k ^ 0x80000000u);
    else out[pos] = k;
  }
}

// ---- unique of sorted keys -----------------------------------------------------
__global__ void __launch_bounds__(kThreads) unique_kernel(const uint32_t* keys, const int* count, int n_total,
                                                          int32_t* out, uint32_t* status, int* tile_counter,
                                                          int* result) {
  __shared__ int s_tile;
  __shared__ uint32_t s_warp[kWarps];
  __shared__ uint32_t s_excl;
  if (threadIdx.x == 0) s_tile = atomicAdd(tile_counter, 1);
  __syncthreads();
  const int tile = s_tile;
  const int m = *count;
  const int base = tile * kTile;
  if (m == 0) {  // nothing but sentinels (or nothing at all)
    if (tile == 0 && threadIdx.x == 0) {
      int u = 0;
      if (n_total > 0) out[u++] = kNoHit;
      *result = u;
    }
    return;
  }
  if (base >= m) return;
  const int valid = min(kTile, m - base);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // thread t owns keys base + t*16 .. +15 (blocked)
  uint32_t flags = 0, cnt = 0;
  uint32_t k[kItems];
#pragma unroll
  for (int r = 0; r < kItems; ++r) {
    const int li = threadIdx.x * kItems + r;
    if (li < valid) {
      const int gi = base + li;
      k[r] = keys[gi];
      const bool start = gi == 0 || keys[gi - 1] != k[r];
      if (start) { flags |= 1u << r; ++cnt; }
    }
  }
  uint32_t incl = cnt;
  for (int off = 1; off < 32; off <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off) incl += t;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t run = 0;
    for (int w = 0; w < kWarps; ++w) { const uint32_t v = s_warp[w]; s_warp[w] = run; run += v; }
    uint32_t* st = status + tile;
    if (tile == 0) {
      st_volatile(st, kFlagPrefix | run);
      s_excl = 0;
    } else {
      st_volatile(st, kFlagAgg | run);
      const uint32_t excl = look_back(status, tile, 1, 0);
      st_volatile(st, kFlagPrefix | ((excl + run) & kValueMask));
      s_excl = excl;
    }
    if (base + valid == m) {  // last tile: totals and the NO_HIT sentinel
      int u = min((int)(s_excl + run), m);
      if (m < n_total) out[u++] = kNoHit;
      *result = u;
    }
  }
  __syncthreads();
  uint32_t pos = s_excl + s_warp[warp] + incl - cnt;
#pragma unroll
  for (int r = 0; r < kItems; ++r)
    if ((flags & (1u << r)) && pos < (uint32_t)m) out[pos++] = (int32_t)(k[r] ^ 0x80000000u);
}

// ---- inclusive scan (wrapping int32) ---------------------------------------------
__global__ void __launch_bounds__(kThreads) scan_kernel(int32_t* data, int n, unsigned long long* status,
                                                        int* tile_counter) {
  __shared__ int s_tile;
  __shared__ uint32_t s_warp[kWarps];
  __shared__ uint32_t s_excl;
  if (threadIdx.x == 0) s_tile = atomicAdd(tile_counter, 1);
  __syncthreads();
  const int tile = s_tile;
  const int base = tile * kTile;
  if (base >= n) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint32_t v[kItems], sum = 0;
#pragma unroll
  for (int r = 0; r < kItems; ++r) {
    const int i = base + threadIdx.x * kItems + r;
    v[r] = i < n ? (uint32_t)data[i] : 0u;
    sum += v[r];
  }
  uint32_t incl = sum;
  for (int off = 1; off < 32; off <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off) incl += t;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t run = 0;
    for (int w = 0; w < kWarps; ++w) { const uint32_t t = s_warp[w]; s_warp[w] = run; run += t; }
    const unsigned long long agg = 1ull << 32, pre = 2ull << 32;
    unsigned long long* st = status + tile;
    if (tile == 0) {
      *(volatile unsigned long long*)st = pre | run;
      s_excl = 0;
    } else {
      *(volatile unsigned long long*)st = agg | run;
      uint32_t excl = 0;
      for (int j = tile - 1; j >= 0; --j) {
        unsigned long long s;
        long long spins = 0;
        while (((s = ld_volatile64(status + j)) >> 32) == 0) {
          if (++spins > kSpinLimit) { atomicExch(&g_error_flag, 1); break; }
        }
        excl += (uint32_t)s;
        if ((s >> 32) == 2 || (s >> 32) == 0) break;
      }
      *(volatile unsigned long long*)st = pre | (uint32_t)(excl + run);
      s_excl = excl;
    }
  }
  __syncthreads();
  uint32_t run = s_excl + s_warp[warp] + incl - sum;
#pragma unroll
  for (int r = 0; r < kItems; ++r) {
    const int i = base + threadIdx.x * kItems + r;
    run += v[r];
    if (i < n) data[i] = (int32_t)run;
  }
}

int grid_for(int n) {
  const int tiles = (n + kTile - 1) / kTile;
  return tiles > 0 ? tiles : 1;
}

cudaError_t run_passes(SortScratchLayout& l, int n, uint32_t*& cur, uint32_t*& other, int32_t* final_out,
                       cudaStream_t s) {
  cudaError_t e;
  hist_offsets_kernel<<<1, kBuckets, 0, s>>>(l.hist);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  const size_t tiles = ((size_t)n + kTile - 1) / kTile + 1;
  for (int p = 0; p < kPasses; ++p) {
    if ((e = cudaMemsetAsync(l.status, 0, tiles * kBuckets * 4, s)) != cudaSuccess) return e;
    const bool last = p == kPasses - 1;
    digit_kernel<<<grid_for(n), kThreads, 0, s>>>(cur, other, l.count, 8 * p, l.hist + p * kBuckets, l.status,
                                                 l.tile_counter + p, last, last ? final_out : nullptr);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    std::swap(cur, other);
  }
  return cudaSuccess;
}

}  // namespace

int* device_error_flag() {
  int* p = nullptr;
  cudaGetSymbolAddress((void**)&p, g_error_flag);
  return p;
}

size_t sort_scratch_bytes(int n) { return layout(nullptr, n).bytes; }
size_t feedback_scratch_bytes(int n) { return layout(nullptr, n).bytes; }
size_t scan_scratch_bytes(int n) { return (((size_t)n + kTile - 1) / kTile + 1) * 8 + 256; }

cudaError_t feedback_unique_device(const int32_t* words, int n, int nib, int32_t* unique_out, int* counts_dev,
                                   void* scratch, size_t scratch_bytes, cudaStream_t s) {
  SortScratchLayout l = layout(scratch, n);
  if (scratch_bytes < l.bytes) return cudaErrorInvalidValue;
  cudaError_t e;
  if ((e = cudaMemsetAsync(l.hist, 0, kPasses * kBuckets * 4, s)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(l.tile_counter, 0, 16 * 4, s)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(l.count, 0, 4 * 4, s)) != cudaSuccess) return e;
  int grid = grid_for(n);
  if (grid > 152 * 8) grid = 152 * 8;
  compact_kernel<true><<<grid, kThreads, 0, s>>>(words, n, nib, l.keys_a, l.count, l.hist);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  uint32_t* cur = l.keys_a;
  uint32_t* other = l.keys_b;
  if ((e = run_passes(l, n, cur, other, nullptr, s)) != cudaSuccess) return e;
  const size_t tiles = ((size_t)n + kTile - 1) / kTile + 1;
  if ((e = cudaMemsetAsync(l.status, 0, tiles * 4, s)) != cudaSuccess) return e;
  unique_kernel<<<grid_for(n), kThreads, 0, s>>>(cur, l.count, n, unique_out, l.status, l.tile_counter + kPasses,
                                                 counts_dev);
  return cudaGetLastError();
}

cudaError_t sort_i32_device(int32_t* data, int n, void* scratch, size_t scratch_bytes, cudaStream_t s) {
  if (n <= 1) return cudaSuccess;
  SortScratchLayout l = layout(scratch, n);
  if (scratch_bytes < l.bytes) return cudaErrorInvalidValue;
  cudaError_t e;
  if ((e = cudaMemsetAsync(l.hist, 0, kPasses * kBuckets * 4, s)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(l.tile_counter, 0, 16 * 4, s)) != cudaSuccess) return e;
  if ((e = launch_fill_i32(l.count, n, 1, s)) != cudaSuccess) return e;
  int grid = grid_for(n);
  if (grid > 152 * 8) grid = 152 * 8;
  compact_kernel<false><<<grid, kThreads, 0, s>>>(data, n, 0, l.keys_a, nullptr, l.hist);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  uint32_t* cur = l.keys_a;
  uint32_t* other = l.keys_b;
  return run_passes(l, n, cur, other, data, s);
}

cudaError_t scan_i32_device(int32_t* data, int n, void* scratch, size_t scratch_bytes, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  if (scratch_bytes < scan_scratch_bytes(n)) return cudaErrorInvalidValue;
  const size_t tiles = ((size_t)n + kTile - 1) / kTile + 1;
  unsigned long long* status = static_cast<unsigned long long*>(scratch);
  int* counter = reinterpret_cast<int*>(static_cast<uint8_t*>(scratch) + tiles * 8);
  cudaError_t e;
  if ((e = cudaMemsetAsync(scratch, 0, tiles * 8 + 16, s)) != cudaSuccess) return e;
  scan_kernel<<<grid_for(n), kThreads, 0, s>>>(data, n, status, counter);
  return cudaGetLastError();
}

}  // namespace rayt
