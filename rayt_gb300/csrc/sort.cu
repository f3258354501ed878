// Feedback primitives: stream compaction, LSD radix sort and unique of int32
// feedback words, and an inclusive scan.
//
// The reference does this with a work-group merge sort plus log2(N/wg) global
// merge passes (rayt/GPU algorithms/kernels/merge_sort.cl:2-73), an
// adjacent-difference flag, a Hillis-Steele scan of log2(N) full passes
// (rayt/GPU algorithms/kernels/scan.cl:2-12) and a scatter
// (rayt/GPU_renderer/kernels/feedback_compression.cl:4-34).  Here:
//   compact_kernel   drops NO_HIT words, applies NodeToBlock, maps each word
//                    to an unsigned key (x ^ 0x80000000 keeps signed order),
//                    builds all four 8-bit digit histograms and the key range
//                    in the same read,
//   hist_offsets     digit offsets; for feedback unique, chooses the path:
//   bitmap path      (the keys span at most 32 values per input word and at
//                    most 2^26) a bitmap over [min, max], whose set bits read
//                    in order are the sorted unique set: range_hist and
//                    range_partition split the keys into 256 ranges
//                    (unstable), bucket_bitmap builds each range's slice of the
//                    bitmap in shared memory (so frequent keys cost no global
//                    atomics), bitmap_unique writes the set bits in order,
//   radix path       (wider ranges, and GPUSort) four stable digit_kernel
//                    passes (persistent CTAs, tiles of 8192 keys brought into
//                    shared memory by bulk async copies a tile ahead, ranking
//                    through per-warp peer masks in shared memory, per-digit
//                    decoupled look-back, scatter staged through shared
//                    memory) and unique_kernel (run starts counted per tile
//                    with a look-back prefix).
// The kernels of the path not taken return at once.  Tiles are claimed in
// order from an atomic counter, by one CTA per tile (the scan) or by
// persistent CTAs until the device-side count runs out (the digit passes,
// feedback unique), so a tile only waits on tiles claimed by running CTAs.
// The sort's look-back words
// are tagged with a per-call epoch and the pass, so its table is never
// cleared.  Every wait is bounded and sets an error flag instead of hanging.
#include <algorithm>

#include "internal.h"

namespace rayt {
namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kItems = 16;
constexpr int kTile = kThreads * kItems;  // 4096 keys
constexpr int kBuckets = 256;
constexpr int kPasses = 4;
// histogram rows: the four digits, then the range buckets' counts and offsets
constexpr int kHistRows = kPasses + 2;
constexpr int kRangeCounts = kPasses * kBuckets, kRangeOffsets = (kPasses + 1) * kBuckets;
// the range partition's per-bucket cursors, one per 128-byte line, so that
// claims on different buckets (every tile claims from most of them) never
// contend for one line
constexpr int kCursorStride = 32;
// tile counters: digit passes 0-3, unique, bitmap unique, range histogram done
// count, bucket items
constexpr int kCtrUnique = 4, kCtrBitmapUnique = 5, kCtrRangeDone = 6, kCtrBuckets = 7;
// the bitmap path keeps one range bucket's bitmap (span / 256 bits) in shared memory
constexpr int kMaxSpanLog2 = 26;
constexpr long long kSpinLimit = 1ll << 26;  // polls, a backstop to the time limit

__device__ int g_error_flag;
// Time limit of every wait on another CTA's result (ns): a correct wait ends in
// microseconds, so one that lasts this long sets g_error_flag and gives up.
__device__ unsigned long long g_wait_ns = 1000000000ull;

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
// True once a wait that began at `start` has run out of polls or time.
__device__ __forceinline__ bool wait_over(long long& spins, unsigned long long start) {
  return ++spins > kSpinLimit || ((spins & 63) == 0 && global_ns() - start > g_wait_ns);
}
// Call counter of the sort/unique kernels.  Their look-back words carry the
// tag epoch * 8 + pass, so words left by earlier calls never look published
// and the look-back table needs no clearing between passes or calls.
__device__ uint32_t g_epoch;

__device__ __forceinline__ unsigned long long ld_volatile64(const unsigned long long* p) {
  return *(const volatile unsigned long long*)p;
}
__device__ __forceinline__ void st_volatile64(unsigned long long* p, unsigned long long v) {
  *(volatile unsigned long long*)p = v;
}

// Look-back words: [63:34] tag, [33:32] 1 = tile aggregate, 2 = inclusive
// prefix, [31:0] value.
__device__ __forceinline__ unsigned long long lb_word(uint32_t tag, uint32_t flag, uint32_t value) {
  return ((unsigned long long)tag << 34) | ((unsigned long long)flag << 32) | value;
}

// Sum of the values published by tiles before `tile` for one lane of a
// look-back table with `stride` words per tile.  Predecessors are read
// kLookAhead at a time (independent loads in flight together), then consumed
// newest first until an inclusive prefix appears; a word not yet published is
// polled (bounded) before the walk goes on.
constexpr int kLookAhead = 4;
__device__ __forceinline__ bool lb_ready(unsigned long long w, uint32_t tag) {
  return (uint32_t)(w >> 34) == tag && ((w >> 32) & 3u) != 0;
}
__device__ uint32_t look_back(const unsigned long long* status, int tile, int stride, int lane, uint32_t tag) {
  uint32_t excl = 0;
  for (int j = tile - 1; j >= 0; j -= kLookAhead) {
    const int k = min(kLookAhead, j + 1);
    unsigned long long w[kLookAhead];
#pragma unroll
    for (int i = 0; i < kLookAhead; ++i)
      if (i < k) w[i] = ld_volatile64(status + (size_t)(j - i) * stride + lane);
#pragma unroll
    for (int i = 0; i < kLookAhead; ++i) {
      if (i >= k) break;
      long long spins = 0;
      const unsigned long long start = lb_ready(w[i], tag) ? 0 : global_ns();
      while (!lb_ready(w[i], tag)) {
        if (wait_over(spins, start)) {
          atomicExch(&g_error_flag, 1);
          return excl;
        }
        __nanosleep(32);  // a polling warp yields its issue slots to the SM's other warps
        w[i] = ld_volatile64(status + (size_t)(j - i) * stride + lane);
      }
      excl += (uint32_t)w[i];
      if (((w[i] >> 32) & 3u) == 2u) return excl;
    }
  }
  return excl;
}

// Sum of the values published by tiles before `tile` in a table of one word
// per tile, looked back by a whole warp: lane i reads tile j - i, so one round
// trip covers 32 predecessors.  The ready prefix of lanes up to the first
// inclusive prefix is summed; a round that meets an unpublished word first
// consumes the ready lanes before it and polls again (bounded).  All 32 lanes
// call it and get the same result.
__device__ uint32_t warp_look_back(const unsigned long long* status, int tile, uint32_t tag) {
  const int lane = threadIdx.x & 31;
  uint32_t excl = 0;
  int j = tile - 1;
  long long spins = 0;
  unsigned long long start = 0;
  while (j >= 0) {
    const int t = j - lane;
    const unsigned long long w = t >= 0 ? ld_volatile64(status + t) : 0ull;
    const bool ready = t < 0 || lb_ready(w, tag);
    const bool incl = t < 0 || (ready && ((w >> 32) & 3u) == 2u);
    const unsigned not_ready = __ballot_sync(0xffffffffu, !ready);
    const unsigned incl_mask = __ballot_sync(0xffffffffu, incl);
    const int first_nr = not_ready ? __ffs(not_ready) - 1 : 32;
    const int first_incl = incl_mask ? __ffs(incl_mask) - 1 : 32;
    const int take = first_nr <= first_incl ? first_nr : first_incl + 1;  // lanes consumed by this read
    uint32_t v = lane < take && t >= 0 ? (uint32_t)w : 0u;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    excl += v;
    if (first_incl < first_nr) return excl;  // reached an inclusive prefix (or the first tile)
    j -= take;
    if (take == 0) {  // the nearest unpublished word: poll it
      if (start == 0) start = global_ns();
      if (wait_over(spins, start)) {
        if (lane == 0) atomicExch(&g_error_flag, 1);
        return excl;
      }
    } else {
      spins = 0;
      start = 0;
    }
  }
  return excl;
}

// Called by one warp: turns the per-warp counts s_warp[0..kWarps) into
// exclusive offsets (s_warp[kWarps] = the tile's total), publishes the tile's
// aggregate, looks back, publishes the inclusive prefix and returns the
// tile's exclusive prefix.
__device__ uint32_t tile_prefix(uint32_t* s_warp, unsigned long long* status, int tile, uint32_t tag) {
  const int lane = threadIdx.x & 31;
  const uint32_t c = lane < kWarps ? s_warp[lane] : 0u;
  uint32_t incl = c;
  for (int off = 1; off < 32; off <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off) incl += t;
  }
  const uint32_t run = __shfl_sync(0xffffffffu, incl, 31);
  __syncwarp();
  if (lane < kWarps) s_warp[lane] = incl - c;
  if (lane == 0) s_warp[kWarps] = run;
  unsigned long long* st = status + tile;
  if (tile == 0) {
    if (lane == 0) st_volatile64(st, lb_word(tag, 2u, run));
    return 0;
  }
  if (lane == 0) st_volatile64(st, lb_word(tag, 1u, run));
  const uint32_t excl = warp_look_back(status, tile, tag);
  if (lane == 0) st_volatile64(st, lb_word(tag, 2u, excl + run));
  return excl;
}

struct SortScratchLayout {
  uint32_t* keys_a;
  uint32_t* keys_b;
  uint32_t* hist;                 // kPasses * kBuckets counts, then turned into offsets
  unsigned long long* status;     // tiles * kBuckets tagged look-back words
  int* tile_counter;              // kPasses + 2 counters
  int* count;                     // [0] compacted keys, [1] unique count
  uint32_t* cursors;              // kBuckets range-partition cursors, kCursorStride words apart
  uint32_t* range;                // [0] max of ~key, [1] max key, [2] path (kBitmapPath), [3] bitmap words,
                                  // [4] range-bucket shift
  size_t bitmap_bits;             // unique-by-bitmap capacity: the bitmap lives in keys_b
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
  l.hist = reinterpret_cast<uint32_t*>(b + off); off += up(kHistRows * kBuckets * 4);
  l.status = reinterpret_cast<unsigned long long*>(b + off); off += up(tiles * kBuckets * 8);
  l.tile_counter = reinterpret_cast<int*>(b + off); off += up(16 * 4);
  l.count = reinterpret_cast<int*>(b + off); off += up(4 * 4);
  l.range = reinterpret_cast<uint32_t*>(b + off); off += up(8 * 4);
  l.cursors = reinterpret_cast<uint32_t*>(b + off); off += up(kBuckets * kCursorStride * 4);
  l.bitmap_bits = (((size_t)n * 4 + 16) / 16) * 16 * 8;  // whole 16-byte units of keys_b
  l.bytes = off;
  return l;
}

// ---- compaction + histograms -------------------------------------------------
// NodeToBlock's division of a node index (0 <= x < 2^31) by nodes_in_block d
// without a hardware divide: q = floor(x * M / 2^64) with M = ceil(2^64 / d).
// For x < 2^31 and d < 2^32 the product's excess x * (M - 2^64/d) / 2^64 is
// below 1/d, so the floor equals floor(x / d) exactly (Granlund & Montgomery,
// "Division by invariant integers using multiplication", 1994).  d = 1 passes
// x through.
struct Divider {
  unsigned long long m;  // 0: d == 1
};
inline Divider make_divider(uint32_t d) {
  Divider v;
  v.m = d <= 1 ? 0ull : ~0ull / d + 1ull;
  return v;
}
__device__ __forceinline__ uint32_t divide(uint32_t x, Divider v) {
  return v.m ? (uint32_t)__umul64hi((unsigned long long)x, v.m) : x;
}

// Tiles of 4096 words, grid-strided over the resident CTAs.  A thread owns 16
// words of a tile, read as four 16-byte loads when `words` is 16-byte aligned
// (scalar loads otherwise, and for the last, partial tile).  The next tile's
// loads are issued before the current tile is processed, so memory latency
// overlaps the work.  The per-word loop only drops NO_HIT words: each warp
// appends the words it keeps to its own 1024-word region of shared memory.
// NodeToBlock, the key mapping and the four 8-bit digit histograms run when
// the regions are flushed, on the kept words with every lane busy (at 10%
// kept words, doing them per word cost three quarters of the instructions of
// an issue-bound kernel).  The CTA flushes, claiming its output range with
// one atomicAdd on `claim`, only when a region could not take another tile or
// after its last tile; the regions go out coalesced.  Input words are read
// once, with evict-first loads, so they do not push the compacted keys (read
// again by the digit passes) out of L2.  Keys leave a warp in any order: only
// sorted keys leave the sort.
constexpr int kRegion = 1024;  // keys per warp region; a tile adds at most 512

template <bool kVec>
__device__ __forceinline__ void load_words(int32_t (&w)[kItems], const int32_t* words, uint32_t n, uint32_t first) {
  // thread's words: first + r * 128 + j, r, j = 0..3
  if (kVec && first + (kItems * 32 - 4 * (threadIdx.x & 31)) <= n) {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int4 v = __ldcs(reinterpret_cast<const int4*>(words + first + r * 128));
      w[4 * r] = v.x; w[4 * r + 1] = v.y; w[4 * r + 2] = v.z; w[4 * r + 3] = v.w;
    }
  } else {
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const uint32_t i = first + r * 128 + j;
        w[4 * r + j] = i < n ? __ldcs(words + i) : kNoHit;
      }
  }
}

template <bool kCompact, bool kVec>
__global__ void __launch_bounds__(kThreads) compact_kernel(const int32_t* words, int n_words, int nib, Divider div,
                                                           uint32_t* keys, int* claim, uint32_t* hist,
                                                           uint32_t* range) {
  __shared__ uint32_t sh[kPasses][kBuckets];
  __shared__ uint32_t s_range[2];  // max of ~key (so the minimum), max key
  __shared__ uint32_t s_keys[kWarps * kRegion];
  __shared__ uint32_t s_fill[2][kWarps];  // by tile parity: a warp may write the next tile's entry early
  __shared__ uint32_t s_base;
  for (int i = threadIdx.x; i < kPasses * kBuckets; i += kThreads) (&sh[0][0])[i] = 0;
  if (threadIdx.x < 2) s_range[threadIdx.x] = 0;
  uint32_t not_min = 0, max_key = 0;
  const uint32_t n = (uint32_t)n_words;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned lt = (1u << lane) - 1;
  const uint32_t mine = warp * (kItems * 32) + lane * 4;  // offset of the thread's first word in a tile
  uint32_t* region = s_keys + warp * kRegion;
  const uint32_t stride = gridDim.x * kTile;  // tiles of n < 2^31 words: base + stride stays below 2^32
  int32_t cur[kItems], nxt[kItems];
  uint32_t base = blockIdx.x * kTile;
  load_words<kVec>(cur, words, n, base + mine);
  uint32_t fill = 0;  // keys in this warp's region
  __syncthreads();    // histograms zeroed
  for (int parity = 0; base < n; base += stride, parity ^= 1) {
    const uint32_t next = base + stride;
    load_words<kVec>(nxt, words, n, next + mine);
#pragma unroll
    for (int q = 0; q < kItems; ++q) {
      const bool keep = kCompact ? cur[q] != kNoHit  // words past the end were loaded as NO_HIT
                                 : base + mine + (q >> 2) * 128 + (q & 3) < n;
      const unsigned mask = __ballot_sync(0xffffffffu, keep);
      if (keep) region[fill + __popc(mask & lt)] = (uint32_t)cur[q];
      fill += __popc(mask);
    }
#pragma unroll
    for (int q = 0; q < kItems; ++q) cur[q] = nxt[q];
    if (lane == 0) s_fill[parity][warp] = fill;
    __syncthreads();
    bool flush = next >= n;
#pragma unroll
    for (int k = 0; k < kWarps; ++k) flush = flush || s_fill[parity][k] > kRegion - kItems * 32;
    if (!flush) continue;
    if (threadIdx.x == 0) {
      uint32_t total = 0;
      for (int k = 0; k < kWarps; ++k) total += s_fill[parity][k];
      s_base = (uint32_t)atomicAdd(claim, (int)total);
    }
    __syncthreads();
    uint32_t out = s_base;
    for (int k = 0; k < warp; ++k) out += s_fill[parity][k];
    for (uint32_t j = lane; j < fill; j += 32) {
      int32_t v = (int32_t)region[j];
      if (kCompact && v > 0 && nib > 0) v = (int32_t)(((divide((uint32_t)((v >> 1) - 1), div) + 1) << 1) | (v & 1));
      const uint32_t key = (uint32_t)v ^ 0x80000000u;
#pragma unroll
      for (int p = 0; p < kPasses; ++p) atomicAdd(&sh[p][(key >> (8 * p)) & 255u], 1u);
      not_min = max(not_min, ~key);
      max_key = max(max_key, key);
      keys[out + j] = key;
    }
    fill = 0;
    __syncthreads();  // s_base is reused by the next flush
  }
  if (range) {
    not_min = __reduce_max_sync(0xffffffffu, not_min);
    max_key = __reduce_max_sync(0xffffffffu, max_key);
    if (lane == 0) {
      atomicMax(&s_range[0], not_min);
      atomicMax(&s_range[1], max_key);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kPasses * kBuckets; i += kThreads) {
    const uint32_t v = (&sh[0][0])[i];
    if (v) atomicAdd(hist + i, v);
  }
  if (range && threadIdx.x < 2 && s_range[threadIdx.x]) atomicMax(range + threadIdx.x, s_range[threadIdx.x]);
}

// Compaction launch: 16-byte loads when `words` allows them.
template <bool kCompact>
cudaError_t launch_compact(int grid, const int32_t* words, int n, int nib, uint32_t* keys, int* claim,
                           uint32_t* hist, uint32_t* range, cudaStream_t s) {
  const Divider div = make_divider((uint32_t)nib);
  if ((reinterpret_cast<uintptr_t>(words) & 15) == 0)
    compact_kernel<kCompact, true><<<grid, kThreads, 0, s>>>(words, n, nib, div, keys, claim, hist, range);
  else
    compact_kernel<kCompact, false><<<grid, kThreads, 0, s>>>(words, n, nib, div, keys, claim, hist, range);
  return cudaGetLastError();
}

// Unique-by-bitmap: when the kept keys span at most `bitmap_bits` values (and
// at most 2^26), a bitmap over [min, max] read in order is the sorted unique
// set, and the radix passes are skipped.  range[2] holds the choice.
constexpr uint32_t kBitmapPath = 1;

// hist counts -> exclusive offsets (one CTA of 256 threads); opens a new epoch
// for the look-back words of this call.  With `range`, also chooses between
// the radix passes and the bitmap.
__global__ void hist_offsets_kernel(uint32_t* hist, const int* count, uint32_t* range,
                                    unsigned long long bitmap_bits) {
  if (range && threadIdx.x == 0) {
    const int m = *count;
    const unsigned long long span = (unsigned long long)range[1] - (unsigned long long)(~range[0]) + 1ull;
    const bool bitmap = m > 0 && span <= bitmap_bits && span <= (1ull << kMaxSpanLog2);
    range[2] = bitmap ? kBitmapPath : 0u;
    range[3] = bitmap ? (uint32_t)((span + 31) / 32) : 0u;
    const int bits = span > 1 ? 64 - __clzll((long long)(span - 1)) : 0;  // bits of the largest key - min
    range[4] = bits > 8 ? (uint32_t)(bits - 8) : 0u;
  }
  // warp p scans digit row p: 8 counts per lane, then a warp scan
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp < kPasses) {
    uint32_t* row = hist + warp * kBuckets;
    uint32_t v[8], sum = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) { v[k] = row[lane * 8 + k]; sum += v[k]; }
    uint32_t incl = sum;
    for (int off = 1; off < 32; off <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, incl, off);
      if (lane >= off) incl += t;
    }
    uint32_t run = incl - sum;
#pragma unroll
    for (int k = 0; k < 8; ++k) { row[lane * 8 + k] = run; run += v[k]; }
  }
  if (threadIdx.x == 0) g_epoch = (g_epoch + 1) & ((1u << 27) - 1);
}

// ---- bulk async copies into shared memory ------------------------------------
// A tile of keys arrives in shared memory by one cp.async.bulk (the copy
// engine moves it; no thread holds it in registers), and its completion is an
// mbarrier phase with a transaction count.
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
}
// Makes the barriers' initialisation visible to the copy engine.
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
// Waits for the phase of `bar` with parity `parity`; false (error flag set)
// when the wait runs out.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  long long spins = 0;
  const unsigned long long start = global_ns();
  while (!mbar_try_wait(bar, parity)) {
    if (wait_over(spins, start)) {
      atomicExch(&g_error_flag, 1);
      return false;
    }
  }
  return true;
}
// Copies `bytes` (a multiple of 16, both addresses 16-byte aligned) from
// global to shared memory; the copy completes the current phase of `bar`.
// Shared memory last touched by the threads is handed to the copy engine by
// the proxy fence.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, unsigned long long* bar) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

// ---- one stable counting pass over 8 bits ------------------------------------
// Persistent CTAs of 512 threads claim tiles of 8192 keys in order from
// tile_counter until the keys run out (the count is read on the device: for
// feedback unique only the compaction knows it).  A CTA claims its next tile
// when it starts the current one, and the next tile's keys come into the
// other half of a double buffer by one bulk async copy while the current tile
// is ranked, looked back and written out.  (A next tile is always above its
// CTA's current one, so the lowest unfinished tile is always some CTA's
// current tile and every look-back ends.)  Per tile:
// - ranking (stable), a warp's 512 keys in 16 rounds of 32: the lanes of a
//   round holding the same digit find one another through a per-warp table of
//   peer masks in shared memory (each lane ORs its bit into its digit's word;
//   one shared atomic instead of eight ballots and the selects between them,
//   which had made the pass issue-bound at 4.9 warp instructions per key); the
//   group's first lane adds the group to the warp's count of that digit with
//   one atomic, clears the mask word and shares the old count; ranks follow
//   lane order inside the group, and rounds apply in order;
// - the per-digit counts over warps become offsets; the tile's count per digit
//   is published at once (the look-back's aggregate); the 256 counts are
//   scanned into the tile-local start of each digit run, which is added into
//   the per-warp offsets;
// - the keys (held in registers since the ranking) are staged in tile-local
//   sorted order in place, in the buffer they came from (one shared load of
//   the warp's offset per key);
// - one thread per digit looks back for the digit run's global position;
// - each digit run goes out contiguously.
// 8192-key tiles halve the look-back's walk per key twice over 4096-key ones:
// half the tiles, and half as many tiles in flight behind a tile's
// predecessors.  With `range` (feedback unique), skipped on the bitmap path.
constexpr int kDigitThreads = 512;
constexpr int kDigitWarps = kDigitThreads / 32;
constexpr int kDigitTile = kDigitThreads * kItems;  // 8192 keys
// shared memory: two tile buffers, per-warp counts and peer masks, the run
// starts and offsets, 8 warp totals, two mbarriers and the next tile's index
constexpr int kDigitSmemBytes = (2 * kDigitTile + 2 * kDigitWarps * kBuckets + 2 * kBuckets + 8) * 4 + 32;

// Bytes copied for tile t of m keys: the partial last tile is rounded up to 16
// bytes (the key buffers carry 16 bytes of padding).
__device__ __forceinline__ uint32_t digit_tile_bytes(int t, int m) {
  const int valid = min(kDigitTile, m - t * kDigitTile);
  return (uint32_t)((valid * 4 + 15) & ~15);
}

template <bool kFull>
__device__ __forceinline__ void rank_tile(const uint32_t* s_tile_keys, uint32_t (&keys)[kItems],
                                          uint32_t (&ranks)[kItems / 2], uint32_t* s_count, uint32_t* s_peers,
                                          int shift, int valid, int w0, int lane) {
#pragma unroll
  for (int r = 0; r < kItems; ++r) {
    const int li = w0 + r * 32 + lane;
    const bool ok = kFull || li < valid;
    keys[r] = s_tile_keys[li];  // past `valid` a stale word, not used
    const uint32_t d = (keys[r] >> shift) & 255u;
    if (ok) atomicOr(&s_peers[d], 1u << lane);
    __syncwarp();
    const unsigned peers = ok ? s_peers[d] : (1u << lane);
    __syncwarp();  // every lane has read its mask before the leader clears it
    const int leader = __ffs(peers) - 1;
    uint32_t before = 0;
    if (ok && lane == leader) {
      s_peers[d] = 0u;
      before = atomicAdd(&s_count[d], (uint32_t)__popc(peers));
    }
    before = __shfl_sync(0xffffffffu, before, leader);
    __syncwarp();  // the cleared mask is in place before the next round's ORs
    const uint32_t rank = before + __popc(peers & ((1u << lane) - 1));
    ranks[r / 2] = (r & 1) ? ranks[r / 2] | (rank << 16) : rank;  // two 16-bit ranks (< 512) per word
  }
}

__global__ void __launch_bounds__(kDigitThreads, 2) digit_kernel(const uint32_t* in, uint32_t* out, const int* count,
                                                              int shift, const uint32_t* digit_base,
                                                              unsigned long long* status, int* tile_counter, int pass,
                                                              bool last, int32_t* final_out, const uint32_t* range) {
  extern __shared__ __align__(128) uint32_t smem[];
  uint32_t* s_warp = smem + 2 * kDigitTile;         // [warp][digit] counts, then offsets
  uint32_t* s_peers = s_warp + kDigitWarps * kBuckets;  // [warp][digit] peer masks of a round
  uint32_t* s_start = s_peers + kDigitWarps * kBuckets; // tile-local start of each digit run
  uint32_t* s_off = s_start + kBuckets;                 // global position - tile-local position
  uint32_t* s_wsum = s_off + kBuckets;                  // per digit warp: its digits' counts summed
  unsigned long long* s_bar = reinterpret_cast<unsigned long long*>(s_wsum + 8);
  int* s_next = reinterpret_cast<int*>(s_bar + 2);
  if (range && range[2] == kBitmapPath) return;
  const int m = *count;
  const uint32_t tag = g_epoch * 8u + (uint32_t)pass;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int w0 = warp * (kItems * 32);  // warp `warp` ranks keys [w0, w0 + 512) of a tile
  for (int i = threadIdx.x; i < 2 * kDigitWarps * kBuckets; i += kDigitThreads) s_warp[i] = 0;
  if (threadIdx.x == 0) {
    mbar_init(&s_bar[0]);
    mbar_init(&s_bar[1]);
    mbar_init_fence();
    const int t = atomicAdd(tile_counter, 1);
    *s_next = t;
    if ((long long)t * kDigitTile < m) bulk_load(smem, in + (size_t)t * kDigitTile, digit_tile_bytes(t, m), &s_bar[0]);
  }
  __syncthreads();
  int tile = *s_next;
  __syncthreads();  // every thread has read s_next before it is rewritten
  uint32_t phases = 0u;  // bit b: parity of buffer b's next completion
  int b = 0;
  while ((long long)tile * kDigitTile < m) {
    const int valid = min(kDigitTile, m - tile * kDigitTile);
    uint32_t* s_tile_keys = smem + b * kDigitTile;
    if (threadIdx.x == 0) *s_next = atomicAdd(tile_counter, 1);  // read after (A)
    const bool landed = mbar_wait(&s_bar[b], (phases >> b) & 1u);
    uint32_t keys[kItems], ranks[kItems / 2];
    if (valid == kDigitTile)
      rank_tile<true>(s_tile_keys, keys, ranks, s_warp + warp * kBuckets, s_peers + warp * kBuckets, shift, valid, w0,
                      lane);
    else
      rank_tile<false>(s_tile_keys, keys, ranks, s_warp + warp * kBuckets, s_peers + warp * kBuckets, shift, valid,
                       w0, lane);
    // (A) every read of this buffer is done.  A wait that ran out (error flag
    // set) ends the CTA, after its copy has landed (bounded), so that nothing
    // lands in shared memory after the CTA has left.
    if (!__syncthreads_and(landed)) {
      if (threadIdx.x == 0) mbar_wait(&s_bar[b], (phases >> b) & 1u);
      return;
    }
    phases ^= 1u << b;
    const int next = *s_next;
    if (threadIdx.x == 0 && (long long)next * kDigitTile < m)  // the other buffer was drained before the last tile ended
      bulk_load(smem + (b ^ 1) * kDigitTile, in + (size_t)next * kDigitTile, digit_tile_bytes(next, m), &s_bar[b ^ 1]);
    // per digit: exclusive prefix over warps and the tile's count; the count
    // is published at once so later tiles' look-backs can pass this one
    // The 256 digit threads (8 warps) also scan the tile's counts: within the
    // warp by shuffles, across warps through the warp totals after (B).
    uint32_t tile_count = 0, incl = 0;
    if (threadIdx.x < kBuckets) {
      const int d = threadIdx.x;
      uint32_t run = 0;
#pragma unroll
      for (int w = 0; w < kDigitWarps; ++w) {
        const uint32_t v = s_warp[w * kBuckets + d];
        s_warp[w * kBuckets + d] = run;
        run += v;
      }
      tile_count = run;
      st_volatile64(status + (size_t)tile * kBuckets + d, lb_word(tag, tile == 0 ? 2u : 1u, run));
      incl = run;
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += t;
      }
      if (lane == 31) s_wsum[warp] = incl;
    }
    __syncthreads();  // (B)
    // tile-local start of each digit run, folded into the per-warp offsets so
    // that staging reads one word per key
    if (threadIdx.x < kBuckets) {
      const int d = threadIdx.x;
      uint32_t start = incl - tile_count;
      for (int k = 0; k < warp; ++k) start += s_wsum[k];
      s_start[d] = start;
#pragma unroll
      for (int w = 0; w < kDigitWarps; ++w) s_warp[w * kBuckets + d] += start;
    }
    __syncthreads();  // (C)
    {  // stage keys in tile-local sorted order, in place: every read of the buffer finished before (A)
      const uint32_t* s_pos = s_warp + warp * kBuckets;
#pragma unroll
      for (int r = 0; r < kItems; ++r) {
        const int li = w0 + r * 32 + lane;
        if (valid == kDigitTile || li < valid) {
          const uint32_t k = keys[r];
          const uint32_t rank = (r & 1) ? ranks[r / 2] >> 16 : ranks[r / 2] & 0xffffu;
          s_tile_keys[s_pos[(k >> shift) & 255u] + rank] = k;
        }
      }
    }
    // global position of each digit run: look-back over earlier tiles
    if (threadIdx.x < kBuckets) {
      const int d = threadIdx.x;
      uint32_t excl = 0;
      if (tile != 0) {
        excl = look_back(status, tile, kBuckets, d, tag);
        st_volatile64(status + (size_t)tile * kBuckets + d, lb_word(tag, 2u, excl + tile_count));
      }
      s_off[d] = digit_base[d] + excl - s_start[d];
    }
    __syncthreads();  // (D)
    // contiguous write-out of each digit run; the counts are cleared for the
    // next tile on the way (the write-out does not read them)
    for (int i = threadIdx.x; i < kDigitWarps * kBuckets; i += kDigitThreads) s_warp[i] = 0;
    if (valid == kDigitTile) {
#pragma unroll
      for (int k = 0; k < kItems; ++k) {
        const int i = threadIdx.x + k * kDigitThreads;
        const uint32_t key = s_tile_keys[i];
        const uint32_t pos = s_off[(key >> shift) & 255u] + (uint32_t)i;
        if (pos >= (uint32_t)m) continue;  // only after a look-back gave up (error flag set)
        if (last && final_out) final_out[pos] = (int32_t)(key ^ 0x80000000u);
        else out[pos] = key;
      }
    } else {
      for (int i = threadIdx.x; i < valid; i += kDigitThreads) {
        const uint32_t key = s_tile_keys[i];
        const uint32_t pos = s_off[(key >> shift) & 255u] + (uint32_t)i;
        if (pos >= (uint32_t)m) continue;
        if (last && final_out) final_out[pos] = (int32_t)(key ^ 0x80000000u);
        else out[pos] = key;
      }
    }
    __syncthreads();  // (E) the buffer, the run starts and offsets and the counts are reused
    tile = next;
    b ^= 1;
  }
}

// ---- unique of sorted keys -----------------------------------------------------
// Persistent like digit_kernel, and pipelined the same way: a tile's run-start
// keys are compacted into shared memory (each warp into its own range), the
// next tile (claimed at the start of this one) is loaded, and only then does
// the tile's look-back for its output position run.
__global__ void __launch_bounds__(kThreads) unique_kernel(const uint32_t* keys, const int* count, int n_total,
                                                          int32_t* out, unsigned long long* status,
                                                          int* tile_counter, int* result, const uint32_t* range) {
  __shared__ int s_tile;
  __shared__ uint32_t s_warp[kWarps + 1];
  __shared__ uint32_t s_excl;
  __shared__ uint32_t s_starts[kTile];
  if (range[2] == kBitmapPath) return;
  const int m = *count;
  const uint32_t tag = g_epoch * 8u + 4u;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (m == 0) {  // nothing but sentinels (or nothing at all)
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      int u = 0;
      if (n_total > 0) out[u++] = kNoHit;
      *result = u;
    }
    return;
  }
  // warp `warp` owns keys [w0, w0 + 512) of a tile, 32 per round (coalesced);
  // a key starts a run when it differs from the key before it
  const int w0 = warp * (kItems * 32);
  const unsigned lt = (1u << lane) - 1;
  if (threadIdx.x == 0) s_tile = atomicAdd(tile_counter, 1);
  __syncthreads();
  int tile = s_tile;
  __syncthreads();  // every thread has read s_tile
  if ((long long)tile * kTile >= m) return;
  uint32_t k[kItems];
  uint32_t prev_last = 0;  // the key before this warp's first key
  {
    const long long b = (long long)tile * kTile + w0;
#pragma unroll
    for (int r = 0; r < kItems; ++r) k[r] = b + r * 32 + lane < m ? __ldg(keys + b + r * 32 + lane) : 0u;
    if (lane == 0 && b > 0 && b < m) prev_last = __ldg(keys + b - 1);
  }
  for (;;) {
    const int base = tile * kTile;
    const int valid = min(kTile, m - base);
    if (threadIdx.x == 0) s_tile = atomicAdd(tile_counter, 1);  // the next tile
    uint32_t cnt = 0;
#pragma unroll
    for (int r = 0; r < kItems; ++r) {
      const int li = w0 + r * 32 + lane;
      uint32_t prev = __shfl_up_sync(0xffffffffu, k[r], 1);
      if (lane == 0) prev = prev_last;
      prev_last = __shfl_sync(0xffffffffu, k[r], 31);
      const bool start = li < valid && (base + li == 0 || prev != k[r]);
      const unsigned starts = __ballot_sync(0xffffffffu, start);
      if (start) s_starts[w0 + cnt + __popc(starts & lt)] = k[r];
      cnt += __popc(starts);
    }
    if (lane == 0) s_warp[warp] = cnt;
    __syncthreads();
    const int next = s_tile;
    const long long next_base = (long long)next * kTile;
    {  // the next tile's keys are in flight during the look-back and write-out
      const long long b = next_base + w0;
#pragma unroll
      for (int r = 0; r < kItems; ++r) k[r] = b + r * 32 + lane < m ? __ldg(keys + b + r * 32 + lane) : 0u;
      prev_last = lane == 0 && b > 0 && b < m ? __ldg(keys + b - 1) : 0u;
    }
    if (warp == 0) {
      const uint32_t excl = tile_prefix(s_warp, status, tile, tag);
      if (lane == 0 && base + valid == m) {  // last tile: totals and the NO_HIT sentinel
        int u = min((int)(excl + s_warp[kWarps]), m);
        if (m < n_total) out[u++] = kNoHit;
        *result = u;
      }
      if (lane == 0) s_excl = excl;
    }
    __syncthreads();
    const uint32_t pos = s_excl + s_warp[warp];
    for (uint32_t j = lane; j < cnt; j += 32)
      if (pos + j < (uint32_t)m) out[pos + j] = (int32_t)(s_starts[w0 + j] ^ 0x80000000u);
    __syncthreads();  // shared state is reused by the next tile
    if (next_base >= m) return;
    tile = next;
  }
}

// ---- unique by bitmap ------------------------------------------------------------
// Bit b of the bitmap stands for key min + b.  All three kernels return at once
// on the radix path.
__global__ void __launch_bounds__(kThreads) bitmap_clear_kernel(const uint32_t* range, uint4* bitmap) {
  if (range[2] != kBitmapPath) return;
  const size_t n4 = ((size_t)range[3] + 3) / 4;
  for (size_t i = blockIdx.x * (size_t)kThreads + threadIdx.x; i < n4; i += (size_t)gridDim.x * kThreads)
    bitmap[i] = make_uint4(0u, 0u, 0u, 0u);
}

// Histogram of the range buckets (top 8 bits of key - min) of the kept keys;
// the last CTA to finish turns the counts into offsets (no CTA waits).
__global__ void __launch_bounds__(kThreads) range_hist_kernel(const uint32_t* keys, const int* count,
                                                              const uint32_t* range, uint32_t* hist, int* done,
                                                              uint32_t* cursors) {
  __shared__ uint32_t sh[kBuckets];
  __shared__ bool s_last;
  if (range[2] != kBitmapPath) return;
  const uint32_t m = (uint32_t)*count, lo = ~range[0];
  const int shift = (int)range[4];
  sh[threadIdx.x] = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  for (uint32_t i0 = blockIdx.x * kThreads * 8u; i0 < m; i0 += gridDim.x * kThreads * 8u) {
    uint32_t k[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const uint32_t i = i0 + r * kThreads + threadIdx.x;
      k[r] = i < m ? __ldg(keys + i) : 0u;
    }
#pragma unroll
    for (int r = 0; r < 8; ++r) {  // one shared atomic per distinct bucket per warp: frequent keys share one
      const bool ok = i0 + r * kThreads + threadIdx.x < m;
      const uint32_t b = ok ? (k[r] - lo) >> shift : 0x100u + (uint32_t)lane;
      const unsigned peers = __match_any_sync(0xffffffffu, b);
      if (ok && lane == __ffs(peers) - 1) atomicAdd(&sh[b], (uint32_t)__popc(peers));
    }
  }
  __syncthreads();
  if (sh[threadIdx.x]) atomicAdd(hist + kRangeCounts + threadIdx.x, sh[threadIdx.x]);
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(done, 1) == (int)gridDim.x - 1;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  const uint32_t c = *(volatile uint32_t*)(hist + kRangeCounts + threadIdx.x);
  sh[threadIdx.x] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t run = 0;
    for (int d = 0; d < kBuckets; ++d) { const uint32_t v = sh[d]; sh[d] = run; run += v; }
  }
  __syncthreads();
  hist[kRangeOffsets + threadIdx.x] = sh[threadIdx.x];
  cursors[threadIdx.x * kCursorStride] = sh[threadIdx.x];
}

// Range partition of the bitmap path.  Unstable (the bitmap does not care
// about order): tiles of 4096 keys, grid-strided; a key's slot in its range
// bucket comes from a shared per-tile count (one atomic per distinct bucket
// per warp), the tile claims one range per bucket from the bucket's cursor,
// and the keys are staged in shared memory in bucket order so each bucket's
// run goes out contiguously while the next tile's keys load.  No CTA waits on
// another.
__global__ void __launch_bounds__(kThreads, 4) range_partition_kernel(const uint32_t* in, uint32_t* out,
                                                                   const int* count, const uint32_t* range,
                                                                   uint32_t* cursors) {
  __shared__ uint32_t s_cnt[kBuckets];    // per-tile count, then the tile-local start of each bucket
  __shared__ uint32_t s_base[kBuckets];   // global start of each bucket's run
  __shared__ uint32_t s_keys[kTile];
  if (range[2] != kBitmapPath) return;
  const uint32_t m = (uint32_t)*count, lo = ~range[0];
  const int shift = (int)range[4];
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1;
  const uint32_t stride = gridDim.x * (uint32_t)kTile;
  uint32_t k[kItems];
#pragma unroll
  for (int r = 0; r < kItems; ++r) {
    const uint32_t i = blockIdx.x * (uint32_t)kTile + r * kThreads + threadIdx.x;
    k[r] = i < m ? __ldg(in + i) : 0u;
  }
  for (uint32_t base = blockIdx.x * (uint32_t)kTile; base < m; base += stride) {
    const uint32_t valid = min((uint32_t)kTile, m - base);
    s_cnt[threadIdx.x] = 0;
    __syncthreads();
    uint32_t slot[kItems / 2];  // two 16-bit slots (< 4096) per word
#pragma unroll
    for (int r = 0; r < kItems; ++r) {
      const bool ok = r * kThreads + threadIdx.x < valid;
      const uint32_t b = ok ? (k[r] - lo) >> shift : 0x100u + (uint32_t)lane;
      const unsigned peers = __match_any_sync(0xffffffffu, b);
      const int leader = __ffs(peers) - 1;
      uint32_t first = 0;
      if (ok && lane == leader) first = atomicAdd(&s_cnt[b], (uint32_t)__popc(peers));
      first = __shfl_sync(0xffffffffu, first, leader);
      const uint32_t sl = first + __popc(peers & lt);
      slot[r / 2] = (r & 1) ? slot[r / 2] | (sl << 16) : sl;
    }
    __syncthreads();
    {
      const uint32_t c = s_cnt[threadIdx.x];
      if (c) s_base[threadIdx.x] = atomicAdd(cursors + threadIdx.x * kCursorStride, c);
    }
    __syncthreads();
    if (threadIdx.x < 32) {  // tile-local bucket starts: exclusive scan of 256 counts by one warp
      uint32_t v[8], sum = 0;
#pragma unroll
      for (int q = 0; q < 8; ++q) { v[q] = s_cnt[lane * 8 + q]; sum += v[q]; }
      uint32_t incl = sum;
      for (int off = 1; off < 32; off <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += t;
      }
      uint32_t run = incl - sum;
      __syncwarp();
#pragma unroll
      for (int q = 0; q < 8; ++q) { s_cnt[lane * 8 + q] = run; run += v[q]; }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kItems; ++r)
      if (r * kThreads + threadIdx.x < valid)
        s_keys[s_cnt[(k[r] - lo) >> shift] + ((r & 1) ? slot[r / 2] >> 16 : slot[r / 2] & 0xffffu)] = k[r];
    // the next tile's keys are in flight during the write-out
#pragma unroll
    for (int r = 0; r < kItems; ++r) {
      const uint32_t i = base + stride + r * kThreads + threadIdx.x;
      k[r] = i < m ? __ldg(in + i) : 0u;
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < valid; i += kThreads) {
      const uint32_t key = s_keys[i];
      const uint32_t b = (key - lo) >> shift;
      out[s_base[b] + i - s_cnt[b]] = key;
    }
    __syncthreads();  // shared state is reused by the next tile
  }
}

// One range bucket's bitmap slice (at most 2^18 bits) built in shared memory
// from its partitioned keys (a shared atomicOr only for bits not yet set),
// then OR-ed into the global bitmap word by word
// (only words with bits set; a word shared with a neighbouring bucket is
// combined by the atomic).  Work items are chunks of kChunk keys of one
// bucket, claimed from a counter, so a bucket holding most keys (feedback is
// Zipf-like) is spread over many CTAs.
constexpr int kChunk = 16384;
constexpr int kSliceWords = (1 << (kMaxSpanLog2 - 8)) / 32 + 1;
__global__ void __launch_bounds__(kThreads) bucket_bitmap_kernel(const uint32_t* keys, const uint32_t* range,
                                                                 const uint32_t* hist, uint32_t* bitmap,
                                                                 int* item_counter) {
  __shared__ uint32_t s_bits[kSliceWords];
  __shared__ uint32_t s_first[kBuckets + 1];  // first item of each bucket; [256] = all items
  __shared__ int s_item;
  if (range[2] != kBitmapPath) return;
  const uint32_t lo = ~range[0];
  const int shift = (int)range[4];
  const int lane = threadIdx.x & 31;
  {  // items per bucket, scanned by one warp
    const uint32_t c = hist[kRangeCounts + threadIdx.x];
    s_first[threadIdx.x] = (c + kChunk - 1) / kChunk;
    __syncthreads();
    if (threadIdx.x < 32) {
      uint32_t v[8], sum = 0;
#pragma unroll
      for (int k = 0; k < 8; ++k) { v[k] = s_first[lane * 8 + k]; sum += v[k]; }
      uint32_t incl = sum;
      for (int off = 1; off < 32; off <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += t;
      }
      uint32_t run = incl - sum;
      __syncwarp();
#pragma unroll
      for (int k = 0; k < 8; ++k) { s_first[lane * 8 + k] = run; run += v[k]; }
      if (lane == 31) s_first[kBuckets] = run;
    }
    __syncthreads();
  }
  const uint32_t items = s_first[kBuckets];
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(item_counter, 1);
    __syncthreads();
    const uint32_t item = (uint32_t)s_item;
    if (item >= items) return;
    int b = 0;  // the bucket: last with s_first[b] <= item
    for (int step = kBuckets / 2; step > 0; step >>= 1)
      if (s_first[b + step] <= item) b += step;
    const uint32_t count = hist[kRangeCounts + b];
    const uint32_t first = hist[kRangeOffsets + b] + (item - s_first[b]) * kChunk;
    const uint32_t end = hist[kRangeOffsets + b] + min(count, (item - s_first[b] + 1) * kChunk);
    const uint32_t bit0 = (uint32_t)b << shift;  // the bucket's first bit
    const uint32_t w0 = bit0 >> 5;
    const int words = (int)(((bit0 + (1u << shift) - 1) >> 5) - w0 + 1);
    for (int i = threadIdx.x; i < words; i += kThreads) s_bits[i] = 0;
    __syncthreads();
    for (uint32_t r0 = first; r0 < end; r0 += kThreads * 8) {  // the same rounds for every thread
      uint32_t k[8];
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        const uint32_t i = r0 + r * kThreads + threadIdx.x;
        k[r] = i < end ? __ldg(keys + i) : 0u;
      }
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        if (r0 + r * kThreads + threadIdx.x >= end) continue;
        const uint32_t bit = k[r] - lo;
        const uint32_t word = (bit >> 5) - w0, mask = 1u << (bit & 31);
        // a bit already set costs a (broadcast) load, not an atomic: frequent
        // keys stop contending once set; two lanes racing both OR the same bit
        if ((s_bits[word] & mask) == 0) atomicOr(s_bits + word, mask);
      }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < words; i += kThreads)
      if (s_bits[i]) atomicOr(bitmap + w0 + i, s_bits[i]);
    __syncthreads();  // s_bits / s_item are reused by the next item
  }
}

// The set bits in order, as signed words: tiles of 1024 bitmap words (4 per
// thread, one 16-byte load), a CTA scan of the per-thread bit counts and a
// look-back for the tile's output position.  Persistent like unique_kernel.
// The last tile writes the count and the NO_HIT sentinel when any word was
// NO_HIT.
constexpr int kBitmapTile = kThreads * 4;
__global__ void __launch_bounds__(kThreads) bitmap_unique_kernel(const uint32_t* bitmap, const int* count,
                                                                 int n_total, const uint32_t* range, int32_t* out,
                                                                 unsigned long long* status, int* tile_counter,
                                                                 int* result) {
  __shared__ int s_tile;
  __shared__ uint32_t s_warp[kWarps + 1];
  __shared__ uint32_t s_excl;
  if (range[2] != kBitmapPath) return;
  const uint32_t n_words = range[3], lo = ~range[0];
  const int m = *count;
  const uint32_t tag = g_epoch * 8u + 5u;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (;;) {
    if (threadIdx.x == 0) s_tile = atomicAdd(tile_counter, 1);
    __syncthreads();
    const int tile = s_tile;
    const size_t base = (size_t)tile * kBitmapTile;
    if (base >= n_words) return;
    const size_t first = base + (size_t)threadIdx.x * 4;
    uint32_t w[4];
    if (first + 4 <= n_words) {
      const uint4 v = __ldg(reinterpret_cast<const uint4*>(bitmap + first));
      w[0] = v.x; w[1] = v.y; w[2] = v.z; w[3] = v.w;
    } else {
#pragma unroll
      for (int r = 0; r < 4; ++r) w[r] = first + r < n_words ? __ldg(bitmap + first + r) : 0u;
    }
    const uint32_t cnt = __popc(w[0]) + __popc(w[1]) + __popc(w[2]) + __popc(w[3]);
    uint32_t incl = cnt;
    for (int off = 1; off < 32; off <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, incl, off);
      if (lane >= off) incl += t;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      const uint32_t excl = tile_prefix(s_warp, status, tile, tag);
      if (lane == 0 && base + kBitmapTile >= n_words) {  // last tile
        int u = min((int)(excl + s_warp[kWarps]), m);
        if (m < n_total) out[u++] = kNoHit;
        *result = u;
      }
      if (lane == 0) s_excl = excl;
    }
    __syncthreads();
    uint32_t pos = s_excl + s_warp[warp] + incl - cnt;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      uint32_t v = w[r];
      const uint32_t key0 = lo + (uint32_t)(first + r) * 32u;
      while (v) {
        const int b = __ffs(v) - 1;
        v &= v - 1;
        if (pos < (uint32_t)m) out[pos] = (int32_t)((key0 + (uint32_t)b) ^ 0x80000000u);
        ++pos;
      }
    }
    __syncthreads();  // s_tile / s_warp / s_excl are reused by the next tile
  }
}

// ---- inclusive scan (wrapping int32) ---------------------------------------------
// Tiles of 4096 values claimed in order; a tile's prefix comes from a warp-wide
// look-back over a status table cleared per call (tag 0: a cleared word is
// unpublished).  Sums wrap like the reference's int arithmetic.
__global__ void __launch_bounds__(kThreads) scan_kernel(int32_t* data, int n, unsigned long long* status,
                                                        int* tile_counter) {
  __shared__ int s_tile;
  __shared__ uint32_t s_warp[kWarps + 1];
  __shared__ uint32_t s_excl;
  if (threadIdx.x == 0) s_tile = atomicAdd(tile_counter, 1);
  __syncthreads();
  const int tile = s_tile;
  const int base = tile * kTile;
  if (base >= n) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint32_t v[kItems], sum = 0;
  const int first = base + threadIdx.x * kItems;
  if (first + kItems <= n && ((reinterpret_cast<uintptr_t>(data + first) & 15) == 0)) {
#pragma unroll
    for (int r = 0; r < kItems / 4; ++r) {
      const int4 q = reinterpret_cast<const int4*>(data + first)[r];
      v[4 * r] = (uint32_t)q.x; v[4 * r + 1] = (uint32_t)q.y; v[4 * r + 2] = (uint32_t)q.z; v[4 * r + 3] = (uint32_t)q.w;
    }
  } else {
#pragma unroll
    for (int r = 0; r < kItems; ++r) v[r] = first + r < n ? (uint32_t)data[first + r] : 0u;
  }
#pragma unroll
  for (int r = 0; r < kItems; ++r) sum += v[r];
  uint32_t incl = sum;
  for (int off = 1; off < 32; off <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off) incl += t;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    const uint32_t excl = tile_prefix(s_warp, status, tile, 0u);
    if (lane == 0) s_excl = excl;
  }
  __syncthreads();
  uint32_t run = s_excl + s_warp[warp] + incl - sum;
#pragma unroll
  for (int r = 0; r < kItems; ++r) {
    run += v[r];
    v[r] = run;
  }
  if (first + kItems <= n && ((reinterpret_cast<uintptr_t>(data + first) & 15) == 0)) {
#pragma unroll
    for (int r = 0; r < kItems / 4; ++r)
      reinterpret_cast<int4*>(data + first)[r] =
          make_int4((int)v[4 * r], (int)v[4 * r + 1], (int)v[4 * r + 2], (int)v[4 * r + 3]);
  } else {
#pragma unroll
    for (int r = 0; r < kItems; ++r)
      if (first + r < n) data[first + r] = (int32_t)v[r];
  }
}

int grid_for(int n) {
  const int tiles = (n + kTile - 1) / kTile;
  return tiles > 0 ? tiles : 1;
}

// Resident CTAs of persistent kernel K, at most the tiles of n keys.
template <auto K>
int persistent_grid(int n) {
  static int resident = 0;
  if (!resident) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, K, kThreads, 0);
    resident = sms * (per_sm > 0 ? per_sm : 1);
  }
  return std::min(resident, grid_for(n));
}

// Resident digit_kernel CTAs (two per SM), at most the tiles of n keys.
int digit_grid(int n) {
  static int resident = 0;
  if (!resident) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaFuncSetAttribute(digit_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kDigitSmemBytes);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, digit_kernel, kDigitThreads, kDigitSmemBytes);
    resident = sms * (per_sm > 0 ? per_sm : 1);
  }
  return std::max(1, std::min(resident, (n + kDigitTile - 1) / kDigitTile));
}

// The four digit passes.  With `range` (feedback unique) they return at once
// when the bitmap path was chosen.
cudaError_t run_passes(SortScratchLayout& l, int n, uint32_t*& cur, uint32_t*& other, int32_t* final_out,
                       const uint32_t* range, cudaStream_t s) {
  cudaError_t e;
  const int grid = digit_grid(n);
  for (int p = 0; p < kPasses; ++p) {
    const bool last = p == kPasses - 1;
    digit_kernel<<<grid, kDigitThreads, kDigitSmemBytes, s>>>(cur, other, l.count, 8 * p, l.hist + p * kBuckets,
                                                              l.status, l.tile_counter + p, p, last,
                                                              last ? final_out : nullptr, range);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    std::swap(cur, other);
  }
  return cudaSuccess;
}

int compact_grid(int n) {
  static int resident = 0;
  if (!resident) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, compact_kernel<true, true>, kThreads, 0);
    resident = sms * (per_sm > 0 ? per_sm : 1);
  }
  return std::min(resident, grid_for(n));
}

// Waits, as a look-back does, on a word that nothing publishes: the wait must
// give up after g_wait_ns, set the error flag and return.
__global__ void bounded_wait_probe_kernel(const unsigned long long* never) {
  if (threadIdx.x == 0 && blockIdx.x == 0) look_back(never, 1, 1, 0, 1u);
}

}  // namespace

cudaError_t bounded_wait_probe(double limit_s, cudaStream_t s) {
  const unsigned long long limit = (unsigned long long)(limit_s * 1e9), normal = 1000000000ull;
  unsigned long long* never = nullptr;
  cudaError_t e = cudaMalloc(&never, 2 * sizeof(unsigned long long));
  if (e != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(never, 0, 2 * sizeof(unsigned long long), s)) == cudaSuccess &&
      (e = cudaMemcpyToSymbolAsync(g_wait_ns, &limit, sizeof(limit), 0, cudaMemcpyHostToDevice, s)) == cudaSuccess) {
    bounded_wait_probe_kernel<<<1, 32, 0, s>>>(never);
    e = cudaGetLastError();
  }
  cudaError_t e2 = cudaMemcpyToSymbolAsync(g_wait_ns, &normal, sizeof(normal), 0, cudaMemcpyHostToDevice, s);
  cudaError_t e3 = cudaStreamSynchronize(s);
  cudaFree(never);
  return e != cudaSuccess ? e : (e2 != cudaSuccess ? e2 : e3);
}

int* device_error_flag() {
  int* p = nullptr;
  cudaGetSymbolAddress((void**)&p, g_error_flag);
  return p;
}

cudaError_t set_lookback_epoch(uint32_t epoch, cudaStream_t s) {
  // pageable source: the copy reads `epoch` before the call returns
  return cudaMemcpyToSymbolAsync(g_epoch, &epoch, sizeof(epoch), 0, cudaMemcpyHostToDevice, s);
}

size_t sort_scratch_bytes(int n) { return layout(nullptr, n).bytes; }
size_t feedback_scratch_bytes(int n) { return layout(nullptr, n).bytes; }
size_t scan_scratch_bytes(int n) { return (((size_t)n + kTile - 1) / kTile + 1) * 8 + 256; }

cudaError_t feedback_unique_device(const int32_t* words, int n, int nib, int32_t* unique_out, int* counts_dev,
                                   void* scratch, size_t scratch_bytes, cudaStream_t s) {
  SortScratchLayout l = layout(scratch, n);
  if (scratch_bytes < l.bytes) return cudaErrorInvalidValue;
  cudaError_t e;
  if ((e = cudaMemsetAsync(l.hist, 0, kHistRows * kBuckets * 4, s)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(l.tile_counter, 0, 16 * 4, s)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(l.count, 0, 4 * 4, s)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(l.range, 0, 8 * 4, s)) != cudaSuccess) return e;
  const int grid = compact_grid(n);
  if ((e = launch_compact<true>(grid, words, n, nib, l.keys_a, l.count, l.hist, l.range, s)) != cudaSuccess)
    return e;
  hist_offsets_kernel<<<1, kBuckets, 0, s>>>(l.hist, l.count, l.range, l.bitmap_bits);
  // bitmap path (each kernel returns at once on the radix path): range
  // partition keys_a -> keys_b, bitmap in keys_a, its set bits in order
  const int grid_n = std::min(grid, std::max(1, (int)(((size_t)n + 4095) / 4096)));
  range_hist_kernel<<<grid_n, kThreads, 0, s>>>(l.keys_a, l.count, l.range, l.hist, l.tile_counter + kCtrRangeDone,
                                                l.cursors);
  range_partition_kernel<<<grid_n, kThreads, 0, s>>>(l.keys_a, l.keys_b, l.count, l.range, l.cursors);
  bitmap_clear_kernel<<<grid_n, kThreads, 0, s>>>(l.range, reinterpret_cast<uint4*>(l.keys_a));
  bucket_bitmap_kernel<<<persistent_grid<bucket_bitmap_kernel>(n), kThreads, 0, s>>>(
      l.keys_b, l.range, l.hist, l.keys_a, l.tile_counter + kCtrBuckets);
  bitmap_unique_kernel<<<persistent_grid<bitmap_unique_kernel>(n), kThreads, 0, s>>>(
      l.keys_a, l.count, n, l.range, unique_out, l.status, l.tile_counter + kCtrBitmapUnique, counts_dev);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  // radix path (each kernel returns at once on the bitmap path)
  uint32_t* cur = l.keys_a;
  uint32_t* other = l.keys_b;
  if ((e = run_passes(l, n, cur, other, nullptr, l.range, s)) != cudaSuccess) return e;
  unique_kernel<<<persistent_grid<unique_kernel>(n), kThreads, 0, s>>>(cur, l.count, n, unique_out, l.status,
                                                                      l.tile_counter + kCtrUnique, counts_dev,
                                                                      l.range);
  return cudaGetLastError();
}

cudaError_t sort_i32_device(int32_t* data, int n, void* scratch, size_t scratch_bytes, cudaStream_t s) {
  if (n <= 1) return cudaSuccess;
  SortScratchLayout l = layout(scratch, n);
  if (scratch_bytes < l.bytes) return cudaErrorInvalidValue;
  cudaError_t e;
  if ((e = cudaMemsetAsync(l.hist, 0, kPasses * kBuckets * 4, s)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(l.tile_counter, 0, 16 * 4, s)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(l.count, 0, 4 * 4, s)) != cudaSuccess) return e;
  if ((e = launch_fill_i32(l.count, n, 1, s)) != cudaSuccess) return e;  // [0] keys; [2] the compaction's claims
  const int grid = compact_grid(n);
  if ((e = launch_compact<false>(grid, data, n, 0, l.keys_a, l.count + 2, l.hist, nullptr, s)) != cudaSuccess)
    return e;
  hist_offsets_kernel<<<1, kBuckets, 0, s>>>(l.hist, l.count, nullptr, 0);
  uint32_t* cur = l.keys_a;
  uint32_t* other = l.keys_b;
  return run_passes(l, n, cur, other, data, nullptr, s);
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
