// Block upload into the device cache.
//
// The reference rewrites each block's links on the CPU and issues one
// clEnqueueWriteBuffer per channel plus one 4-byte write per parent pointer and
// far pointer (rayt/GPU data/gpu-octree-cache.cpp:102-234,
// gpu-octree-data.cpp:60-93).  Here one kernel scatters a batch of blocks into
// the channel buffers, rewriting stored links into the cache format on the way
// (gpu-octree-cache.cpp:120-141: a loaded, non-fault link becomes a near
// pointer relative to the node itself), and a second kernel applies the
// parent/far-pointer writes, which the host has reduced to the last write per
// address in the reference's order.  The blocks come either from a staging
// area filled by one host-to-device copy of the batch (upload_kernel) or
// straight from the block file mapped into host memory and registered with the
// device (upload_mapped_kernel: no host copy at all).
#include <algorithm>

#include "internal.h"

namespace rayt {
namespace {

constexpr int kThreads = 256;

// One CTA per staged block: a grid-stride copy of each channel section.
__global__ void __launch_bounds__(kThreads) upload_kernel(const __grid_constant__ UploadParams p) {
  const int b = blockIdx.x;
  const size_t nib = (size_t)p.nodes_in_block;
  const uint8_t* src = p.stage + (size_t)b * p.stride;
  if (p.slots[b] < 0) return;  // staged but not placed (read ahead, then not needed)
  const size_t slot = (size_t)p.slots[b];

  // channel 0: node links, stored format -> cache format
  const uint32_t* sl = reinterpret_cast<const uint32_t*>(src);
  uint32_t* dl = reinterpret_cast<uint32_t*>(p.chan[0]) + slot * nib;
  for (size_t n = threadIdx.x; n < nib; n += kThreads) {
    uint32_t l = sl[n];
    const uint32_t mask = l & 255u, fault = (l >> 8) & 1u;
    if (mask && !fault) {
      const uint32_t ptr = l >> 11;
      const uint32_t near_ptr = (1u << 20) + ptr - (uint32_t)n;  // NearPointerValue(n, ptr)
      l = (near_ptr << 11) | (l & (1u << 9)) | mask;             // fault 0, far 0, dup kept
    }
    dl[n] = l;
  }
  // other channels: raw copy, 16 bytes at a time when aligned
  size_t off = nib * 4;
  for (int c = 1; c < p.channels; ++c) {
    const size_t bytes = nib * (size_t)p.chan_bytes[c];
    const uint8_t* s = src + off;
    uint8_t* d = p.chan[c] + slot * bytes;
    if (((reinterpret_cast<uintptr_t>(s) | reinterpret_cast<uintptr_t>(d) | bytes) & 15u) == 0) {
      const uint4* s4 = reinterpret_cast<const uint4*>(s);
      uint4* d4 = reinterpret_cast<uint4*>(d);
      for (size_t i = threadIdx.x; i < bytes / 16; i += kThreads) d4[i] = s4[i];
    } else {
      for (size_t i = threadIdx.x; i < bytes; i += kThreads) d[i] = s[i];
    }
    off += bytes;
  }
}

// NearPointerValue rewrite of one stored link (see upload_kernel).
__device__ __forceinline__ uint32_t cache_link(uint32_t l, uint32_t n) {
  const uint32_t mask = l & 255u, fault = (l >> 8) & 1u;
  if (mask && !fault) l = (((1u << 20) + (l >> 11) - n) << 11) | (l & (1u << 9)) | mask;
  return l;
}

// `parts` CTAs per block, each a contiguous share of every channel section,
// reading the block's content where it lies in the mapped block file (host
// memory the device reads directly).  A read over the host link takes long
// enough that a CTA copies a block's share in a few rounds of loads; a small
// batch (a transaction of a later pass streams a few dozen blocks) spreads
// each block over several CTAs so that more SMs have reads in flight.  A block
// record starts
// at any byte offset, so each warp reads rows of 32 consecutive aligned words,
// every lane its own, and forms the content words with a funnel shift from its
// word and the next lane's (the row's last lane takes the next row's first
// word; after the last row it reads that word itself).  A warp issues four
// rows' loads before it uses them, so that enough reads are in flight over
// the host link.  The aligned words read hold at least one byte of the content
// (or of its block header), so they lie inside the file.
constexpr int kRows = 4;
__global__ void __launch_bounds__(kThreads) upload_mapped_kernel(const __grid_constant__ UploadParams p) {
  const int b = blockIdx.x / p.parts, part = blockIdx.x - b * p.parts;
  if (p.slots[b] < 0) return;  // staged but not placed, or superseded
  const size_t slot = (size_t)p.slots[b];
  const size_t nib = (size_t)p.nodes_in_block;
  const uint8_t* src = p.file + p.file_first + p.file_stride * (uint64_t)(uint32_t)p.block_ids[b];
  const uint32_t mis = (uint32_t)(reinterpret_cast<uintptr_t>(src) & 3u);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  size_t off = 0;  // byte offset of the channel's section in the content
  for (int c = 0; c < p.channels; ++c) {
    const size_t bytes = nib * (size_t)p.chan_bytes[c];
    uint8_t* d = p.chan[c] + slot * bytes;
    if (((off | bytes) & 3u) == 0) {
      const size_t words = bytes / 4, limit = words + (mis ? 1 : 0);
      const uint32_t* a = reinterpret_cast<const uint32_t*>(src + off - mis);
      uint32_t* d4 = reinterpret_cast<uint32_t*>(d);
      // this CTA's words [w0, w1); loads past w1 stay below limit (inside the
      // section, or its one trailing word) and are not stored
      const size_t per = (words + p.parts - 1) / p.parts;
      const size_t w0 = min(words, per * part), w1 = min(words, w0 + per);
      // warp-uniform trip count: each warp takes 32 * kRows words at a time
      for (size_t i0 = w0 + (size_t)warp * 32 * kRows; i0 < w1; i0 += (size_t)kThreads * kRows) {
        uint32_t lo[kRows];
#pragma unroll
        for (int r = 0; r < kRows; ++r) {
          const size_t i = i0 + 32 * r + lane;
          lo[r] = i < limit ? a[i] : 0u;
        }
        uint32_t after = 0u;  // the word after the last row, for its last lane
        if (mis && lane == 31 && i0 + 32 * kRows < limit) after = a[i0 + 32 * kRows];
#pragma unroll
        for (int r = 0; r < kRows; ++r) {
          uint32_t w = lo[r];
          if (mis) {
            uint32_t hi = __shfl_down_sync(0xffffffffu, lo[r], 1);
            const uint32_t next_row = r + 1 < kRows ? __shfl_sync(0xffffffffu, lo[r + 1 < kRows ? r + 1 : r], 0) : after;
            if (lane == 31) hi = next_row;
            w = __funnelshift_r(lo[r], hi, 8u * mis);
          }
          const size_t i = i0 + 32 * r + lane;
          if (i < w1) d4[i] = c == 0 ? cache_link(w, (uint32_t)i) : w;
        }
      }
    } else {  // a section of odd size: bytes (links are always whole words)
      const size_t per = (bytes + p.parts - 1) / p.parts;
      const size_t b0 = min(bytes, per * part), b1 = min(bytes, b0 + per);
      for (size_t i = b0 + threadIdx.x; i < b1; i += kThreads) d[i] = src[off + i];
    }
    off += bytes;
  }
}

__global__ void patch_kernel(const Patch* patches, int n, uint32_t* links, uint32_t* far_ptrs) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const Patch q = patches[i];
  if (q.far) far_ptrs[q.index] = q.value;
  else links[q.index] = q.value;
}

}  // namespace

cudaError_t launch_upload(const UploadParams& p, cudaStream_t s) {
  if (p.blocks <= 0) return cudaSuccess;
  if (p.file) {
    // about two CTAs per SM over the batch, at most 8 per block
    static const int sms = [] {
      int dev = 0, n = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
      return n > 0 ? n : 1;
    }();
    UploadParams q = p;
    q.parts = std::max(1, std::min(8, (2 * sms + p.blocks - 1) / p.blocks));
    upload_mapped_kernel<<<(unsigned)(p.blocks * q.parts), kThreads, 0, s>>>(q);
  } else {
    upload_kernel<<<p.blocks, kThreads, 0, s>>>(p);
  }
  return cudaGetLastError();
}

cudaError_t launch_patches(const Patch* patches, int n, uint32_t* links, uint32_t* far_ptrs, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  patch_kernel<<<(n + 255) / 256, 256, 0, s>>>(patches, n, links, far_ptrs);
  return cudaGetLastError();
}

}  // namespace rayt
