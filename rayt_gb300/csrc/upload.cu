// Block upload into the device cache.
//
// The reference rewrites each block's links on the CPU and issues one
// clEnqueueWriteBuffer per channel plus one 4-byte write per parent pointer and
// far pointer (rayt/GPU data/gpu-octree-cache.cpp:102-234,
// gpu-octree-data.cpp:60-93).  Here a whole transaction's blocks arrive in one
// host-to-device copy into a staging area; one kernel then scatters every block
// into the channel buffers, rewriting stored links into the cache format on the
// way (gpu-octree-cache.cpp:120-141: a loaded, non-fault link becomes a near
// pointer relative to the node itself), and a second kernel applies the
// parent/far-pointer writes, which the host has reduced to the last write per
// address in the reference's order.
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
  upload_kernel<<<p.blocks, kThreads, 0, s>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_patches(const Patch* patches, int n, uint32_t* links, uint32_t* far_ptrs, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  patch_kernel<<<(n + 255) / 256, 256, 0, s>>>(patches, n, links, far_ptrs);
  return cudaGetLastError();
}

}  // namespace rayt
