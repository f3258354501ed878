// Oracle harness: the reference's debug depth view (raytracer.cl, with
// raycast.cl) compiled as C++, run over host copies of a cache's buffers.
#include <cstring>

#include "cl_prelude.h"
namespace clc { namespace k_depth {
#include "raytracer.cl"
}}
#include "clc_exec.h"

void refcl_depth_view(unsigned char* rgba, const unsigned* links, const unsigned* fars, int root,
                      const float* view_proj_inv, float lod_voxel_size, int w, int h) {
  using namespace clc::k_depth;
  clc::Launch L{};
  L.dims = 2;
  L.global[0] = (size_t)w;
  L.global[1] = (size_t)h;
  L.local[0] = 8;
  L.local[1] = 8;
  L.width = w;
  L.height = h;
  clc::float16 m;
  std::memcpy(&m, view_proj_inv, sizeof(m));
  auto* out = reinterpret_cast<clc::uchar4*>(rgba);
  auto* l = const_cast<clc::uint*>(links);
  auto* f = const_cast<clc::uint*>(fars);
  clc::for_each_item(L, [&] { RaytraceKernel(out, l, f, root, m, lod_voxel_size); });
}
