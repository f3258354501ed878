// Oracle harness: the reference's raytracing_pass.cl (with raycast.cl and
// shading.cl) compiled as C++.
#include "cl_prelude.h"
namespace clc { namespace k_pass {
#include "raytracing_pass.cl"
}}
void fakecl_RaytracingPass(const clc::Launch& L, const clc::Args& a) {
  using namespace clc::k_pass;
  auto* fh = a.ptr<int>(0);
  auto* st = a.ptr<TracingState>(1);
  auto* links = a.ptr<clc::uint>(2);
  auto* fars = a.ptr<clc::uint>(3);
  int root = a.val<int>(4);
  auto* nrm = a.ptr<clc::char4>(5);
  auto* col = a.ptr<clc::uchar4>(6);
  clc::for_each_item(L, [&] { RaytracingPass(fh, st, links, fars, root, nrm, col); });
}
