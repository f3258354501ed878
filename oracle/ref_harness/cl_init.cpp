// Oracle harness: the reference's init_tracing_frame.cl compiled as C++.
#include "cl_prelude.h"
namespace clc { namespace k_init {
#include "init_tracing_frame.cl"
static_assert(sizeof(TracingState) == 48, "TracingState layout");
}}
void fakecl_InitTracingFrame(const clc::Launch& L, const clc::Args& a) {
  using namespace clc::k_init;
  auto* st = a.ptr<TracingState>(0);
  auto m = a.val<clc::float16>(1);
  float lod = a.val<float>(2);
  clc::for_each_item(L, [&] { InitTracingFrame(st, m, lod); });
}
