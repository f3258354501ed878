// Oracle harness: the reference's finish_tracing_frame.cl compiled as C++.
#include "cl_prelude.h"
namespace clc { namespace k_finish {
#include "finish_tracing_frame.cl"
}}
void fakecl_FinishTracingFrame(const clc::Launch& L, const clc::Args& a) {
  using namespace clc::k_finish;
  auto* out = a.ptr<clc::uchar4>(0);
  auto* st = a.ptr<TracingState>(1);
  auto bg = a.val<clc::float4>(2);
  auto* nrm = a.ptr<clc::char4>(3);
  auto* col = a.ptr<clc::uchar4>(4);
  clc::for_each_item(L, [&] { FinishTracingFrame(out, st, bg, nrm, col); });
}
