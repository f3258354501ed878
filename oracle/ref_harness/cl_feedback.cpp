// Oracle harness: the reference's feedback_compression.cl compiled as C++.
#include "cl_prelude.h"
namespace clc { namespace k_fb {
#include "feedback_compression.cl"
}}
void fakecl_NodeToBlockKernel(const clc::Launch& L, const clc::Args& a) {
  int n = a.val<int>(0), bs = a.val<int>(1);
  int* d = a.ptr<int>(2);
  clc::for_each_item(L, [&] { clc::k_fb::NodeToBlockKernel(n, bs, d); });
}
void fakecl_DifferenceFlagKernel(const clc::Launch& L, const clc::Args& a) {
  int n = a.val<int>(0);
  int* in = a.ptr<int>(1);
  int* out = a.ptr<int>(2);
  clc::for_each_item(L, [&] { clc::k_fb::DifferenceFlagKernel(n, in, out); });
}
void fakecl_CompressKernel(const clc::Launch& L, const clc::Args& a) {
  int n = a.val<int>(0);
  int* idx = a.ptr<int>(1);
  int* in = a.ptr<int>(2);
  int* out = a.ptr<int>(3);
  clc::for_each_item(L, [&] { clc::k_fb::CompressKernel(n, idx, in, out); });
}
