// Oracle harness: the reference's merge_sort.cl and scan.cl compiled as C++.
// LocalMergeSortKernel uses work-group barriers, so its work-items run as fibers.
#include "cl_prelude.h"
namespace clc { namespace k_sort {
#include "merge_sort.cl"
}}
namespace clc { namespace k_scan {
#include "scan.cl"
}}
namespace {
struct LocalSortArgs { int n; int* data; };
void local_sort_item(void* p) {
  auto* s = static_cast<LocalSortArgs*>(p);
  clc::k_sort::LocalMergeSortKernel(s->n, s->data, reinterpret_cast<int*>(clc::current_local_mem()));
}
}
void fakecl_LocalMergeSortKernel(const clc::Launch& L, const clc::Args& a) {
  LocalSortArgs s{a.val<int>(0), a.ptr<int>(1)};
  clc::for_each_group_with_barriers(L, local_sort_item, &s, a.local(2));
}
void fakecl_GlobalMergeSortPassKernel(const clc::Launch& L, const clc::Args& a) {
  int n = a.val<int>(0), len = a.val<int>(1);
  int* in = a.ptr<int>(2);
  int* out = a.ptr<int>(3);
  clc::for_each_item(L, [&] { clc::k_sort::GlobalMergeSortPassKernel(n, len, in, out); });
}
void fakecl_ScanPassKernel(const clc::Launch& L, const clc::Args& a) {
  int n = a.val<int>(0), len = a.val<int>(1);
  int* in = a.ptr<int>(2);
  int* out = a.ptr<int>(3);
  clc::for_each_item(L, [&] { clc::k_scan::ScanPassKernel(n, len, in, out); });
}
