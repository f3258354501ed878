// Oracle harness: work-item loop for barrier-free kernels.  Rows of the NDRange
// run on OpenMP threads; each thread keeps its own work-item ids.
#pragma once
namespace clc {
template <class F> void for_each_item(const Launch& L, F fn) {
  const long long g0 = (long long)L.global[0];
  const long long g1 = L.dims == 2 ? (long long)L.global[1] : 1;
  const long long total = g0 * g1;
#pragma omp parallel for schedule(dynamic, 1024)
  for (long long i = 0; i < total; ++i) {
    size_t x = (size_t)(i % g0), y = (size_t)(i / g0);
    g_gid[0] = x; g_gid[1] = y;
    g_lid[0] = x % L.local[0]; g_lid[1] = L.dims == 2 ? y % L.local[1] : 0;
    g_lsize[0] = L.local[0]; g_lsize[1] = L.dims == 2 ? L.local[1] : 1;
    g_width = L.width; g_height = L.height;
    fn();
  }
}
}  // namespace clc
