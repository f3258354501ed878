// Oracle harness: the OpenCL C built-ins and vector types the reference's
// kernels use, restated for C++ so that the kernels themselves
// (rayt/GPU_renderer/kernels/*.cl, rayt/GPU algorithms/kernels/*.cl) compile
// and run on host cores.  Test infrastructure only; never part of the product.
//
// Implementation-defined built-ins are pinned here, and the CUDA kernels and the
// oracle restatement use the same definitions:
//   dot(a, b)      = ((a.x*b.x + a.y*b.y) + a.z*b.z) + a.w*b.w, left to right
//   length(v)      = sqrt(dot(v, v))                (IEEE sqrt)
//   normalize(v)   = v / length(v)                  (component-wise IEEE divide)
//   distance(a, b) = length(a - b)
//   vector / scalar is a component-wise IEEE divide (not a reciprocal multiply)
//   min/max(x, y)  = OpenCL definitions: y < x ? y : x and x < y ? y : x
//   log(x)         = the C library's logf (OpenCL allows 3 ulp; only the debug
//                    depth view uses it, and is compared within 1 LSB)
// The kernels are built with -ffp-contract=off so no multiply-add is fused.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstddef>
#include <vector>

namespace clc {

typedef unsigned int uint;
typedef unsigned char uchar;
typedef unsigned short ushort;

struct float4 {
  float x, y, z, w;
  float4() {}
  template <class A, class B, class C, class D>
  float4(A a, B b, C c, D d) : x((float)a), y((float)b), z((float)c), w((float)d) {}
};
struct uchar4 {
  uchar x, y, z, w;
  uchar4() {}
  template <class A, class B, class C, class D>
  uchar4(A a, B b, C c, D d) : x((uchar)a), y((uchar)b), z((uchar)c), w((uchar)d) {}
};
struct char4 {
  signed char x, y, z, w;
  char4() {}
  template <class A, class B, class C, class D>
  char4(A a, B b, C c, D d)
      : x((signed char)a), y((signed char)b), z((signed char)c), w((signed char)d) {}
};
struct uint2 {
  uint x, y;
  uint2() {}
  template <class A, class B>
  uint2(A a, B b) : x((uint)a), y((uint)b) {}
};
struct float16 {
  float s0, s1, s2, s3, s4, s5, s6, s7, s8, s9, sa, sb, sc, sd, se, sf;
};
static_assert(sizeof(float4) == 16, "float4 layout");
static_assert(sizeof(float16) == 64, "float16 layout");

inline float4 operator+(float4 a, float4 b) { return float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline float4 operator-(float4 a, float4 b) { return float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
inline float4 operator*(float4 a, float4 b) { return float4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
inline float4 operator/(float4 a, float4 b) { return float4(a.x / b.x, a.y / b.y, a.z / b.z, a.w / b.w); }
inline float4 operator*(float4 a, float s) { return float4(a.x * s, a.y * s, a.z * s, a.w * s); }
inline float4 operator*(float s, float4 a) { return float4(s * a.x, s * a.y, s * a.z, s * a.w); }
inline float4 operator/(float4 a, float s) { return float4(a.x / s, a.y / s, a.z / s, a.w / s); }
inline float4 operator-(float4 a) { return float4(-a.x, -a.y, -a.z, -a.w); }
inline float4& operator+=(float4& a, float4 b) { a = a + b; return a; }

inline float fabs(float v) { return std::fabs(v); }
inline float copysign(float a, float b) { return std::copysign(a, b); }
inline float fmin(float a, float b) { return std::fmin(a, b); }
inline float fmax(float a, float b) { return std::fmax(a, b); }
inline float sqrt(float v) { return std::sqrt(v); }
inline float log(float v) { return std::log(v); }  // natural log in float (libm logf)
inline float min(float a, float b) { return b < a ? b : a; }
inline float max(float a, float b) { return a < b ? b : a; }
inline int min(int a, int b) { return b < a ? b : a; }
inline int max(int a, int b) { return a < b ? b : a; }
inline float4 min(float4 a, float4 b) { return float4(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z), min(a.w, b.w)); }
inline float4 max(float4 a, float4 b) { return float4(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z), max(a.w, b.w)); }
inline float dot(float4 a, float4 b) {
  float r = a.x * b.x;
  r = r + a.y * b.y;
  r = r + a.z * b.z;
  r = r + a.w * b.w;
  return r;
}
inline float length(float4 v) { return std::sqrt(dot(v, v)); }
inline float4 normalize(float4 v) { return v / length(v); }
inline float distance(float4 a, float4 b) { return length(a - b); }

inline int as_int(float f) { int r; std::memcpy(&r, &f, 4); return r; }
inline uint as_uint(float f) { uint r; std::memcpy(&r, &f, 4); return r; }
inline float as_float(int i) { float r; std::memcpy(&r, &i, 4); return r; }
inline float as_float(uint i) { float r; std::memcpy(&r, &i, 4); return r; }

// ---- work-item state -------------------------------------------------------
extern thread_local size_t g_gid[2], g_lid[2], g_lsize[2];
extern thread_local int g_width, g_height;
inline size_t get_global_id(int d) { return g_gid[d]; }
inline size_t get_local_id(int d) { return g_lid[d]; }
inline size_t get_local_size(int d) { return g_lsize[d]; }
#define CLK_LOCAL_MEM_FENCE 1
void barrier(int flags);

// One NDRange as the reference's CLKernel::Run1D/Run2D shapes it.
struct Launch {
  int dims;
  size_t global[2];
  size_t local[2];
  int width, height;  // the kernel program's -D WIDTH / -D HEIGHT
};

// Raw kernel arguments, as clSetKernelArg received them.
struct Args {
  const std::vector<std::vector<char>>* raw;
  const std::vector<int>* local_bytes;
  template <class T> T* ptr(int i) const {
    void* p;
    std::memcpy(&p, (*raw)[i].data(), sizeof(void*));
    return reinterpret_cast<T*>(p);
  }
  template <class T> T val(int i) const {
    T v;
    std::memcpy(&v, (*raw)[i].data(), sizeof(T));
    return v;
  }
  int local(int i) const { return (*local_bytes)[i]; }
};

// Runs fn once per work-item of L (no barriers inside fn).
template <class F> void for_each_item(const Launch& L, F fn);
// Runs fn once per work-item, one work-group at a time, with barrier() support
// (work-items are fibers; each barrier() yields to the next work-item).
void for_each_group_with_barriers(const Launch& L, void (*fn)(void*), void* ctx,
                                  int local_mem_bytes);
// The running work-group's __local memory (valid inside the fn above).
char* current_local_mem();

}  // namespace clc

#include "clc_exec.h"
