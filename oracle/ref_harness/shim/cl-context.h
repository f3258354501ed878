// Oracle harness: host-only stand-in for the reference's OpenCL context wrapper
// ("CL util/cl-context.h" in the reference).  Everything the fake runtime does is
// synchronous, so WaitForAll has nothing to wait for.  Test infrastructure only.
#pragma once
#include "common.h"
#include <cstdint>
#include <vector>
#include <string>

typedef unsigned long cl_mem_flags;
typedef void* cl_mem;
typedef void* cl_event;
typedef int32_t cl_int;
typedef float cl_float16[16];
#define CL_MEM_READ_WRITE 1
#define CL_MEM_WRITE_ONLY 2
#define CL_MEM_READ_ONLY 4

namespace rayt {
class CLContext {
 public:
  CLContext() {}
  ~CLContext() {}
  void WaitForAll() {}
};
}  // namespace rayt
