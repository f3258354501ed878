// Oracle harness: macros that let an OpenCL C kernel file compile as C++ inside
// namespace clc.  WIDTH/HEIGHT, which the reference passes as -D options when it
// builds a kernel program, become the launch's runtime values.
#pragma once
#include "clc.h"
#define __kernel
#define __global
#define __local
#define __private
#define WIDTH (::clc::g_width)
#define HEIGHT (::clc::g_height)
#define MAX_ALLOWED_TRACING_STATE_SIZE 48
