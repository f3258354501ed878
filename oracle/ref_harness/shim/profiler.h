// Oracle harness: the reference's profiling macros compiled out.
#pragma once
#include "common.h"
#include "stopwatch.h"
#define PROFILE_TIMER_START(name)
#define PROFILE_TIMER_STOP()
#define PROFILE_TIMER_COMMIT(name)
#define PROFILE_VALUE_ADD(name, value)
#define PROFILE_VALUE_COMMIT_SET(name, value)
#define PROFILE_VALUE_COMMIT(name)
