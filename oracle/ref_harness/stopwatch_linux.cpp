// Oracle harness: a Linux clock for the reference's Stopwatch class (the
// reference's util/stopwatch.cpp only has Windows and macOS branches).
#include "stopwatch.h"
#include <chrono>
namespace rayt {
static long long now_ns() {
  return std::chrono::duration_cast<std::chrono::nanoseconds>(
             std::chrono::steady_clock::now().time_since_epoch()).count();
}
Stopwatch::Stopwatch() { Restart(); }
Stopwatch::~Stopwatch() {}
double Stopwatch::TimeSinceRestart() const { return (now_ns() - start_time) * 1e-9; }
double Stopwatch::Restart() {
  long long t = now_ns();
  double r = (t - start_time) * 1e-9;
  start_time = t;
  return r;
}
void Stopwatch::ReportAndRestart(const char*) { Restart(); }
void Stopwatch::ReportIfGreaterAndRestart(const char*, double) { Restart(); }
}
