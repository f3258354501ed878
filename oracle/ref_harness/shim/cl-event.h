// Oracle harness: no-op events (the fake runtime executes every command
// synchronously when it is enqueued).  Test infrastructure only.
#pragma once
#include "cl-context.h"
#include "array.h"  // the reference header pulls this in transitively

#define PROFILE_CL_EVENT(event, name)
#define PROFILE_CL_EVENTS_FINISH()

namespace rayt {
class CLEvent {
 public:
  CLEvent() {}
  CLEvent(cl_event) {}
  void reset(cl_event) {}
  cl_event event() const { return nullptr; }
  void WaitFor() const {}
};

class CLEventList {
 public:
  void Clear() { n_ = 0; }
  void Add(const CLEvent&) { ++n_; }
  int size() const { return n_; }
  void WaitFor() const {}
  const cl_event* events() const { return nullptr; }
 private:
  int n_ = 0;
};
}  // namespace rayt
