// Oracle harness: a CLBuffer backed by host memory (zero-initialised).
// Same member functions as the reference's "CL util/cl-buffer.h"; every
// transfer completes before it returns.  Test infrastructure only.
#pragma once
#include <boost/shared_ptr.hpp>
#include "cl-context.h"
#include "cl-event.h"

namespace rayt {
class CLBuffer {
 public:
  CLBuffer(cl_mem_flags flags, int size, boost::shared_ptr<CLContext> context);
  ~CLBuffer();
  cl_mem buffer() const;
  int size() const;
  void CopyFrom(CLBuffer& buf, int src_start, int dest_start, int length,
                const CLEventList* wait_list, CLEvent* out_event);
  void CopyFrom(CLBuffer& buf, const CLEventList* wait_list, CLEvent* out_event);
  void Write(int start, int length, const void* data, bool blocking,
             const CLEventList* wait_list, CLEvent* out_event);
  void Read(int start, int length, void* data, const CLEventList* wait_list,
            CLEvent* out_event);
  void Read(int start, int length, void* data) const;

 private:
  mutable std::vector<char> mem_;
  CLBuffer(const CLBuffer&) = delete;
  void operator=(const CLBuffer&) = delete;
};
}  // namespace rayt
