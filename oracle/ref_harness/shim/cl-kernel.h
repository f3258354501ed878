// Oracle harness: CLKernel that runs the reference's .cl kernels, compiled as
// C++, on host threads.  Arguments are captured as raw bytes exactly as the
// reference passes them to clSetKernelArg; the NDRange is shaped exactly like
// the reference's Run1D/Run2D.  Test infrastructure only.
#pragma once
#include "cl-context.h"
#include "cl-buffer.h"
#include "mat.h"

namespace rayt {
class CLKernel {
 public:
  CLKernel(std::string file_name, std::string params, std::string kernel_name,
           boost::shared_ptr<CLContext> context);
  CLKernel(std::string include_dir, std::string file_name, std::string params,
           std::string kernel_name, boost::shared_ptr<CLContext> context);
  ~CLKernel();
  int work_group_size() const;
  void SetArg(int index, int size, void* data);
  void SetLocalBufferArg(int index, int size);
  void SetIntArg(int index, int val);
  void SetFloat4Arg(int index, fvec3 xyz, float w);
  void SetFloatArg(int index, float val);
  void SetBufferArg(int index, const CLBuffer* buf);
  void SetFloat16Arg(int index, fmat4 mat);
  void Run1D(int size, const CLEventList* wait_list, CLEvent* out_event);
  void Run2D(int size0, int size1, const CLEventList* wait_list, CLEvent* out_event);

 private:
  std::string name_;
  int width_ = 0, height_ = 0;
  std::vector<std::vector<char>> args_;
  std::vector<int> local_bytes_;
  void Dispatch(int dims, const size_t* global, const size_t* local);
  CLKernel(const CLKernel&) = delete;
  void operator=(const CLKernel&) = delete;
};
}  // namespace rayt
