// Oracle harness: host implementation of the fake OpenCL runtime (CLBuffer,
// CLKernel) that the reference's unmodified host code links against.
// Kernels are dispatched by name to the reference's .cl sources compiled as
// C++ (cl_*.cpp).  Test infrastructure only.
#include "cl-kernel.h"
#include "clc.h"
#include <ucontext.h>
#include <map>
#include <functional>
#include <cstdio>

namespace clc {
thread_local size_t g_gid[2], g_lid[2], g_lsize[2];
thread_local int g_width, g_height;

// ---- fibers for kernels that call barrier() --------------------------------
struct Group {
  std::vector<ucontext_t> ctx;
  std::vector<std::vector<char>> stacks;
  std::vector<char> done;
  ucontext_t main;
  int cur = 0;
  void (*fn)(void*) = nullptr;
  void* arg = nullptr;
  size_t base[2];
  size_t lsize[2];
  int width, height;
  std::vector<char> local_mem;
};
static thread_local Group* g_group = nullptr;

static void set_ids(Group& g, int i) {
  g_lid[0] = (size_t)i % g.lsize[0];
  g_lid[1] = (size_t)i / g.lsize[0];
  g_gid[0] = g.base[0] + g_lid[0];
  g_gid[1] = g.base[1] + g_lid[1];
  g_lsize[0] = g.lsize[0];
  g_lsize[1] = g.lsize[1];
  g_width = g.width;
  g_height = g.height;
}

static void trampoline() {
  Group& g = *g_group;
  g.fn(g.arg);
  g.done[g.cur] = 1;
}

void barrier(int) {
  Group& g = *g_group;
  swapcontext(&g.ctx[g.cur], &g.main);
  set_ids(g, g.cur);
}

char* current_local_mem() { return g_group->local_mem.data(); }

void for_each_group_with_barriers(const Launch& L, void (*fn)(void*), void* arg,
                                  int local_mem_bytes) {
  const size_t ng0 = L.global[0] / L.local[0];
  const size_t ng1 = L.dims == 2 ? L.global[1] / L.local[1] : 1;
  const int items = (int)(L.local[0] * (L.dims == 2 ? L.local[1] : 1));
  const long long ngroups = (long long)(ng0 * ng1);
#pragma omp parallel
  {
    Group g;
    g.ctx.resize(items);
    g.stacks.assign(items, std::vector<char>(64 * 1024));
    g.done.resize(items);
    g.local_mem.assign(local_mem_bytes > 0 ? local_mem_bytes : 1, 0);
    g_group = &g;
#pragma omp for schedule(dynamic, 1)
    for (long long gi = 0; gi < ngroups; ++gi) {
      g.fn = fn;
      g.arg = arg;
      g.base[0] = (size_t)(gi % (long long)ng0) * L.local[0];
      g.base[1] = (size_t)(gi / (long long)ng0) * (L.dims == 2 ? L.local[1] : 1);
      g.lsize[0] = L.local[0];
      g.lsize[1] = L.dims == 2 ? L.local[1] : 1;
      g.width = L.width;
      g.height = L.height;
      for (int i = 0; i < items; ++i) {
        getcontext(&g.ctx[i]);
        g.ctx[i].uc_stack.ss_sp = g.stacks[i].data();
        g.ctx[i].uc_stack.ss_size = g.stacks[i].size();
        g.ctx[i].uc_link = &g.main;
        makecontext(&g.ctx[i], trampoline, 0);
        g.done[i] = 0;
      }
      bool live = true;
      while (live) {
        live = false;
        for (int i = 0; i < items; ++i) {
          if (g.done[i]) continue;
          g.cur = i;
          set_ids(g, i);
          swapcontext(&g.main, &g.ctx[i]);
          if (!g.done[i]) live = true;
        }
      }
    }
    g_group = nullptr;
  }
}
}  // namespace clc

// ---- kernel entry points compiled from the reference's .cl sources ----------
using KernelRunner = void (*)(const clc::Launch&, const clc::Args&);
void fakecl_InitTracingFrame(const clc::Launch&, const clc::Args&);
void fakecl_RaytracingPass(const clc::Launch&, const clc::Args&);
void fakecl_FinishTracingFrame(const clc::Launch&, const clc::Args&);
void fakecl_NodeToBlockKernel(const clc::Launch&, const clc::Args&);
void fakecl_DifferenceFlagKernel(const clc::Launch&, const clc::Args&);
void fakecl_CompressKernel(const clc::Launch&, const clc::Args&);
void fakecl_LocalMergeSortKernel(const clc::Launch&, const clc::Args&);
void fakecl_GlobalMergeSortPassKernel(const clc::Launch&, const clc::Args&);
void fakecl_ScanPassKernel(const clc::Launch&, const clc::Args&);

static const std::map<std::string, KernelRunner>& kernel_table() {
  static const std::map<std::string, KernelRunner> t = {
      {"InitTracingFrame", fakecl_InitTracingFrame},
      {"RaytracingPass", fakecl_RaytracingPass},
      {"FinishTracingFrame", fakecl_FinishTracingFrame},
      {"NodeToBlockKernel", fakecl_NodeToBlockKernel},
      {"DifferenceFlagKernel", fakecl_DifferenceFlagKernel},
      {"CompressKernel", fakecl_CompressKernel},
      {"LocalMergeSortKernel", fakecl_LocalMergeSortKernel},
      {"GlobalMergeSortPassKernel", fakecl_GlobalMergeSortPassKernel},
      {"ScanPassKernel", fakecl_ScanPassKernel},
  };
  return t;
}

// Observers the harness installs to snapshot buffers after a named kernel ran.
std::function<void(const std::string&, const clc::Args&)> g_fakecl_after_kernel;

namespace rayt {

// ---- CLBuffer ----------------------------------------------------------------
CLBuffer::CLBuffer(cl_mem_flags, int size, boost::shared_ptr<CLContext>) : mem_((size_t)size) {}
CLBuffer::~CLBuffer() {}
cl_mem CLBuffer::buffer() const { return mem_.empty() ? nullptr : (cl_mem)mem_.data(); }
int CLBuffer::size() const { return (int)mem_.size(); }
void CLBuffer::CopyFrom(CLBuffer& buf, int src_start, int dest_start, int length,
                        const CLEventList*, CLEvent*) {
  if (src_start < 0 || dest_start < 0 || src_start + length > buf.size() || dest_start + length > size())
    crash("fake CL: CopyFrom out of range");
  std::memmove(mem_.data() + dest_start, buf.mem_.data() + src_start, (size_t)length);
}
void CLBuffer::CopyFrom(CLBuffer& buf, const CLEventList* w, CLEvent* e) {
  CopyFrom(buf, 0, 0, std::min(size(), buf.size()), w, e);
}
void CLBuffer::Write(int start, int length, const void* data, bool, const CLEventList*, CLEvent*) {
  if (start < 0 || start + length > size()) crash("fake CL: Write out of range");
  std::memcpy(mem_.data() + start, data, (size_t)length);
}
void CLBuffer::Read(int start, int length, void* data, const CLEventList*, CLEvent*) {
  if (start < 0 || start + length > size()) crash("fake CL: Read out of range");
  std::memcpy(data, mem_.data() + start, (size_t)length);
}
void CLBuffer::Read(int start, int length, void* data) const {
  if (start < 0 || start + length > size()) crash("fake CL: Read out of range");
  std::memcpy(data, mem_.data() + start, (size_t)length);
}

// ---- CLKernel ----------------------------------------------------------------
static int param_value(const std::string& params, const char* key) {
  std::string k = std::string("-D ") + key + "=";
  size_t p = params.find(k);
  return p == std::string::npos ? 0 : atoi(params.c_str() + p + k.size());
}

CLKernel::CLKernel(std::string, std::string params, std::string kernel_name,
                   boost::shared_ptr<CLContext>)
    : name_(kernel_name) {
  width_ = param_value(params, "WIDTH");
  height_ = param_value(params, "HEIGHT");
  if (!kernel_table().count(name_)) crash("fake CL: unknown kernel " + name_);
}
CLKernel::CLKernel(std::string, std::string file_name, std::string params,
                   std::string kernel_name, boost::shared_ptr<CLContext> context)
    : CLKernel(file_name, params, kernel_name, context) {}
CLKernel::~CLKernel() {}

// The fake device reports 256 work-items per group (a typical OpenCL GPU value).
int CLKernel::work_group_size() const { return 256; }

void CLKernel::SetArg(int index, int size, void* data) {
  if ((int)args_.size() <= index) {
    args_.resize(index + 1);
    local_bytes_.resize(index + 1, 0);
  }
  args_[index].assign((size_t)std::max(size, 0), 0);
  if (data) std::memcpy(args_[index].data(), data, (size_t)size);
  local_bytes_[index] = data ? 0 : size;
}
void CLKernel::SetLocalBufferArg(int index, int size) { SetArg(index, size, nullptr); }
void CLKernel::SetIntArg(int index, int val) { SetArg(index, sizeof(int), &val); }
void CLKernel::SetFloat4Arg(int index, fvec3 xyz, float w) {
  float v[4] = {xyz.x, xyz.y, xyz.z, w};
  SetArg(index, sizeof(v), v);
}
void CLKernel::SetFloatArg(int index, float val) { SetArg(index, sizeof(float), &val); }
void CLKernel::SetBufferArg(int index, const CLBuffer* buf) {
  cl_mem mem = buf ? buf->buffer() : nullptr;
  SetArg(index, sizeof(cl_mem), &mem);
}
void CLKernel::SetFloat16Arg(int index, fmat4 mat) { SetArg(index, sizeof(cl_float16), mat.m); }

void CLKernel::Dispatch(int dims, const size_t* global, const size_t* local) {
  clc::Launch L;
  L.dims = dims;
  L.global[0] = global[0];
  L.global[1] = dims == 2 ? global[1] : 1;
  L.local[0] = local[0];
  L.local[1] = dims == 2 ? local[1] : 1;
  L.width = width_;
  L.height = height_;
  clc::Args a{&args_, &local_bytes_};
  kernel_table().at(name_)(L, a);
  if (g_fakecl_after_kernel) g_fakecl_after_kernel(name_, a);
}

// Same NDRange shaping as the reference's CLKernel::Run1D.
void CLKernel::Run1D(int size, const CLEventList*, CLEvent*) {
  int wg = work_group_size();
  size_t global = (size_t)((size + wg - 1) / wg * wg);
  size_t local = (size_t)wg;
  if (global == 0) return;
  Dispatch(1, &global, &local);
}

// Same NDRange shaping as the reference's CLKernel::Run2D.
void CLKernel::Run2D(int size0, int size1, const CLEventList*, CLEvent*) {
  int wg = work_group_size();
  int s0 = 1;
  while (s0 < size0 && s0 * s0 < wg) s0 *= 2;
  s0 = std::min(s0, size0);
  int s1 = std::min(wg / s0, size1);
  size_t local[2] = {(size_t)s0, (size_t)s1};
  size_t global[2] = {(size_t)((size0 + s0 - 1) / s0 * s0), (size_t)((size1 + s1 - 1) / s1 * s1)};
  Dispatch(2, global, local);
}

}  // namespace rayt
