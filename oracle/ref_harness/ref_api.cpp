// Oracle harness: C entry points over the reference's own classes, compiled
// from the reference sources against the fake OpenCL runtime.  Used only to
// generate and check golden fixtures in the development container (the
// reference sources are not available anywhere else).  Test infrastructure.
#include <cstdlib>
#include <functional>
#include <string>
#include <vector>
#include "gpu-ray-tracer.h"
#include "stored-octree-builder.h"
#include "stored-octree-loader.h"
#include "stored-octree-test.h"
#include "gpu-sort.h"
#include "gpu-scan.h"
#include "camera.h"
#include "clc.h"
#include "../../rayt_gb300/csrc/scene_source.h"

extern std::function<void(const std::string&, const clc::Args&)> g_fakecl_after_kernel;
void refcl_depth_view(unsigned char* rgba, const unsigned* links, const unsigned* fars, int root,
                      const float* view_proj_inv, float lod_voxel_size, int w, int h);

using namespace rayt;

namespace {

class TerrainAdapter : public StoredOctreeBuilderDataSource<rayt_scene::TerrainNode> {
 public:
  explicit TerrainAdapter(rayt_scene::TerrainSource* s) : s_(s) {}
  rayt_scene::TerrainNode GetRoot() override { return s_->GetRoot(); }
  std::vector<std::pair<int, rayt_scene::TerrainNode>> GetChildren(rayt_scene::TerrainNode& n) override {
    return s_->GetChildren(n);
  }
  void GetNodeData(rayt_scene::TerrainNode& n,
                   const std::vector<std::pair<int, rayt_scene::TerrainNode*>>& c, void* out) override {
    s_->GetNodeData(n, c, out);
  }
 private:
  rayt_scene::TerrainSource* s_;
};

struct Session {
  boost::shared_ptr<CLContext> ctx;
  boost::shared_ptr<StoredOctreeLoader> loader;
  boost::shared_ptr<GPUOctreeCacheManager> cache;
};

struct Renderer {
  Session* s;
  int w, h;
  boost::shared_ptr<GPURayTracer> rt;
  std::vector<std::vector<int>> pass_words;      // faults_and_hits after each pass
  std::vector<unsigned long long> pass_links;   // FNV-1a of node links + far pointers seen by each pass
};

unsigned long long fnv(const void* p, size_t n, unsigned long long h = 1469598103934665603ULL) {
  const unsigned char* b = static_cast<const unsigned char*>(p);
  for (size_t i = 0; i < n; ++i) {
    h ^= b[i];
    h *= 1099511628211ULL;
  }
  return h;
}

Camera make_camera(const float* c) {
  Camera cam;
  cam.set_yaw(c[0]);
  cam.set_pitch(c[1]);
  cam.set_roll(c[2]);
  cam.set_position(fvec3(c[3], c[4], c[5]));
  cam.set_field_of_view(c[6]);
  cam.set_aspect_ratio(c[7]);
  return cam;
}

}  // namespace

extern "C" {

void ref_srand(unsigned seed) { srand(seed); }
int ref_rand() { return rand(); }

int ref_build_sphere(const char* path, float cx, float cy, float cz, float r, int level, int nib) {
  WriteTestOctreeSphere(fvec3(cx, cy, cz), r, level, path, nib);
  return 0;
}

int ref_check_sphere_with_loader(const char* path, float cx, float cy, float cz, float r, int level) {
  CheckTestOctreeSphereWithLoader(fvec3(cx, cy, cz), r, level, path);  // crash() exits on failure
  return 0;
}

// params: depth, seed, base_cells, octaves, spheres, sphere_seed, min_radius, max_radius
int ref_build_terrain(const char* path, const int* params, int nib) {
  rayt_scene::TerrainParams p;
  p.depth = params[0];
  p.seed = (uint32_t)params[1];
  p.base_cells = params[2];
  p.octaves = params[3];
  p.spheres = params[4];
  p.sphere_seed = (uint32_t)params[5];
  p.min_radius = params[6];
  p.max_radius = params[7];
  rayt_scene::TerrainSource src(p);
  TerrainAdapter a(&src);
  StoredOctreeChannelSet cs;
  cs.AddChannel(StoredOctreeChannel(4, "normals"));
  cs.AddChannel(StoredOctreeChannel(4, "colors"));
  BuildOctree(path, nib, cs, &a);
  return 0;
}

void* ref_session_open(const char* path, int max_blocks) {
  Session* s = new Session();
  s->ctx.reset(new CLContext());
  s->loader.reset(new StoredOctreeLoader(path));
  if (max_blocks <= 0) max_blocks = (int)s->loader->header().blocks_count;
  s->cache.reset(new GPUOctreeCacheManager(max_blocks, s->loader, s->ctx));
  s->cache->InitialFillCache();
  return s;
}
void ref_session_close(void* p) { delete static_cast<Session*>(p); }
int ref_session_root(void* p) { return static_cast<Session*>(p)->cache->root_node_index(); }
int ref_session_blocks(void* p) { return (int)static_cast<Session*>(p)->loader->header().blocks_count; }
int ref_session_nib(void* p) { return static_cast<Session*>(p)->cache->data()->nodes_in_block(); }
int ref_session_max_blocks(void* p) { return static_cast<Session*>(p)->cache->data()->max_blocks_count(); }

// Reads a whole device buffer: channel by name, or "far pointers".
int ref_session_read(void* p, const char* name, void* out, long long bytes) {
  Session* s = static_cast<Session*>(p);
  const CLBuffer* b = nullptr;
  if (std::string(name) == "far pointers")
    b = s->cache->data()->far_pointers_buffer();
  else if (s->cache->data()->ChannelByName(name))
    b = s->cache->data()->ChannelByName(name)->cl_buffer();
  if (!b || bytes > b->size()) return -1;
  b->Read(0, (int)bytes, out);
  return 0;
}

// RaytraceKernel (raytracer.cl, the reference's debug depth view) over the
// session's cache as it is: RGBA8, w x h.
int ref_session_depth_view(void* p, const float* view_proj_inv, float lod_voxel_size, int w, int h,
                           unsigned char* out) {
  Session* s = static_cast<Session*>(p);
  const CLBuffer* lb = s->cache->data()->ChannelByName("node links")->cl_buffer();
  const CLBuffer* fb = s->cache->data()->far_pointers_buffer();
  std::vector<unsigned> links(lb->size() / 4), fars(fb->size() / 4);
  lb->Read(0, (int)lb->size(), links.data());
  fb->Read(0, (int)fb->size(), fars.data());
  refcl_depth_view(out, links.data(), fars.data(), s->cache->root_node_index(), view_proj_inv, lod_voxel_size, w, h);
  return 0;
}

void* ref_renderer_create(void* sess, int w, int h, float lod_voxel_size, double frame_time_limit) {
  Renderer* r = new Renderer();
  r->s = static_cast<Session*>(sess);
  r->w = w;
  r->h = h;
  r->rt.reset(new GPURayTracer(r->s->cache, w, h, r->s->ctx));
  r->rt->set_lod_voxel_size(lod_voxel_size);
  r->rt->set_frame_time_limit(frame_time_limit);
  return r;
}
void ref_renderer_destroy(void* p) { delete static_cast<Renderer*>(p); }

// camera: yaw, pitch, roll, x, y, z, fov, aspect.  Fills view_proj_inv (16
// floats, row-major) with the matrix the reference passes to InitTracingFrame.
void ref_camera_matrix(const float* camera, float* view_proj_inv) {
  fmat4 m = make_camera(camera).ViewProjectionMatrix().Inverse();
  for (int i = 0; i < 16; ++i) view_proj_inv[i] = m.m[i];
}

int ref_render_frame(void* p, const float* camera) {
  Renderer* r = static_cast<Renderer*>(p);
  r->pass_words.clear();
  r->pass_links.clear();
  const long long nodes = (long long)ref_session_max_blocks(r->s) * ref_session_nib(r->s);
  g_fakecl_after_kernel = [r, nodes](const std::string& name, const clc::Args& a) {
    if (name != "RaytracingPass") return;
    const int* words = a.ptr<int>(0);
    r->pass_words.emplace_back(words, words + (size_t)r->w * r->h);
    unsigned long long hsh = fnv(a.ptr<unsigned>(2), (size_t)nodes * 4);
    hsh = fnv(a.ptr<unsigned>(3), (size_t)ref_session_max_blocks(r->s) * 8 * 4, hsh);
    r->pass_links.push_back(hsh);
  };
  r->rt->RenderFrame(make_camera(camera));
  g_fakecl_after_kernel = nullptr;
  return (int)r->pass_words.size();
}
int ref_frame_image(void* p, unsigned char* out) {
  Renderer* r = static_cast<Renderer*>(p);
  r->rt->out_image()->Read(0, 4 * r->w * r->h, out);
  return 0;
}
int ref_frame_pass_words(void* p, int pass, int* out) {
  Renderer* r = static_cast<Renderer*>(p);
  if (pass < 0 || pass >= (int)r->pass_words.size()) return -1;
  std::memcpy(out, r->pass_words[pass].data(), r->pass_words[pass].size() * 4);
  return 0;
}
unsigned long long ref_frame_pass_links_hash(void* p, int pass) {
  Renderer* r = static_cast<Renderer*>(p);
  return r->pass_links.at(pass);
}

// GPUSort / GPUScan on a host array through the reference classes.
int ref_sort(int* data, int n) {
  boost::shared_ptr<CLContext> ctx(new CLContext());
  GPUSort srt(n, ctx);
  CLBuffer buf(0, n * 4, ctx);
  buf.Write(0, n * 4, data, true, NULL, NULL);
  srt.Sort(buf);
  buf.Read(0, n * 4, data);
  return 0;
}
int ref_scan(int* data, int n) {
  boost::shared_ptr<CLContext> ctx(new CLContext());
  GPUScan scan(n, ctx);
  CLBuffer buf(0, n * 4, ctx);
  buf.Write(0, n * 4, data, true, NULL, NULL);
  scan.Scan(buf);
  buf.Read(0, n * 4, data);
  return 0;
}

// The reference feedback extractor's GetUnique sequence
// (ray-tracing-feedback-extractor.cpp:44-98) over a host array of words:
// NodeToBlock -> GPUSort -> DifferenceFlag -> GPUScan -> Compress.
// Returns the unique count (including a trailing NO_HIT when present).
int ref_feedback_unique(int* words, int n, int nodes_in_block, int* unique_out) {
  boost::shared_ptr<CLContext> ctx(new CLContext());
  CLBuffer data(0, n * 4, ctx), index(0, n * 4, ctx), uniq(0, n * 4, ctx);
  data.Write(0, n * 4, words, true, NULL, NULL);
  CLKernel n2b("GPU_renderer/kernels", "feedback_compression.cl", "", "NodeToBlockKernel", ctx);
  CLKernel flag("GPU_renderer/kernels", "feedback_compression.cl", "", "DifferenceFlagKernel", ctx);
  CLKernel comp("GPU_renderer/kernels", "feedback_compression.cl", "", "CompressKernel", ctx);
  n2b.SetIntArg(0, n);
  n2b.SetIntArg(1, nodes_in_block);
  n2b.SetBufferArg(2, &data);
  n2b.Run1D(n, NULL, NULL);
  GPUSort srt(n, ctx);
  srt.Sort(data);
  flag.SetIntArg(0, n);
  flag.SetBufferArg(1, &data);
  flag.SetBufferArg(2, &index);
  flag.Run1D(n, NULL, NULL);
  GPUScan scan(n, ctx);
  scan.Scan(index);
  int count = 0;
  index.Read((n - 1) * 4, 4, &count, NULL, NULL);
  comp.SetIntArg(0, n);
  comp.SetBufferArg(1, &index);
  comp.SetBufferArg(2, &data);
  comp.SetBufferArg(3, &uniq);
  comp.Run1D(n, NULL, NULL);
  ++count;
  uniq.Read(0, count * 4, unique_out, NULL, NULL);
  data.Read(0, n * 4, words, NULL, NULL);
  return count;
}

}  // extern "C"
