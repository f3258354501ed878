/*
 * rayt_gb300 - C ABI of the GB300 (sm_103a) per-frame path of rayt: primary-ray
 * sparse-voxel-octree traversal against a device block cache, miss/hit
 * feedback, compaction + radix sort + unique of requested block IDs, and
 * upload of streamed blocks into the cache.
 *
 * The reference has no FFI: its boundary is the C++ class API of the OpenCL
 * renderer.  Each entry point below names the reference member it replaces
 * (paths relative to the reference project).  Plain pointers and sizes only.
 *
 * Conventions
 *  - Every call returns RAYT_OK (0) or a negative RAYT_E_* status; the message
 *    of the last failure on the calling thread is rayt_last_error().  Nothing
 *    exits the process (the reference calls crash() -> exit(),
 *    rayt/util/common.h:43-53).
 *  - Handles are opaque and single-threaded (one host thread per handle), as
 *    the reference's classes are.
 *  - Device pointers returned by the library are borrowed: valid until the
 *    owning handle is destroyed (images: until the next frame).
 *  - A "stream" argument is a cudaStream_t passed as void*; NULL means the
 *    library's own stream for that handle (or the legacy default stream for
 *    the stand-alone primitives).
 */
#ifndef RAYT_GB300_H_
#define RAYT_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RAYT_OK 0
#define RAYT_E_ARG (-1)      /* invalid argument or size */
#define RAYT_E_IO (-2)       /* file read/write failed */
#define RAYT_E_FORMAT (-3)   /* block file is malformed */
#define RAYT_E_OOM (-4)      /* host or device allocation failed */
#define RAYT_E_CUDA (-5)     /* CUDA runtime error */
#define RAYT_E_TIMEOUT (-6)  /* a bounded device wait gave up */
#define RAYT_E_STATE (-7)    /* call not valid in the current state */
#define RAYT_E_LIMIT (-8)    /* size beyond a documented format/ABI limit */

/* NO_HIT feedback word (rayt/GPU_renderer/kernels/common.cl:14). */
#define RAYT_NO_HIT 0x7fffffff

const char* rayt_last_error(void);
/* Library version string. */
const char* rayt_version(void);

/* ------------------------------------------------------------------------ */
/* Block file: replaces StoredOctreeLoader (rayt/CPU data/stored-octree-loader.h:14-38). */

typedef struct rayt_tree rayt_tree;

typedef struct {
  uint32_t nodes_in_block;   /* StoredOctreeHeader::nodes_in_block */
  uint32_t blocks_count;     /* StoredOctreeHeader::blocks_count */
  uint32_t root_block_index; /* StoredOctreeHeader::root_block_index */
  uint32_t block_stride;     /* bytes per block record (header + content) */
  uint32_t channels_count;   /* including "node links" */
  uint32_t content_bytes;    /* StoredOctreeLoader::BytesInBlockContent() */
  uint64_t header_bytes;     /* file offset of block 0 */
} rayt_tree_info;

typedef struct {
  uint16_t parent_pointer_index;
  uint16_t pointed_child_index;
  uint32_t parent_pointer_value;
} rayt_block_root;

typedef struct { /* StoredOctreeBlockHeader (rayt/CPU data/stored-octree-block.h:7-23) */
  uint32_t block_index;
  uint32_t parent_block_index;
  uint32_t roots_count;
  rayt_block_root roots[8];
} rayt_block_header;

/* StoredOctreeLoader(file) + ReadHeader (stored-octree-loader.cpp:9-19,60-98). */
int rayt_tree_open(const char* path, rayt_tree** out);
void rayt_tree_close(rayt_tree* tree);
/* StoredOctreeLoader::header() (stored-octree-loader.h:19). */
int rayt_tree_info_get(const rayt_tree* tree, rayt_tree_info* out);
/* StoredOctreeHeader::channels[i] (stored-octree-channel-set.h:26-27). */
int rayt_tree_channel(const rayt_tree* tree, int index, int* bytes_in_node, char* name, int name_capacity);
/* StoredOctreeLoader::LoadBlock (stored-octree-loader.cpp:31-58); content may be NULL. */
int rayt_tree_load_block(rayt_tree* tree, uint32_t block_index, rayt_block_header* header,
                         void* content, size_t content_bytes);

/* ------------------------------------------------------------------------ */
/* Scene building: the reference's BuildOctree (rayt/CPU data/stored-octree-builder.h:40-41)
 * fed by the sphere known-answer source (rayt/scene sources/stored-octree-test.cpp:317-323)
 * or the seeded heightfield/sphere benchmark source. */

typedef struct {
  int depth;          /* grid of 2^depth voxels per axis */
  uint32_t seed;      /* heightfield seed */
  int base_cells;     /* value-noise cells across the scene at octave 0 */
  int octaves;        /* fBm octaves (lacunarity 2, gain 0.5) */
  int spheres;        /* number of voxelised sphere shells */
  uint32_t sphere_seed;
  int min_radius;     /* sphere radius range in voxels (log-uniform) */
  int max_radius;
} rayt_terrain_params;

/* WriteTestOctreeSphere (stored-octree-test.cpp:317-323). */
int rayt_build_sphere_test(const char* path, float cx, float cy, float cz, float radius, int depth,
                           int nodes_in_block, uint32_t* blocks_out);
/* BuildOctree over the heightfield(+spheres) source, channels "normals" and "colors". */
int rayt_build_terrain(const char* path, const rayt_terrain_params* params, int nodes_in_block,
                       uint32_t* blocks_out, uint64_t* nodes_out);

/* ------------------------------------------------------------------------ */
/* Device block cache: replaces GPUOctreeCacheManager + GPUOctreeCache + GPUOctreeData
 * (rayt/GPU data/gpu-octree-cache-manager.h:14-68, gpu-octree-cache.h:10-113,
 * gpu-octree-data.h:14-52).  Device layout is the reference's cache format
 * (rayt/doc/cache data format.txt): one buffer per channel of
 * max_blocks * nodes_in_block nodes, plus max_blocks * 8 far pointers. */

typedef struct rayt_cache rayt_cache;

/* GPUOctreeCacheManager(max_blocks_count, loader, context); max_blocks <= 0 means
 * every block of the file.  The cache keeps the tree open until the cache is
 * destroyed (like the reference's shared loader), so rayt_tree_close may come
 * first.  Renderers and
 * servers may share a cache (one LRU, one CUDA stream), one at a time: like
 * the reference's single-threaded frame loop, a cache is not used by two host
 * threads at once (a server's scheduler thread counts as one). */
int rayt_cache_create(rayt_tree* tree, int max_blocks, rayt_cache** out);
void rayt_cache_destroy(rayt_cache* cache);
/* GPUOctreeCacheManager::InitialFillCache (gpu-octree-cache-manager.cpp:60-108). */
int rayt_cache_initial_fill(rayt_cache* cache);
/* GPUOctreeCacheManager::root_node_index (gpu-octree-cache-manager.cpp:41-43). */
int rayt_cache_root_node_index(const rayt_cache* cache, int* out);
/* GPUOctreeCache::loaded_blocks_count / max_blocks_count. */
int rayt_cache_blocks(const rayt_cache* cache, int* loaded, int* max_blocks);
/* GPUOctreeData::ChannelByName(name)->cl_buffer() / far_pointers_buffer()
 * (gpu-octree-data.cpp:24-31).  name "far pointers" selects the far-pointer buffer. */
int rayt_cache_device_buffer(rayt_cache* cache, const char* name, void** device_ptr, size_t* bytes);
/* Copies a cache buffer to host memory (test and tooling helper). */
int rayt_cache_read_buffer(rayt_cache* cache, const char* name, void* host, size_t bytes);
/* Session / transaction protocol (gpu-octree-cache-manager.h:24-57). */
int rayt_cache_start_session(rayt_cache* cache);
int rayt_cache_start_transaction(rayt_cache* cache);
int rayt_cache_mark_block_used(rayt_cache* cache, int block_index_in_cache);
int rayt_cache_mark_parent_used(rayt_cache* cache, int block_index_in_cache);
int rayt_cache_request_block(rayt_cache* cache, int block_index);
int rayt_cache_transaction_filled(const rayt_cache* cache, int* out);
int rayt_cache_session_filled(const rayt_cache* cache, int* out);
int rayt_cache_end_transaction(rayt_cache* cache);
int rayt_cache_end_session(rayt_cache* cache);

typedef struct {
  int64_t uploaded_blocks;   /* blocks streamed into the cache */
  int64_t pointer_patches;   /* parent link writes (load and unload) */
  int64_t far_pointer_writes;
  int64_t bytes_h2d;         /* host->device bytes for block uploads */
  int64_t bytes_read;        /* bytes read from the block file */
  double io_seconds;         /* host time spent reading the file */
  double io_wait_seconds;    /* host time a transaction waited for its block reads */
  double place_seconds;      /* host time placing blocks (slot choice, links, patches) */
  double flush_seconds;      /* host time submitting copies and upload kernels */
  int64_t mapped;            /* 1: the device reads blocks from the block file mapped into
                                host memory (no host copy); 0: blocks are read with pread
                                into pinned staging and copied (RAYT_BLOCK_IO=read, or the
                                file could not be mapped and registered) */
} rayt_cache_stats;
int rayt_cache_stats_get(const rayt_cache* cache, rayt_cache_stats* out);

/* ------------------------------------------------------------------------ */
/* Renderer: replaces GPURayTracer (rayt/GPU_renderer/gpu-ray-tracer.h:11-55). */

typedef struct rayt_renderer rayt_renderer;

typedef struct { /* Camera (rayt/scene/camera.h:11-76) */
  float yaw, pitch, roll;      /* degrees */
  float position[3];
  float field_of_view;         /* horizontal, degrees */
  float aspect_ratio;          /* width / height */
  float near_clip_plane;       /* the reference's default is 0.01 */
} rayt_camera;

/* Camera::ViewProjectionMatrix().Inverse() (camera.cpp:23-28, mat.cpp:20-107):
 * the 16 floats (row-major) the reference passes to InitTracingFrame. */
int rayt_camera_view_proj_inv(const rayt_camera* camera, float out[16]);

/* GPURayTracer(cache_manager, frame_width, frame_height, context). */
int rayt_renderer_create(rayt_cache* cache, int width, int height, rayt_renderer** out);
void rayt_renderer_destroy(rayt_renderer* r);
/* set_frame_time_limit / set_lod_voxel_size (gpu-ray-tracer.h:17-23). */
int rayt_renderer_set_frame_time_limit(rayt_renderer* r, double seconds);
int rayt_renderer_set_lod_voxel_size(rayt_renderer* r, float size);
/* No counterpart in the reference (its todo list, msvs/rayt/todo.txt:5:
 * "Decrease LOD when cache is too small").  When on, a frame whose session
 * filled the cache makes the next frame render with grow x the voxel size (at
 * most max_lod_voxel_size); a frame that did not shrinks it by shrink, down to
 * the size set with rayt_renderer_set_lod_voxel_size.  Off by default;
 * rayt_frame_stats.lod_voxel_size reports the size each frame used. */
int rayt_renderer_set_lod_pressure(rayt_renderer* r, int on, float max_lod_voxel_size, float grow, float shrink);
/* Deterministic frame end: at most max_passes tracing passes (0 = no cap).  The
 * cap is applied where the reference applies its wall-clock limit. */
int rayt_renderer_set_max_passes(rayt_renderer* r, int max_passes);
/* Seeds the hit-window generator; it is the glibc rand() sequence after
 * srand(seed), which the reference's feedback extractor draws from
 * (ray-tracing-feedback-extractor.cpp:147). */
int rayt_renderer_seed(rayt_renderer* r, uint32_t seed);
/* Replay each pass's device work (feedback reset, traversal, feedback unique)
 * from a CUDA graph built once per pass kind (default on; recording passes
 * uses plain launches).  Results do not depend on it. */
int rayt_renderer_use_graphs(rayt_renderer* r, int on);
/* Keep each pass's dense per-pixel feedback words for rayt_renderer_pass_words. */
int rayt_renderer_record_passes(rayt_renderer* r, int on);
/* GPURayTracer::RenderFrame(camera) (gpu-ray-tracer.cpp:66-227), given the
 * camera's view_proj_inv matrix. */
int rayt_render_frame(rayt_renderer* r, const float view_proj_inv[16]);
/* The CUDA stream (cudaStream_t) the renderer and its cache run on, for
 * callers that order their own work or timing events after a frame. */
int rayt_renderer_stream(rayt_renderer* r, void** stream);
/* GPURayTracer::out_image(): RGBA8 frame, row 0 at the bottom. */
int rayt_renderer_image(rayt_renderer* r, void** device_rgba);
int rayt_renderer_read_image(rayt_renderer* r, void* host_rgba, size_t bytes);
/* Dense feedback words of pass `pass` of the last frame (recording on); views
 * follow one another in view order. */
int rayt_renderer_pass_words(rayt_renderer* r, int pass, int32_t* host_words, size_t count);

/* Depth and hit-node output (no counterpart in the reference, which keeps the
 * hit distance only inside a pass: raytracing_pass.cl:43,50-51,
 * raycast.cl:157-163).  Off by default; when on, every frame also writes per
 * pixel (same layout as the image, row 0 at the bottom):
 *   depth     float: the distance along the (normalised) ray direction from
 *             the camera to what the pixel shows, in octree units (the octree
 *             is the unit cube): the t at which each earlier pass stopped the
 *             ray on a fault, plus the final hit's t, summed in float in pass
 *             order.  +inf for a miss, NaN for an error (the iteration limit,
 *             shown red).  A ray still faulted when the frame ends (shaded
 *             with its fault's parent node) gets the distance where it stopped.
 *   hit node  int32: the cache node index (slot * nodes_in_block + node) that
 *             shaded the pixel - the hit node, or the fault's parent node for a
 *             ray still faulted at the end - -1 for a miss, -2 for an error.
 * Turning it on allocates both buffers (and 4 bytes per ray record). */
int rayt_renderer_set_depth_output(rayt_renderer* r, int on);
/* No counterpart in the reference (its out_image() is a device buffer that
 * GPURayTracer's caller draws with OpenGL, gpu-ray-tracer.h:20).  Host
 * delivery for a headless caller: from the next frame on, RenderFrame also
 * leaves the frame's RGBA8 image (width * height * 4 bytes, row 0 at the
 * bottom) in host_rgba by the time it returns, as rayt_renderer_read_image
 * would copy it.  The first pass's pixels are copied on a separate stream
 * while the host decodes feedback and streams blocks; the pixels that later
 * passes and the finish write go to host_rgba as well.  host_rgba must be
 * page-locked (cudaHostAlloc, or host memory registered with cudaHostRegister),
 * 4-byte aligned, and stay valid until delivery is switched off (NULL) or the
 * renderer is destroyed; one-view renderers only.  The device image stays
 * valid too. */
int rayt_renderer_set_host_image(rayt_renderer* r, void* host_rgba, size_t bytes);
/* Device pointers of view `view`'s depth (float) and hit-node (int32) buffers;
 * either out pointer may be NULL.  RAYT_E_STATE if depth output was never on. */
int rayt_renderer_depth(rayt_renderer* r, int view, void** device_depth, void** device_hit_nodes);
/* Copies view `view`'s depth and/or hit nodes (count >= its pixels) to host
 * memory; either host pointer may be NULL. */
int rayt_renderer_read_depth(rayt_renderer* r, int view, float* host_depth, int32_t* host_hit_nodes, size_t count);

/* Batched form (no counterpart in the reference, which renders one view per
 * RenderFrame).  A renderer over n_views views (1..512) of any sizes; each
 * frame traces all views in the same persistent launches and one cache
 * session, so their feedback is merged into one request list per pass and the
 * pass loop ends as RenderFrame's does.  Once the cache holds every block the
 * views touch, each view's image equals a one-view frame of that camera. */
int rayt_renderer_create_views(rayt_cache* cache, int n_views, const int* widths, const int* heights,
                               rayt_renderer** out);
/* One frame of every view; view_proj_inv holds n_views matrices of 16 floats. */
int rayt_render_views(rayt_renderer* r, const float* view_proj_inv, int n_views);
int rayt_renderer_view_count(const rayt_renderer* r);
int rayt_renderer_view_image(rayt_renderer* r, int view, void** device_rgba);
int rayt_renderer_read_view_image(rayt_renderer* r, int view, void* host_rgba, size_t bytes);
/* Traversal launch shape: a warp's 32 first-pass rays cover a
 * (1 << tile_w_log2) x (32 >> tile_w_log2) pixel tile.  refill = 32: one
 * thread per ray over a grid covering all rays.  refill < 32: a persistent
 * kernel (ctas_per_sm resident CTAs per SM, 0 = as many as fit) whose warps
 * take rays from a work counter, stop their rays every step_budget traversal
 * iterations and hand new rays to idle lanes once at least `refill` of them
 * are idle.  Default {2, 32, 0, 16}.  Results do not depend on the shape. */
int rayt_renderer_set_launch_shape(rayt_renderer* r, int tile_w_log2, int refill, int ctas_per_sm, int step_budget);
int rayt_renderer_get_launch_shape(const rayt_renderer* r, int shape[4]);
/* Times first passes over the given view matrices (as rayt_renderer_time_pass)
 * for every launch shape of a fixed candidate set, keeps the fastest and
 * returns it in best ({tile_w_log2, refill, ctas_per_sm, step_budget}). */
int rayt_renderer_autotune(rayt_renderer* r, const float* view_proj_inv, int reps, int best[4]);

typedef struct {
  int passes;                /* tracing passes of the last frame */
  int faults;                /* fault blocks reported over the frame */
  int uploaded_blocks;       /* blocks uploaded during the frame */
  int session_filled;        /* SessionFilledCache() at frame end */
  int64_t rays_traced;       /* ray casts over the frame (all passes) */
  float gpu_ms_trace;        /* device time of tracing passes */
  float gpu_ms_feedback;     /* device time of feedback unique */
  float gpu_ms_upload;       /* device time of upload kernels and copies */
  double frame_ms;           /* host wall time of the frame */
  int kernel_launches;       /* library kernels launched for the frame */
  int64_t bytes_h2d;         /* host->device bytes of the frame (block uploads) */
  int64_t bytes_d2h;         /* device->host bytes of the frame (feedback read-back) */
  double host_ms_wait;       /* host time blocked on the GPU (pass synchronisations) */
  double host_ms_decode;     /* host time in feedback decode, LRU marks and requests */
  double host_ms_load;       /* host time in EndTransaction: block reads, linking, upload issue */
  float lod_voxel_size;      /* the LOD voxel size the frame rendered with */
} rayt_frame_stats;
int rayt_renderer_stats(const rayt_renderer* r, rayt_frame_stats* out);

/* The reference's debug depth view (RaytraceKernel, rayt/GPU_renderer/kernels/
 * raytracer.cl:18-71, not wired into its application): rays from the near
 * plane, one pass over the cache as it is, no feedback or loads.  RGBA8 into
 * device_rgba (width x height, row 0 at the bottom): red where a ray faults or
 * errs, black where it misses, else grey = 255 * (1 - log-depth in [0.01, 5]).
 * Runs on `stream` (null: the cache's stream) and returns when done. */
int rayt_cache_depth_view(rayt_cache* cache, const float view_proj_inv[16], float lod_voxel_size, int width,
                          int height, void* device_rgba, void* stream);
/* Traces one pass from view_proj_inv (one matrix per view) against the cache
 * as it is (no feedback, no uploads) and counts node-link and far-pointer
 * fetches: the algorithmic byte count of the traversal roofline.  counts =
 * {rays, link fetches, far fetches, iterations, hits, faults}. */
int rayt_renderer_count_fetches(rayt_renderer* r, const float* view_proj_inv, int64_t counts[6]);
/* Times `reps` back-to-back first passes (ray setup + traversal + shading) on
 * the renderer's stream with CUDA events; returns milliseconds per pass. */
int rayt_renderer_time_pass(rayt_renderer* r, const float* view_proj_inv, int reps, float* ms_per_pass);

/* ------------------------------------------------------------------------ */
/* Served form (no counterpart in the reference).  Frame requests of up to 64
 * clients against one shared cache, with continuous batching: every
 * scheduling tick is one pass over all requests in flight (new requests'
 * first passes and older requests' faulted rays in the same launches), one
 * feedback unique and one cache transaction.  Clients are admitted while
 * framebuffer memory is free; requests while ray-record capacity is free, one
 * per client at a time, in arrival order.  Faulted rays restart from the
 * camera, so a request that ends without hitting its pass cap has exactly the
 * image of a fully resident cache, whatever else shared its ticks. */

typedef struct rayt_server rayt_server;
typedef struct {
  int max_clients;             /* 1..64 */
  int64_t framebuffer_bytes;   /* device memory for all client framebuffers */
  int64_t max_rays_in_flight;  /* ray records held between passes (request admission) */
  int max_passes;              /* tracing passes per request before its faulted rays are shaded */
  float lod_voxel_size;
  int deliver_to_host;         /* copy every finished frame to the client's pinned host image
                                  (a request is done once its image is there; the copies
                                  overlap the following ticks) */
} rayt_server_config;
typedef struct {
  uint64_t request;
  int client;
  int passes;                  /* tracing passes the request took */
  int truncated;               /* 1: rays still faulting at the end were shaded with their fault parent */
  double submit_s, admit_s, done_s;  /* steady-clock seconds */
} rayt_request_info;
typedef struct {
  int64_t submitted, completed, ticks, rays_traced, faults, kernel_launches, bytes_d2h;
  int64_t uploaded_blocks;   /* blocks streamed into the shared cache by ticks */
  double host_ms_wait;       /* host time blocked on the GPU (tick passes), summed over ticks */
  double host_ms_lru;        /* feedback decode, LRU marks and block requests */
  double host_ms_load;       /* EndTransaction: block reads, placement (evictions), upload issue */
  double gpu_ms_upload;      /* device time of block uploads (copies, upload and patch kernels) */
} rayt_server_stats;

int rayt_server_create(rayt_cache* cache, const rayt_server_config* cfg, rayt_server** out);
void rayt_server_destroy(rayt_server* s);
/* RAYT_E_LIMIT when no slot or framebuffer memory is free.  Add and remove
 * clients while the scheduler thread is stopped. */
int rayt_server_add_client(rayt_server* s, int width, int height, int* client);
int rayt_server_remove_client(rayt_server* s, int client);
int rayt_server_seed(rayt_server* s, uint32_t seed);
/* Queues a frame of `client` (thread-safe). */
int rayt_server_submit(rayt_server* s, int client, const float view_proj_inv[16], uint64_t* request);
/* One scheduling tick on the calling thread; *finished = requests it ended. */
int rayt_server_step(rayt_server* s, int* finished);
/* Scheduler thread running ticks while requests are queued or in flight. */
int rayt_server_start(rayt_server* s);
int rayt_server_stop(rayt_server* s);
/* Blocks until `request` ended (running ticks itself when no scheduler thread
 * runs); each request's info is returned once. */
int rayt_server_wait(rayt_server* s, uint64_t request, double timeout_s, rayt_request_info* out);
/* The client's framebuffer: its last finished frame until its next request
 * is admitted. */
int rayt_server_client_image(rayt_server* s, int client, void** device_rgba);
int rayt_server_read_client_image(rayt_server* s, int client, void* host_rgba, size_t bytes);
/* With deliver_to_host: the pinned host copy of the client's last finished frame. */
int rayt_server_host_image(rayt_server* s, int client, const void** host_rgba);
int rayt_server_stats_get(const rayt_server* s, rayt_server_stats* out);

/* ------------------------------------------------------------------------ */
/* Feedback primitives on device arrays of int32. */

/* GPUSort::Sort (rayt/GPU algorithms/gpu-sort.cpp:16-49): ascending signed
 * sort in place (LSD radix sort, 8-bit digits, decoupled look-back). */
int rayt_sort_i32(int32_t* device_data, int n, void* stream);
/* GPUScan::Scan (rayt/GPU algorithms/gpu-scan.cpp:15-43): inclusive prefix
 * sum in place, wrapping int32 arithmetic. */
int rayt_scan_i32(int32_t* device_data, int n, void* stream);
/* RayTracingFeedbackExtractor::GetUnique (ray-tracing-feedback-extractor.cpp:44-98):
 * NodeToBlock (when nodes_in_block > 0), then the sorted unique values
 * (signed ascending, RAYT_NO_HIT last when present) into device_unique (n
 * entries of room); *unique_count (host) receives the count.  Computed as
 * stream compaction, then, when the kept values span at most 32 per input
 * word and at most 2^26, a bitmap over their range read in order; otherwise
 * an LSD radix sort and unique.  The scratch memory is a device buffer the
 * library keeps per device and grows on demand.  The device work is captured
 * once as a CUDA graph and replayed while the pointers, n and nodes_in_block
 * repeat (one graph per device is kept).  device_words is not modified. */
int rayt_feedback_unique(const int32_t* device_words, int n, int nodes_in_block,
                         int32_t* device_unique, int* unique_count, void* stream);

/* No counterpart in the reference.  rayt_feedback_unique's computation for
 * callers that cannot let the library allocate device memory (an application
 * that owns all of HBM through its own allocator or reservation, or a frame
 * loop that cannot absorb the device-wide wait of cudaFree).  It calls no
 * cudaMalloc/cudaFree: its scratch is a fixed __device__ array of about
 * 17 MiB that each GPU loading the library keeps until exit, sized for n up
 * to RAYT_FEEDBACK_UNIQUE_NOALLOC_MAX_WORDS (larger n returns RAYT_E_LIMIT).
 * All calls on a device share that array: calls whose GPU work overlaps race.
 * The library serialises its own calls: this entry point, rayt_sort_i32,
 * rayt_scan_i32 and rayt_feedback_unique take one lock and return after their
 * stream finished (they share a device error flag and look-back epoch).  The
 * first call on a device looks up the array's address and zeroes the array on
 * `stream`; make it before any stream capture.
 * Returns after the result is on the device and *unique_count is set. */
#define RAYT_FEEDBACK_UNIQUE_NOALLOC_MAX_WORDS (1 << 21)
int rayt_feedback_unique_noalloc(const int32_t* device_words, int n, int nodes_in_block,
                                 int32_t* device_unique, int* unique_count, void* stream);

/* No counterpart in the reference.  Failure detection self-test: every wait
 * of a kernel on another CTA's result (the sort's look-back) gives up after a
 * time limit (1 s), sets a device error flag and returns, and the call reports
 * RAYT_E_TIMEOUT with the context still usable.  This runs one such wait on a
 * word nothing ever publishes, with a limit of limit_s seconds, and returns
 * RAYT_OK when the wait gave up and was reported as it must. */
int rayt_selftest_bounded_wait(double limit_s, void* stream);

/* No counterpart in the reference.  Testing hook for the look-back epoch of
 * the sort/unique kernels: their look-back words are tagged with a 27-bit
 * per-call epoch, and before the epoch would repeat (after 2^27 - 1 calls on
 * a device) the library clears every look-back table of the device and
 * restarts it.  This sets the current device's epoch (and the library's count
 * of calls since the last clear) to `calls`, so a test can make the restart
 * happen within a few calls. */
int rayt_testing_set_lookback_epoch(uint32_t calls);

/* No counterpart in the reference.  Testing hook for the renderer's feedback
 * marks: rayt_cache_mark_block_used for every slot of hits, then
 * rayt_cache_mark_parent_used for every slot of dup_hits, applied the way a
 * frame applies a pass's marks (one batch that leaves the LRU list and the
 * session/transaction markers as the calls one by one would; slots out of
 * range are skipped, as those calls refuse them).  Needs an open transaction. */
int rayt_testing_cache_mark_batch(rayt_cache* cache, const int* hits, int n_hits, const int* dup_hits, int n_dup);

#ifdef __cplusplus
}
#endif
#endif /* RAYT_GB300_H_ */
