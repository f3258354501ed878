"""rayt_gb300: the GB300 (sm_103a) per-frame path of rayt behind its C ABI.

This module loads rayt_gb300/_lib/librayt_gb300.so (built by
rayt_gb300/build.py) and mirrors the reference's C++ classes for this path
with the same names and argument meaning:

    StoredOctreeLoader      rayt/CPU data/stored-octree-loader.h:14-38
    GPUOctreeCacheManager   rayt/GPU data/gpu-octree-cache-manager.h:14-68
    GPURayTracer            rayt/GPU_renderer/gpu-ray-tracer.h:11-55
    GPUSort / GPUScan       rayt/GPU algorithms/gpu-sort.h, gpu-scan.h
    feedback_unique         RayTracingFeedbackExtractor::GetUnique
    Camera                  rayt/scene/camera.h:11-76

Errors raise RaytError (the reference calls crash(), which exits).  There is
no CPU fallback: without the built library or a GPU, calls fail loudly.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "librayt_gb300.so")

RAYT_OK = 0
NO_HIT = 0x7FFFFFFF
_ERRORS = {-1: "RAYT_E_ARG", -2: "RAYT_E_IO", -3: "RAYT_E_FORMAT", -4: "RAYT_E_OOM", -5: "RAYT_E_CUDA",
           -6: "RAYT_E_TIMEOUT", -7: "RAYT_E_STATE", -8: "RAYT_E_LIMIT"}


class RaytError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (_ERRORS.get(code, code), msg))
        self.code = code


class TreeInfo(C.Structure):
    _fields_ = [("nodes_in_block", C.c_uint32), ("blocks_count", C.c_uint32), ("root_block_index", C.c_uint32),
                ("block_stride", C.c_uint32), ("channels_count", C.c_uint32), ("content_bytes", C.c_uint32),
                ("header_bytes", C.c_uint64)]


class BlockRoot(C.Structure):
    _fields_ = [("parent_pointer_index", C.c_uint16), ("pointed_child_index", C.c_uint16),
                ("parent_pointer_value", C.c_uint32)]


class BlockHeader(C.Structure):
    _fields_ = [("block_index", C.c_uint32), ("parent_block_index", C.c_uint32), ("roots_count", C.c_uint32),
                ("roots", BlockRoot * 8)]


class TerrainParams(C.Structure):
    _fields_ = [("depth", C.c_int), ("seed", C.c_uint32), ("base_cells", C.c_int), ("octaves", C.c_int),
                ("spheres", C.c_int), ("sphere_seed", C.c_uint32), ("min_radius", C.c_int), ("max_radius", C.c_int)]


class CacheStats(C.Structure):
    _fields_ = [("uploaded_blocks", C.c_int64), ("pointer_patches", C.c_int64), ("far_pointer_writes", C.c_int64),
                ("bytes_h2d", C.c_int64), ("bytes_read", C.c_int64), ("io_seconds", C.c_double),
                ("io_wait_seconds", C.c_double), ("place_seconds", C.c_double), ("flush_seconds", C.c_double),
                ("mapped", C.c_int64)]


class FrameStats(C.Structure):
    _fields_ = [("passes", C.c_int), ("faults", C.c_int), ("uploaded_blocks", C.c_int), ("session_filled", C.c_int),
                ("rays_traced", C.c_int64), ("gpu_ms_trace", C.c_float), ("gpu_ms_feedback", C.c_float),
                ("gpu_ms_upload", C.c_float), ("frame_ms", C.c_double), ("kernel_launches", C.c_int),
                ("bytes_h2d", C.c_int64), ("bytes_d2h", C.c_int64), ("host_ms_wait", C.c_double),
                ("host_ms_decode", C.c_double), ("host_ms_load", C.c_double), ("lod_voxel_size", C.c_float)]


class ServerConfig(C.Structure):
    _fields_ = [("max_clients", C.c_int), ("framebuffer_bytes", C.c_int64), ("max_rays_in_flight", C.c_int64),
                ("max_passes", C.c_int), ("lod_voxel_size", C.c_float), ("deliver_to_host", C.c_int)]


class RequestInfo(C.Structure):
    _fields_ = [("request", C.c_uint64), ("client", C.c_int), ("passes", C.c_int), ("truncated", C.c_int),
                ("submit_s", C.c_double), ("admit_s", C.c_double), ("done_s", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [(k, C.c_int64) for k in ["submitted", "completed", "ticks", "rays_traced", "faults",
                                         "kernel_launches", "bytes_d2h", "uploaded_blocks"]] + [
        (k, C.c_double) for k in ["host_ms_wait", "host_ms_lru", "host_ms_load", "gpu_ms_upload"]]


class CameraStruct(C.Structure):
    _fields_ = [("yaw", C.c_float), ("pitch", C.c_float), ("roll", C.c_float), ("position", C.c_float * 3),
                ("field_of_view", C.c_float), ("aspect_ratio", C.c_float), ("near_clip_plane", C.c_float)]


_lib = None


def lib():
    """The loaded product library (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RaytError(-7, "native library not built: %s (run rayt_gb300/build.py)" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    vp, i32, u32, f32 = C.c_void_p, C.c_int, C.c_uint32, C.c_float
    sig = {
        "rayt_last_error": (C.c_char_p, []),
        "rayt_version": (C.c_char_p, []),
        "rayt_tree_open": (i32, [C.c_char_p, C.POINTER(vp)]),
        "rayt_tree_close": (None, [vp]),
        "rayt_tree_info_get": (i32, [vp, C.POINTER(TreeInfo)]),
        "rayt_tree_channel": (i32, [vp, i32, C.POINTER(i32), C.c_char_p, i32]),
        "rayt_tree_load_block": (i32, [vp, u32, C.POINTER(BlockHeader), vp, C.c_size_t]),
        "rayt_build_sphere_test": (i32, [C.c_char_p, f32, f32, f32, f32, i32, i32, C.POINTER(u32)]),
        "rayt_build_terrain": (i32, [C.c_char_p, C.POINTER(TerrainParams), i32, C.POINTER(u32), C.POINTER(C.c_uint64)]),
        "rayt_cache_create": (i32, [vp, i32, C.POINTER(vp)]),
        "rayt_cache_destroy": (None, [vp]),
        "rayt_cache_initial_fill": (i32, [vp]),
        "rayt_cache_root_node_index": (i32, [vp, C.POINTER(i32)]),
        "rayt_cache_blocks": (i32, [vp, C.POINTER(i32), C.POINTER(i32)]),
        "rayt_cache_device_buffer": (i32, [vp, C.c_char_p, C.POINTER(vp), C.POINTER(C.c_size_t)]),
        "rayt_cache_read_buffer": (i32, [vp, C.c_char_p, vp, C.c_size_t]),
        "rayt_cache_start_session": (i32, [vp]),
        "rayt_cache_start_transaction": (i32, [vp]),
        "rayt_cache_mark_block_used": (i32, [vp, i32]),
        "rayt_cache_mark_parent_used": (i32, [vp, i32]),
        "rayt_cache_request_block": (i32, [vp, i32]),
        "rayt_cache_transaction_filled": (i32, [vp, C.POINTER(i32)]),
        "rayt_cache_session_filled": (i32, [vp, C.POINTER(i32)]),
        "rayt_cache_end_transaction": (i32, [vp]),
        "rayt_cache_end_session": (i32, [vp]),
        "rayt_cache_stats_get": (i32, [vp, C.POINTER(CacheStats)]),
        "rayt_camera_view_proj_inv": (i32, [C.POINTER(CameraStruct), C.POINTER(f32)]),
        "rayt_renderer_create": (i32, [vp, i32, i32, C.POINTER(vp)]),
        "rayt_renderer_destroy": (None, [vp]),
        "rayt_renderer_set_frame_time_limit": (i32, [vp, C.c_double]),
        "rayt_renderer_set_lod_voxel_size": (i32, [vp, f32]),
        "rayt_renderer_set_max_passes": (i32, [vp, i32]),
        "rayt_renderer_seed": (i32, [vp, u32]),
        "rayt_renderer_record_passes": (i32, [vp, i32]),
        "rayt_renderer_use_graphs": (i32, [vp, i32]),
        "rayt_renderer_set_lod_pressure": (i32, [vp, i32, f32, f32, f32]),
        "rayt_render_frame": (i32, [vp, C.POINTER(f32)]),
        "rayt_renderer_image": (i32, [vp, C.POINTER(vp)]),
        "rayt_renderer_stream": (i32, [vp, C.POINTER(vp)]),
        "rayt_renderer_read_image": (i32, [vp, vp, C.c_size_t]),
        "rayt_renderer_pass_words": (i32, [vp, i32, vp, C.c_size_t]),
        "rayt_renderer_set_depth_output": (i32, [vp, i32]),
        "rayt_renderer_set_host_image": (i32, [vp, vp, C.c_size_t]),
        "rayt_renderer_depth": (i32, [vp, i32, C.POINTER(vp), C.POINTER(vp)]),
        "rayt_renderer_read_depth": (i32, [vp, i32, C.POINTER(f32), C.POINTER(i32), C.c_size_t]),
        "rayt_renderer_stats": (i32, [vp, C.POINTER(FrameStats)]),
        "rayt_renderer_count_fetches": (i32, [vp, C.POINTER(f32), C.POINTER(C.c_int64)]),
        "rayt_renderer_time_pass": (i32, [vp, C.POINTER(f32), i32, C.POINTER(f32)]),
        "rayt_renderer_create_views": (i32, [vp, i32, C.POINTER(i32), C.POINTER(i32), C.POINTER(vp)]),
        "rayt_render_views": (i32, [vp, C.POINTER(f32), i32]),
        "rayt_renderer_view_count": (i32, [vp]),
        "rayt_renderer_view_image": (i32, [vp, i32, C.POINTER(vp)]),
        "rayt_renderer_read_view_image": (i32, [vp, i32, vp, C.c_size_t]),
        "rayt_renderer_set_launch_shape": (i32, [vp, i32, i32, i32, i32]),
        "rayt_renderer_get_launch_shape": (i32, [vp, C.POINTER(i32)]),
        "rayt_renderer_autotune": (i32, [vp, C.POINTER(f32), i32, C.POINTER(i32)]),
        "rayt_cache_depth_view": (i32, [vp, C.POINTER(f32), f32, i32, i32, vp, vp]),
        "rayt_selftest_bounded_wait": (i32, [C.c_double, vp]),
        "rayt_testing_set_lookback_epoch": (i32, [u32]),
        "rayt_testing_cache_mark_batch": (i32, [vp, C.POINTER(i32), i32, C.POINTER(i32), i32]),
        "rayt_server_create": (i32, [vp, C.POINTER(ServerConfig), C.POINTER(vp)]),
        "rayt_server_destroy": (None, [vp]),
        "rayt_server_add_client": (i32, [vp, i32, i32, C.POINTER(i32)]),
        "rayt_server_remove_client": (i32, [vp, i32]),
        "rayt_server_seed": (i32, [vp, u32]),
        "rayt_server_submit": (i32, [vp, i32, C.POINTER(f32), C.POINTER(C.c_uint64)]),
        "rayt_server_step": (i32, [vp, C.POINTER(i32)]),
        "rayt_server_start": (i32, [vp]),
        "rayt_server_stop": (i32, [vp]),
        "rayt_server_wait": (i32, [vp, C.c_uint64, C.c_double, C.POINTER(RequestInfo)]),
        "rayt_server_client_image": (i32, [vp, i32, C.POINTER(vp)]),
        "rayt_server_read_client_image": (i32, [vp, i32, vp, C.c_size_t]),
        "rayt_server_host_image": (i32, [vp, i32, C.POINTER(vp)]),
        "rayt_server_stats_get": (i32, [vp, C.POINTER(ServerStats)]),
        "rayt_sort_i32": (i32, [vp, i32, vp]),
        "rayt_scan_i32": (i32, [vp, i32, vp]),
        "rayt_feedback_unique": (i32, [vp, i32, i32, vp, C.POINTER(i32), vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _check(rc):
    if rc != RAYT_OK:
        raise RaytError(rc, lib().rayt_last_error().decode())
    return rc


def _mat(view_proj_inv):
    m = np.ascontiguousarray(np.asarray(view_proj_inv, dtype=np.float32).reshape(16))
    return m, m.ctypes.data_as(C.POINTER(C.c_float))


def _mats(view_proj_invs, n):
    m = np.ascontiguousarray(np.asarray(view_proj_invs, dtype=np.float32).reshape(n * 16))
    return m, m.ctypes.data_as(C.POINTER(C.c_float))


# ---------------------------------------------------------------------------
def build_sphere_test(path, center, radius, depth, nodes_in_block):
    """WriteTestOctreeSphere (rayt/scene sources/stored-octree-test.cpp:317-323)."""
    n = C.c_uint32()
    _check(lib().rayt_build_sphere_test(os.fsencode(path), center[0], center[1], center[2], radius, depth,
                                        nodes_in_block, C.byref(n)))
    return n.value


def build_terrain(path, depth, nodes_in_block=4096, seed=1, base_cells=4, octaves=6, spheres=0, sphere_seed=2,
                  min_radius=8, max_radius=256):
    """BuildOctree over the seeded heightfield (+ sphere shells) source."""
    p = TerrainParams(depth, seed, base_cells, octaves, spheres, sphere_seed, min_radius, max_radius)
    nb, nn = C.c_uint32(), C.c_uint64()
    _check(lib().rayt_build_terrain(os.fsencode(path), C.byref(p), nodes_in_block, C.byref(nb), C.byref(nn)))
    return nb.value, nn.value


class Camera:
    """Camera (rayt/scene/camera.h): yaw/pitch/roll in degrees, horizontal FOV."""

    def __init__(self, yaw=0.0, pitch=0.0, roll=0.0, position=(0.0, 0.0, 0.0), field_of_view=90.0,
                 aspect_ratio=4.0 / 3.0, near_clip_plane=0.01):
        self.yaw, self.pitch, self.roll = yaw, pitch, roll
        self.position = tuple(position)
        self.field_of_view, self.aspect_ratio, self.near_clip_plane = field_of_view, aspect_ratio, near_clip_plane

    def view_proj_inv(self):
        c = CameraStruct(self.yaw, self.pitch, self.roll, (C.c_float * 3)(*self.position), self.field_of_view,
                         self.aspect_ratio, self.near_clip_plane)
        out = (C.c_float * 16)()
        _check(lib().rayt_camera_view_proj_inv(C.byref(c), out))
        return np.array(out[:], dtype=np.float32)


class StoredOctreeLoader:
    def __init__(self, path):
        h = C.c_void_p()
        _check(lib().rayt_tree_open(os.fsencode(path), C.byref(h)))
        self._h = h
        info = TreeInfo()
        _check(lib().rayt_tree_info_get(h, C.byref(info)))
        self.info = info
        self.channels = []
        for i in range(info.channels_count):
            b = C.c_int()
            name = C.create_string_buffer(256)
            _check(lib().rayt_tree_channel(h, i, C.byref(b), name, 256))
            self.channels.append((name.value.decode(), b.value))

    @property
    def handle(self):
        return self._h

    def header(self):
        return self.info

    def BytesInBlockContent(self):
        return self.info.content_bytes

    def LoadBlock(self, index):
        hdr = BlockHeader()
        buf = np.zeros(self.info.content_bytes, np.uint8)
        _check(lib().rayt_tree_load_block(self._h, index, C.byref(hdr), buf.ctypes.data, buf.nbytes))
        return hdr, buf

    def close(self):
        if self._h:
            lib().rayt_tree_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GPUOctreeCacheManager:
    def __init__(self, max_blocks_count, loader):
        self.loader = loader
        h = C.c_void_p()
        _check(lib().rayt_cache_create(loader.handle, max_blocks_count, C.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def InitialFillCache(self):
        _check(lib().rayt_cache_initial_fill(self._h))

    def root_node_index(self):
        v = C.c_int()
        _check(lib().rayt_cache_root_node_index(self._h, C.byref(v)))
        return v.value

    def blocks(self):
        a, b = C.c_int(), C.c_int()
        _check(lib().rayt_cache_blocks(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def depth_view(self, view_proj_inv, lod_voxel_size, width, height, device_out=None):
        """raytracer.cl's debug depth view over the cache as it is; returns an
        (height, width, 4) uint8 array (or fills a device buffer with a
        data_ptr() and returns it)."""
        m, p = _mat(view_proj_inv)
        if device_out is not None:
            _check(lib().rayt_cache_depth_view(self._h, p, lod_voxel_size, width, height, _ptr(device_out), None))
            return device_out
        import torch
        buf = torch.empty((height, width, 4), dtype=torch.uint8, device="cuda")
        _check(lib().rayt_cache_depth_view(self._h, p, lod_voxel_size, width, height, buf.data_ptr(), None))
        return buf.cpu().numpy()

    def read_buffer(self, name, dtype=np.uint8):
        size = C.c_size_t()
        ptr = C.c_void_p()
        _check(lib().rayt_cache_device_buffer(self._h, name.encode(), C.byref(ptr), C.byref(size)))
        out = np.zeros(size.value, np.uint8)
        _check(lib().rayt_cache_read_buffer(self._h, name.encode(), out.ctypes.data, out.nbytes))
        return out.view(dtype)

    def StartRequestSession(self):
        _check(lib().rayt_cache_start_session(self._h))

    def StartRequestTransaction(self):
        _check(lib().rayt_cache_start_transaction(self._h))

    def MarkBlockAsUsed(self, slot):
        _check(lib().rayt_cache_mark_block_used(self._h, slot))

    def MarkParentAsUsed(self, slot):
        _check(lib().rayt_cache_mark_parent_used(self._h, slot))

    def RequestBlock(self, block):
        _check(lib().rayt_cache_request_block(self._h, block))

    def TransactionFilledCache(self):
        v = C.c_int()
        _check(lib().rayt_cache_transaction_filled(self._h, C.byref(v)))
        return bool(v.value)

    def SessionFilledCache(self):
        v = C.c_int()
        _check(lib().rayt_cache_session_filled(self._h, C.byref(v)))
        return bool(v.value)

    def EndRequestTransaction(self):
        _check(lib().rayt_cache_end_transaction(self._h))

    def EndRequestSession(self):
        _check(lib().rayt_cache_end_session(self._h))

    def stats(self):
        s = CacheStats()
        _check(lib().rayt_cache_stats_get(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in CacheStats._fields_}

    def close(self):
        if self._h:
            lib().rayt_cache_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GPURayTracer:
    """GPURayTracer (rayt/GPU_renderer/gpu-ray-tracer.h:11-55).

    GPURayTracer(cache, w, h) is the reference's one-view renderer.
    GPURayTracer.views(cache, [(w, h), ...]) is the batched form: every frame
    (RenderViews) traces all views in the same launches and cache session."""

    def __init__(self, cache_manager, frame_width, frame_height, _sizes=None):
        self.cache = cache_manager
        h = C.c_void_p()
        if _sizes is None:
            self.sizes = [(frame_width, frame_height)]
            _check(lib().rayt_renderer_create(cache_manager.handle, frame_width, frame_height, C.byref(h)))
        else:
            self.sizes = [(int(w), int(hh)) for w, hh in _sizes]
            n = len(self.sizes)
            ws = (C.c_int * n)(*[w for w, _ in self.sizes])
            hs = (C.c_int * n)(*[hh for _, hh in self.sizes])
            _check(lib().rayt_renderer_create_views(cache_manager.handle, n, ws, hs, C.byref(h)))
        self.width, self.height = self.sizes[0]
        self._h = h

    @classmethod
    def views(cls, cache_manager, sizes):
        return cls(cache_manager, 0, 0, _sizes=list(sizes))

    @property
    def n_views(self):
        return len(self.sizes)

    def set_frame_time_limit(self, seconds):
        _check(lib().rayt_renderer_set_frame_time_limit(self._h, seconds))

    def set_lod_voxel_size(self, size):
        _check(lib().rayt_renderer_set_lod_voxel_size(self._h, size))

    def set_max_passes(self, n):
        _check(lib().rayt_renderer_set_max_passes(self._h, n))

    def seed(self, seed):
        _check(lib().rayt_renderer_seed(self._h, seed))

    def set_lod_pressure(self, on=True, max_lod_voxel_size=16.0, grow=1.5, shrink=1.25):
        """Coarser LOD after frames whose session filled the cache (see
        rayt_renderer_set_lod_pressure)."""
        _check(lib().rayt_renderer_set_lod_pressure(self._h, 1 if on else 0, max_lod_voxel_size, grow, shrink))

    def use_graphs(self, on=True):
        _check(lib().rayt_renderer_use_graphs(self._h, 1 if on else 0))

    def record_passes(self, on=True):
        _check(lib().rayt_renderer_record_passes(self._h, 1 if on else 0))

    def RenderFrame(self, camera_or_matrix):
        if isinstance(camera_or_matrix, Camera):
            camera_or_matrix = camera_or_matrix.view_proj_inv()
        m, p = _mat(camera_or_matrix)
        _check(lib().rayt_render_frame(self._h, p))

    def RenderViews(self, matrices):
        """One frame of every view; matrices: n_views view_proj_inv matrices."""
        mats = [c.view_proj_inv() if isinstance(c, Camera) else c for c in matrices]
        m, p = _mats(mats, self.n_views)
        _check(lib().rayt_render_views(self._h, p, self.n_views))

    def set_launch_shape(self, tile_w_log2, refill, ctas_per_sm=0, step_budget=16):
        """See rayt_renderer_set_launch_shape; results do not depend on it."""
        _check(lib().rayt_renderer_set_launch_shape(self._h, tile_w_log2, refill, ctas_per_sm, step_budget))

    def launch_shape(self):
        """(tile_w_log2, refill, ctas_per_sm, step_budget)"""
        out = (C.c_int * 4)()
        _check(lib().rayt_renderer_get_launch_shape(self._h, out))
        return tuple(out[:])

    def autotune(self, matrices, reps=3):
        m, p = _mats(matrices, self.n_views)
        out = (C.c_int * 4)()
        _check(lib().rayt_renderer_autotune(self._h, p, reps, out))
        return tuple(out[:])

    def stream_handle(self):
        """The cudaStream_t (as an int) the renderer runs on."""
        p = C.c_void_p()
        _check(lib().rayt_renderer_stream(self._h, C.byref(p)))
        return p.value or 0

    def out_image_device_ptr(self, view=0):
        p = C.c_void_p()
        _check(lib().rayt_renderer_view_image(self._h, view, C.byref(p)))
        return p.value

    def read_image(self, out=None, view=0):
        w, h = self.sizes[view]
        if out is None:
            out = np.zeros((h, w, 4), np.uint8)
        _check(lib().rayt_renderer_read_view_image(self._h, view, out.ctypes.data, out.nbytes))
        return out

    def pass_words(self, p):
        out = np.zeros(sum(w * h for w, h in self.sizes), np.int32)
        _check(lib().rayt_renderer_pass_words(self._h, p, out.ctypes.data, out.size))
        return out

    def set_host_image(self, address, nbytes=0):
        """Host delivery (rayt_renderer_set_host_image): every frame from the
        next one on also leaves its RGBA8 image at `address` (page-locked
        host memory of at least width * height * 4 bytes, e.g. a pinned torch
        tensor's data_ptr()) when RenderFrame returns; None switches it off."""
        _check(lib().rayt_renderer_set_host_image(self._h, address or None, nbytes if address else 0))

    def set_depth_output(self, on=True):
        """Per-pixel depth and hit-node buffers from the next frame on (see
        rayt_renderer_set_depth_output)."""
        _check(lib().rayt_renderer_set_depth_output(self._h, 1 if on else 0))

    def read_depth(self, view=0):
        """(depth float32 [h, w], hit node int32 [h, w]) of the last frame."""
        w, h = self.sizes[view]
        depth = np.zeros((h, w), np.float32)
        nodes = np.zeros((h, w), np.int32)
        _check(lib().rayt_renderer_read_depth(self._h, view, depth.ctypes.data_as(C.POINTER(C.c_float)),
                                              nodes.ctypes.data_as(C.POINTER(C.c_int32)), w * h))
        return depth, nodes

    def depth_device_ptrs(self, view=0):
        """Device pointers (depth, hit nodes) of a view."""
        d, n = C.c_void_p(), C.c_void_p()
        _check(lib().rayt_renderer_depth(self._h, view, C.byref(d), C.byref(n)))
        return d.value, n.value

    def stats(self):
        s = FrameStats()
        _check(lib().rayt_renderer_stats(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in FrameStats._fields_}

    def count_fetches(self, view_proj_inv):
        m, p = _mats(view_proj_inv, self.n_views)
        out = (C.c_int64 * 6)()
        _check(lib().rayt_renderer_count_fetches(self._h, p, out))
        return dict(zip(["rays", "link_fetches", "far_fetches", "iterations", "hits", "faults"], out[:]))

    def time_pass(self, view_proj_inv, reps):
        m, p = _mats(view_proj_inv, self.n_views)
        ms = C.c_float()
        _check(lib().rayt_renderer_time_pass(self._h, p, reps, C.byref(ms)))
        return ms.value

    def close(self):
        if self._h:
            lib().rayt_renderer_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class RenderServer:
    """Served form: frames of many clients against one shared cache with
    continuous batching (rayt_server_*).  No counterpart in the reference."""

    def __init__(self, cache_manager, max_clients=16, framebuffer_bytes=1 << 30, max_rays_in_flight=1 << 25,
                 max_passes=8, lod_voxel_size=1.0, deliver_to_host=False):
        self.cache = cache_manager
        cfg = ServerConfig(max_clients, framebuffer_bytes, max_rays_in_flight, max_passes, lod_voxel_size,
                           1 if deliver_to_host else 0)
        h = C.c_void_p()
        _check(lib().rayt_server_create(cache_manager.handle, C.byref(cfg), C.byref(h)))
        self._h = h
        self.sizes = {}

    def add_client(self, width, height):
        c = C.c_int()
        _check(lib().rayt_server_add_client(self._h, width, height, C.byref(c)))
        self.sizes[c.value] = (width, height)
        return c.value

    def remove_client(self, client):
        _check(lib().rayt_server_remove_client(self._h, client))
        self.sizes.pop(client, None)

    def seed(self, seed):
        _check(lib().rayt_server_seed(self._h, seed))

    def submit(self, client, camera_or_matrix):
        if isinstance(camera_or_matrix, Camera):
            camera_or_matrix = camera_or_matrix.view_proj_inv()
        m, p = _mat(camera_or_matrix)
        r = C.c_uint64()
        _check(lib().rayt_server_submit(self._h, client, p, C.byref(r)))
        return r.value

    def step(self):
        n = C.c_int()
        _check(lib().rayt_server_step(self._h, C.byref(n)))
        return n.value

    def start(self):
        _check(lib().rayt_server_start(self._h))

    def stop(self):
        _check(lib().rayt_server_stop(self._h))

    def wait(self, request, timeout=60.0):
        info = RequestInfo()
        _check(lib().rayt_server_wait(self._h, request, timeout, C.byref(info)))
        return {k: getattr(info, k) for k, _ in RequestInfo._fields_}

    def read_image(self, client, out=None):
        w, h = self.sizes[client]
        if out is None:
            out = np.zeros((h, w, 4), np.uint8)
        _check(lib().rayt_server_read_client_image(self._h, client, out.ctypes.data, out.nbytes))
        return out

    def host_image(self, client):
        """Zero-copy view of the pinned host copy of the client's last frame."""
        w, h = self.sizes[client]
        p = C.c_void_p()
        _check(lib().rayt_server_host_image(self._h, client, C.byref(p)))
        return np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_uint8)), shape=(h, w, 4))

    def stats(self):
        s = ServerStats()
        _check(lib().rayt_server_stats_get(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in ServerStats._fields_}

    def close(self):
        if self._h:
            lib().rayt_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- feedback primitives on device arrays (any object with a device pointer) --
def _ptr(x):
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    return int(x)


def GPUSort(device_array, n, stream=None):
    """GPUSort::Sort: ascending signed int32 sort in place."""
    _check(lib().rayt_sort_i32(_ptr(device_array), n, stream))


def GPUScan(device_array, n, stream=None):
    """GPUScan::Scan: inclusive prefix sum in place (wrapping int32)."""
    _check(lib().rayt_scan_i32(_ptr(device_array), n, stream))


def feedback_unique(device_words, n, nodes_in_block, device_unique_out, stream=None):
    """GetUnique: returns the unique count; the values land in device_unique_out."""
    cnt = C.c_int()
    _check(lib().rayt_feedback_unique(_ptr(device_words), n, nodes_in_block, _ptr(device_unique_out),
                                      C.byref(cnt), stream))
    return cnt.value
