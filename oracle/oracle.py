"""ORACLE - test infrastructure only (tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py).  ctypes wrapper over oracle/_build/
librayt_oracle.so, the CPU restatement of the reference's per-frame path in
oracle/rayt_oracle.cpp.  The product package never imports this module."""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "librayt_oracle.so")
_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("oracle not built: %s" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        vp, i32 = C.c_void_p, C.c_int
        sig = {
            "oracle_last_error": (C.c_char_p, []),
            "oracle_tree_open": (vp, [C.c_char_p]),
            "oracle_tree_close": (None, [vp]),
            "oracle_tree_blocks": (i32, [vp]),
            "oracle_tree_nib": (i32, [vp]),
            "oracle_cache_create": (vp, [vp, i32]),
            "oracle_cache_destroy": (None, [vp]),
            "oracle_cache_initial_fill": (i32, [vp]),
            "oracle_cache_root": (i32, [vp]),
            "oracle_cache_loaded": (i32, [vp]),
            "oracle_cache_max_blocks": (i32, [vp]),
            "oracle_cache_read": (i32, [vp, i32, vp, C.c_longlong]),
            "oracle_cache_counters": (None, [vp, C.POINTER(C.c_longlong)]),
            "oracle_renderer_create": (vp, [vp, i32, i32, C.c_float, C.c_double, i32]),
            "oracle_renderer_create_views": (vp, [vp, i32, C.POINTER(i32), C.POINTER(i32), C.c_float, C.c_double, i32]),
            "oracle_frame_view_image": (i32, [vp, i32, vp]),
            "oracle_renderer_destroy": (None, [vp]),
            "oracle_renderer_record": (None, [vp, i32]),
            "oracle_render_frame": (i32, [vp, C.POINTER(C.c_float)]),
            "oracle_frame_image": (i32, [vp, vp]),
            "oracle_frame_pass_words": (i32, [vp, i32, vp]),
            "oracle_frame_depth": (i32, [vp, vp, vp]),
            "oracle_renderer_counters": (None, [vp, C.POINTER(C.c_longlong)]),
            "oracle_trace_once": (i32, [vp, C.POINTER(C.c_float), vp, vp]),
            "oracle_depth_view": (i32, [vp, C.POINTER(C.c_float), C.c_float, i32, i32, vp]),
            "oracle_sort": (None, [vp, i32]),
            "oracle_scan": (None, [vp, i32]),
            "oracle_feedback_unique": (i32, [vp, i32, i32, vp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _m(mat):
    m = np.ascontiguousarray(np.asarray(mat, np.float32).reshape(16))
    return m, m.ctypes.data_as(C.POINTER(C.c_float))


class OracleScene:
    """Block file + cache + renderer on the CPU (reference semantics)."""

    def __init__(self, path, max_blocks=0, width=0, height=0, lod=1.0, time_limit=1e30, max_passes=0, views=None):
        L = lib()
        self.tree = L.oracle_tree_open(os.fsencode(path))
        if not self.tree:
            raise RuntimeError("oracle: " + L.oracle_last_error().decode())
        self.cache = L.oracle_cache_create(self.tree, max_blocks)
        if L.oracle_cache_initial_fill(self.cache) != 0:
            raise RuntimeError("oracle: " + L.oracle_last_error().decode())
        self.nib = L.oracle_tree_nib(self.tree)
        self.max_blocks = L.oracle_cache_max_blocks(self.cache)
        self.w, self.h = width, height
        self.views = None
        if views:
            # several views traced together per frame (the batched form)
            self.views = [(int(a), int(b)) for a, b in views]
            n = len(self.views)
            ws = (C.c_int * n)(*[a for a, _ in self.views])
            hs = (C.c_int * n)(*[b for _, b in self.views])
            self.w, self.h = self.views[0]
            self.r = L.oracle_renderer_create_views(self.cache, n, ws, hs, lod, time_limit, max_passes)
        else:
            self.r = L.oracle_renderer_create(self.cache, width, height, lod, time_limit, max_passes) if width else None

    def root(self):
        return lib().oracle_cache_root(self.cache)

    def record(self, on=True):
        lib().oracle_renderer_record(self.r, 1 if on else 0)

    def render(self, mat):
        m, p = _m(mat)
        n = lib().oracle_render_frame(self.r, p)
        if n < 0:
            raise RuntimeError("oracle: " + lib().oracle_last_error().decode())
        img = np.zeros((self.h, self.w, 4), np.uint8)
        lib().oracle_frame_image(self.r, img.ctypes.data)
        return n, img

    def render_views(self, mats):
        """One frame of every view; returns (passes, [image per view])."""
        m = np.ascontiguousarray(np.asarray(mats, np.float32).reshape(len(self.views) * 16))
        n = lib().oracle_render_frame(self.r, m.ctypes.data_as(C.POINTER(C.c_float)))
        if n < 0:
            raise RuntimeError("oracle: " + lib().oracle_last_error().decode())
        imgs = []
        for v, (w, h) in enumerate(self.views):
            img = np.zeros((h, w, 4), np.uint8)
            lib().oracle_frame_view_image(self.r, v, img.ctypes.data)
            imgs.append(img)
        return n, imgs

    def pass_words(self, i):
        out = np.zeros(sum(a * b for a, b in self.views) if self.views else self.w * self.h, np.int32)
        if lib().oracle_frame_pass_words(self.r, i, out.ctypes.data) != 0:
            raise IndexError(i)
        return out

    def depth(self):
        """(depth, hit node) of the last frame: one (h, w) pair per view (a
        single pair without views)."""
        n = sum(a * b for a, b in self.views) if self.views else self.w * self.h
        depth = np.zeros(n, np.float32)
        nodes = np.zeros(n, np.int32)
        lib().oracle_frame_depth(self.r, depth.ctypes.data, nodes.ctypes.data)
        if not self.views:
            return depth.reshape(self.h, self.w), nodes.reshape(self.h, self.w)
        out, o = [], 0
        for w, h in self.views:
            out.append((depth[o:o + w * h].reshape(h, w), nodes[o:o + w * h].reshape(h, w)))
            o += w * h
        return out

    def render_size(self, w, h, mat, lod=1.0):
        """A one-view frame of size (w, h) over this scene's cache, by a second
        renderer kept per size (for a resident cache: the frame any renderer
        would draw).  Returns (passes, image)."""
        if not hasattr(self, "_extra"):
            self._extra = {}
        if (w, h) not in self._extra:
            self._extra[w, h] = lib().oracle_renderer_create(self.cache, w, h, lod, 1e30, 0)
        r = self._extra[w, h]
        m, p = _m(mat)
        n = lib().oracle_render_frame(r, p)
        if n < 0:
            raise RuntimeError("oracle: " + lib().oracle_last_error().decode())
        img = np.zeros((h, w, 4), np.uint8)
        lib().oracle_frame_image(r, img.ctypes.data)
        return n, img

    def trace_once(self, mat):
        m, p = _m(mat)
        words = np.zeros(self.w * self.h, np.int32)
        rgba = np.zeros((self.h, self.w, 4), np.uint8)
        lib().oracle_trace_once(self.r, p, words.ctypes.data, rgba.ctypes.data)
        return words, rgba

    def depth_view(self, mat, lod, w, h):
        """raytracer.cl's debug depth view over the cache as it is."""
        m, p = _m(mat)
        out = np.zeros((h, w, 4), np.uint8)
        lib().oracle_depth_view(self.cache, p, lod, w, h, out.ctypes.data)
        return out

    def counters(self):
        out = (C.c_longlong * 6)()
        lib().oracle_renderer_counters(self.r, out)
        return dict(zip(["rays", "link_fetches", "far_fetches", "iterations", "hits", "faults"], out[:]))

    def read(self, channel, nbytes):
        out = np.zeros(nbytes, np.uint8)
        if lib().oracle_cache_read(self.cache, channel, out.ctypes.data, nbytes) != 0:
            raise ValueError("bad oracle cache read")
        return out

    def close(self):
        L = lib()
        for r in getattr(self, "_extra", {}).values():
            L.oracle_renderer_destroy(r)
        self._extra = {}
        if self.r:
            L.oracle_renderer_destroy(self.r)
            self.r = None
        if self.cache:
            L.oracle_cache_destroy(self.cache)
            self.cache = None
        if self.tree:
            L.oracle_tree_close(self.tree)
            self.tree = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def sort(a):
    a = np.ascontiguousarray(a, np.int32).copy()
    lib().oracle_sort(a.ctypes.data, a.size)
    return a


def scan(a):
    a = np.ascontiguousarray(a, np.int32).copy()
    lib().oracle_scan(a.ctypes.data, a.size)
    return a


def feedback_unique(words, nib):
    w = np.ascontiguousarray(words, np.int32).copy()
    out = np.zeros(max(1, w.size), np.int32)
    n = lib().oracle_feedback_unique(w.ctypes.data, w.size, nib, out.ctypes.data)
    return out[:n].copy()
