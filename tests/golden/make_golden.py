"""Generates the golden fixtures in tests/golden/ by running the REFERENCE's own
code: its builder, loader, block cache, renderer, feedback extractor, GPU sort
and scan, camera, and its .cl kernels compiled as C++, all linked against the
fake OpenCL runtime in oracle/ref_harness/ (oracle/build_ref.sh builds it into
oracle/_ref/librayt_ref.so).  Only the development container has the reference
sources, so this script runs there; the fixtures it writes are committed.

    RAYT_REFERENCE=<reference checkout> python tests/golden/make_golden.py [part ...]

Parts (default: every part but builder_large): builder, sphere_cache, frames,
depth, sort_scan, feedback, cameras, and builder_large (the depth-12 benchmark
scene through the reference builder: a multi-GB file and several minutes).
golden.json keeps the entries of parts that were not regenerated.
"""
import ctypes as C
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from tests.golden.common import (BUILDER_CASES, CAMERA_SWEEP, DEPTH_CASES, FRAME_CASES, LARGE_BUILDER_CASES,  # noqa: E402
                                 SPHERE_CACHE_CASES, camera_sweep, canonical_tree_bytes, canonical_tree_sha,
                                 feedback_words, sha)

REF = os.path.join(ROOT, "oracle", "_ref", "librayt_ref.so")


def load_ref():
    subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_ref.sh")], check=True, stdout=subprocess.DEVNULL)
    L = C.CDLL(REF)
    vp = C.c_void_p
    L.ref_session_open.restype = vp
    L.ref_renderer_create.restype = vp
    L.ref_renderer_create.argtypes = [vp, C.c_int, C.c_int, C.c_float, C.c_double]
    for f in ["ref_session_root", "ref_session_blocks", "ref_session_nib", "ref_session_max_blocks",
              "ref_session_close", "ref_renderer_destroy"]:
        getattr(L, f).argtypes = [vp]
    L.ref_render_frame.argtypes = [vp, vp]
    L.ref_frame_image.argtypes = [vp, vp]
    L.ref_frame_pass_words.argtypes = [vp, C.c_int, vp]
    L.ref_frame_pass_links_hash.argtypes = [vp, C.c_int]
    L.ref_frame_pass_links_hash.restype = C.c_ulonglong
    L.ref_session_read.argtypes = [vp, C.c_char_p, vp, C.c_longlong]
    L.ref_build_sphere.argtypes = [C.c_char_p] + [C.c_float] * 4 + [C.c_int, C.c_int]
    L.ref_build_terrain.argtypes = [C.c_char_p, vp, C.c_int]
    L.ref_camera_matrix.argtypes = [vp, vp]
    L.ref_sort.argtypes = [vp, C.c_int]
    L.ref_scan.argtypes = [vp, C.c_int]
    L.ref_feedback_unique.argtypes = [vp, C.c_int, C.c_int, vp]
    L.ref_session_depth_view.argtypes = [vp, vp, C.c_float, C.c_int, C.c_int, vp]
    return L


def build(L, case, path):
    if case["kind"] == "sphere":
        cx, cy, cz = case["center"]
        L.ref_build_sphere(path.encode(), cx, cy, cz, case["radius"], case["depth"], case["nib"])
    else:
        p = case["terrain"]
        arr = (C.c_int * 8)(p["depth"], p["seed"], p["base_cells"], p["octaves"], p["spheres"], p["sphere_seed"],
                            p["min_radius"], p["max_radius"])
        L.ref_build_terrain(path.encode(), arr, case["nib"])


def cache_hashes(L, s, channels):
    mb = L.ref_session_max_blocks(s)
    nib = L.ref_session_nib(s)
    out = {}
    for name, b in channels:
        buf = np.zeros(mb * nib * b, np.uint8)
        assert L.ref_session_read(s, name.encode(), buf.ctypes.data, buf.size) == 0
        out[name] = sha(buf)
    far = np.zeros(mb * 8 * 4, np.uint8)
    assert L.ref_session_read(s, b"far pointers", far.ctypes.data, far.size) == 0
    out["far pointers"] = sha(far)
    return out


def ref_matrix(L, cam, aspect):
    m = np.zeros(16, np.float32)
    cam_arr = np.array(list(cam) + [aspect], np.float32)
    L.ref_camera_matrix(cam_arr.ctypes.data, m.ctypes.data)
    return m, cam_arr


class Trees:
    """Reference-built trees of BUILDER_CASES, built on first use."""

    def __init__(self, L, tmp):
        self.L, self.tmp, self.paths = L, tmp, {}

    def __getitem__(self, name):
        if name not in self.paths:
            path = os.path.join(self.tmp, name + ".tree")
            build(self.L, BUILDER_CASES[name], path)
            self.paths[name] = path
        return self.paths[name]


def part_builder(L, golden, trees):
    golden["builder"] = {}
    for name in BUILDER_CASES:
        data = canonical_tree_bytes(trees[name])
        golden["builder"][name] = {"sha256": sha(np.frombuffer(data, np.uint8)), "bytes": len(data)}


def part_builder_large(L, golden, trees):
    """The benchmark scenes too large to commit or to build in the CPU tests:
    only the canonical hash of the reference builder's file is kept."""
    golden.setdefault("builder_large", {})
    for name, case in LARGE_BUILDER_CASES.items():
        path = os.path.join(trees.tmp, name + ".tree")
        build(L, case, path)
        digest, size = canonical_tree_sha(path)
        golden["builder_large"][name] = {"sha256": digest, "bytes": size}
        os.unlink(path)


def part_sphere_cache(L, golden, trees):
    golden["sphere_cache"] = {}
    for name, case in SPHERE_CACHE_CASES.items():
        s = L.ref_session_open(trees[case["tree"]].encode(), case["max_blocks"])
        golden["sphere_cache"][name] = {
            "root": L.ref_session_root(s),
            "hashes": cache_hashes(L, s, [("node links", 4), ("node index", 4), ("node index % 211", 1)]),
        }
        L.ref_session_close(s)


def part_frames(L, golden, trees):
    golden["frames"] = {}
    images = {}
    for name, case in FRAME_CASES.items():
        L.ref_srand(case["seed"])
        s = L.ref_session_open(trees[case["tree"]].encode(), case["max_blocks"])
        w, h = case["size"]
        r = L.ref_renderer_create(s, w, h, case["lod"], 1e30)
        frames = []
        for cam in case["cameras"]:
            m, cam_arr = ref_matrix(L, cam, w / h)
            npass = L.ref_render_frame(r, cam_arr.ctypes.data)
            img = np.zeros((h, w, 4), np.uint8)
            L.ref_frame_image(r, img.ctypes.data)
            words = []
            for p in range(npass):
                wd = np.zeros(w * h, np.int32)
                L.ref_frame_pass_words(r, p, wd.ctypes.data)
                words.append(sha(wd))
            frames.append({
                "matrix": [float(x) for x in m],
                "passes": npass,
                "image_sha256": sha(img),
                "surface_pixels": int((~((img[..., 0] == 0) & (img[..., 1] == 216) & (img[..., 2] == 255))).sum()),
                "pass_words_sha256": words,
                "cache": cache_hashes(L, s, [("node links", 4), ("normals", 4), ("colors", 4)]),
                "root": L.ref_session_root(s),
            })
            if case.get("keep_images"):
                images["%s_%d" % (name, len(frames) - 1)] = img
        golden["frames"][name] = frames
        L.ref_renderer_destroy(r)
        L.ref_session_close(s)
    if images:
        np.savez_compressed(os.path.join(HERE, "frame_images.npz"), **images)


def part_depth(L, golden, trees):
    """The debug depth view (raytracer.cl) over freshly filled caches."""
    depth = {}
    for name, case in DEPTH_CASES.items():
        s = L.ref_session_open(trees[case["tree"]].encode(), case["max_blocks"])
        w, h = case["size"]
        m, _ = ref_matrix(L, case["camera"], w / h)
        img = np.zeros((h, w, 4), np.uint8)
        L.ref_session_depth_view(s, m.ctypes.data, case["lod"], w, h, img.ctypes.data)
        depth[name + "_matrix"] = m
        depth[name + "_image"] = img
        L.ref_session_close(s)
    np.savez_compressed(os.path.join(HERE, "depth_views.npz"), **depth)


def part_sort_scan(L, golden, trees):
    """GPUSort / GPUScan known-answer runs (test-application.cpp:150-240):
    n = 2013, values rand() % 201 - 100 after srand(seed), 10 trials."""
    L.ref_srand(12345)
    sort_in, sort_out, scan_out = [], [], []
    for _ in range(10):
        a = np.array([L.ref_rand() % 201 - 100 for _ in range(2013)], np.int32)
        b = a.copy()
        L.ref_sort(b.ctypes.data, b.size)
        c = a.copy()
        L.ref_scan(c.ctypes.data, c.size)
        sort_in.append(a)
        sort_out.append(b)
        scan_out.append(c)
    np.savez_compressed(os.path.join(HERE, "sort_scan.npz"), inputs=np.stack(sort_in), sorted=np.stack(sort_out),
                        scanned=np.stack(scan_out))


def part_feedback(L, golden, trees):
    """Feedback unique (GetUnique) on synthetic feedback words."""
    fb = {}
    for key, (n, nib, seed) in {"small": (5000, 37, 5), "c2_like": (1 << 16, 4096, 6),
                                "all_nohit": (4096, 4096, 7), "no_nohit": (3000, 64, 8)}.items():
        words = feedback_words(n, seed, no_hit=(key != "no_nohit"), all_nohit=(key == "all_nohit"))
        w = words.copy()
        out = np.zeros(n, np.int32)
        cnt = L.ref_feedback_unique(w.ctypes.data, n, nib, out.ctypes.data)
        fb[key + "_words"] = words
        fb[key + "_unique"] = out[:cnt].copy()
        fb[key + "_nib"] = np.array([nib], np.int32)
    np.savez_compressed(os.path.join(HERE, "feedback_unique.npz"), **fb)


def part_cameras(L, golden, trees):
    """Camera::ViewProjectionMatrix().Inverse() for a seeded sweep of cameras
    (rayt/scene/camera.cpp:23-28, rayt/util/mat.cpp:20-107)."""
    cams = camera_sweep(CAMERA_SWEEP["count"], CAMERA_SWEEP["seed"])
    out = np.zeros((len(cams), 16), np.float32)
    for i, c in enumerate(cams):
        out[i], _ = ref_matrix(L, c[:7], c[7])
    np.savez_compressed(os.path.join(HERE, "cameras.npz"), cameras=cams, matrices=out)


PARTS = {"builder": part_builder, "sphere_cache": part_sphere_cache, "frames": part_frames, "depth": part_depth,
         "sort_scan": part_sort_scan, "feedback": part_feedback, "cameras": part_cameras,
         "builder_large": part_builder_large}
DEFAULT_PARTS = [p for p in PARTS if p != "builder_large"]


def main(parts):
    if not os.environ.get("RAYT_REFERENCE"):
        sys.exit("set RAYT_REFERENCE to the reference checkout (the directory holding rayt/)")
    unknown = [p for p in parts if p not in PARTS]
    if unknown:
        sys.exit("unknown parts %s (known: %s)" % (unknown, ", ".join(PARTS)))
    L = load_ref()
    gpath = os.path.join(HERE, "golden.json")
    golden = json.load(open(gpath)) if os.path.exists(gpath) else {}
    trees = Trees(L, tempfile.mkdtemp(prefix="rayt_golden_"))
    devnull = os.open(os.devnull, os.O_WRONLY)
    saved = os.dup(1)
    os.dup2(devnull, 1)  # the reference prints build reports and fill progress
    try:
        for p in parts:
            PARTS[p](L, golden, trees)
    finally:
        os.dup2(saved, 1)
        os.close(devnull)
    with open(gpath, "w") as f:
        json.dump(golden, f, indent=1, sort_keys=True)
    print("wrote golden fixtures (%s) to %s" % (", ".join(parts), HERE))


if __name__ == "__main__":
    main(sys.argv[1:] or DEFAULT_PARTS)
