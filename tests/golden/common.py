"""Case definitions and helpers shared by the golden-fixture generator and the
tests.  Everything here is integer or byte arithmetic, so it gives the same
result on every host."""
import hashlib

import numpy as np

NO_HIT = 0x7FFFFFFF


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).view(np.uint8).tobytes()).hexdigest()


def canonical_tree_bytes(path):
    """The file with the root records past roots_count zeroed: the reference
    leaves whatever its reused block header held there, and nothing reads them
    (rayt/CPU data/stored-octree-builder-impl.h:166-201)."""
    b = bytearray(open(path, "rb").read())
    nib, blocks, root, stride, nch = np.frombuffer(bytes(b[:20]), "<u4")
    pos = 20
    for _ in range(int(nch)):
        ln = int.from_bytes(b[pos + 4:pos + 8], "little")
        pos += 8 + ln
    for i in range(int(blocks)):
        o = pos + int(stride) * i
        rc = int.from_bytes(b[o + 8:o + 12], "little")
        for r in range(rc, 8):
            b[o + 12 + 8 * r:o + 20 + 8 * r] = bytes(8)
    return bytes(b)


def canonical_tree_sha(path, chunk_blocks=4096):
    """(sha256, bytes) of canonical_tree_bytes(path), streamed block by block
    so multi-GB files need not fit in memory."""
    h = hashlib.sha256()
    size = 0
    with open(path, "rb") as f:
        head = f.read(20)
        nib, blocks, root, stride, nch = np.frombuffer(head, "<u4")
        rest = b""
        for _ in range(int(nch)):
            rec = f.read(8)
            ln = int.from_bytes(rec[4:8], "little")
            rest += rec + f.read(ln)
        h.update(head + rest)
        size += len(head) + len(rest)
        stride = int(stride)
        left = int(blocks)
        while left:
            k = min(left, chunk_blocks)
            buf = np.frombuffer(f.read(stride * k), np.uint8).copy()
            if buf.size != stride * k:
                raise ValueError("truncated tree file")
            rec = buf.reshape(k, stride)
            rc = rec[:, 8:12].copy().view("<u4").ravel()
            for r in range(8):
                rec[rc <= r, 12 + 8 * r:20 + 8 * r] = 0
            h.update(rec.tobytes())
            size += rec.size
            left -= k
        tail = f.read()
        h.update(tail)
        size += len(tail)
    return h.hexdigest(), size


def _terrain(depth, spheres=0, min_radius=8, max_radius=256, seed=1, sphere_seed=2):
    return {"depth": depth, "seed": seed, "base_cells": 4, "octaves": 6, "spheres": spheres,
            "sphere_seed": sphere_seed, "min_radius": min_radius, "max_radius": max_radius}


# Trees built by the reference builder (the sphere cases are the reference's
# own test parameters, rayt/application/test-application.cpp:134-148,262-291).
BUILDER_CASES = {
    "sphere3": {"kind": "sphere", "center": [0.3, 0.4, 0.65], "radius": 0.23, "depth": 3, "nib": 131},
    "sphere7": {"kind": "sphere", "center": [0.5, 0.5, 0.5], "radius": 0.3, "depth": 7, "nib": 111},
    "sphere11": {"kind": "sphere", "center": [0.3, 0.4, 0.65], "radius": 0.23, "depth": 11, "nib": 737},
    "terrain8s": {"kind": "terrain", "terrain": _terrain(8, spheres=60, min_radius=2, max_radius=24), "nib": 512},
    "terrain10": {"kind": "terrain", "terrain": _terrain(10), "nib": 4096},
}

# The benchmark scenes (1080p flythrough and 64-view workloads: depth 12, the
# fBm heightfield plus 2000 sphere shells of radius 8..256 voxels, 4096-node
# blocks).  Too large to commit or to build in the CPU tests: the golden file
# keeps the canonical hash of the reference builder's output, and the GPU
# tests compare the product builder's file with it.
LARGE_BUILDER_CASES = {
    "terrain12s": {"kind": "terrain", "terrain": _terrain(12, spheres=2000, min_radius=8, max_radius=256),
                   "nib": 4096},
}

# Camera::ViewProjectionMatrix().Inverse() over a seeded sweep of cameras.
CAMERA_SWEEP = {"count": 512, "seed": 5}


def camera_sweep(count, seed):
    """count x 8 float32: yaw, pitch, roll, x, y, z, horizontal fov, aspect."""
    rng = np.random.default_rng(seed)
    out = np.zeros((count, 8), np.float32)
    out[:, 0] = rng.uniform(-360, 360, count)
    out[:, 1] = rng.uniform(-90, 90, count)
    out[:, 2] = rng.uniform(-180, 180, count)
    out[:, 3:6] = rng.uniform(-1, 2, (count, 3))
    out[:, 6] = rng.uniform(20, 120, count)
    wh = rng.integers(1, 4096, (count, 2))
    out[:, 7] = wh[:, 0] / wh[:, 1]
    return out


# Cache contents after InitialFillCache (the reference's OctreeGPUTest /
# TestBuilder checks, stored-octree-test.cpp:212-233).
SPHERE_CACHE_CASES = {
    "sphere3_all": {"tree": "sphere3", "max_blocks": 0},
    "sphere7_all": {"tree": "sphere7", "max_blocks": 0},
    "sphere7_partial": {"tree": "sphere7", "max_blocks": 100},
}

# camera = yaw, pitch, roll, x, y, z, horizontal fov (aspect = width / height)
C1_CAMERA = [45.0, -30.0, 0.0, -0.06, 0.66, 1.06, 60.0]
FRAME_CASES = {
    # streaming: a cache far smaller than the tree, several frames in a row
    "stream8": {"tree": "terrain8s", "max_blocks": 200, "size": [96, 64], "lod": 1.0, "seed": 11,
                "keep_images": True,
                "cameras": [C1_CAMERA, [30.0, -25.0, 0.0, 0.1, 0.6, 1.1, 60.0], [80.0, -40.0, 5.0, 0.0, 0.8, 0.7, 70.0],
                            [200.0, -35.0, 0.0, 0.9, 0.7, -0.1, 60.0]]},
    "stream8_lod0": {"tree": "terrain8s", "max_blocks": 40, "size": [64, 48], "lod": 0.0, "seed": 3,
                     "keep_images": True,
                     "cameras": [[10.0, -20.0, 0.0, 0.3, 0.5, 1.0, 60.0], [120.0, -45.0, 0.0, 0.8, 0.7, 0.9, 75.0]]},
    # the CPU-runnable configuration: depth 10, 512 x 512, whole tree resident
    "c1": {"tree": "terrain10", "max_blocks": 0, "size": [512, 512], "lod": 1.0, "seed": 1, "cameras": [C1_CAMERA]},
    "stream8_300": {"tree": "terrain8s", "max_blocks": 300, "size": [96, 64], "lod": 1.0, "seed": 12,
                    "cameras": [C1_CAMERA, [30.0, -25.0, 0.0, 0.1, 0.6, 1.1, 60.0],
                                [80.0, -40.0, 5.0, 0.0, 0.8, 0.7, 70.0]]},
    # the same scene streamed through a cache of 600 of its 758 blocks
    "c1_stream": {"tree": "terrain10", "max_blocks": 600, "size": [256, 256], "lod": 1.0, "seed": 21,
                  "cameras": [C1_CAMERA, [30.0, -25.0, 0.0, 0.1, 0.6, 1.1, 60.0],
                              [200.0, -35.0, 0.0, 0.9, 0.7, -0.1, 60.0]]},
}

# raytracer.cl's debug depth view over the cache right after InitialFillCache
# (resident trees, and a partial cache whose faults show red)
DEPTH_CASES = {
    "resident_c1": {"tree": "terrain10", "max_blocks": 0, "size": [160, 120], "lod": 1.0, "camera": C1_CAMERA},
    "resident_lod0": {"tree": "terrain10", "max_blocks": 0, "size": [96, 80], "lod": 0.0,
                      "camera": [30.0, -25.0, 0.0, 0.1, 0.6, 1.1, 60.0]},
    "partial8s": {"tree": "terrain8s", "max_blocks": 60, "size": [128, 72], "lod": 1.0,
                  "camera": [80.0, -40.0, 5.0, 0.0, 0.8, 0.7, 70.0]},
    "sphere_lod4": {"tree": "sphere7", "max_blocks": 0, "size": [64, 64], "lod": 4.0,
                    "camera": [200.0, -35.0, 0.0, 0.9, 0.7, -0.1, 60.0]},
}


def _splitmix(x):
    x = (x + np.uint64(0x9E3779B97F4A7C15)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    z = x
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def feedback_words(n, seed, no_hit=True, all_nohit=False, id_bits=24):
    """Feedback words in the reference's encoding: NO_HIT (90% when no_hit),
    fault words -id-1 and hit words ((id+1)<<1)|dup, ids skewed toward small
    values so that about half are duplicates."""
    with np.errstate(over="ignore"):
        i = np.arange(n, dtype=np.uint64) + np.uint64(seed) * np.uint64(0x100000001B3)
        r1 = _splitmix(i)
        r2 = _splitmix(r1)
        r3 = _splitmix(r2)
    k = (r2 % np.uint64(id_bits)).astype(np.int64) + 1
    ids = (r3 & ((np.uint64(1) << k.astype(np.uint64)) - np.uint64(1))).astype(np.int64)
    fault = (r1 >> np.uint64(7)) & np.uint64(1)
    dup = (r1 >> np.uint64(9)) & np.uint64(1)
    words = np.where(fault == 1, -ids - 1, ((ids + 1) << 1) | dup.astype(np.int64))
    if no_hit:
        words = np.where((r1 % np.uint64(10)) != 0, NO_HIT, words)
    if all_nohit:
        words[:] = NO_HIT
    return words.astype(np.int32)
