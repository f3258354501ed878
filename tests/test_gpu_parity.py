"""GPU parity: the CUDA path through the C ABI against the golden fixtures made
by the reference's own code and against the CPU oracle.  Bit-exact throughout:
node IDs, feedback words, RGBA8 pixels and cache buffers are integers."""
import os

import numpy as np
import pytest

import rayt_gb300 as R
from tests.conftest import libc_srand
from tests.golden.common import C1_CAMERA, FRAME_CASES, SPHERE_CACHE_CASES, sha

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _scene(path, max_blocks, w, h, lod=1.0, seed=1):
    ld = R.StoredOctreeLoader(path)
    cm = R.GPUOctreeCacheManager(max_blocks, ld)
    cm.InitialFillCache()
    rt = R.GPURayTracer(cm, w, h)
    rt.set_lod_voxel_size(lod)
    rt.set_frame_time_limit(1e30)
    rt.seed(seed)
    return ld, cm, rt


def _matrix(cam, w, h):
    c = R.Camera(cam[0], cam[1], cam[2], cam[3:6], cam[6], w / h)
    return c.view_proj_inv()


@pytest.mark.parametrize("name", sorted(SPHERE_CACHE_CASES))
def test_sphere_cache_contents(trees, golden, name):
    """InitialFillCache leaves the reference's exact cache buffers
    (links rewritten to the cache format, far pointers, channels)."""
    case = SPHERE_CACHE_CASES[name]
    ld = R.StoredOctreeLoader(trees[case["tree"]])
    cm = R.GPUOctreeCacheManager(case["max_blocks"], ld)
    cm.InitialFillCache()
    g = golden["sphere_cache"][name]
    assert cm.root_node_index() == g["root"]
    for cname in ["node links", "node index", "node index % 211", "far pointers"]:
        assert sha(cm.read_buffer(cname)) == g["hashes"][cname], cname


@pytest.mark.parametrize("name", sorted(FRAME_CASES))
def test_frames_match_reference(trees, golden, name):
    """Every frame of every golden case: pass count, each pass's feedback
    words, the image and the cache buffers afterwards."""
    case = FRAME_CASES[name]
    w, h = case["size"]
    ld, cm, rt = _scene(trees[case["tree"]], case["max_blocks"], w, h, case["lod"], case["seed"])
    rt.record_passes(True)
    for i, g in enumerate(golden["frames"][name]):
        rt.RenderFrame(np.array(g["matrix"], np.float32))
        st = rt.stats()
        assert st["passes"] == g["passes"], "frame %d" % i
        for p in range(st["passes"]):
            assert sha(rt.pass_words(p)) == g["pass_words_sha256"][p], "frame %d pass %d" % (i, p)
        assert sha(rt.read_image()) == g["image_sha256"], "frame %d" % i
        assert cm.root_node_index() == g["root"]
        for cname in ["node links", "normals", "colors", "far pointers"]:
            assert sha(cm.read_buffer(cname)) == g["cache"][cname], "frame %d %s" % (i, cname)


def _oracle_frame(path, max_blocks, w, h, mats, lod=1.0, seed=1):
    from oracle import oracle as O
    sc = O.OracleScene(path, max_blocks, w, h, lod)
    libc_srand(seed)
    out = [sc.render(m) for m in mats]
    counters = sc.counters()
    sc.close()
    return out, counters


@pytest.mark.parametrize("size", [(1920, 1080), (333, 77), (1, 1), (8, 4), (1000, 1)])
def test_resident_frame_vs_oracle(trees, size):
    """Odd and full-HD frame sizes on the resident depth-10 scene."""
    w, h = size
    m = _matrix(C1_CAMERA, w, h)
    (ref,), _ = _oracle_frame(trees["terrain10"], 0, w, h, [m])
    ld, cm, rt = _scene(trees["terrain10"], 0, w, h)
    rt.RenderFrame(m)
    np.testing.assert_array_equal(rt.read_image(), ref[1])
    assert rt.stats()["passes"] == ref[0]


EDGE_CAMERAS = {
    "looking_away": [225.0, 30.0, 0.0, -0.5, 1.5, 1.5, 60.0],       # every ray misses
    "inside_volume": [10.0, -5.0, 0.0, 0.5, 0.45, 0.5, 90.0],        # origin inside the octree
    "straight_down": [0.0, -90.0, 0.0, 0.5, 1.2, 0.5, 40.0],         # axis-aligned rays (epsilon clamp)
    "axis_x": [-90.0, 0.0, 0.0, -0.2, 0.3, 0.5, 30.0],
    "grazing": [45.0, -1.0, 0.0, -0.1, 0.42, 1.1, 120.0],            # long shallow rays
    "rolled": [30.0, -20.0, 45.0, 0.1, 0.7, 1.2, 60.0],
}


@pytest.mark.parametrize("name", sorted(EDGE_CAMERAS))
@pytest.mark.parametrize("lod", [0.0, 1.0, 4.0])
def test_edge_cameras_vs_oracle(trees, name, lod):
    w, h = 160, 120
    m = _matrix(EDGE_CAMERAS[name], w, h)
    (ref,), _ = _oracle_frame(trees["terrain10"], 0, w, h, [m], lod=lod)
    ld, cm, rt = _scene(trees["terrain10"], 0, w, h, lod=lod)
    rt.RenderFrame(m)
    np.testing.assert_array_equal(rt.read_image(), ref[1])


def test_streaming_sequence_vs_oracle(trees):
    """A longer streamed flythrough at 320x180 (cache 250 of 790 blocks)."""
    w, h = 320, 180
    cams = [[a, -25.0 - 0.2 * a, 0.0, 0.5 - 0.6 * np.sin(np.radians(a)), 0.7, 0.5 + 0.6 * np.cos(np.radians(a)), 60.0]
            for a in range(0, 360, 30)]
    mats = [_matrix(c, w, h) for c in cams]
    refs, _ = _oracle_frame(trees["terrain8s"], 250, w, h, mats, seed=99)
    ld, cm, rt = _scene(trees["terrain8s"], 250, w, h, seed=99)
    for i, (m, ref) in enumerate(zip(mats, refs)):
        rt.RenderFrame(m)
        assert rt.stats()["passes"] == ref[0], i
        np.testing.assert_array_equal(rt.read_image(), ref[1], err_msg="frame %d" % i)


def test_fetch_counts_match_oracle(trees):
    """The algorithmic byte count of the roofline (node-link and far-pointer
    fetches per ray) is the same on the GPU as in the oracle."""
    from oracle import oracle as O
    w, h = 512, 512
    m = _matrix(C1_CAMERA, w, h)
    sc = O.OracleScene(trees["terrain10"], 0, w, h, 1.0)
    sc.trace_once(m)
    oc = sc.counters()
    sc.close()
    ld, cm, rt = _scene(trees["terrain10"], 0, w, h)
    gc = rt.count_fetches(m)
    for k in ["rays", "link_fetches", "far_fetches", "iterations", "hits", "faults"]:
        assert gc[k] == oc[k], k


def test_pass_cap_stops_frame(trees):
    w, h = 96, 64
    m = _matrix(C1_CAMERA, w, h)
    ld, cm, rt = _scene(trees["terrain8s"], 300, w, h)
    rt.set_max_passes(2)
    rt.RenderFrame(m)
    assert rt.stats()["passes"] <= 2


@pytest.mark.parametrize("name", sorted(__import__("tests.golden.common", fromlist=["DEPTH_CASES"]).DEPTH_CASES))
def test_depth_view_matches_reference(trees, name):
    """rayt_cache_depth_view against the reference's raytracer.cl run by the
    harness: red (fault/error) and black (miss) exact, grey within 1 LSB
    (CUDA's logf against the C library's)."""
    from tests.golden.common import DEPTH_CASES
    case = DEPTH_CASES[name]
    d = np.load(os.path.join(GOLDEN, "depth_views.npz"))
    w, h = case["size"]
    ld = R.StoredOctreeLoader(trees[case["tree"]])
    cm = R.GPUOctreeCacheManager(case["max_blocks"], ld)
    cm.InitialFillCache()
    img = cm.depth_view(d[name + "_matrix"], case["lod"], w, h)
    ref = d[name + "_image"]
    assert np.array_equal(img[..., 3], ref[..., 3])
    red = (ref[..., 0] == 255) & (ref[..., 1] == 0) & (ref[..., 2] == 0)
    assert np.array_equal(red, (img[..., 0] == 255) & (img[..., 1] == 0) & (img[..., 2] == 0))
    assert np.abs(img.astype(int) - ref.astype(int)).max() <= 1


def test_lod_pressure_policy(trees):
    """Decrease LOD when the cache is too small (the reference's todo): with
    the policy on, frames whose session filled the cache coarsen the next
    frame's voxel size until a frame fits; with it off the size never moves."""
    w, h = 256, 256
    m = _matrix(C1_CAMERA, w, h)
    runs = {}
    for on in (False, True):
        ld, cm, rt = _scene(trees["terrain10"], 80, w, h)
        rt.set_lod_pressure(on, max_lod_voxel_size=32.0, grow=2.0, shrink=1.25)
        seq = []
        for _ in range(10):
            rt.RenderFrame(m)
            st = rt.stats()
            seq.append((st["lod_voxel_size"], st["session_filled"]))
        runs[on] = seq
    off, on = runs[False], runs[True]
    assert all(l == 1.0 for l, _ in off)
    assert off[0][1] == 1  # the cache is too small for this frame at voxel size 1
    assert on[0] == off[0]
    f32 = np.float32
    for (l0, f0), (l1, _) in zip(on, on[1:]):  # grows after a filled session, never beyond the cap (float math)
        assert f32(l1) == (min(f32(32.0), f32(l0) * f32(2.0)) if f0 else max(f32(1.0), f32(l0) / f32(1.25)))
    assert any(f == 0 for _, f in on)  # a coarser frame fits in the cache


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.mark.parametrize("name,max_passes", [("stream8", 0), ("stream8_lod0", 0), ("c1_stream", 0), ("stream8", 2)])
def test_depth_output_vs_oracle(trees, name, max_passes):
    """Depth and hit-node buffers of streamed frames equal the oracle's bit for
    bit (depth compared as float bits: a faulted ray's advances add up in the
    same order), including rays a pass cap leaves faulted, which end with the
    distance where they stopped and their fault's parent node."""
    from oracle import oracle as O
    case = FRAME_CASES[name]
    w, h = case["size"]
    mats = [_matrix(c, w, h) for c in case["cameras"]]
    libc_srand(case["seed"])
    sc = O.OracleScene(trees[case["tree"]], case["max_blocks"], w, h, case["lod"], max_passes=max_passes)
    ld, cm, rt = _scene(trees[case["tree"]], case["max_blocks"], w, h, case["lod"], case["seed"])
    rt.set_max_passes(max_passes)
    rt.set_depth_output(True)
    capped = 0
    for i, m in enumerate(mats):
        passes, ref = sc.render(m)
        dref, nref = sc.depth()
        rt.RenderFrame(m)
        st = rt.stats()
        assert st["passes"] == passes, i
        capped += int(max_passes > 0 and passes == max_passes and st["faults"] > 0)
        np.testing.assert_array_equal(rt.read_image(), ref, err_msg="frame %d" % i)
        d, n = rt.read_depth()
        np.testing.assert_array_equal(n, nref, err_msg="frame %d hit nodes" % i)
        np.testing.assert_array_equal(_bits(d), _bits(dref), err_msg="frame %d depth" % i)
    assert np.isposinf(dref).any() and np.isfinite(dref).any()
    if max_passes:
        assert capped > 0  # some frame ended at the cap with rays still faulted
    sc.close()


def test_depth_output_resident_full_hd(trees):
    """1920x1080 on the resident depth-10 scene: depth bits and hit nodes equal
    the oracle's on every pixel; turning the output off leaves the image alone."""
    from oracle import oracle as O
    w, h = 1920, 1080
    m = _matrix(C1_CAMERA, w, h)
    sc = O.OracleScene(trees["terrain10"], 0, w, h, 1.0)
    _, ref = sc.render(m)
    dref, nref = sc.depth()
    sc.close()
    ld, cm, rt = _scene(trees["terrain10"], 0, w, h)
    rt.set_depth_output(True)
    rt.RenderFrame(m)
    d, n = rt.read_depth()
    np.testing.assert_array_equal(n, nref)
    np.testing.assert_array_equal(_bits(d), _bits(dref))
    np.testing.assert_array_equal(rt.read_image(), ref)
    rt.set_depth_output(False)
    rt.RenderFrame(m)
    np.testing.assert_array_equal(rt.read_image(), ref)
