"""GPU parity of the batched form (several views per frame in the same
persistent traversal launches and cache session) and of the traversal launch
shapes: the oracle's batched restatement for streamed frames, the one-view
oracle for resident frames, and identical results for every launch shape."""
import numpy as np
import pytest

import rayt_gb300 as R
from tests.conftest import libc_srand
from tests.golden.common import C1_CAMERA

pytestmark = pytest.mark.gpu

SIZES = [(160, 120), (33, 17), (1, 1), (128, 72), (64, 64), (200, 3)]


def _cams(n, phase=0.0):
    out = []
    for v in range(n):
        a = 30.0 + 40 * v + phase
        out.append([a, -20.0 - 5 * (v % 4), 0.0, 0.5 - 0.6 * np.sin(np.radians(a)), 0.7,
                    0.5 + 0.6 * np.cos(np.radians(a)), 60.0])
    return out


def _matrix(cam, w, h):
    return R.Camera(cam[0], cam[1], cam[2], cam[3:6], cam[6], w / h).view_proj_inv()


def _gpu_views(path, max_blocks, sizes, seed=1, lod=1.0):
    ld = R.StoredOctreeLoader(path)
    cm = R.GPUOctreeCacheManager(max_blocks, ld)
    cm.InitialFillCache()
    rt = R.GPURayTracer.views(cm, sizes)
    rt.set_lod_voxel_size(lod)
    rt.set_frame_time_limit(1e30)
    rt.seed(seed)
    return ld, cm, rt


def test_batched_resident_equals_single_views(trees):
    """Resident cache: every view equals the one-view oracle frame."""
    from oracle import oracle as O
    mats = [_matrix(c, w, h) for c, (w, h) in zip(_cams(len(SIZES)), SIZES)]
    ld, cm, rt = _gpu_views(trees["terrain10"], 0, SIZES)
    rt.RenderViews(mats)
    for v, ((w, h), m) in enumerate(zip(SIZES, mats)):
        sc = O.OracleScene(trees["terrain10"], 0, w, h)
        _, ref = sc.render(m)
        sc.close()
        np.testing.assert_array_equal(rt.read_image(view=v), ref, err_msg="view %d" % v)


def test_batched_streaming_vs_oracle(trees):
    """Streamed frames (cache 250 of 790 blocks): passes, every pass's merged
    feedback words and every view's image equal the oracle's batched frame."""
    from oracle import oracle as O
    frames = [[_matrix(c, w, h) for c, (w, h) in zip(_cams(len(SIZES), 25.0 * f), SIZES)] for f in range(6)]
    libc_srand(17)
    sc = O.OracleScene(trees["terrain8s"], 250, views=SIZES)
    sc.record(True)
    ld, cm, rt = _gpu_views(trees["terrain8s"], 250, SIZES, seed=17)
    rt.record_passes(True)
    for f, mats in enumerate(frames):
        n, imgs = sc.render_views(mats)
        rt.RenderViews(mats)
        assert rt.stats()["passes"] == n, "frame %d" % f
        for p in range(n):
            np.testing.assert_array_equal(rt.pass_words(p), sc.pass_words(p), err_msg="frame %d pass %d" % (f, p))
        for v in range(len(SIZES)):
            np.testing.assert_array_equal(rt.read_image(view=v), imgs[v], err_msg="frame %d view %d" % (f, v))
    sc.close()


def test_one_view_batch_equals_plain_renderer(trees):
    w, h = 96, 64
    mats = [_matrix(c, w, h) for c in _cams(5)]
    ld, cm, rt = _gpu_views(trees["terrain8s"], 120, [(w, h)], seed=9)
    ld2 = R.StoredOctreeLoader(trees["terrain8s"])
    cm2 = R.GPUOctreeCacheManager(120, ld2)
    cm2.InitialFillCache()
    rt2 = R.GPURayTracer(cm2, w, h)
    rt2.set_lod_voxel_size(1.0)
    rt2.set_frame_time_limit(1e30)
    rt2.seed(9)
    for m in mats:
        rt.RenderViews([m])
        rt2.RenderFrame(m)
        assert rt.stats()["passes"] == rt2.stats()["passes"]
        np.testing.assert_array_equal(rt.read_image(), rt2.read_image())


@pytest.mark.parametrize("shape", [(0, 1, 0, 1), (2, 8, 0, 7), (3, 16, 0, 16), (4, 24, 4, 64), (5, 32, 1, 0), (2, 32, 0, 16),
                                   (3, 4, 2, 3), (3, 32, 0, 16)])
def test_launch_shapes_same_result(trees, shape):
    """Tile shape, refill threshold and CTAs per SM change the schedule only."""
    from oracle import oracle as O
    w, h = 257, 131
    m = _matrix(C1_CAMERA, w, h)
    libc_srand(4)
    sc = O.OracleScene(trees["terrain8s"], 200, w, h)
    n, ref = sc.render(m)
    sc.close()
    ld = R.StoredOctreeLoader(trees["terrain8s"])
    cm = R.GPUOctreeCacheManager(200, ld)
    cm.InitialFillCache()
    rt = R.GPURayTracer(cm, w, h)
    rt.set_lod_voxel_size(1.0)
    rt.set_frame_time_limit(1e30)
    rt.seed(4)
    rt.set_launch_shape(*shape)
    assert rt.launch_shape() == shape
    rt.RenderFrame(m)
    assert rt.stats()["passes"] == n
    np.testing.assert_array_equal(rt.read_image(), ref)


def test_autotune_keeps_results(trees):
    sizes = [(320, 180), (64, 64)]
    mats = [_matrix(c, w, h) for c, (w, h) in zip(_cams(2), sizes)]
    ld, cm, rt = _gpu_views(trees["terrain10"], 0, sizes)
    rt.RenderViews(mats)
    before = [rt.read_image(view=v).copy() for v in range(2)]
    best = rt.autotune(mats, reps=1)
    assert rt.launch_shape() == best
    assert 2 <= best[0] <= 5 and 1 <= best[1] <= 32 and len(best) == 4
    rt.RenderViews(mats)
    for v in range(2):
        np.testing.assert_array_equal(rt.read_image(view=v), before[v])


def test_batched_argument_errors(trees):
    ld, cm, rt = _gpu_views(trees["terrain10"], 0, [(8, 8), (4, 4)])
    with pytest.raises(R.RaytError):
        rt.RenderFrame(np.eye(4, dtype=np.float32))
    with pytest.raises(R.RaytError):
        rt.set_launch_shape(6, 16, 0)
    with pytest.raises(R.RaytError):
        rt.set_launch_shape(3, 0, 0)
    with pytest.raises(R.RaytError):
        rt.set_launch_shape(3, 16, 0, 0)


def test_graphs_match_plain_launches(trees):
    """Pass graphs (default) and plain launches give the same frames, including
    after a launch-shape change that rebuilds the graphs."""
    sizes = [(96, 64), (33, 17), (128, 72)]
    frames = [[_matrix(c, w, h) for c, (w, h) in zip(_cams(len(sizes), 30.0 * f), sizes)] for f in range(6)]
    runs = []
    for graphs in (True, False):
        ld, cm, rt = _gpu_views(trees["terrain8s"], 150, sizes, seed=23)
        rt.use_graphs(graphs)
        out = []
        for f, mats in enumerate(frames):
            if f == 3:
                rt.set_launch_shape(3, 32, 0, 16)
            rt.RenderViews(mats)
            out.append((rt.stats()["passes"], [rt.read_image(view=v).copy() for v in range(len(sizes))]))
        runs.append(out)
    for f, (a, b) in enumerate(zip(*runs)):
        assert a[0] == b[0], "frame %d" % f
        for v in range(len(sizes)):
            np.testing.assert_array_equal(a[1][v], b[1][v], err_msg="frame %d view %d" % (f, v))


def test_batched_depth_output_vs_oracle(trees):
    """Streamed batched frames with depth output on: every view's depth bits
    and hit nodes equal the oracle's batched frame."""
    from oracle import oracle as O
    frames = [[_matrix(c, w, h) for c, (w, h) in zip(_cams(len(SIZES), 25.0 * f), SIZES)] for f in range(4)]
    libc_srand(23)
    sc = O.OracleScene(trees["terrain8s"], 250, views=SIZES)
    ld, cm, rt = _gpu_views(trees["terrain8s"], 250, SIZES, seed=23)
    rt.set_depth_output(True)
    for f, mats in enumerate(frames):
        n, imgs = sc.render_views(mats)
        ref = sc.depth()
        rt.RenderViews(mats)
        assert rt.stats()["passes"] == n, "frame %d" % f
        for v in range(len(SIZES)):
            d, nodes = rt.read_depth(view=v)
            np.testing.assert_array_equal(nodes, ref[v][1], err_msg="frame %d view %d" % (f, v))
            np.testing.assert_array_equal(d.view(np.uint32), ref[v][0].view(np.uint32),
                                          err_msg="frame %d view %d" % (f, v))
            np.testing.assert_array_equal(rt.read_image(view=v), imgs[v], err_msg="frame %d view %d" % (f, v))
    sc.close()
