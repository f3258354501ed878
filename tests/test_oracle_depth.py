"""CPU tests of the oracle's depth output (the per-pixel distance to what a
pixel shows, and the cache node that shaded it), which the GPU tests compare
the CUDA path with bit for bit.  The reference keeps the hit distance only
inside a pass (rayt/GPU_renderer/kernels/raytracing_pass.cl:43,50-51), so
these pin the definition by its properties: a miss is +inf with node -1, a hit
is finite and positive, the hit-node IDs are exactly the nodes of the feedback
words, and a streamed frame (whose rays restart at their faults and add up
their advances) agrees with a resident frame of the same camera within 1e-5
relative depth."""
import numpy as np

from tests.conftest import libc_srand
from tests.golden.common import C1_CAMERA, NO_HIT

CAMS = [C1_CAMERA, [30.0, -25.0, 0.0, 0.1, 0.6, 1.1, 60.0], [200.0, -35.0, 0.0, 0.9, 0.7, -0.1, 60.0]]


def _matrix(cam, w, h):
    import rayt_gb300 as R
    return R.Camera(cam[0], cam[1], cam[2], cam[3:6], cam[6], w / h).view_proj_inv()


def test_depth_definition_on_a_resident_frame(trees):
    """Resident cache, one pass: the hit node is the word's node, depth the hit t."""
    from oracle import oracle as O
    w, h = 128, 96
    sc = O.OracleScene(trees["terrain10"], 0, w, h, 1.0)
    sc.record(True)
    m = _matrix(C1_CAMERA, w, h)
    passes, img = sc.render(m)
    assert passes == 1
    depth, nodes = sc.depth()
    words = sc.pass_words(0).reshape(h, w)
    sc.close()
    hit = words != NO_HIT
    assert hit.any() and (~hit).any()
    np.testing.assert_array_equal(nodes[hit], (words[hit] >> 1) - 1)
    assert np.all(nodes[~hit] == -1) and np.all(np.isposinf(depth[~hit]))
    assert np.all(np.isfinite(depth[hit])) and np.all(depth[hit] > 0)
    bg = (img[..., 0] == 0) & (img[..., 1] == 216) & (img[..., 2] == 255)
    np.testing.assert_array_equal(bg, ~hit)


def test_streamed_depth_agrees_with_resident(trees):
    """Frames streamed through a small cache (rays stop at faults and resume
    from there) against the same cameras with every block resident: where
    both frames hit, depths agree within 1e-5 relative."""
    from oracle import oracle as O
    w, h = 96, 64
    mats = [_matrix(c, w, h) for c in CAMS]
    full = O.OracleScene(trees["terrain8s"], 0, w, h, 1.0)
    libc_srand(3)
    part = O.OracleScene(trees["terrain8s"], 300, w, h, 1.0)
    streamed_any = False
    for m in mats:
        full.render(m)
        dr, nr = full.depth()
        passes, _ = part.render(m)
        ds, ns = part.depth()
        streamed_any |= passes > 1
        both = (nr >= 0) & (ns >= 0)
        assert both.mean() > 0.3
        np.testing.assert_allclose(ds[both], dr[both], rtol=1e-5)
        assert np.array_equal(np.isposinf(ds), np.isposinf(dr))
    assert streamed_any
    full.close()
    part.close()
