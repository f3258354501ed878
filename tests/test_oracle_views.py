"""CPU tests of the oracle's batched form (several views traced together per
frame).  With every block resident a view's image cannot depend on the other
views, so each must equal the one-view frame of its camera; with streaming the
views share one request list per pass, which the GPU tests pin against this
restatement."""
import numpy as np

from tests.conftest import libc_srand
from tests.golden.common import C1_CAMERA

SIZES = [(64, 48), (33, 17), (1, 1), (40, 40)]


def _cams(n):
    return [[30.0 + 40 * v, -20.0 - 5 * v, 0.0, 0.5 - 0.6 * np.sin(np.radians(30 + 40 * v)), 0.7,
             0.5 + 0.6 * np.cos(np.radians(30 + 40 * v)), 60.0] for v in range(n)]


def _matrix(cam, w, h):
    import rayt_gb300 as R
    return R.Camera(cam[0], cam[1], cam[2], cam[3:6], cam[6], w / h).view_proj_inv()


def test_oracle_views_resident_equal_single_views(trees):
    from oracle import oracle as O
    mats = [_matrix(c, w, h) for c, (w, h) in zip(_cams(len(SIZES)), SIZES)]
    sc = O.OracleScene(trees["terrain10"], 0, views=SIZES)
    _, imgs = sc.render_views(mats)
    sc.close()
    for (w, h), m, img in zip(SIZES, mats, imgs):
        one = O.OracleScene(trees["terrain10"], 0, w, h)
        _, ref = one.render(m)
        one.close()
        np.testing.assert_array_equal(img, ref)


def test_oracle_one_view_batch_equals_frame(trees):
    """A batch of one view is the reference's frame, streaming included."""
    from oracle import oracle as O
    w, h = 96, 64
    m = _matrix(C1_CAMERA, w, h)
    libc_srand(5)
    a = O.OracleScene(trees["terrain8s"], 120, views=[(w, h)])
    na, (ia,) = a.render_views([m])
    a.close()
    libc_srand(5)
    b = O.OracleScene(trees["terrain8s"], 120, w, h)
    nb, ib = b.render(m)
    b.close()
    assert na == nb
    np.testing.assert_array_equal(ia, ib)
