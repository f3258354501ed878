"""Host delivery of the frame (rayt_renderer_set_host_image): the image lands
in the caller's page-locked buffer by the time RenderFrame returns.  The first
pass's pixels come by one copy that overlaps the host's feedback decode and
block streaming; later passes and the finish write their pixels there too.
Checked bit for bit against the device image and against a renderer without
delivery on the same frames, for streamed frames of several passes (later
passes write host pixels after the copy) and frames that stop with faulted
rays (the finish writes them)."""
import numpy as np
import pytest

import rayt_gb300 as R
from tests.golden.common import FRAME_CASES

pytestmark = pytest.mark.gpu


def _pinned(nbytes):
    torch = pytest.importorskip("torch")
    return torch.empty(nbytes, dtype=torch.uint8).pin_memory()


def _pair(path, max_blocks, w, h, lod, seed, max_passes=0, extras=False):
    out = []
    for _ in range(2):
        ld = R.StoredOctreeLoader(path)
        cm = R.GPUOctreeCacheManager(max_blocks, ld)
        cm.InitialFillCache()
        rt = R.GPURayTracer(cm, w, h)
        rt.set_lod_voxel_size(lod)
        rt.set_frame_time_limit(1e30)
        rt.seed(seed)
        if max_passes:
            rt.set_max_passes(max_passes)
        if extras:  # depth output, and plain launches (recorded passes) instead of pass graphs
            rt.set_depth_output(True)
            rt.record_passes(True)
        out.append((ld, cm, rt))
    return out


def _matrix(cam, w, h):
    return R.Camera(cam[0], cam[1], cam[2], cam[3:6], cam[6], w / h).view_proj_inv()


@pytest.mark.parametrize("name,max_passes,extras", [("stream8", 0, False), ("stream8_lod0", 0, False),
                                                    ("c1_stream", 0, False), ("stream8", 2, False),
                                                    ("stream8", 0, True)])
def test_host_image_equals_device_image(trees, name, max_passes, extras):
    case = FRAME_CASES[name]
    w, h = case["size"]
    (_, _, plain), (_, _, deliv) = _pair(trees[case["tree"]], case["max_blocks"], w, h, case["lod"], case["seed"],
                                         max_passes, extras)
    buf = _pinned(w * h * 4)
    deliv.set_host_image(buf.data_ptr(), buf.numel())
    multi, stopped = 0, 0
    for cam in case["cameras"] * 2:
        m = _matrix(cam, w, h)
        plain.RenderFrame(m)
        buf.fill_(7)  # stale bytes: every pixel must be delivered again
        deliv.RenderFrame(m)
        host = buf.numpy().reshape(h, w, 4).copy()
        assert np.array_equal(host, deliv.read_image())
        assert np.array_equal(host, plain.read_image())
        if extras:
            dd, dn = deliv.read_depth()
            pd, pn = plain.read_depth()
            assert np.array_equal(np.asarray(dd).view(np.uint32), np.asarray(pd).view(np.uint32))
            assert np.array_equal(dn, pn)
        st = deliv.stats()
        multi += st["passes"] > 1
        stopped += st["passes"] == max_passes
    assert multi > 0  # later passes wrote host pixels after the first pass's copy
    if max_passes:
        assert stopped > 0  # frames cut at the pass cap: the finish wrote host pixels
    deliv.set_host_image(None)
    m = _matrix(case["cameras"][0], w, h)
    buf.fill_(7)
    deliv.RenderFrame(m)
    assert (buf.numpy() == 7).all()  # delivery switched off


def test_host_image_refuses_pageable_memory_and_views(trees):
    case = FRAME_CASES["stream8"]
    w, h = case["size"]
    ld = R.StoredOctreeLoader(trees[case["tree"]])
    cm = R.GPUOctreeCacheManager(case["max_blocks"], ld)
    cm.InitialFillCache()
    rt = R.GPURayTracer(cm, w, h)
    pageable = np.zeros(w * h * 4, np.uint8)
    with pytest.raises(R.RaytError):
        rt.set_host_image(pageable.ctypes.data, pageable.nbytes)
    buf = _pinned(w * h * 4 + 4)
    with pytest.raises(R.RaytError):
        rt.set_host_image(buf.data_ptr(), w * h * 4 - 1)
    with pytest.raises(R.RaytError):  # pixels are written as 4-byte words
        rt.set_host_image(buf.data_ptr() + 1, w * h * 4)
    views = R.GPURayTracer.views(cm, [(w, h), (32, 32)])
    with pytest.raises(R.RaytError):
        views.set_host_image(buf.data_ptr(), buf.numel())
