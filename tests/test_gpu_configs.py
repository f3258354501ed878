"""GPU parity at the benchmarked configurations, on the benchmark scene itself:
the depth-12 fBm heightfield with 2000 sphere shells (4096^3 voxels, 4096-node
blocks, about 6.8 GB), built by the product's parallel builder into the
benchmark's scene directory (so the benchmark run after the tests reuses it).

- the scene's bytes equal the reference builder's (canonical hash committed by
  tests/golden/make_golden.py, part builder_large);
- the 1920x1080 flythrough streamed through a 2 GiB cache (the c3 workload):
  its first frames, pass by pass, against the oracle (feedback words, images,
  depth bits, hit nodes, cache buffers);
- one frame of the 64-view batched workload (c4: view sizes drawn from
  {256^2, 640x480, 1280x720, 1920x1080}, whole tree resident) against the
  oracle's batched frame;
- one served tick mix of the three served client sizes (1280x720, 1920x1080,
  2560x1440) in one server against the oracle's one-view frames.
Everything compared is integer or float bits: tolerance 0."""
import numpy as np
import pytest

import bench
import rayt_gb300 as R
from tests.conftest import libc_srand

pytestmark = pytest.mark.gpu

SHORT_RUN_FRAMES = 25  # frames of a short run: 5 warm-up + 20 timed


@pytest.fixture(scope="module")
def c3_scene(built):
    return bench.scene_path("c3", 0, 1)


@pytest.fixture(scope="module")
def resident_oracle(c3_scene):
    """The oracle over the whole depth-12 tree (about 6.8 GB of host memory)."""
    from oracle import oracle as O
    sizes, _ = bench.batched_views(bench.WORKLOADS["c4"])
    sc = O.OracleScene(c3_scene, 0, views=sizes, lod=1.0)
    yield sc
    sc.close()


def test_scene_bytes_match_reference_builder(c3_scene, golden):
    from tests.golden.common import canonical_tree_sha
    digest, size = canonical_tree_sha(c3_scene)
    g = golden["builder_large"]["terrain12s"]
    assert size == g["bytes"]
    assert digest == g["sha256"]


def test_c3_streamed_frames_vs_oracle(c3_scene):
    cfg = bench.WORKLOADS["c3"]
    # the whole spline in 25 frames: each frame moves 12x as far as in the
    # 300-frame flythrough, so every frame streams hundreds of blocks
    mats = bench.camera_path("c3", SHORT_RUN_FRAMES, cfg["width"], cfg["height"], period=SHORT_RUN_FRAMES)[:4]
    out = bench.frames_parity(c3_scene, cfg, mats, seed=1)
    assert out["frames"] == 4 and out["uploaded_blocks"] > 0
    assert out["passes"] > out["frames"]  # frames streamed blocks and traced again
    assert out["ok"], out


def test_c4_batched_frame_vs_oracle(c3_scene, resident_oracle):
    cfg = bench.WORKLOADS["c4"]
    sizes, seeds = bench.batched_views(cfg)
    f = 5  # the first timed frame of the benchmark's default run
    mats = [bench.camera_path("c4", SHORT_RUN_FRAMES, w, h, seed=sd)[f] for (w, h), sd in zip(sizes, seeds)]
    ld = R.StoredOctreeLoader(c3_scene)
    cm = R.GPUOctreeCacheManager(0, ld)
    cm.InitialFillCache()
    rt = R.GPURayTracer.views(cm, sizes)
    rt.set_lod_voxel_size(cfg["lod"])
    rt.set_frame_time_limit(1e30)
    rt.seed(1)
    rt.set_depth_output(True)
    libc_srand(1)
    n, imgs = resident_oracle.render_views(mats)
    ref_depth = resident_oracle.depth()
    rt.RenderViews(mats)
    assert rt.stats()["passes"] == n == 1  # resident: one pass
    for v in range(len(sizes)):
        np.testing.assert_array_equal(rt.read_image(view=v), imgs[v], err_msg="view %d" % v)
        d, nodes = rt.read_depth(view=v)
        np.testing.assert_array_equal(nodes, ref_depth[v][1], err_msg="view %d" % v)
        np.testing.assert_array_equal(d.view(np.uint32), ref_depth[v][0].view(np.uint32), err_msg="view %d" % v)


def test_c5_client_size_mix_vs_oracle(c3_scene, resident_oracle):
    """Three clients of the served sizes in one server over a 2 GiB cache of
    the depth-12 tree (so their frames fault and share ticks): each request's
    image equals the oracle's resident one-view frame of its camera."""
    sizes = [(1280, 720), (1920, 1080), (2560, 1440)]
    cams = [bench.camera_path("c3", SHORT_RUN_FRAMES, w, h, seed=100 + c) for c, (w, h) in enumerate(sizes)]
    ld = R.StoredOctreeLoader(c3_scene)
    cm = R.GPUOctreeCacheManager(bench.cache_blocks(bench.WORKLOADS["c3"]), ld)
    cm.InitialFillCache()
    px = sum(w * h for w, h in sizes)
    srv = R.RenderServer(cm, max_clients=4, framebuffer_bytes=px * 4 + (1 << 20), max_rays_in_flight=px,
                         max_passes=32, lod_voxel_size=1.0)
    ids = [srv.add_client(w, h) for w, h in sizes]
    for f in (0, 5):
        reqs = [srv.submit(ids[c], cams[c][f]) for c in range(len(sizes))]
        for c, r in enumerate(reqs):
            info = srv.wait(r, timeout=120)
            assert not info["truncated"], (c, f)
            w, h = sizes[c]
            _, ref = resident_oracle.render_size(w, h, cams[c][f])
            np.testing.assert_array_equal(srv.read_image(ids[c]), ref, err_msg="client %d frame %d" % (c, f))
    st = srv.stats()
    srv.close()
    assert st["faults"] > 0 and st["completed"] == 2 * len(sizes)
