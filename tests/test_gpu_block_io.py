"""The two ways streamed blocks reach the device cache give the same cache:
the block file mapped into host memory and read by the upload kernel where it
lies (the default), and pread into pinned staging plus one copy per batch
(RAYT_BLOCK_IO=read).  A block record can start at any byte offset of the
file, so the mapped upload is checked at every alignment, and with a channel
section of odd size."""
import os
import struct

import numpy as np
import pytest

import rayt_gb300 as R

pytestmark = pytest.mark.gpu

ROOT_PARENT = (1 << 24) - 1


def _cache(path, max_blocks, mode):
    old = os.environ.get("RAYT_BLOCK_IO")
    if mode == "read":
        os.environ["RAYT_BLOCK_IO"] = "read"
    else:
        os.environ.pop("RAYT_BLOCK_IO", None)
    try:
        ld = R.StoredOctreeLoader(path)
        cm = R.GPUOctreeCacheManager(max_blocks, ld)
    finally:
        if old is None:
            os.environ.pop("RAYT_BLOCK_IO", None)
        else:
            os.environ["RAYT_BLOCK_IO"] = old
    return ld, cm


def test_default_cache_reads_blocks_from_the_mapped_file(trees):
    ld, cm = _cache(trees["terrain8s"], 250, "mapped")
    assert cm.stats()["mapped"] == 1
    ld2, cm2 = _cache(trees["terrain8s"], 250, "read")
    assert cm2.stats()["mapped"] == 0


def test_streamed_frames_identical_in_both_modes(trees):
    """A streamed flythrough (cache of 250 of 790 blocks, evictions every
    frame): images and every cache buffer equal after each frame."""
    w, h = 320, 180
    mats = []
    for a in range(0, 360, 45):
        c = R.Camera(a, -25.0 - 0.2 * a, 0.0, (0.5 - 0.6 * np.sin(np.radians(a)), 0.7,
                                                0.5 + 0.6 * np.cos(np.radians(a))), 60.0, w / h)
        mats.append(c.view_proj_inv())
    runs = []
    for mode in ("mapped", "read"):
        ld, cm = _cache(trees["terrain8s"], 250, mode)
        cm.InitialFillCache()
        rt = R.GPURayTracer(cm, w, h)
        rt.set_frame_time_limit(1e30)
        rt.seed(99)
        frames = []
        for m in mats:
            rt.RenderFrame(m)
            frames.append((rt.stats()["passes"], rt.read_image().copy(),
                           [cm.read_buffer(n).copy() for n in ("node links", "normals", "colors", "far pointers")]))
        st = cm.stats()
        assert st["mapped"] == (1 if mode == "mapped" else 0)
        assert st["uploaded_blocks"] > 250  # blocks were streamed and evicted
        runs.append(frames)
        rt.close()
        cm.close()
    for i, (a, b) in enumerate(zip(*runs)):
        assert a[0] == b[0], "frame %d passes" % i
        np.testing.assert_array_equal(a[1], b[1], err_msg="frame %d image" % i)
        for k in range(4):
            np.testing.assert_array_equal(a[2][k], b[2][k], err_msg="frame %d buffer %d" % (i, k))


def test_tree_closed_before_its_cache(trees):
    """Closing the tree while a cache still streams from its mapped file is
    allowed: the cache keeps the tree open until it is destroyed.  Frames
    streamed after the close equal frames with the tree left open."""
    w, h = 160, 90
    mats = [R.Camera(a, -30.0, 0.0, (0.5 - 0.6 * np.sin(np.radians(a)), 0.7, 0.5 + 0.6 * np.cos(np.radians(a))),
                     60.0, w / h).view_proj_inv() for a in range(0, 360, 60)]
    images = []
    for close_early in (False, True):
        ld, cm = _cache(trees["terrain8s"], 250, "mapped")
        cm.InitialFillCache()
        if close_early:
            ld.close()
        rt = R.GPURayTracer(cm, w, h)
        rt.set_frame_time_limit(1e30)
        rt.seed(3)
        run = []
        for m in mats:
            rt.RenderFrame(m)
            run.append(rt.read_image().copy())
        assert cm.stats()["uploaded_blocks"] > 250
        images.append(run)
        rt.close()
        cm.close()
    for i, (a, b) in enumerate(zip(*images)):
        np.testing.assert_array_equal(a, b, err_msg="frame %d" % i)


def test_cache_released_before_its_renderer_and_server(trees):
    """Releasing the cache handle while a renderer or a server still uses it
    is allowed: each keeps the cache (its stream and buffers) until it is
    destroyed.  Frames after the release equal frames with it kept."""
    w, h = 160, 90
    mats = [R.Camera(a, -30.0, 0.0, (0.5 - 0.6 * np.sin(np.radians(a)), 0.7, 0.5 + 0.6 * np.cos(np.radians(a))),
                     60.0, w / h).view_proj_inv() for a in range(0, 360, 90)]
    images = []
    for release_early in (False, True):
        ld, cm = _cache(trees["terrain8s"], 250, "mapped")
        cm.InitialFillCache()
        rt = R.GPURayTracer(cm, w, h)
        rt.set_frame_time_limit(1e30)
        rt.seed(3)
        srv = R.RenderServer(cm, max_clients=2, framebuffer_bytes=w * h * 8, max_rays_in_flight=w * h * 2,
                             deliver_to_host=True)
        client = srv.add_client(w, h)
        if release_early:
            cm.close()
            ld.close()
        run = []
        for m in mats:
            rt.RenderFrame(m)
            run.append(rt.read_image().copy())
            srv.wait(srv.submit(client, m), timeout=60)
            run.append(srv.host_image(client).copy())
        images.append(run)
        srv.close()
        rt.close()
        cm.close()
    for i, (a, b) in enumerate(zip(*images)):
        np.testing.assert_array_equal(a, b, err_msg="image %d" % i)


def _write_tree(path, nib, extra_name, extra_bytes, rng):
    """A one-block tree: 'node links' (in-block child links and empty nodes)
    and one more channel; the channel name's length moves the block record's
    offset in the file, so its content starts at any alignment.  Returns the
    stored links and the other channel's bytes."""
    links = np.zeros(nib, np.uint32)
    for n in range(0, nib - 8, 3):  # a node with children n+1.. inside the block
        mask = int(rng.integers(1, 256))
        links[n] = (mask | ((n + 1) << 11)) & 0xFFFFFFFF
        links[n] |= int(rng.integers(0, 2)) << 9  # duplicate flag kept
    extra = rng.integers(0, 256, nib * extra_bytes).astype(np.uint8)
    name = extra_name.encode()
    chans = struct.pack("<2I", 4, len(b"node links")) + b"node links" + struct.pack("<2I", extra_bytes, len(name)) + name
    content = links.tobytes() + extra.tobytes()
    stride = 76 + len(content)
    header = struct.pack("<5I", nib, 1, 0, stride, 2)
    block = struct.pack("<3I", 0, ROOT_PARENT, 1) + struct.pack("<HHI", 0, 0, 0) + b"\0" * (8 * 7)
    assert len(block) == 76
    with open(path, "wb") as f:
        f.write(header + chans + block + content)
    return links, extra, len(header) + len(chans) + 76


def _expected_links(links):
    out = links.copy()
    for n, l in enumerate(links):
        l = int(l)
        mask, fault = l & 255, (l >> 8) & 1
        if mask and not fault:
            near = (1 << 20) + (l >> 11) - n
            out[n] = ((near << 11) | (l & (1 << 9)) | mask) & 0xFFFFFFFF
    return out


@pytest.mark.parametrize("mode", ["mapped", "read"])
@pytest.mark.parametrize("name_len", [1, 2, 3, 4])
@pytest.mark.parametrize("extra_bytes, nib", [(4, 64), (1, 37), (3, 64)])
def test_block_upload_at_any_alignment(tmp_path, built, mode, name_len, extra_bytes, nib):
    rng = np.random.default_rng(name_len * 100 + extra_bytes * 10 + nib)
    path = os.path.join(str(tmp_path), "t.tree")
    links, extra, content_at = _write_tree(path, nib, "x" * name_len, extra_bytes, rng)
    ld, cm = _cache(path, 1, mode)
    assert cm.stats()["mapped"] == (1 if mode == "mapped" else 0)
    cm.InitialFillCache()
    got = cm.read_buffer("node links", np.uint32)[:nib]
    np.testing.assert_array_equal(got, _expected_links(links), err_msg="content at byte %d" % content_at)
    np.testing.assert_array_equal(cm.read_buffer("x" * name_len)[:nib * extra_bytes], extra)
