"""CPU tests of host logic and the C ABI (no GPU calls)."""
import ctypes
import os
import re
import struct

import numpy as np
import pytest

import rayt_gb300 as R

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "rayt_gb300.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|void|const char\s*\*|size_t)\s+\**(rayt_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol(built):
    names = declared_symbols()
    assert len(names) >= 40
    L = ctypes.CDLL(R.LIB_PATH)
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_version_and_error_string(built):
    assert b"sm_103a" in R.lib().rayt_version()
    with pytest.raises(R.RaytError) as e:
        R.StoredOctreeLoader("/nonexistent/file.tree")
    assert e.value.code == -2 and "cannot open" in str(e.value)


def _parse_header(path):
    b = open(path, "rb").read()
    nib, blocks, root, stride, nch = struct.unpack("<5I", b[:20])
    pos, ch = 20, []
    for _ in range(nch):
        bn, ln = struct.unpack("<2I", b[pos:pos + 8])
        ch.append((b[pos + 8:pos + 8 + ln].decode(), bn))
        pos += 8 + ln
    return nib, blocks, root, stride, ch, pos, b


def test_loader_matches_file_layout(trees):
    for name in ["sphere7", "terrain8s"]:
        nib, blocks, root, stride, ch, hdr, raw = _parse_header(trees[name])
        ld = R.StoredOctreeLoader(trees[name])
        assert (ld.info.nodes_in_block, ld.info.blocks_count, ld.info.root_block_index) == (nib, blocks, root)
        assert ld.channels == ch and ld.channels[0] == ("node links", 4)
        assert ld.info.header_bytes == hdr and ld.info.block_stride == stride
        for bi in [0, blocks // 2, blocks - 1]:
            h, content = ld.LoadBlock(bi)
            o = hdr + stride * bi
            assert h.block_index == bi
            assert (h.block_index, h.parent_block_index, h.roots_count) == struct.unpack("<3I", raw[o:o + 12])
            assert bytes(content) == raw[o + 76:o + 76 + ld.info.content_bytes]
        with pytest.raises(R.RaytError) as e:
            ld.LoadBlock(blocks)
        assert e.value.code == -1


def test_loader_rejects_corrupt_files(trees, tmp_path):
    raw = open(trees["sphere3"], "rb").read()
    bad = tmp_path / "bad.tree"
    for blob, code in [(raw[:10], -3),                                         # truncated header
                       (struct.pack("<5I", 0, 1, 0, 100, 1) + raw[20:], -3),   # zero nodes_in_block
                       (raw[:20] + struct.pack("<2I", 4, 5) + b"links" + raw[38:], -3)]:  # first channel misnamed
        bad.write_bytes(blob)
        with pytest.raises(R.RaytError) as e:
            R.StoredOctreeLoader(str(bad))
        assert e.value.code == code
    # a block record cut short reads as an I/O error on LoadBlock
    bad.write_bytes(raw[:-100])
    ld = R.StoredOctreeLoader(str(bad))
    with pytest.raises(R.RaytError) as e:
        ld.LoadBlock(ld.info.blocks_count - 1)
    assert e.value.code == -2


def test_builder_rejects_bad_arguments(built, tmp_path):
    with pytest.raises(R.RaytError):
        R.build_terrain(str(tmp_path / "x.tree"), 0)
    with pytest.raises(R.RaytError):
        R.build_terrain(str(tmp_path / "x.tree"), 6, nodes_in_block=4)
    with pytest.raises(R.RaytError):
        R.build_terrain("/nonexistent/dir/x.tree", 6)


def test_terrain_with_spheres_is_deterministic(built, tmp_path):
    a, b = tmp_path / "a.tree", tmp_path / "b.tree"
    na = R.build_terrain(str(a), 7, 1024, spheres=20, min_radius=2, max_radius=16)
    nb = R.build_terrain(str(b), 7, 1024, spheres=20, min_radius=2, max_radius=16)
    assert na == nb and a.read_bytes() == b.read_bytes()
    assert R.build_terrain(str(b), 7, 1024)[1] < na[1]  # spheres add nodes


def test_camera_helper_matches_reference(golden):
    """The camera helper builds the reference's float matrix and inverts it with
    the reference's float cofactor method: the 16 floats of every golden frame
    camera are the reference's own, bit for bit."""
    from tests.golden.common import FRAME_CASES
    for name, case in FRAME_CASES.items():
        w, h = case["size"]
        for cam, g in zip(case["cameras"], golden["frames"][name]):
            c = R.Camera(cam[0], cam[1], cam[2], cam[3:6], cam[6], w / h)
            m = np.asarray(c.view_proj_inv(), np.float32)
            ref = np.array(g["matrix"], np.float32)
            np.testing.assert_array_equal(m.view(np.uint32), ref.view(np.uint32))


def test_camera_helper_sweep_matches_reference():
    """512 seeded cameras (any yaw/roll, pitch -90..90, FOV 20..120, aspect
    from 1..4095-pixel sides) against Camera::ViewProjectionMatrix().Inverse()
    run by the reference harness: bit for bit."""
    from tests.golden.common import CAMERA_SWEEP, camera_sweep
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "cameras.npz"))
    cams = camera_sweep(CAMERA_SWEEP["count"], CAMERA_SWEEP["seed"])
    np.testing.assert_array_equal(cams, d["cameras"])
    got = np.zeros_like(d["matrices"])
    for i, c in enumerate(cams):
        got[i] = R.Camera(c[0], c[1], c[2], c[3:6], c[6], c[7]).view_proj_inv()
    np.testing.assert_array_equal(got.view(np.uint32), d["matrices"].view(np.uint32))


def test_shading_light_constants_are_the_references():
    """The traversal kernel shades with the three light directions of
    shading.cl:7-32 as float constants; recomputed here as the reference
    computes them per call in IEEE float: normalize(v) = v / sqrt(dot(v, v))
    (dot left to right, correctly rounded sqrt and division), times w."""
    src = open(os.path.join(ROOT, "rayt_gb300", "csrc", "trace.cu")).read()
    m = re.search(r"const float l\[3\]\[3\] = \{(.*?)\};", src, re.S)
    got = [float.fromhex(t.rstrip("f")) for t in re.findall(r"-?0x[0-9a-f.]+p-?\d+f", m.group(1))]
    f = np.float32
    want = []
    for (x, y, z), w in [((2, -2, 3), .6), ((-3, -3, -2), .5), ((1, 2.5, -1), .3)]:
        x, y, z, w = f(x), f(y), f(z), f(w)
        d = f(f(f(f(x * x) + f(y * y)) + f(z * z)) + f(f(0) * f(0)))
        ln = np.sqrt(d, dtype=np.float32)
        want += [float(f(f(c / ln) * w)) for c in (x, y, z)]
    assert got == want


def test_normal_component_division_identity():
    """x / 127 for every char normal component x: the kernel's product with the
    rounded reciprocal plus one fused residual correction equals the IEEE
    quotient (libm's fmaf stands in for the GPU's fused multiply-add)."""
    libm = ctypes.CDLL("libm.so.6")
    fmaf = libm.fmaf
    fmaf.restype = ctypes.c_float
    fmaf.argtypes = [ctypes.c_float] * 3
    f = np.float32
    r = f(1) / f(127)
    for x in range(-128, 128):
        q0 = f(x) * r
        e = f(fmaf(float(-q0), 127.0, float(x)))
        q1 = f(fmaf(float(e), float(r), float(q0)))
        assert q1.view(np.uint32) == (f(x) / f(127)).view(np.uint32), x
