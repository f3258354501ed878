"""CPU tests: the product's block-file builder and the CPU oracle against the
golden fixtures produced by the reference's own code (tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

from tests.conftest import libc_srand
from tests.golden.common import (BUILDER_CASES, FRAME_CASES, SPHERE_CACHE_CASES, canonical_tree_bytes, sha)

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("name", sorted(BUILDER_CASES))
def test_builder_golden(trees, golden, name):
    """Block files are byte-identical to the reference builder's (unused root
    records masked, see canonical_tree_bytes)."""
    data = canonical_tree_bytes(trees[name])
    g = golden["builder"][name]
    assert len(data) == g["bytes"]
    assert sha(np.frombuffer(data, np.uint8)) == g["sha256"]


@pytest.mark.parametrize("name", sorted(SPHERE_CACHE_CASES))
def test_oracle_sphere_cache(trees, golden, name):
    from oracle import oracle as O
    case = SPHERE_CACHE_CASES[name]
    sc = O.OracleScene(trees[case["tree"]], case["max_blocks"])
    g = golden["sphere_cache"][name]
    assert sc.root() == g["root"]
    n = sc.max_blocks * sc.nib
    for ch, (cname, b) in enumerate([("node links", 4), ("node index", 4), ("node index % 211", 1)]):
        assert sha(sc.read(ch, n * b)) == g["hashes"][cname], cname
    assert sha(sc.read(-1, sc.max_blocks * 32)) == g["hashes"]["far pointers"]
    sc.close()


@pytest.mark.parametrize("name", sorted(FRAME_CASES))
def test_oracle_frames(trees, golden, name):
    """Images, every pass's feedback words and the cache buffers after every
    frame match the reference pipeline, including streaming and eviction."""
    from oracle import oracle as O
    case = FRAME_CASES[name]
    w, h = case["size"]
    sc = O.OracleScene(trees[case["tree"]], case["max_blocks"], w, h, case["lod"])
    sc.record(True)
    libc_srand(case["seed"])
    imgs = np.load(os.path.join(GOLDEN, "frame_images.npz")) if case.get("keep_images") else None
    for i, g in enumerate(golden["frames"][name]):
        n, img = sc.render(np.array(g["matrix"], np.float32))
        assert n == g["passes"]
        for p in range(n):
            assert sha(sc.pass_words(p)) == g["pass_words_sha256"][p], "pass %d" % p
        if imgs is not None:
            np.testing.assert_array_equal(img, imgs["%s_%d" % (name, i)])
        assert sha(img) == g["image_sha256"]
        assert sc.root() == g["root"]
        nodes = sc.max_blocks * sc.nib
        for ch, cname in enumerate(["node links", "normals", "colors"]):
            assert sha(sc.read(ch, nodes * 4)) == g["cache"][cname], cname
        assert sha(sc.read(-1, sc.max_blocks * 32)) == g["cache"]["far pointers"]
    sc.close()


def test_oracle_sort_scan_golden(built):
    """The reference's GPUSort/GPUScan known-answer runs (n = 2013, values
    rand() % 201 - 100; test-application.cpp:150-240)."""
    from oracle import oracle as O
    d = np.load(os.path.join(GOLDEN, "sort_scan.npz"))
    for a, s, c in zip(d["inputs"], d["sorted"], d["scanned"]):
        np.testing.assert_array_equal(O.sort(a), s)
        np.testing.assert_array_equal(O.scan(a), c)
        np.testing.assert_array_equal(s, np.sort(a))
        np.testing.assert_array_equal(c, np.cumsum(a).astype(np.int32))


def test_oracle_feedback_unique_golden(built):
    from oracle import oracle as O
    d = np.load(os.path.join(GOLDEN, "feedback_unique.npz"))
    for key in ["small", "c2_like", "all_nohit", "no_nohit"]:
        out = O.feedback_unique(d[key + "_words"], int(d[key + "_nib"][0]))
        np.testing.assert_array_equal(out, d[key + "_unique"], err_msg=key)


@pytest.mark.parametrize("seed", range(6))
def test_oracle_feedback_unique_properties(built, seed):
    """The oracle's restatement of GetUnique (merge sort, flag, Hillis-Steele
    scan, compress) on random words of every kind (NO_HIT, faults, hits with
    and without the duplicate bit, the int32 extremes) equals NodeToBlock then
    numpy's sorted unique; n includes sizes around the reference's work-group
    size and powers of two."""
    from oracle import oracle as O
    rng = np.random.default_rng(seed)
    for n in [1, 2, 255, 256, 257, 1023, 4096, 5000]:
        nib = int(rng.choice([0, 1, 7, 512, 4096]))
        kind = rng.integers(0, 4, n)
        words = np.where(kind == 0, 0x7FFFFFFF,
                         np.where(kind == 1, -rng.integers(1, 1 << 20, n),
                                  (rng.integers(1, 1 << 24, n) << 1) | rng.integers(0, 2, n))).astype(np.int64)
        if n > 3:
            words[:3] = [-2**31, 2**30 - 1, 0x7FFFFFFF]
        words = words.astype(np.int32)
        conv = words.astype(np.int64)
        hit = (conv > 0) & (conv != 0x7FFFFFFF)
        if nib > 0:
            conv[hit] = ((((conv[hit] >> 1) - 1) // nib + 1) << 1) | (conv[hit] & 1)
        np.testing.assert_array_equal(O.feedback_unique(words, nib), np.unique(conv).astype(np.int32),
                                      err_msg="n=%d nib=%d" % (n, nib))


def test_golden_inputs_regenerate(built):
    """The committed feedback inputs are what common.feedback_words produces."""
    from tests.golden.common import feedback_words
    d = np.load(os.path.join(GOLDEN, "feedback_unique.npz"))
    np.testing.assert_array_equal(d["small_words"], feedback_words(5000, 5))
    np.testing.assert_array_equal(d["no_nohit_words"], feedback_words(3000, 8, no_hit=False))


@pytest.mark.parametrize("name", sorted(__import__("tests.golden.common", fromlist=["DEPTH_CASES"]).DEPTH_CASES))
def test_oracle_depth_view(trees, name):
    """The oracle's restatement of raytracer.cl (the reference's debug depth
    view) against the reference kernel run by the harness: red (fault or
    error) and black (miss) pixels exact, grey within 1 LSB (log is the C
    library's)."""
    from oracle import oracle as O
    from tests.golden.common import DEPTH_CASES
    case = DEPTH_CASES[name]
    d = np.load(os.path.join(GOLDEN, "depth_views.npz"))
    w, h = case["size"]
    sc = O.OracleScene(trees[case["tree"]], case["max_blocks"])
    img = sc.depth_view(d[name + "_matrix"], case["lod"], w, h)
    sc.close()
    ref = d[name + "_image"]
    assert np.array_equal(img[..., 3], ref[..., 3])
    red = (ref[..., 0] == 255) & (ref[..., 1] == 0)
    assert np.array_equal(red, (img[..., 0] == 255) & (img[..., 1] == 0))
    assert np.abs(img.astype(int) - ref.astype(int)).max() <= 1
