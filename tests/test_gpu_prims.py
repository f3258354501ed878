"""GPU parity of the feedback primitives (sort, scan, unique) against the
reference's known-answer runs, the oracle and numpy."""
import os

import numpy as np
import pytest

import rayt_gb300 as R
from tests.golden.common import NO_HIT, feedback_words

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, np.int32)).cuda()


def host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


def test_sort_scan_known_answers(built):
    d = np.load(os.path.join(GOLDEN, "sort_scan.npz"))
    for a, s, c in zip(d["inputs"], d["sorted"], d["scanned"]):
        x = dev(a)
        R.GPUSort(x, a.size)
        np.testing.assert_array_equal(host(x), s)
        y = dev(a)
        R.GPUScan(y, a.size)
        np.testing.assert_array_equal(host(y), c)


@pytest.mark.parametrize("n", [1, 2, 31, 4095, 4096, 4097, 65537, (1 << 20) + 3, 1 << 24])
def test_sort_sizes(built, n):
    rng = np.random.default_rng(n)
    a = rng.integers(-2**31, 2**31 - 1, size=n, dtype=np.int64).astype(np.int32)
    a[: n // 3] = a[0]  # long run of equal keys
    x = dev(a)
    R.GPUSort(x, n)
    np.testing.assert_array_equal(host(x), np.sort(a))


def test_sort_extremes(built):
    a = np.array([2**31 - 1, -2**31, 0, -1, 1, -2**31, 2**31 - 1] * 1000, np.int32)
    x = dev(a)
    R.GPUSort(x, a.size)
    np.testing.assert_array_equal(host(x), np.sort(a))


@pytest.mark.parametrize("n", [1, 4096, 4097, 1000003])
def test_scan_sizes_wrap(built, n):
    rng = np.random.default_rng(n)
    a = rng.integers(-2**31, 2**31 - 1, size=n, dtype=np.int64).astype(np.int32)
    y = dev(a)
    R.GPUScan(y, n)
    with np.errstate(over="ignore"):
        ref = np.cumsum(a.astype(np.int64)).astype(np.uint64).astype(np.uint32).view(np.int32)
    np.testing.assert_array_equal(host(y), ref)


def _unique(words, nib):
    import torch
    w = dev(words)
    out = torch.zeros(max(1, words.size), dtype=torch.int32, device="cuda")
    cnt = R.feedback_unique(w, words.size, nib, out)
    res = host(out)[:cnt]
    np.testing.assert_array_equal(host(w), words)  # input untouched
    return res


def test_feedback_unique_golden(built):
    d = np.load(os.path.join(GOLDEN, "feedback_unique.npz"))
    for key in ["small", "c2_like", "all_nohit", "no_nohit"]:
        np.testing.assert_array_equal(_unique(d[key + "_words"], int(d[key + "_nib"][0])), d[key + "_unique"],
                                      err_msg=key)


@pytest.mark.parametrize("n,nib", [(1, 1), (100, 0), (4096 * 3 + 5, 4096), (1 << 20, 512)])
def test_feedback_unique_vs_oracle(built, n, nib):
    from oracle import oracle as O
    words = feedback_words(n, n + nib)
    np.testing.assert_array_equal(_unique(words, nib), O.feedback_unique(words, nib))


@pytest.mark.parametrize("n", [1 << 24, (1 << 26) + 12345])
def test_feedback_unique_large_properties(built, n):
    """At sizes the oracle's merge sort is too slow for: strictly increasing
    output, NO_HIT last exactly when present, and the same value set as numpy."""
    words = feedback_words(n, 77)
    u = _unique(words, 4096)
    conv = words.astype(np.int64)
    hit = (conv > 0) & (conv != NO_HIT)
    conv[hit] = ((((conv[hit] >> 1) - 1) // 4096 + 1) << 1) | (conv[hit] & 1)
    np.testing.assert_array_equal(u, np.unique(conv).astype(np.int32))
    assert np.all(np.diff(u.astype(np.int64)) > 0) and u[-1] == NO_HIT


def _np_unique(words, nib):
    conv = words.astype(np.int64)
    hit = (conv > 0) & (conv != NO_HIT)
    if nib > 0:
        conv[hit] = ((((conv[hit] >> 1) - 1) // nib + 1) << 1) | (conv[hit] & 1)
    return np.unique(conv).astype(np.int32)


def _bitmap_path(words, nib):
    """True when feedback unique takes the bitmap path: the kept keys span at
    most 2^26 values and at most the bitmap's capacity, 8 bits per byte of one
    (n + 4)-word key buffer in whole 16-byte units."""
    u = _np_unique(words, nib).astype(np.int64)
    u = u[u != NO_HIT]
    cap = ((words.size * 4 + 16) // 16) * 16 * 8
    return u.size > 0 and int(u.max() - u.min() + 1) <= min(cap, 1 << 26)


@pytest.mark.parametrize("case", ["narrow", "narrow_no_nohit", "one_key", "top_end", "bottom_end", "wide_small_n",
                                  "cap_exact", "cap_plus_one", "zipf_heavy", "span_2_26", "span_over_2_26",
                                  "wide_large_n"])
def test_feedback_unique_bitmap_and_radix_paths(built, case):
    """Feedback unique takes the bitmap path when the kept keys span at most 32
    values per input word and the radix passes otherwise; both give the sorted
    unique set."""
    rng = np.random.default_rng(sum(map(ord, case)))
    n, nib = 200_000, 0
    if case == "narrow":
        words = rng.integers(-5000, 5000, n).astype(np.int32)
        words[rng.random(n) < 0.7] = NO_HIT
        path = True
    elif case == "narrow_no_nohit":
        words, nib, path = feedback_words(n, 3, no_hit=False, id_bits=12), 64, True
    elif case == "one_key":
        words = np.full(n, -77, np.int32)
        words[::3] = NO_HIT
        path = True
    elif case == "top_end":
        words = (2**31 - 2 - rng.integers(0, 3000, n)).astype(np.int32)
        path = True
    elif case == "bottom_end":
        words = (-2**31 + rng.integers(0, 3000, n)).astype(np.int32)
        path = True
    elif case == "wide_small_n":
        n = 5000
        words = rng.integers(-2**31, 2**31 - 1, n, dtype=np.int64).astype(np.int32)
        path = False
    elif case in ("cap_exact", "cap_plus_one"):
        n = 1000
        cap = ((n * 4 + 16) // 16) * 16 * 8
        words = np.full(n, NO_HIT, np.int32)
        words[10] = -100000
        words[500] = -100000 + cap - 1 + (case == "cap_plus_one")
        words[700] = -100000 + 5
        path = case == "cap_exact"
    elif case == "wide_large_n":  # the radix passes at scale: keys over the whole int32 range
        n = (1 << 22) + 5
        words = rng.integers(-2**31, 2**31 - 1, n, dtype=np.int64).astype(np.int32)
        words[rng.random(n) < 0.5] = NO_HIT
        words[:1000] = words[1000:2000]  # some repeats
        path = False
    elif case in ("span_2_26", "span_over_2_26"):  # the widest bitmap (2^18-bit range slices), and one past it
        n = (1 << 21) + 77
        words = rng.integers(-(1 << 25), (1 << 25) - 1, n).astype(np.int32)
        words[0], words[1] = -(1 << 25), (1 << 25) - 1 + (case == "span_over_2_26")
        path = case == "span_2_26"
    else:  # zipf_heavy: a few keys repeated very often, as feedback is
        n = 1 << 22
        ids = np.minimum(rng.zipf(1.3, n), 1 << 20)
        words = np.where(rng.random(n) < 0.5, -ids, (ids << 1) | 1).astype(np.int32)
        nib, path = 1, True
    assert _bitmap_path(words, nib) == path
    np.testing.assert_array_equal(_unique(words, nib), _np_unique(words, nib))


@pytest.mark.parametrize("offset", [1, 2, 3])
def test_unaligned_inputs(built, offset):
    """Input arrays that start off a 16-byte boundary take the scalar-load
    compaction; results equal the aligned ones."""
    import torch
    n = 3 * 4096 + 777
    words = feedback_words(n, 5)
    pad = dev(np.concatenate([np.zeros(offset, np.int32), words]))
    out = torch.zeros(n, dtype=torch.int32, device="cuda")
    cnt = R.feedback_unique(pad[offset:], n, 4096, out)
    np.testing.assert_array_equal(host(out)[:cnt], _unique(words, 4096))
    rng = np.random.default_rng(offset)
    a = rng.integers(-2**31, 2**31 - 1, size=n, dtype=np.int64).astype(np.int32)
    x = dev(np.concatenate([np.full(offset, 7, np.int32), a]))
    R.GPUSort(x[offset:], n)
    got = host(x)
    np.testing.assert_array_equal(got[offset:], np.sort(a))
    assert np.all(got[:offset] == 7)


@pytest.mark.parametrize("nib", [1, 2, 3, 7, 1000, 1024, 4096, 8192, 10000, 65535, 65536])
def test_node_to_block_division_edges(built, nib):
    """NodeToBlock divides node indices by nodes_in_block with a multiply-high;
    node indices at block edges and up to 2^30 - 2 give the exact quotient."""
    nodes = [0, 1, nib - 1, nib, nib + 1, 2 * nib - 1, (1 << 30) - 2, (1 << 30) - 3, 123456789, (1 << 29) + 7]
    nodes += list(np.random.default_rng(nib).integers(0, (1 << 30) - 1, size=5000))
    nodes = np.array([x for x in nodes if 0 <= x <= (1 << 30) - 2], np.int64)
    dup = np.arange(nodes.size) & 1
    words = (((nodes + 1) << 1) | dup).astype(np.int32)
    words = np.concatenate([words, np.array([NO_HIT, -5, -1], np.int32)])
    conv = words.astype(np.int64)
    hit = (conv > 0) & (conv != NO_HIT)
    conv[hit] = ((((conv[hit] >> 1) - 1) // nib + 1) << 1) | (conv[hit] & 1)
    np.testing.assert_array_equal(_unique(words, nib), np.unique(conv).astype(np.int32))


def test_bounded_wait_gives_up_and_context_survives(built):
    """Failure detection without a fault: a wait on a word nothing publishes
    gives up after its time limit, the call reports it, and the next sort on
    the same context is correct."""
    import time
    t = time.time()
    assert R.lib().rayt_selftest_bounded_wait(0.02, None) == 0
    assert time.time() - t < 5.0
    a = np.random.default_rng(3).integers(-1000, 1000, size=100000).astype(np.int32)
    x = dev(a)
    R.GPUSort(x, a.size)
    np.testing.assert_array_equal(host(x), np.sort(a))


def test_feedback_unique_cached_graph_replays(built):
    """rayt_feedback_unique replays its cached graph while the pointers, n and
    nodes_in_block repeat.  The same input and output buffers, refilled
    between calls so the bitmap and radix paths alternate: every result equals
    numpy's, so nothing of one call (path choice, counts) is baked in."""
    import torch
    n, nib = 300_000, 512
    w = torch.zeros(n, dtype=torch.int32, device="cuda")
    out = torch.zeros(n, dtype=torch.int32, device="cuda")
    rng = np.random.default_rng(41)
    paths = []
    for k in range(8):
        if k % 2 == 0:  # narrow keys: bitmap path
            words = feedback_words(n, 100 + k, id_bits=14)
        else:  # keys over the whole int32 range: radix passes
            words = rng.integers(-2**31, 2**31 - 1, n, dtype=np.int64).astype(np.int32)
            words[rng.random(n) < 0.6] = NO_HIT
            words[:500] = words[500:1000]
        paths.append(_bitmap_path(words, nib))
        w.copy_(torch.from_numpy(words))
        cnt = R.feedback_unique(w, n, nib, out)
        np.testing.assert_array_equal(host(out)[:cnt], _np_unique(words, nib), err_msg="call %d" % k)
    assert paths == [True, False] * 4


def test_lookback_epoch_restart(built):
    """The sort/unique look-back tags carry a 27-bit per-call epoch; before it
    would repeat, every look-back table of the device is cleared and the epoch
    restarts.  Driven to the restart through the testing hook: sorts and
    feedback uniques across it stay exact, and so does a large call after a
    run of small ones (whose stale look-back words a repeated tag would read)."""
    import torch
    L = R.lib()
    big = feedback_words(1 << 22, 9, id_bits=30)  # wide: radix passes over many tiles
    small = feedback_words(5000, 10)
    try:
        assert L.rayt_testing_set_lookback_epoch((1 << 27) - 4) == 0
        for k in range(8):
            words = big if k in (0, 7) else small
            np.testing.assert_array_equal(_unique(words, 4096), _np_unique(words, 4096), err_msg="call %d" % k)
            a = np.random.default_rng(k).integers(-2**31, 2**31 - 1, 70000, dtype=np.int64).astype(np.int32)
            x = dev(a)
            R.GPUSort(x, a.size)
            np.testing.assert_array_equal(host(x), np.sort(a), err_msg="sort %d" % k)
    finally:
        torch.cuda.synchronize()
