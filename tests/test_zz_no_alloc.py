"""rayt_feedback_unique_noalloc through the C ABI: the same unique arrays as
rayt_feedback_unique on two calls in a row (the second call must not see the
first call's leftovers in the shared static scratch), and the size limit.

This file is collected last on purpose: if it fails, a run that stops at the
first failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

from tests.golden.common import feedback_words

pytestmark = pytest.mark.gpu

MAX_WORDS = 1 << 21  # RAYT_FEEDBACK_UNIQUE_NOALLOC_MAX_WORDS


def _abi():
    import rayt_gb300 as R
    L = R.lib()
    f = L.rayt_feedback_unique_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.POINTER(C.c_int), C.c_void_p]
    g = L.rayt_feedback_unique
    g.restype = C.c_int
    g.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.POINTER(C.c_int), C.c_void_p]
    return L, f, g


def _run(fn, words, nib):
    import torch
    d_in = torch.from_numpy(words).cuda()
    d_out = torch.full((max(1, words.size),), -7, dtype=torch.int32, device="cuda")
    cnt = C.c_int(-1)
    torch.cuda.synchronize()
    rc = fn(d_in.data_ptr(), words.size, nib, d_out.data_ptr(), C.byref(cnt), None)
    torch.cuda.synchronize()
    return rc, d_out.cpu().numpy()[:max(cnt.value, 0)], cnt.value


def test_noalloc_matches_allocating_entry_point_twice(built):
    L, noalloc, existing = _abi()
    # two calls in a row with different inputs: a larger one, then a smaller
    # one whose result would show stale data from the first if any leaked
    for n, nib, seed in [(MAX_WORDS, 4096, 31), (300001, 512, 32)]:
        words = feedback_words(n, seed)
        rc_a, got, cnt_a = _run(noalloc, words, nib)
        assert rc_a == 0, L.rayt_last_error()
        rc_b, want, cnt_b = _run(existing, words, nib)
        assert rc_b == 0, L.rayt_last_error()
        assert cnt_a == cnt_b and cnt_a > 0
        np.testing.assert_array_equal(got, want)


def test_noalloc_rejects_sizes_beyond_its_limit(built):
    L, noalloc, _ = _abi()
    cnt = C.c_int(-1)
    rc = noalloc(C.c_void_p(16), MAX_WORDS + 1, 4096, C.c_void_p(16), C.byref(cnt), None)
    assert rc == -8  # RAYT_E_LIMIT, before any GPU work
    assert b"MAX_WORDS" in L.rayt_last_error()
