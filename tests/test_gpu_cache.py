"""Block-file validation on load: a block whose links leave the block or name a
block past the last one is refused with RAYT_E_FORMAT before it reaches the
cache (the traversal never sees it).  And the renderer's batched feedback
marks against the same marks one by one through the C ABI."""
import ctypes as C
import os
import shutil
import struct

import numpy as np
import pytest

import rayt_gb300 as R

pytestmark = pytest.mark.gpu


def _corrupt(src, dst, kind):
    """Copies the tree file and breaks one link of one non-root block: a child
    link made to reach past the block's end, or a fault link made to name a
    block past the last one.  Returns the corrupted block's index."""
    shutil.copyfile(src, dst)
    info = R.StoredOctreeLoader(src).info
    nib, blocks = info.nodes_in_block, info.blocks_count
    with open(dst, "r+b") as f:
        for b in range(blocks):
            if b == info.root_block_index:
                continue
            base = info.header_bytes + info.block_stride * b + 76
            f.seek(base)
            links = np.frombuffer(f.read(4 * nib), np.uint32)
            used = (links & 255) != 0
            fault = ((links >> 8) & 1) == 1
            cand = np.nonzero(used & (fault if kind == "fault" else ~fault))[0]
            if cand.size == 0:
                continue
            n = int(cand[0])
            l = int(links[n])
            if kind == "child":  # two children starting at the block's last node: one past the end
                l = (l & ~255 & ((1 << 11) - 1)) | 0x3 | ((nib - 1) << 11)
            else:  # a fault link to block index blocks_count
                l = (l & ((1 << 11) - 1)) | (blocks << 11)
            f.seek(base + 4 * n)
            f.write(struct.pack("<I", l))
            return b
    raise AssertionError("no link of that kind in the tree")


@pytest.mark.parametrize("kind", ["child", "fault"])
def test_corrupt_block_is_refused(trees, tmp_path, kind):
    dst = os.path.join(str(tmp_path), "bad.tree")
    _corrupt(trees["terrain8s"], dst, kind)
    ld = R.StoredOctreeLoader(dst)
    cm = R.GPUOctreeCacheManager(0, ld)  # room for every block: the bad one is loaded
    with pytest.raises(R.RaytError) as e:
        cm.InitialFillCache()
    assert e.value.code == -3  # RAYT_E_FORMAT
    assert ("past the end of its block" if kind == "child" else "past the last block") in str(e.value)


def test_valid_tree_loads_and_reloads(trees):
    """The same tree unmodified fills the whole cache; a second cache over the
    same loader (blocks read again) fills identically."""
    ld = R.StoredOctreeLoader(trees["terrain8s"])
    a = R.GPUOctreeCacheManager(0, ld)
    a.InitialFillCache()
    b = R.GPUOctreeCacheManager(0, ld)
    b.InitialFillCache()
    assert a.blocks() == b.blocks()


def _marks_then_requests(ld, cap, hits, dups, requests, batched):
    """A full cache of `cap` slots; one transaction that marks `hits` and
    `dups` (one by one through the C ABI, or as the renderer's batch) and then
    requests blocks until the transaction fills.  Returns the markers' states
    after the marks and the cache's buffers after the transaction."""
    c = R.GPUOctreeCacheManager(cap, ld)
    c.InitialFillCache()
    filled_by_fill = c.stats()["uploaded_blocks"]
    c.StartRequestSession()
    c.StartRequestTransaction()
    if batched:
        h = np.ascontiguousarray(hits, np.int32)
        d = np.ascontiguousarray(dups, np.int32)
        I = C.POINTER(C.c_int)
        R._check(R.lib().rayt_testing_cache_mark_batch(c.handle, h.ctypes.data_as(I), h.size,
                                                        d.ctypes.data_as(I), d.size))
    else:
        for s in hits:
            try:
                c.MarkBlockAsUsed(int(s))
            except R.RaytError:
                pass
        for s in dups:
            try:
                c.MarkParentAsUsed(int(s))
            except R.RaytError:
                pass
    filled = (c.TransactionFilledCache(), c.SessionFilledCache())
    asked = 0
    for b in requests:
        if c.TransactionFilledCache():
            break
        try:
            c.RequestBlock(int(b))
            asked += 1
        except R.RaytError:  # its parent is not resident
            pass
    c.EndRequestTransaction()
    c.EndRequestSession()
    out = [c.read_buffer(n) for n in ("node links", "normals", "colors", "far pointers")]
    loaded = c.stats()["uploaded_blocks"] - filled_by_fill
    c.close()
    return filled, asked, loaded, out


@pytest.mark.parametrize("seed,frac", [(1, 0.1), (2, 0.4), (3, 0.9), (4, 3.0), (5, -1)])
def test_batched_feedback_marks_equal_one_by_one(trees, seed, frac):
    """The renderer applies a pass's LRU marks (MarkBlockAsUsed per hit block,
    then MarkParentAsUsed per duplicate hit) as one batch.  On a full cache the
    marks decide which slots the following requests evict, so the batch must
    leave the LRU list and the markers exactly as the calls one by one: same
    filled flags, same evictions, same cache bytes.  Random slots with repeats
    and out-of-range values, a few to thousands of marks."""
    ld = R.StoredOctreeLoader(trees["terrain8s"])
    cap = 300  # of 793 blocks: the fill takes every slot, so each load evicts
    rng = np.random.default_rng(seed)
    n = int(cap * frac) if frac > 0 else cap
    hits = rng.integers(-2, cap + 2, size=n)
    if frac < 0:  # every slot marked: both markers reach the LRU front
        hits = np.concatenate([rng.integers(0, cap, size=50), rng.permutation(cap)])
    dups = rng.integers(-2, cap + 2, size=max(1, n // 4))
    requests = rng.permutation(ld.info.blocks_count)[:600]
    a = _marks_then_requests(ld, cap, hits, dups, requests, batched=False)
    b = _marks_then_requests(ld, cap, hits, dups, requests, batched=True)
    assert a[0] == b[0]
    if frac < 0:
        assert a[0] == (True, True)
    assert a[1] == b[1] and a[2] == b[2]
    for x, y in zip(a[3], b[3]):
        assert np.array_equal(x, y)
    if 0 < frac < 1:
        assert a[2] > 0  # requests loaded blocks, each evicting the LRU front
