"""Block-file validation on load: a block whose links leave the block or name a
block past the last one is refused with RAYT_E_FORMAT before it reaches the
cache (the traversal never sees it)."""
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
