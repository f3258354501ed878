"""CPU test: the parallel block-file builder writes the same bytes for every
thread count (frontier subtrees are packed on workers with block-local
numbering and relocated in the serial builder's order)."""
import hashlib
import os

import pytest


@pytest.mark.parametrize("kind", ["terrain", "sphere"])
def test_builder_bytes_do_not_depend_on_threads(tmp_path, built, kind, monkeypatch):
    import rayt_gb300 as R
    digests = []
    for threads in (1, 2, 5):
        monkeypatch.setenv("RAYT_BUILD_THREADS", str(threads))
        path = str(tmp_path / ("%s_%d.tree" % (kind, threads)))
        if kind == "terrain":
            R.build_terrain(path, 8, 512, spheres=40, min_radius=2, max_radius=20)
        else:
            R.build_sphere_test(path, (0.5, 0.5, 0.5), 0.4, 8, 300)
        with open(path, "rb") as f:
            digests.append(hashlib.sha256(f.read()).hexdigest())
        os.remove(path)
    assert len(set(digests)) == 1
