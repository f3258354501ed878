"""CPU tests of bench.py's multi-rank plumbing (replicas only: every rank
renders the same workload on its own GPU; ranks meet only in a barrier and in
the max/sum reductions of the timing).  Two gloo ranks on 127.0.0.1."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, scene_dir, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RAYT_SCENE_DIR": scene_dir})
    sys.path.insert(0, ROOT)
    import bench as B
    B.SCENE_DIR = scene_dir
    r, w, local = B.dist_setup(world, backend="gloo")
    assert (r, w, local) == (rank, world, rank)
    # timing reductions: the job's time is the slowest rank's, throughput the total
    t = B.max_over_ranks(1.0 + rank, w)
    s = B.sum_over_ranks(10.0 * (rank + 1), w)
    # the scene is built once (rank 0) and the other ranks wait for its marker
    B.WORKLOADS["tiny"] = {"depth": 5, "spheres": 3, "width": 8, "height": 8, "cache_bytes": 0, "lod": 1.0}
    path = B.scene_path("tiny", local, w)
    B.barrier(w)
    out.put((rank, t, s, os.path.exists(path), os.path.getsize(path)))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_gloo_ranks(tmp_path, built):
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, str(tmp_path), q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [2.0, 2.0]      # max over ranks
    assert [r[2] for r in res] == [30.0, 30.0]    # sum over ranks
    assert all(r[3] for r in res) and res[0][4] == res[1][4] > 0  # one scene, seen by both


def test_flythrough_frames_sit_at_the_configured_spacing(built):
    """c3 is 300 frames along one loop of its spline: a run of any length
    renders the first frames of that flythrough at the same spacing (the
    cameras of a 25-frame run are the first 25 of a 303-frame run), frame i
    wraps around the closed loop after 300, and a period equal to the run
    spreads the run over the whole loop."""
    sys.path.insert(0, ROOT)
    import numpy as np
    import bench as B
    w, h = 1920, 1080
    short = B.camera_path("c3", 25, w, h, period=B.C3_PATH_FRAMES)
    long_ = B.camera_path("c3", 303, w, h, period=B.C3_PATH_FRAMES)
    assert np.array_equal(np.array(short), np.array(long_[:25]))
    assert np.array_equal(np.array(long_[300:303]), np.array(long_[0:3]))
    loop = B.camera_path("c3", 25, w, h)
    assert np.array_equal(np.array(loop[0]), np.array(short[0]))
    assert not np.array_equal(np.array(loop[1]), np.array(short[1]))  # 12x the camera motion per frame
