"""Benchmark of the per-frame path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload c3|c1|c2|c2r|c4|c5|c5p]

The default workload is c3, the configuration the Mrays/s-at-1080p metric is
quoted on.

A step is one frame of the plain per-frame path (RenderFrame: traversal
passes, feedback unique, cache transaction with block streaming, finish) for
the frame workloads, and one compaction + radix sort + unique of the feedback
words for c2.  Workloads (synthetic seeded scenes built by the block-file
builder; no public dataset is involved):
  c1  depth-10 fBm heightfield (1024^3), 512x512, whole tree resident
  c3  depth-12 heightfield + sphere shells (4096^3), 1920x1080 flythrough of
      300 frames along a seeded Catmull-Rom spline (a shorter run times the
      start of it at the same frame spacing), block cache capped at 2 GiB,
      blocks streamed from the file
  c2  2^28 feedback words: 90% NO_HIT, Zipf(1.1) block IDs over 2^24
  c2r the same with block IDs over 2^28: the kept keys span more than 2^26
      values, so unique runs the LSD radix passes instead of the bitmap
  c4  the c3 scene, 64 views per frame of sizes drawn from {256^2, 640x480,
      1280x720, 1920x1080} (seed 7), view v on its own spline (seed 7 + v),
      through the batched renderer; the plain per-view path is timed beside it
  c5  depth-14 heightfield + spheres (16384^3, 16384-node blocks), 16 clients
      of sizes drawn from {1280x720, 1920x1080, 2560x1440} (seed 100), client
      c on its own spline (seed 100 + c), frame requests Poisson at 60 Hz per
      client (seed 11), through the server (continuous batching, 40 GiB shared
      cache) and through the plain per-frame path on the same schedule
  c5p c5 with a 6 GiB shared cache, below the tree: shared-LRU eviction

--impl reference times the reference algorithm's CPU implementation (the
oracle restatement in oracle/, all host threads) on the same workload.
With --gpus N > 1 (torchrun), every rank renders the same workload on its own
GPU (replicas; the path has no cross-GPU step) and value is the total.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

HBM_FALLBACK_GBS = 6800.0
SCENE_DIR = os.environ.get("RAYT_SCENE_DIR", "/tmp/rayt_bench_scenes")
C1_CAMERA = [45.0, -30.0, 0.0, -0.06, 0.66, 1.06, 60.0]
C3_PATH_FRAMES = 300  # the C3 flythrough: 300 frames along one loop of the spline

WORKLOADS = {
    "c1": {"depth": 10, "spheres": 0, "width": 512, "height": 512, "cache_bytes": 0, "lod": 1.0},
    "c3": {"depth": 12, "spheres": 2000, "width": 1920, "height": 1080, "cache_bytes": 2 << 30, "lod": 1.0},
    # 64 views per frame; the cache holds the whole tree (about 6.5 GB), so a
    # frame measures batched traversal + feedback rather than streaming
    "c4": {"depth": 12, "spheres": 2000, "width": 0, "height": 0, "cache_bytes": 0, "lod": 1.0, "views": 64,
           "sizes": [(256, 256), (640, 480), (1280, 720), (1920, 1080)], "size_seed": 7},
    # 16 clients, Poisson 60 Hz each, against one shared 40 GiB cache.  The
    # cache format's 21-bit far-pointer slots address fewer than 2^18 blocks,
    # so the scene uses 16384-node blocks: 40 GiB is 218453 of them (3.6 G
    # nodes, node indices unsigned 32-bit), more than the whole tree
    "c5": {"depth": 14, "spheres": 2000, "width": 0, "height": 0, "cache_bytes": 40 << 30, "nib": 16384,
           "lod": 1.0,
           "clients": 16, "sizes": [(1280, 720), (1920, 1080), (2560, 1440)], "size_seed": 100,
           "rate_hz": 60.0, "arrival_seed": 11, "seconds": 2.0, "closed_frames": 20, "max_passes": 8},
}
# The served workload under cache pressure: the same scene and clients with a
# 6 GiB cache, well below the tree, so the clients' blocks evict one another
# from the shared LRU
WORKLOADS["c5p"] = dict(WORKLOADS["c5"], cache_bytes=6 << 30)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=0)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c3", choices=["c1", "c2", "c2r", "c3", "c4", "c5", "c5p"])
    ap.add_argument("--cpu-seconds", type=float, default=20.0, help="budget of the CPU baseline sample")
    ap.add_argument("--spheres", type=int, default=None, help="override the workload's sphere count")
    ap.add_argument("--cache-mib", type=int, default=None, help="override the workload's cache size")
    ap.add_argument("--depth", type=int, default=None, help="override the workload's octree depth")
    ap.add_argument("--c2-log2n", type=int, default=28, help="c2: 2^k feedback words (profiling uses a smaller k)")
    ap.add_argument("--parity-frames", type=int, default=5,
                    help="frame workloads: after timing, compare this many timed frames (and the warm-up frames "
                         "before them) with the oracle, untimed; 0 skips the check")
    a = ap.parse_args()
    if a.workload in WORKLOADS:
        if a.spheres is not None:
            WORKLOADS[a.workload]["spheres"] = a.spheres
        if a.cache_mib is not None:
            WORKLOADS[a.workload]["cache_bytes"] = a.cache_mib << 20
        if a.depth is not None:
            WORKLOADS[a.workload]["depth"] = a.depth
    return a


# ---------------------------------------------------------------------------
def dist_setup(n, backend="nccl"):
    """Rank, world size and local rank from the torchrun environment; one
    process group for the barrier and the timing reductions (NCCL on the GPU
    box, gloo in the CPU tests)."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def _reduce(x, world, op):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=op)
    return float(t.item())


def max_over_ranks(x, world):
    import torch.distributed as dist
    return _reduce(x, world, dist.ReduceOp.MAX) if world > 1 else x


def sum_over_ranks(x, world):
    import torch.distributed as dist
    return _reduce(x, world, dist.ReduceOp.SUM) if world > 1 else x


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for k, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(k)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def hbm_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return HBM_FALLBACK_GBS, "fallback"


class roofline_range:
    """NVTX range "roofline" around the launches the roofline object times, so
    an ncu capture can select exactly them (--nvtx --nvtx-include roofline/)."""

    def __enter__(self):
        import torch
        torch.cuda.nvtx.range_push("roofline")

    def __exit__(self, *exc):
        import torch
        torch.cuda.nvtx.range_pop()


def profile_values(name):
    """'key: number' lines of the committed ncu summary profiles/<name>.md."""
    out = {}
    try:
        for line in open(os.path.join(ROOT, "profiles", name + ".md")):
            k, sep, v = line.partition(":")
            if sep and k.strip() in ("traffic_bytes_per_launch", "alg_bytes_per_launch"):
                try:
                    out[k.strip()] = float(v)
                except ValueError:
                    pass
    except OSError:
        pass
    return out


def profile_traffic(name):
    """DRAM bytes per launch of the traversal kernel from the committed ncu
    summary (profiles/<name>.md, line 'traffic_bytes_per_launch: N')."""
    return profile_values(name).get("traffic_bytes_per_launch")


def scaled_traffic(name, alg_bytes):
    """DRAM bytes of the timed launch: the profiled launch's DRAM bytes
    (profiles/<name>.md) scaled by the ratio of the two launches' algorithmic
    bytes, when the profile records its own ('alg_bytes_per_launch: N'); the
    factor is 1 when the profile captured the same camera.  Returns (bytes,
    rule)."""
    v = profile_values(name)
    t, a = v.get("traffic_bytes_per_launch"), v.get("alg_bytes_per_launch")
    if t is None:
        return None, "no profile"
    if not a:
        return t, "profiled launch as is"
    return round(t * alg_bytes / a), "profiled DRAM bytes x (algorithmic bytes of this launch / of the profiled launch)"


# ---------------------------------------------------------------------------
def scene_path(wl, local_rank, world):
    cfg = WORKLOADS[wl]
    os.makedirs(SCENE_DIR, exist_ok=True)
    nib = cfg.get("nib", 4096)
    path = os.path.join(SCENE_DIR, "terrain_d%d_s%d_n%d.tree" % (cfg["depth"], cfg["spheres"], nib))
    done = path + ".ok"
    if local_rank == 0 and not os.path.exists(done):
        import rayt_gb300 as R
        t = time.time()
        R.build_terrain(path + ".tmp", cfg["depth"], nib, spheres=cfg["spheres"], min_radius=8, max_radius=256)
        os.replace(path + ".tmp", path)
        open(done, "w").write("%.1f\n" % (time.time() - t))
    barrier(world)
    while not os.path.exists(done):
        time.sleep(0.5)
    return path


def camera_path(wl, frames, w, h, seed=3, period=None):
    """C1: one fixed camera.  C3/C4: a Catmull-Rom spline through 8 control
    points drawn with `seed` inside the scene, looking along the path and 25 deg
    down (C3 seed 3; C4 view v seed 7 + v).  Frame i sits at (i mod period) /
    period of the closed loop; period defaults to `frames` (the whole loop in
    the frames asked for)."""
    import rayt_gb300 as R
    if wl == "c1":
        c = R.Camera(C1_CAMERA[0], C1_CAMERA[1], C1_CAMERA[2], C1_CAMERA[3:6], C1_CAMERA[6], w / h)
        m = c.view_proj_inv()
        return [m] * frames
    rng = np.random.default_rng(seed)
    pts = np.stack([rng.uniform(0.15, 0.85, 8), rng.uniform(0.62, 0.85, 8), rng.uniform(0.15, 0.85, 8)], 1)
    pts = np.concatenate([pts, pts[:3]])  # closed loop

    def spline(u):
        seg = min(int(u), len(pts) - 4)
        t = u - seg
        p0, p1, p2, p3 = pts[seg:seg + 4]
        return 0.5 * ((2 * p1) + (-p0 + p2) * t + (2 * p0 - 5 * p1 + 4 * p2 - p3) * t * t
                      + (-p0 + 3 * p1 - 3 * p2 + p3) * t * t * t)

    out = []
    span = len(pts) - 3
    period = max(1, period or frames)
    for i in range(frames):
        u = span * (i % period) / period
        p = spline(u)
        q = spline(min(span - 1e-3, u + 0.01))
        d = q - p
        yaw = math.degrees(math.atan2(d[0], -d[2]))
        c = R.Camera(yaw, -25.0, 0.0, tuple(float(v) for v in p), 60.0, w / h)
        out.append(c.view_proj_inv())
    return out


def cache_blocks(cfg):
    """Cache blocks for the workload's cache bytes (12 bytes a node), at most
    2^18 - 1 (the cache format's far-pointer slots); 0 = the whole tree."""
    if not cfg["cache_bytes"]:
        return 0
    return int(min(cfg["cache_bytes"] // (cfg.get("nib", 4096) * 12), (1 << 18) - 1))


# ---------------------------------------------------------------------------
def frames_parity(path, cfg, mats, seed=1, timed=None, timed_first=0):
    """Untimed parity check of the per-frame path on the workload itself: the
    oracle and a fresh GPU cache + renderer (feedback words recorded, depth
    output on) render the same frames from the same initial fill with the same
    hit-window seed, and every frame's pass count, every pass's per-pixel
    feedback words, image, depth bits and hit nodes are compared, then the
    cache buffers after the last frame.  `timed` holds images the timed run
    produced for frames timed_first, timed_first + 1, ...; they are compared
    with the oracle's frames too."""
    import ctypes

    import rayt_gb300 as R
    from oracle import oracle as O
    w, h = cfg["width"], cfg["height"]
    blocks = cache_blocks(cfg)
    t0 = time.time()
    ld = R.StoredOctreeLoader(path)
    cm = R.GPUOctreeCacheManager(blocks, ld)
    cm.InitialFillCache()
    rt = R.GPURayTracer(cm, w, h)
    rt.set_lod_voxel_size(cfg["lod"])
    rt.set_frame_time_limit(1e30)
    rt.seed(seed)
    rt.record_passes(True)
    rt.set_depth_output(True)
    sc = O.OracleScene(path, blocks, w, h, cfg["lod"], 1e30)
    sc.record(True)
    ctypes.CDLL(None).srand(ctypes.c_uint(seed))
    out = {"frames": 0, "pixels_differing": 0, "passes_equal": True, "pass_words_equal": True,
           "depth_bits_equal": True, "hit_nodes_differing": 0, "timed_frames_checked": 0,
           "timed_pixels_differing": 0, "passes": 0, "uploaded_blocks": 0}
    for i, m in enumerate(mats):
        n, img = sc.render(m)
        dref, nref = sc.depth()
        rt.RenderFrame(m)
        st = rt.stats()
        out["frames"] += 1
        out["passes"] += n
        out["uploaded_blocks"] += st["uploaded_blocks"]
        out["passes_equal"] &= st["passes"] == n
        out["pixels_differing"] += int((rt.read_image() != img).any(axis=2).sum())
        for p in range(min(n, st["passes"])):
            out["pass_words_equal"] &= bool(np.array_equal(rt.pass_words(p), sc.pass_words(p)))
        d, nodes = rt.read_depth()
        out["depth_bits_equal"] &= bool(np.array_equal(d.view(np.uint32), dref.view(np.uint32)))
        out["hit_nodes_differing"] += int((nodes != nref).sum())
        k = i - timed_first
        if timed is not None and 0 <= k < len(timed):
            out["timed_frames_checked"] += 1
            out["timed_pixels_differing"] += int((timed[k] != img).any(axis=2).sum())
    nodes = sc.max_blocks * sc.nib
    same = True
    for ch, name in enumerate(["node links", "normals", "colors"]):
        same &= bool(np.array_equal(cm.read_buffer(name), sc.read(ch, nodes * 4)))
    same &= bool(np.array_equal(cm.read_buffer("far pointers"), sc.read(-1, sc.max_blocks * 32)))
    out["cache_buffers_equal"] = same
    out["seconds"] = round(time.time() - t0, 1)
    sc.close()
    del rt, cm, ld
    out["ok"] = bool(out["passes_equal"] and out["pass_words_equal"] and out["depth_bits_equal"] and same
                     and out["pixels_differing"] == 0 and out["hit_nodes_differing"] == 0
                     and out["timed_pixels_differing"] == 0)
    return out


def run_cpu_frames(path, cfg, mats, budget_s, warm=()):
    """The oracle (reference algorithm on host cores) over the same frames, until
    the frames run out or the time budget is spent, after rendering the
    warm-up frames `warm` untimed (the cache then holds what the GPU arm's
    cache held when its timing began).  Returns (rays, seconds, frames,
    setup_seconds)."""
    import ctypes

    from oracle import oracle as O
    w, h = cfg["width"], cfg["height"]
    t0 = time.time()
    sc = O.OracleScene(path, cache_blocks(cfg), w, h, cfg["lod"], 1e30)
    ctypes.CDLL(None).srand(ctypes.c_uint(1))
    for m in warm:
        sc.render(m)
    setup = time.time() - t0
    rays, el, n = 0, 0.0, 0
    for m in mats:
        t = time.time()
        sc.render(m)
        el += time.time() - t
        rays += w * h
        n += 1
        if el > budget_s:
            break
    sc.close()
    return rays, el, n, setup


def bench_frames(args, rank, world, local):
    import torch

    import rayt_gb300 as R
    wl = args.workload
    cfg = WORKLOADS[wl]
    w, h = cfg["width"], cfg["height"]
    steps = args.steps or (300 if wl == "c3" else 200)
    path = scene_path(wl, local, world)
    # C3 is 300 frames along its spline: whatever the number of frames run,
    # they sit at that spacing (a short run covers the start of the flythrough
    # at the configured camera speed, not the whole loop at a higher one)
    mats = camera_path(wl, args.warmup + steps, w, h, period=C3_PATH_FRAMES if wl == "c3" else None)
    threads = os.cpu_count() or 1

    if args.impl == "reference":
        if rank != 0:
            return None
        rays, el, n, setup = run_cpu_frames(path, cfg, mats[args.warmup:], args.cpu_seconds * 3,
                                            warm=mats[:args.warmup])
        v = rays / el / 1e6
        sample = ("%d of %d frames at %dx%d after the same %d warm-up frames (oracle, OpenMP)"
                  % (n, steps, w, h, args.warmup))
        return {"metric": "Mrays/s at %dx%d (frames of the per-frame path)" % (w, h), "value": round(v, 3),
                "unit": "Mrays/s", "impl": "reference", "n_gpus": 1, "steps": n, "warmup": args.warmup,
                "ms_per_step": round(el / n * 1e3, 3), "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": wl, "width": w, "height": h, "depth": cfg["depth"],
                           "spheres": cfg["spheres"], "cache_blocks": cache_blocks(cfg)},
                "cpu_baseline": {"value": round(v, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
                                 "sample": sample},
                "e2e": {"value": round(v, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}

    torch.cuda.set_device(local)
    ld = R.StoredOctreeLoader(path)

    def renderer(host_image=None):
        """A fresh cache (InitialFillCache) and renderer that have rendered the
        warm-up frames; host_image: deliver every frame there."""
        c = R.GPUOctreeCacheManager(cache_blocks(cfg), ld)
        t0 = time.time()
        c.InitialFillCache()
        fill = time.time() - t0
        r = R.GPURayTracer(c, w, h)
        r.set_lod_voxel_size(cfg["lod"])
        r.set_frame_time_limit(1e30)
        r.seed(1)  # the hit-window generator; the parity check replays the same sequence
        if host_image is not None:
            r.set_host_image(host_image.data_ptr(), host_image.numel())
        for i in range(args.warmup):
            r.RenderFrame(mats[i])
        return c, r, fill

    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # > L2 (129 MB)
    timed_imgs = []  # the first parity_frames timed images, checked against the oracle afterwards

    # device-timed frames (value): each frame's image stays in device memory;
    # the wall clock around RenderFrame plus a read-back of the image after
    # the call is reported beside the end-to-end number (e2e_read_after)
    pinned_after = torch.empty((h, w, 4), dtype=torch.uint8).pin_memory()
    cm, rt, fill_s = renderer()
    stream = torch.cuda.ExternalStream(rt.stream_handle())
    torch.cuda.synchronize()
    barrier(world)
    clocks = ClockSampler(local)
    clocks.start()
    cs0 = cm.stats()
    ms_dev, wall_after = 0.0, 0.0
    passes, launches, h2d, uploaded, trace_ms = 0, 0, 0, 0, 0.0
    part_ms = {k: 0.0 for k in ("gpu_ms_feedback", "gpu_ms_upload", "host_ms_wait", "host_ms_decode", "host_ms_load")}
    lat = []
    for i in range(args.warmup, args.warmup + steps):
        with torch.cuda.stream(stream):
            flush.fill_(i & 255)  # L2 holds nothing of the previous frame
        stream.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t = time.perf_counter()
        e0.record(stream)
        rt.RenderFrame(mats[i])
        e1.record(stream)
        R._check(R.lib().rayt_renderer_read_image(rt._h, pinned_after.data_ptr(), pinned_after.numel()))
        wall_after += time.perf_counter() - t
        e1.synchronize()
        d = e0.elapsed_time(e1)
        ms_dev += d
        lat.append(d)
        st = rt.stats()
        passes += st["passes"]
        launches += st["kernel_launches"]
        h2d += st["bytes_h2d"]
        uploaded += st["uploaded_blocks"]
        trace_ms += st["gpu_ms_trace"]
        for k in part_ms:
            part_ms[k] += st[k]
    torch.cuda.synchronize()
    cs1 = cm.stats()
    n_cache_blocks = cm.blocks()[1]

    # roofline of the dominant kernel (first-pass traversal) on the last camera
    m_last = mats[args.warmup + steps - 1]
    fetch = rt.count_fetches(m_last)
    with roofline_range():
        pass_ms = rt.time_pass(m_last, 5)
    rt.close()
    cm.close()

    # end to end (e2e): the same frames from a fresh cache through the public
    # API, every frame's RGBA8 image delivered to pinned host memory inside
    # RenderFrame (rayt_renderer_set_host_image), wall clock per frame
    pinned = torch.empty((h, w, 4), dtype=torch.uint8).pin_memory()
    cm, rt, _ = renderer(host_image=pinned)
    stream = torch.cuda.ExternalStream(rt.stream_handle())
    torch.cuda.synchronize()
    barrier(world)
    wall, d2h = 0.0, 0
    for i in range(args.warmup, args.warmup + steps):
        with torch.cuda.stream(stream):
            flush.fill_(i & 255)
        stream.synchronize()
        t = time.perf_counter()
        rt.RenderFrame(mats[i])
        wall += time.perf_counter() - t
        if len(timed_imgs) < args.parity_frames:
            timed_imgs.append(pinned.numpy().copy())
        d2h += rt.stats()["bytes_d2h"]  # the image and the feedback read-backs
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    rt.close()
    cm.close()
    t_dev = max_over_ranks(ms_dev / 1e3, world)
    t_wall = max_over_ranks(wall, world)
    t_wall_after = max_over_ranks(wall_after, world)
    rays = float(w * h * steps)
    total_rays = sum_over_ranks(rays, world)
    # block streaming over the timed frames: block content and patches moved
    # to the device, bytes of the block file read, and the rate the upload
    # launches moved them at (their device time)
    up_ms = part_ms["gpu_ms_upload"]
    streaming = {"h2d_bytes_per_frame": int(h2d / steps),
                 "file_bytes_per_frame": int((cs1["bytes_read"] - cs0["bytes_read"]) / steps),
                 "upload_gbs": round(h2d / (up_ms / 1e3) / 1e9, 1) if up_ms > 0 else None,
                 "block_source": "block file mapped into host memory, read by the upload kernel"
                                 if cs1["mapped"] else "pread into pinned staging, one copy per batch"}

    alg_bytes = 4 * fetch["link_fetches"] + 4 * fetch["far_fetches"] + 16 * fetch["rays"]
    achieved = alg_bytes / (pass_ms / 1e3) / 1e9
    peak, peak_kind = hbm_peak()
    traffic, traffic_rule = scaled_traffic("trace_kernel_%s" % wl, alg_bytes)

    cpu = None
    if rank == 0:
        crays, cel, cn, _ = run_cpu_frames(path, cfg, mats[args.warmup:], args.cpu_seconds, warm=mats[:args.warmup])
        cpu = {"value": round(crays / cel / 1e6, 3), "unit": "Mrays/s", "cores": os.cpu_count() or 1, "kind": "port",
               "sample": "%d frames at %dx%d of the same workload after the same %d warm-up frames (oracle, OpenMP)"
                         % (cn, w, h, args.warmup)}
    parity = None
    if rank == 0 and args.parity_frames > 0:
        parity = frames_parity(path, cfg, mats[:args.warmup + args.parity_frames], seed=1, timed=timed_imgs,
                               timed_first=args.warmup)
    if rank != 0:
        return None
    lat_sorted = np.sort(np.array(lat))
    return {
        "metric": "Mrays/s at %dx%d (frames of the per-frame path)" % (w, h),
        "value": round(total_rays / t_dev / 1e6, 3), "unit": "Mrays/s", "n_gpus": world, "steps": steps,
        "warmup": args.warmup, "ms_per_step": round(t_dev / steps * 1e3, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": wl, "width": w, "height": h, "depth": cfg["depth"], "spheres": cfg["spheres"],
                   "nodes_in_block": 4096, "cache_blocks": n_cache_blocks, "tree_blocks": ld.info.blocks_count,
                   "lod_voxel_size": cfg["lod"], "l2": "flushed between frames (256 MiB write)",
                   "parallelism": "replicas" if world > 1 else "single GPU", "initial_fill_s": round(fill_s, 2)},
        "e2e": {"value": round(total_rays / t_wall / 1e6, 3), "unit": "Mrays/s",
                "h2d_bytes_per_step": int(h2d / steps) + 64, "d2h_bytes_per_step": int(d2h / steps),
                "how": "wall clock around RenderFrame with the image delivered to pinned host memory inside the call"},
        "e2e_read_after": {"value": round(total_rays / t_wall_after / 1e6, 3), "unit": "Mrays/s",
                           "how": "wall clock around RenderFrame and a read-back of the image after it returns"},
        "frame_latency_ms": {"p50": round(float(np.percentile(lat_sorted, 50)), 4),
                             "p99": round(float(np.percentile(lat_sorted, 99)), 4)},
        "frames": {"passes_per_frame": round(passes / steps, 3), "uploaded_blocks_per_frame": round(uploaded / steps, 2),
                   "trace_ms_per_frame": round(trace_ms / steps, 4),
                   **{k.replace("_ms_", "_") + "_ms_per_frame": round(v / steps, 4) for k, v in part_ms.items()}},
        "streaming": streaming,
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic, "traffic_rule": traffic_rule,
                     "peak_source": peak_kind,
                     "kernel": "trace_kernel<first pass>", "launch_ms": round(pass_ms, 4),
                     "alg_bytes": int(alg_bytes), "bytes_per_ray": round(alg_bytes / fetch["rays"], 2),
                     "link_fetches_per_ray": round(fetch["link_fetches"] / fetch["rays"], 3),
                     "iterations_per_ray": round(fetch["iterations"] / fetch["rays"], 3)},
        "cpu_baseline": cpu,
        "parity": parity,
        "gpu_launches": int(launches),
        "clocks": clk,
    }


def batched_views(cfg):
    """C4: view v's size (drawn uniformly with seed 7) and camera spline seed."""
    rng = np.random.default_rng(cfg["size_seed"])
    pick = rng.integers(0, len(cfg["sizes"]), size=cfg["views"])
    return [tuple(cfg["sizes"][k]) for k in pick], [cfg["size_seed"] + v for v in range(cfg["views"])]


def bench_batched(args, rank, world, local):
    """C4: every frame renders 64 views of mixed sizes through one batched
    renderer (rayt_render_views: one traversal launch per pass for all views,
    pass graphs, launch shape from the autotuner).  Also times the same frames
    through the plain per-frame path, one RenderFrame per view."""
    import torch

    import rayt_gb300 as R
    wl = "c4"
    cfg = WORKLOADS[wl]
    steps = args.steps or 20
    path = scene_path(wl, local, world)
    sizes, seeds = batched_views(cfg)
    n = len(sizes)
    frames = args.warmup + steps
    per_view = [camera_path(wl, frames, w, h, seed=sd) for (w, h), sd in zip(sizes, seeds)]
    mats = [[per_view[v][f] for v in range(n)] for f in range(frames)]
    rays_per_frame = sum(w * h for w, h in sizes)
    threads = os.cpu_count() or 1
    metric = "Mrays/s, 64 views per frame (batched form, depth 12)"

    def cpu_frames(budget):
        from oracle import oracle as O
        sc = O.OracleScene(path, cache_blocks(cfg), views=sizes, lod=cfg["lod"])
        el, k = 0.0, 0
        for f in range(args.warmup, frames):
            t = time.time()
            sc.render_views(mats[f])
            el += time.time() - t
            k += 1
            if el > budget:
                break
        sc.close()
        return k * rays_per_frame, el, k

    if args.impl == "reference":
        if rank != 0:
            return None
        rays, el, k = cpu_frames(args.cpu_seconds * 3)
        v = rays / el / 1e6
        return {"metric": metric, "value": round(v, 3), "unit": "Mrays/s", "impl": "reference", "n_gpus": 1,
                "steps": k, "warmup": 0, "ms_per_step": round(el / k * 1e3, 3), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": wl, "views": n, "rays_per_frame": rays_per_frame, "depth": cfg["depth"]},
                "cpu_baseline": {"value": round(v, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
                                 "sample": "%d frames of 64 views (oracle, OpenMP)" % k},
                "e2e": {"value": round(v, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}

    torch.cuda.set_device(local)
    ld = R.StoredOctreeLoader(path)
    cm = R.GPUOctreeCacheManager(cache_blocks(cfg), ld)
    t0 = time.time()
    cm.InitialFillCache()
    fill_s = time.time() - t0
    rt = R.GPURayTracer.views(cm, sizes)
    rt.set_lod_voxel_size(cfg["lod"])
    rt.set_frame_time_limit(1e30)
    t0 = time.time()
    shape = rt.autotune(mats[0], reps=1)
    tune_s = time.time() - t0
    stream = torch.cuda.ExternalStream(rt.stream_handle())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    pinned = [torch.empty((h, w, 4), dtype=torch.uint8).pin_memory() for w, h in sizes]
    for f in range(args.warmup):
        rt.RenderViews(mats[f])
    torch.cuda.synchronize()
    barrier(world)
    clocks = ClockSampler(local)
    clocks.start()
    ms_dev, wall, launches, passes, lat = 0.0, 0.0, 0, 0, []
    for f in range(args.warmup, frames):
        with torch.cuda.stream(stream):
            flush.fill_(f & 255)
        stream.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t = time.perf_counter()
        e0.record(stream)
        rt.RenderViews(mats[f])
        e1.record(stream)
        for v in range(n):  # end to end: every view's image to pinned host memory
            R._check(R.lib().rayt_renderer_read_view_image(rt._h, v, pinned[v].data_ptr(), pinned[v].numel()))
        wall += time.perf_counter() - t
        e1.synchronize()
        d = e0.elapsed_time(e1)
        ms_dev += d
        lat.append(d)
        st = rt.stats()
        launches += st["kernel_launches"]
        passes += st["passes"]
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    t_dev = max_over_ranks(ms_dev / 1e3, world)
    t_wall = max_over_ranks(wall, world)
    total_rays = sum_over_ranks(float(rays_per_frame * steps), world)

    # the same frames through the plain path: one renderer per view size, one
    # RenderFrame per view
    plain = {}
    for sz in set(sizes):
        r1 = R.GPURayTracer(cm, sz[0], sz[1])
        r1.set_lod_voxel_size(cfg["lod"])
        r1.set_frame_time_limit(1e30)
        plain[sz] = r1
    for v in range(n):
        plain[sizes[v]].RenderFrame(mats[0][v])
    torch.cuda.synchronize()
    t = time.perf_counter()
    for f in range(args.warmup, frames):
        for v in range(n):
            plain[sizes[v]].RenderFrame(mats[f][v])
    torch.cuda.synchronize()
    t_plain = time.perf_counter() - t

    # roofline of the first pass over all views
    fetch = rt.count_fetches(mats[frames - 1])
    with roofline_range():
        pass_ms = rt.time_pass(mats[frames - 1], 3)
    alg_bytes = 4 * fetch["link_fetches"] + 4 * fetch["far_fetches"] + 16 * fetch["rays"]
    achieved = alg_bytes / (pass_ms / 1e3) / 1e9
    peak, peak_kind = hbm_peak()
    cpu = None
    if rank == 0:
        crays, cel, ck = cpu_frames(args.cpu_seconds)
        cpu = {"value": round(crays / cel / 1e6, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
               "sample": "%d frames of the 64 views (oracle, OpenMP)" % ck}
    if rank != 0:
        return None
    lat_sorted = np.sort(np.array(lat))
    return {
        "metric": metric, "value": round(total_rays / t_dev / 1e6, 3), "unit": "Mrays/s", "n_gpus": world,
        "steps": steps, "warmup": args.warmup, "ms_per_step": round(t_dev / steps * 1e3, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": wl, "views": n, "rays_per_frame": rays_per_frame, "depth": cfg["depth"],
                   "spheres": cfg["spheres"], "cache_blocks": cm.blocks()[1], "tree_blocks": ld.info.blocks_count,
                   "sizes": {"%dx%d" % k: sizes.count(k) for k in sorted(set(sizes))},
                   "launch_shape": list(shape), "autotune_s": round(tune_s, 2), "graphs": True,
                   "l2": "flushed between frames (256 MiB write)", "initial_fill_s": round(fill_s, 2),
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "e2e": {"value": round(total_rays / t_wall / 1e6, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 64 * 16 * 4,
                "d2h_bytes_per_step": rays_per_frame * 4},
        "frame_latency_ms": {"p50": round(float(np.percentile(lat_sorted, 50)), 4),
                             "p99": round(float(np.percentile(lat_sorted, 99)), 4)},
        "plain_per_view": {"value": round(rays_per_frame * steps / t_plain / 1e6, 3), "unit": "Mrays/s",
                           "note": "same frames, one RenderFrame per view (wall clock)"},
        "frames": {"passes_per_frame": round(passes / steps, 3)},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": None,
                     "traffic_rule": "not captured: the workload holds 6.8 GB on the device, beyond the size of a "
                                     "counter capture",
                     "peak_source": peak_kind, "kernel": "trace_kernel<first pass>, all 64 views", "launch_ms": round(pass_ms, 4),
                     "bytes_per_ray": round(alg_bytes / fetch["rays"], 2)},
        "cpu_baseline": cpu, "gpu_launches": int(launches), "clocks": clk}


def served_schedule(cfg):
    """C5: client sizes, per-client cameras and the merged Poisson arrival
    schedule [(t, client, frame index)] over cfg["seconds"]."""
    rng = np.random.default_rng(cfg["size_seed"])
    pick = rng.integers(0, len(cfg["sizes"]), size=cfg["clients"])
    sizes = [tuple(cfg["sizes"][k]) for k in pick]
    arr = np.random.default_rng(cfg["arrival_seed"])
    sched = []
    for c in range(cfg["clients"]):
        t, f = 0.0, 0
        while True:
            t += arr.exponential(1.0 / cfg["rate_hz"])
            if t >= cfg["seconds"]:
                break
            sched.append((t, c, f))
            f += 1
    sched.sort()
    return sizes, sched


def _pcts(lat_ms):
    a = np.sort(np.asarray(lat_ms, dtype=np.float64))
    return round(float(np.percentile(a, 50)), 3), round(float(np.percentile(a, 99)), 3)


def bench_served(args, rank, world, local):
    """C5: the served form (RenderServer: scheduler thread, continuous
    batching, shared cache) against the plain per-frame path (one
    GPURayTracer per client, RenderFrame per request in arrival order), on the
    same Poisson schedule (open loop: latency) and with every client keeping
    one frame outstanding (closed loop: throughput).  Every phase has a wall
    clock cap; progress goes to stderr."""
    import threading

    import torch

    import rayt_gb300 as R
    wl = args.workload
    cfg = WORKLOADS[wl]
    closed_frames = args.steps or cfg["closed_frames"]
    path = scene_path(wl, local, world)
    sizes, sched = served_schedule(cfg)
    nclients = cfg["clients"]
    frames_per_client = [1 + max([f for (_, c, f) in sched if c == cc] + [0]) for cc in range(nclients)]
    nframes = max(frames_per_client + [closed_frames + args.warmup]) + 1
    cams = [camera_path("c3", nframes, w, h, seed=cfg["size_seed"] + c) for c, (w, h) in enumerate(sizes)]
    pixels = [w * h for w, h in sizes]
    metric = "frames/s at 16 clients (served, continuous batching), depth 14" + (
        ", %d GiB cache (evicting)" % (cfg["cache_bytes"] >> 30) if wl == "c5p" else "")
    threads = os.cpu_count() or 1
    t_begin = time.time()

    def log(msg):
        sys.stderr.write("[c5 %7.1fs] %s\n" % (time.time() - t_begin, msg))
        sys.stderr.flush()

    def cpu_sample(budget):
        """The oracle on the schedule's requests of one client size, one after
        another, with a 32768-block cache (it streams like the reference)."""
        from oracle import oracle as O
        w, h = sizes[0]
        sc = O.OracleScene(path, 32768, w, h, cfg["lod"])
        el, k = 0.0, 0
        for (t, c, f) in sched:
            if sizes[c] != (w, h):
                continue
            tt = time.time()
            sc.render(cams[c][f])
            el += time.time() - tt
            k += 1
            if el > budget:
                break
        sc.close()
        return k, el

    if args.impl == "reference":
        if rank != 0:
            return None
        k, el = cpu_sample(args.cpu_seconds * 3)
        v = k / el
        return {"metric": metric, "value": round(v, 3), "unit": "frames/s", "impl": "reference", "n_gpus": 1,
                "steps": k, "warmup": 0, "ms_per_step": round(el / k * 1e3, 3), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": wl, "clients": nclients, "depth": cfg["depth"]},
                "cpu_baseline": {"value": round(v, 3), "unit": "frames/s", "cores": threads, "kind": "port",
                                 "sample": "%d %dx%d requests of the schedule (oracle, OpenMP)" % ((k,) + sizes[0])},
                "e2e": {"value": round(v, 3), "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}

    torch.cuda.set_device(local)
    log("scene ready")
    ld = R.StoredOctreeLoader(path)
    cm = R.GPUOctreeCacheManager(cache_blocks(cfg), ld)
    t0 = time.time()
    cm.InitialFillCache()
    fill_s = time.time() - t0
    loaded, cap_blocks = cm.blocks()
    log("initial fill %.1fs: %d of %d tree blocks in a %d-block cache" % (fill_s, loaded, ld.info.blocks_count,
                                                                          cap_blocks))
    fb_bytes = sum(((p + 63) // 64) * 64 * 4 for p in pixels) + (1 << 20)

    state = {"cm": cm}

    def fresh_cache():
        """Every timed phase starts from the same cache state: a new cache
        after InitialFillCache (the previous one is released first)."""
        state["cm"].close()
        c = R.GPUOctreeCacheManager(cache_blocks(cfg), ld)
        c.InitialFillCache()
        state["cm"] = c
        return c

    def make_server(deliver):
        srv = R.RenderServer(fresh_cache(), max_clients=nclients, framebuffer_bytes=fb_bytes,
                             max_rays_in_flight=sum(pixels), max_passes=cfg["max_passes"], lod_voxel_size=cfg["lod"],
                             deliver_to_host=deliver)
        ids = [srv.add_client(w, h) for w, h in sizes]
        return srv, ids

    def closed_served(srv, ids, first, frames, cap_s):
        """Closed loop: every client's frames first..first+frames-1 are queued
        at once; the server admits one request per client at a time, in order,
        so each client always has its next frame waiting and no host thread's
        wake-up sits between a client's frames.  Returns (frames, seconds)."""
        srv.start()
        t = time.perf_counter()
        reqs = [srv.submit(ids[c], cams[c][f]) for f in range(first, first + frames) for c in range(nclients)]
        done = 0
        for r in reqs:
            srv.wait(r, timeout=cap_s + 60)
            done += 1
        el = time.perf_counter() - t
        srv.stop()
        return done, el

    def served_closed(deliver):
        srv, ids = make_server(deliver)
        closed_served(srv, ids, 0, args.warmup, 60)
        n, el = closed_served(srv, ids, args.warmup, closed_frames, 60)
        st = srv.stats()
        srv.close()
        return n, el, st

    barrier(world)
    clocks = ClockSampler(local)
    clocks.start()
    n_served, el_served, st = served_closed(False)
    log("served closed loop: %d frames in %.3fs, %d ticks, %d blocks uploaded" % (n_served, el_served, st["ticks"],
                                                                                 st["uploaded_blocks"]))
    n_served_e2e, el_served_e2e, _ = served_closed(True)
    log("served closed loop, delivered to host: %d frames in %.3fs" % (n_served_e2e, el_served_e2e))
    # open loop: the Poisson schedule
    srv, ids = make_server(True)
    reqs = []
    srv.start()
    t_start = time.perf_counter()
    for (t, c, f) in sched:
        dt = t_start + t - time.perf_counter()
        if dt > 0:
            time.sleep(dt)
        reqs.append(srv.submit(ids[c], cams[c][f]))
    infos = [srv.wait(r, timeout=120) for r in reqs]
    srv.stop()
    sst = srv.stats()
    srv.close()
    lat_served = [(i["done_s"] - i["submit_s"]) * 1e3 for i in infos]
    span_served = max(i["done_s"] for i in infos) - min(i["submit_s"] for i in infos)
    log("served open loop: %d requests over %.3fs" % (len(infos), span_served))

    # plain per-frame path: one renderer per client on one cache
    pinned = [torch.empty((h, w, 4), dtype=torch.uint8).pin_memory() for w, h in sizes]
    rts = []

    def plain_renderers(deliver):
        """One renderer per client on a fresh cache; with deliver, each frame's
        image lands in the client's pinned buffer inside RenderFrame, as the
        server delivers (rayt_renderer_set_host_image)."""
        for rt in rts:
            rt.close()
        rts.clear()
        c = fresh_cache()
        for k, (w, h) in enumerate(sizes):
            rt = R.GPURayTracer(c, w, h)
            rt.set_lod_voxel_size(cfg["lod"])
            rt.set_frame_time_limit(1e30)
            rt.set_max_passes(cfg["max_passes"])
            if deliver:
                rt.set_host_image(pinned[k].data_ptr(), pinned[k].numel())
            rts.append(rt)
        return c

    def plain_frame(c, f):
        rts[c].RenderFrame(cams[c][f])

    def closed_plain(deliver, cap_s):
        """The same frames in the same order, one RenderFrame each, from the
        same cache state (fresh cache, the same warm-up frames)."""
        pc = plain_renderers(deliver)
        up0 = pc.stats()["uploaded_blocks"]
        for f in range(args.warmup):
            for c in range(nclients):
                plain_frame(c, f)
        torch.cuda.synchronize()
        n, t_end = 0, time.perf_counter() + cap_s
        up1 = pc.stats()["uploaded_blocks"]
        t = time.perf_counter()
        for f in range(args.warmup, args.warmup + closed_frames):
            if time.perf_counter() > t_end:
                break
            for c in range(nclients):
                plain_frame(c, f)
                n += 1
        torch.cuda.synchronize()
        return n, time.perf_counter() - t, pc.stats()["uploaded_blocks"] - up1

    n_plain, el_plain, up_plain = closed_plain(False, 60)
    n_plain_e2e, el_plain_e2e, _ = closed_plain(True, 60)
    log("plain closed loop: %d frames in %.3fs, %d blocks uploaded (%d in %.3fs delivered)"
        % (n_plain, el_plain, up_plain, n_plain_e2e, el_plain_e2e))
    plain_renderers(True)
    lat_plain = []
    t_start = time.perf_counter()
    for (t, c, f) in sched:
        dt = t_start + t - time.perf_counter()
        if dt > 0:
            time.sleep(dt)
        plain_frame(c, f)
        lat_plain.append((time.perf_counter() - (t_start + t)) * 1e3)
        if time.perf_counter() - t_start > 60:
            break
    span_plain = time.perf_counter() - t_start
    clk = clocks.stop()
    log("plain open loop: %d of %d requests in %.3fs" % (len(lat_plain), len(sched), span_plain))

    # roofline of the first pass on the largest client view
    big = max(range(nclients), key=lambda c: pixels[c])
    fetch = rts[big].count_fetches(cams[big][0])
    with roofline_range():
        pass_ms = rts[big].time_pass(cams[big][0], 3)
    alg_bytes = 4 * fetch["link_fetches"] + 4 * fetch["far_fetches"] + 16 * fetch["rays"]
    achieved = alg_bytes / (pass_ms / 1e3) / 1e9
    peak, peak_kind = hbm_peak()
    cpu = None
    if rank == 0:
        k, el = cpu_sample(args.cpu_seconds)
        cpu = {"value": round(k / el, 3), "unit": "frames/s", "cores": threads, "kind": "port",
               "sample": "%d %dx%d requests of the schedule (oracle, OpenMP)" % ((k,) + sizes[0])}
        log("cpu sample done")
    if rank != 0:
        return None
    sp50, sp99 = _pcts(lat_served)
    pp50, pp99 = _pcts(lat_plain)
    value = n_served / el_served
    mean_px = sum(pixels) / nclients
    return {
        "metric": metric, "value": round(value, 2), "unit": "frames/s", "n_gpus": world,
        "steps": n_served, "warmup": args.warmup, "ms_per_step": round(el_served / n_served * 1e3, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": wl, "clients": nclients, "depth": cfg["depth"], "spheres": cfg["spheres"],
                   "nodes_in_block": cfg["nib"],
                   "sizes": {"%dx%d" % k: sizes.count(k) for k in sorted(set(sizes))},
                   "rate_hz_per_client": cfg["rate_hz"], "schedule_s": cfg["seconds"], "requests": len(sched),
                   "cache_blocks": cap_blocks, "tree_blocks": ld.info.blocks_count, "blocks_loaded": loaded,
                   "max_passes": cfg["max_passes"], "initial_fill_s": round(fill_s, 2),
                   "l2": "inputs (the cache, GBs) larger than L2", "parallelism": "single GPU"},
        "e2e": {"value": round(n_served_e2e / el_served_e2e, 2), "unit": "frames/s", "h2d_bytes_per_step": 64,
                "d2h_bytes_per_step": int(mean_px * 4)},
        "served": {"closed_loop_frames_s": round(value, 2),
                   "closed_loop_mrays_s": round(n_served * mean_px / el_served / 1e6, 1),
                   "closed_loop_ticks": int(st["ticks"]),
                   "closed_loop_uploaded_blocks": int(st["uploaded_blocks"]),
                   "host_ms_per_tick": {k: round(st["host_ms_" + k] / max(1, st["ticks"]), 4)
                                        for k in ("wait", "lru", "load")},
                   "open_loop": {"offered_frames_s": round(len(sched) / cfg["seconds"], 1),
                                 "frames_s": round(len(infos) / span_served, 1), "p50_ms": sp50, "p99_ms": sp99,
                                 "passes_mean": round(float(np.mean([i["passes"] for i in infos])), 3),
                                 "truncated": int(sum(i["truncated"] for i in infos)),
                                 "ticks": int(sst["ticks"])}},
        "plain": {"closed_loop_frames_s": round(n_plain / el_plain, 2),
                  "closed_loop_e2e_frames_s": round(n_plain_e2e / el_plain_e2e, 2),
                  "closed_loop_uploaded_blocks": int(up_plain),
                  "closed_loop_mrays_s": round(n_plain * mean_px / el_plain / 1e6, 1),
                  "open_loop": {"frames_s": round(len(lat_plain) / span_plain, 1), "p50_ms": pp50, "p99_ms": pp99,
                                "served_requests": len(lat_plain)}},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": None,
                     "traffic_rule": "not captured: the workload holds 6-40 GiB on the device, beyond the size of a "
                                     "counter capture",
                     "peak_source": peak_kind, "kernel": "trace_kernel<first pass>, %dx%d client view" % sizes[big],
                     "launch_ms": round(pass_ms, 4), "bytes_per_ray": round(alg_bytes / fetch["rays"], 2)},
        "cpu_baseline": cpu, "gpu_launches": int(st["kernel_launches"]), "clocks": clk}


# ---------------------------------------------------------------------------
def zipf_words(n, seed=5, blocks=1 << 24, s=1.1):
    """C2 input: 90% NO_HIT, the rest block IDs ~ Zipf(s) over [0, blocks)
    (continuous inversion), half as fault words -id-1, half as hit words
    ((id+1)<<1)|dup."""
    rng = np.random.default_rng(seed)
    out = np.full(n, 0x7FFFFFFF, np.int32)
    m = n // 10
    idx = rng.choice(n, size=m, replace=False) if n <= (1 << 22) else rng.integers(0, n, size=m)
    u = rng.random(m)
    a = 1.0 - s
    ids = np.floor((1.0 + u * (blocks ** a - 1.0)) ** (1.0 / a)).astype(np.int64) - 1
    ids = np.clip(ids, 0, blocks - 1)
    fault = rng.random(m) < 0.5
    dup = rng.integers(0, 2, size=m)
    out[idx] = np.where(fault, -ids - 1, ((ids + 1) << 1) | dup).astype(np.int32)
    return out


def c2_path(words, nib):
    """(kept words, bitmap path taken, key span) of one feedback-unique call:
    the library takes the bitmap path when the kept keys (after NodeToBlock)
    span at most 32 values per input word and at most 2^26."""
    w = words[words != 0x7FFFFFFF].astype(np.int64)
    hit = w > 0
    w[hit] = ((((w[hit] >> 1) - 1) // nib + 1) << 1) | (w[hit] & 1)
    if w.size == 0:
        return 0, False, 0
    span = int(w.max() - w.min() + 1)
    cap = ((words.size * 4 + 16) // 16) * 16 * 8
    return int(w.size), span <= cap and span <= (1 << 26), span


def time_primitives(R, n, steps):
    """GPUSort and GPUScan (in place) on n uniform random int32, each call on a
    fresh copy of the input; CUDA events around the call only."""
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(13)
    src = torch.randint(-2**31, 2**31 - 1, (n,), dtype=torch.int32, device="cuda", generator=g)
    x = torch.empty_like(src)
    out = {}
    for name, fn in (("GPUSort", R.GPUSort), ("GPUScan", R.GPUScan)):
        ms = 0.0
        reps = max(3, min(steps, 10))
        for k in range(reps + 2):
            x.copy_(src)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn(x, n)
            e1.record()
            e1.synchronize()
            if k >= 2:
                ms += e0.elapsed_time(e1)
        ms /= reps
        out[name] = {"n": n, "ms": round(ms, 4), "gkeys_s": round(n / ms / 1e6, 2), "calls": reps,
                     "input": "uniform random int32, in place"}
    del src, x
    return out


def bench_c2(args, rank, world, local):
    import torch

    import rayt_gb300 as R
    n = 1 << args.c2_log2n
    steps = args.steps or 20
    wl = args.workload
    # c2r: block IDs over 2^28 instead of 2^24, so the kept keys span more than
    # 2^26 values and unique takes the LSD radix passes instead of the bitmap
    words = zipf_words(n, blocks=(1 << 28) if wl == "c2r" else (1 << 24))
    if args.impl == "reference":
        if rank != 0:
            return None
        from oracle import oracle as O
        sub = words[: 1 << 22]
        t = time.time()
        k = 0
        while time.time() - t < args.cpu_seconds and k < steps:
            O.feedback_unique(sub, 4096)
            k += 1
        el = (time.time() - t) / k
        v = sub.size / el / 1e9
        return {"metric": "Gkeys/s feedback compaction+sort+unique (2^%d words%s)" % (args.c2_log2n, ", radix path" if wl == "c2r" else ""), "value": round(v, 4),
                "unit": "Gkeys/s", "impl": "reference", "n_gpus": 1, "steps": k, "warmup": 0,
                "ms_per_step": round(el * 1e3, 3), "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "int32", "data": "synthetic",
                "config": {"workload": wl, "n": n, "sample_n": sub.size},
                "cpu_baseline": {"value": round(v, 4), "unit": "Gkeys/s", "cores": os.cpu_count() or 1, "kind": "port",
                                 "sample": "2^22 of the 2^28 words per step (merge sort + Hillis-Steele scan)"},
                "e2e": {"value": round(v, 4), "unit": "Gkeys/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    torch.cuda.set_device(local)
    d_words = torch.from_numpy(words).cuda()
    d_out = torch.empty(n, dtype=torch.int32, device="cuda")
    host_words = torch.from_numpy(words).pin_memory()
    for _ in range(args.warmup):
        R.feedback_unique(d_words, n, 4096, d_out)
    torch.cuda.synchronize()
    barrier(world)
    clocks = ClockSampler(local)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    cnt = 0
    for _ in range(steps):
        cnt = R.feedback_unique(d_words, n, 4096, d_out)
    e1.record()
    torch.cuda.synchronize()
    t_dev = max_over_ranks(e0.elapsed_time(e1) / 1e3, world)
    prims = time_primitives(R, n, steps)
    # end to end: words from pinned host memory, unique array back to host
    t = time.perf_counter()
    for _ in range(steps):
        d_words.copy_(host_words, non_blocking=True)
        c = R.feedback_unique(d_words, n, 4096, d_out)
        d_out[:c].cpu()
    t_e2e = max_over_ranks(time.perf_counter() - t, world)
    clk = clocks.stop()
    m, bitmap, span = c2_path(words, 4096)
    if bitmap:  # compaction, range histogram, partition, bucket bitmaps, bitmap clear/write/read, unique out
        alg = 4 * n + 4 * m + 4 * m + 8 * m + 4 * m + 3 * ((span + 31) // 32) * 4 + 4 * cnt
    else:  # compaction, four digit passes, unique
        alg = 4 * n + 4 * m + 32 * m + 4 * m + 4 * cnt
    achieved = alg / (t_dev / steps) / 1e9
    peak, kind = hbm_peak()
    if rank != 0:
        return None
    if bitmap:  # the bitmap path's profile was taken at 2^26 and scaled to 2^28 in the summary
        traffic, traffic_rule = (profile_traffic("sort_c2"), "profiled at 2^26 words, x4") if n == 1 << 28 else \
            (None, "no profile at this size")
    else:
        traffic, traffic_rule = scaled_traffic("sort_c2r", alg)
    # CPU baseline: the reference's merge sort + Hillis-Steele scan pipeline
    # (oracle) on a 2^22-word sample of the same words
    from oracle import oracle as O
    sub = words[: 1 << 22]
    t = time.time()
    k = 0
    while k < 1 or (time.time() - t < args.cpu_seconds and k < steps):
        O.feedback_unique(sub, 4096)
        k += 1
    cpu = {"value": round(sub.size * k / (time.time() - t) / 1e9, 4), "unit": "Gkeys/s", "cores": os.cpu_count() or 1,
           "kind": "port", "sample": "%d calls on 2^22 of the words (merge sort + Hillis-Steele scan)" % k}
    return {"metric": "Gkeys/s feedback compaction+sort+unique (2^%d words%s)" % (args.c2_log2n, ", radix path" if wl == "c2r" else ""),
            "value": round(sum_over_ranks(n * steps, world) / t_dev / 1e9, 4), "unit": "Gkeys/s", "n_gpus": world,
            "steps": steps, "warmup": args.warmup, "ms_per_step": round(t_dev / steps * 1e3, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
            "config": {"workload": wl, "n": n, "kept": m, "unique": cnt, "key_span": span,
                       "block_ids": (1 << 28) if wl == "c2r" else (1 << 24),
                       "l2": "inputs (%d MiB) larger than L2" % (4 * n >> 20) if 4 * n > (129 << 20) else "inputs in L2"},
            "e2e": {"value": round(n * steps / t_e2e / 1e9, 4), "unit": "Gkeys/s", "h2d_bytes_per_step": 4 * n,
                    "d2h_bytes_per_step": 4 * cnt},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": traffic, "traffic_rule": traffic_rule,
                         "peak_source": kind,
                         "kernel": ("compaction + range partition + bucket bitmaps + bitmap unique (one call)" if bitmap
                                    else "compaction + 4 digit passes + unique (one call)")},
            "cpu_baseline": cpu, "gpu_launches": steps * 12, "clocks": clk, "primitives": prims}


def main():
    args = parse()
    if args.impl == "reference":
        # the CPU arm: rank 0 alone runs it; other ranks exit without work
        if int(os.environ.get("RANK", "0")) != 0:
            return
        rank, world, local = 0, 1, 0
    else:
        rank, world, local = dist_setup(args.gpus)
    if args.workload in ("c2", "c2r"):
        out = bench_c2(args, rank, world, local)
    elif args.workload == "c4":
        out = bench_batched(args, rank, world, local)
    elif args.workload in ("c5", "c5p"):
        out = bench_served(args, rank, world, local)
    else:
        out = bench_frames(args, rank, world, local)
    if rank == 0 and out is not None:
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
