"""Benchmark of the GB300 splat pipeline (one JSON line on stdout).

Workload (default): the hill-like scene of 1,048,576 Gaussians (seed 1) rendered at 1920x1080, fov 50 deg -- the
plain single-frame forward configuration.  A step is one frame of the plain per-view path through the C ABI:
project -> onesweep depth sort -> tile binning (+ tile sort, ranges) -> front-to-back composite, lit view.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--config hill|cornell] [--impl ours|reference]

value      views/s over all ranks, device time: CUDA events around each frame on the render stream, the L2 flushed
           (a 256 MiB write) between frames outside the timed region, inputs resident in HBM.
e2e        the same metric through the public API with host buffers: each step uploads the frame's RenderFrame and
           part records and reads the W x H x 4 fp32 image back into pinned host memory, wall clock.
roofline   the dominant kernel (by device time) against its bound; the sort is reported beside it against HBM.
cpu_baseline  the CPU restatement (oracle/, a port of the reference algorithm) timed on this host's cores (rank 0).
--impl reference  the CPU restatement of the reference pipeline alone (the reference's WGSL needs WebGPU, which is
           not available on this machine), all host threads, each step one full frame of the same workload.
Replicas only on N > 1: every rank renders its own frames, no collective on the data path.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

MEASURED = ROOT / "MEASURED_PEAKS.json"
FALLBACK_HBM = 6800.0  # GB/s
# shade; project, 2 depth-sort passes, binning (counts, offsets and entries in one pass), 2 tile-sort passes, ranges,
# composite
KERNELS_PER_FRAME = 9
# DRAM bytes per Gaussian of one shade_kernel launch (read + write), from ncu on the 1,048,576-Gaussian frame
SHADE_DRAM_BYTES_PER_G = (464.748544e6 + 22.484992e6) / 1048576


def max_over_ranks(value: float, dist, device: str) -> float:
    """The slowest rank's time (replicas: every rank renders its own frames; the job takes as long as the slowest)."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replicas_throughput(world: int, ms_per_step: float) -> float:
    """Whole-job views/s: each of the world ranks finishes one view per step of the slowest rank."""
    return world * 1000.0 / ms_per_step


def peaks():
    if MEASURED.exists():
        m = json.loads(MEASURED.read_text())
        return float(m["hbm_gbs"]), float(m.get("sm_max_mhz", 2070.0)), "measured"
    return FALLBACK_HBM, 2070.0, "fallback"


class ClockSampler:
    """nvidia-smi clock and throttle-reason samples every 200 ms while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_scene(name):
    from splatlight_gb300 import scene
    return scene.hill() if name == "hill" else scene.cornell()


def frame_for(s, view_mode):
    from splatlight_gb300 import camera
    return camera.make_frame(s.eye, s.target, s.up, s.fov_deg, s.width, s.height, s.count, far=s.far,
                             view_mode=view_mode, n_emit=len(s.emitters))


def workload_desc(s):
    sun = f", sun with {s.sun_res}^2 maps, sky ambient {s.sky_ambient:g}" if s.sun is not None else ""
    return (f"{s.name}: {s.count:,} Gaussians + {len(s.emitters)} emitters ({s.shadow_res}^2 light map){sun}, "
            f"{s.width}x{s.height}, fov {s.fov_deg:g} deg, lit view; plain per-view path, per frame the lighting pass "
            f"(opacity maps cached: static scene) + project/sort/bin/composite")


def cpu_frame_seconds(s, cache, threads):
    """One full frame of the CPU restatement on `threads` host threads: the lighting pass (shade_emit + env_direct;
    the opacity maps of the static scene come from `cache`, as on the GPU) then project, sort, bin, composite."""
    from oracle import oracle
    f = frame_for(s, 3)
    t0 = time.perf_counter()
    colour, _, _, _ = oracle.lighting(s, threads=threads, cached=cache)
    oracle.render(s.gaussians, s.parts, f, emitters=s.emitters, colour=colour, threads=threads, want_entries=False)
    return time.perf_counter() - t0


def cpu_cache(s, threads):
    """iso_init and the opacity maps of the static scene, computed once (untimed)."""
    from oracle import oracle
    _, lamp_t, env_t, nodes = oracle.lighting(s, threads=threads)
    return lamp_t, env_t, nodes


MIX_RES = [(256, 256), (512, 512), (1280, 720), (1920, 1080)]


def batch_mix(n_views=64, seed=7):
    """The ragged batch workload: 4 scenes (cornell-like 100k and 400k Gaussians, seed 0; hill-like 1M and 2M, seed
    1), n_views views round-robin over them, each with a resolution drawn from MIX_RES and a camera on a sphere of
    radius U[3, 6] around the scene centre looking at it, lit view."""
    from splatlight_gb300 import camera, scene
    scenes = [scene.cornell(100_000, seed=0), scene.cornell(400_000, seed=0), scene.hill(1_048_576, seed=1),
              scene.hill(2_097_152, seed=1)]
    rng = np.random.default_rng(seed)
    views = []
    for v in range(n_views):
        k = v % len(scenes)
        s = scenes[k]
        W, H = MIX_RES[int(rng.integers(len(MIX_RES)))]
        up = np.asarray(s.up, np.float64)
        while True:
            d = rng.normal(size=3)
            d /= np.linalg.norm(d)
            if abs(float(d @ up)) < 0.95:
                break
        c = np.asarray(s.target, np.float64)
        eye = c + rng.uniform(3.0, 6.0) * d
        f = camera.make_frame(tuple(eye), tuple(c), s.up, s.fov_deg, W, H, s.count, far=s.far, view_mode=3,
                              n_emit=len(s.emitters))
        views.append((k, f, tuple(np.float32(eye))))
    return scenes, views


def run_batch(args, stream, flush):
    """Batched path vs the plain per-view path on the ragged 64-view mix (device time, L2 flushed between steps)."""
    import torch
    from splatlight_gb300.batch import BatchRenderer, View
    from splatlight_gb300.lighting import camera_forward, for_scene
    from splatlight_gb300.renderer import SplatRenderer
    scenes, mix = batch_mix(n_views=args.batch_views)
    rs, ls = [], []
    for s in scenes:
        r = SplatRenderer(s.gaussians, s.parts)
        L = for_scene(r, s)
        L.update(s.eye, camera_forward(s))   # the resident light state: maps at the scene's reference camera
        rs.append(r)
        ls.append(L)
    torch.cuda.synchronize()
    views = [View(k, f, e) for k, f, e in mix]
    sizes = [(int(f["viewport"][1]), int(f["viewport"][0])) for _, f, _ in mix]
    pix = sum(h * w for h, w in sizes)
    B = BatchRenderer(rs, ls, max_views=len(views))
    out = torch.empty(4 * pix, dtype=torch.float32, device="cuda")
    tile, tune_ms = B.autotune(views, reps=2)
    sc = stream.cuda_stream

    def batched():
        return B.render_device(views, out=out, stream=sc)

    plain_out = [torch.empty((h, w, 4), dtype=torch.float32, device="cuda") for h, w in sizes]

    def plain():
        for (k, f, e), o in zip(mix, plain_out):
            ls[k].shade(e, stream=sc)
            rs[k].render(f, out=o, stream=sc)

    def timed(fn, steps):
        ts = []
        for _ in range(steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            b.synchronize()
            ts.append(a.elapsed_time(b))
        return statistics.median(ts)

    for _ in range(max(args.warmup, 3)):
        batched()
        plain()
    torch.cuda.synchronize()
    steps = max(3, min(args.steps, 10))
    ms_b = timed(batched, steps)
    st = B.last_stats
    ms_p = timed(plain, steps)
    # image error of every batched view against the plain per-view path (same light state)
    _, offs = batched()
    torch.cuda.synchronize()
    err = 0.0
    for (h, w), o, po in zip(sizes, offs, plain_out):
        img = out[int(o):int(o) + 4 * h * w].view(h, w, 4)
        err = max(err, float((img - po).abs().max().item()))
    n = len(views)
    res = {"workload": f"{n} lit views over 4 resident scenes (cornell-like 100k, 400k; hill-like 1M, 2M "
                       "Gaussians), resolutions from 256^2, 512^2, 1280x720, 1920x1080, cameras on radius U[3,6] "
                       "spheres; light maps resident per scene",
           "views": n, "pixels": pix, "batched_views_per_s": round(n * 1000.0 / ms_b, 2),
           "batched_ms_per_batch": round(ms_b, 3),
           "plain_views_per_s": round(n * 1000.0 / ms_p, 2), "plain_ms_per_batch": round(ms_p, 3),
           "speedup_vs_plain": round(ms_p / ms_b, 3), "max_abs_err_vs_plain": err,
           "tile": f"{tile[0]}x{tile[1]}", "autotune_ms": {k: round(v, 3) for k, v in tune_ms.items()},
           "slots": int(st.slots), "visible": int(st.visible), "entries": int(st.entries),
           "shaded": int(st.shaded), "reshaded_views": int(st.reshaded_views),
           "max_radiance": round(float(st.max_radiance), 4),
           "graph_replayed": int(st.graph_replayed), "kernels_per_batch": BATCH_KERNELS}
    B.close()
    for L in ls:
        L.close()
    for r in rs:
        r.close()
    return res


SERVE_RES = [(512, 512), (1280, 720), (1920, 1080)]


def serve_scenes():
    """The 6 resident scenes of the serving workload: hill-like, 50k .. 3M Gaussians, seeds 10-15."""
    from splatlight_gb300 import scene
    counts = [50_000, 200_000, 500_000, 1_048_576, 2_097_152, 3_145_728]
    return [scene.hill(n, seed=10 + k) for k, n in enumerate(counts)]


def run_serving(args, rates=(100, 500, 2000)):
    """Poisson arrivals at each rate for --serve-seconds: each request names one of 6 resident scenes, a camera on a
    radius-U[3,8] sphere around the scene centre, a resolution from SERVE_RES and a light scale in U[0.5, 2]; the
    server batches continuously (2 pipelines); latency = result on the host - arrival, wall clock, as the caller's
    polling thread sees it, and beside it the server's own (its completion - its submit, on its clock)."""
    import threading

    import torch
    from splatlight_gb300 import camera
    from splatlight_gb300.lighting import camera_forward, for_scene
    from splatlight_gb300.renderer import SplatRenderer
    from splatlight_gb300._native import SplatlightError
    from splatlight_gb300.server import RenderServer
    scenes = serve_scenes()
    rs, ls = [], []
    for s in scenes:
        r = SplatRenderer(s.gaussians, s.parts)
        L = for_scene(r, s)
        L.update(s.eye, camera_forward(s))
        rs.append(r)
        ls.append(L)
    torch.cuda.synchronize()
    rng = np.random.default_rng(42)

    def request():
        k = int(rng.integers(len(scenes)))
        s = scenes[k]
        W, H = SERVE_RES[int(rng.integers(len(SERVE_RES)))]
        up = np.asarray(s.up, np.float64)
        while True:
            d = rng.normal(size=3)
            d /= np.linalg.norm(d)
            if abs(float(d @ up)) < 0.95:
                break
        c = np.asarray(s.target, np.float64)
        eye = tuple(np.float32(c + rng.uniform(3.0, 8.0) * d))
        f = camera.make_frame(eye, tuple(c), s.up, s.fov_deg, W, H, s.count, far=s.far, view_mode=3,
                              n_emit=len(s.emitters))
        return k, f, eye, float(rng.uniform(0.5, 2.0))

    out = {"workload": "Poisson arrivals over 6 resident hill-like scenes (50k, 200k, 500k, 1M, 2M, 3M Gaussians, "
                       "seeds 10-15), cameras on radius U[3,8] spheres, 512^2 / 1280x720 / 1920x1080, light scale "
                       "U[0.5,2], lit; images delivered to pinned host memory",
           "seconds_per_rate": args.serve_seconds, "rates": []}
    # the pending queue is bounded (512 requests, a few batches' worth): beyond it a request is refused at submit,
    # which keeps the latency of admitted requests bounded when arrivals outrun the device
    srv = RenderServer(rs, ls, max_views=64, pipelines=2, max_slots=48 << 20, max_pixels=24 << 20,
                       max_tiles=1 << 19, result_slots=96, max_pending=512)
    # warm-up: capture the graphs, size the entry buffers
    for k in range(16):
        q = request()
        srv.submit(*q, tag=k)
    got = 0
    while got < 16:
        got += len(srv.poll(wait_us=50000, copy=False))
    # and a paced run (gaps of 0.2-5 ms), so both pipelines capture the graphs of the small capacity classes that
    # single requests and small bursts use before any latency is measured
    for k in range(96):
        srv.submit(*request(), tag=16 + k)
        time.sleep(float(rng.uniform(0.0002, 0.005)))
    while got < 16 + 96:
        got += len(srv.poll(wait_us=50000, copy=False))
    for lam in rates:
        n = max(1, int(lam * args.serve_seconds))
        gaps = rng.exponential(1.0 / lam, size=n)
        reqs = [request() for _ in range(n)]
        arrivals = {}
        done = []
        refused = 0
        stop = threading.Event()

        deadline = [None]

        def poller():
            while not stop.is_set() or len(done) < n - refused:
                for r in srv.poll(wait_us=2000, copy=False):
                    done.append((r.tag, time.perf_counter(), r.status, r.batch_views,
                                 (r.t_done - r.t_submit) * 1000.0))
                if stop.is_set() and len(done) >= n - refused:
                    break
                if deadline[0] is not None and time.perf_counter() > deadline[0]:
                    break

        st0 = srv.stats()
        th = threading.Thread(target=poller)
        th.start()
        t0 = time.perf_counter()
        t_next = t0
        for i, q in enumerate(reqs):
            t_next += gaps[i]
            while True:
                dt = t_next - time.perf_counter()
                if dt <= 0:
                    break
                time.sleep(min(dt, 0.0005))
            arrivals[i] = time.perf_counter()
            try:
                srv.submit(*q, tag=i)
            except SplatlightError as e:
                if e.code != -7:
                    raise
                refused += 1
        t_sub = time.perf_counter()
        deadline[0] = t_sub + 300.0
        stop.set()
        th.join()
        t_end = max(t for _, t, _, _, _ in done)
        lat = np.array([(t - arrivals[tag]) * 1000.0 for tag, t, st, _, _ in done if st == 0])
        lat_srv = np.array([ms for _, _, st, _, ms in done if st == 0])
        fails = sum(1 for _, _, st, _, _ in done if st != 0)
        n_adm = n - refused
        st1 = srv.stats()
        d_batches = st1["batches"] - st0["batches"]
        out["rates"].append({"lambda": lam, "requests": n, "refused_at_admission": refused, "failed": fails,
                             "batches": d_batches,
                             "graph_captures": d_batches - (st1["graph_replays"] - st0["graph_replays"]),
                             "relaunches": st1["relaunches"] - st0["relaunches"],
                             "unfinished": n_adm - len(done),
                             "offered_per_s": round(n / (t_sub - t0), 1),
                             "views_per_s": round(len(done) / (t_end - t0), 1),
                             "p50_ms": round(float(np.percentile(lat, 50)), 2),
                             "p99_ms": round(float(np.percentile(lat, 99)), 2),
                             "server_p50_ms": round(float(np.percentile(lat_srv, 50)), 2),
                             "server_p99_ms": round(float(np.percentile(lat_srv, 99)), 2),
                             "mean_batch": round(float(np.mean([b for _, _, _, b, _ in done])), 1)})
    st = srv.stats()
    out["device_bytes"] = st["device_bytes"]
    out["batches"] = st["batches"]
    out["reshaded_views"] = st["reshaded_views"]
    out["relaunches"] = st["relaunches"]
    srv.close()
    # the plain per-view path on a sample of the same requests, one at a time (the shading pass at the request's eye
    # and the frame; the light scale, a change of light state for the per-view path, is left at 1 there)
    import torch
    sample = [request() for _ in range(128)]
    outs = {}
    for k, f, eye, _ in sample:
        W, H = int(f["viewport"][0]), int(f["viewport"][1])
        outs.setdefault((W, H), torch.empty((H, W, 4), dtype=torch.float32, device="cuda"))
    for k, f, eye, _ in sample[:8]:
        ls[k].shade(eye)
        rs[k].render(f, out=outs[(int(f["viewport"][0]), int(f["viewport"][1]))])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k, f, eye, _ in sample:
        ls[k].shade(eye)
        rs[k].render(f, out=outs[(int(f["viewport"][0]), int(f["viewport"][1]))])
    torch.cuda.synchronize()
    out["plain_per_view_views_per_s"] = round(len(sample) / (time.perf_counter() - t0), 1)
    best = max(x["views_per_s"] for x in out["rates"])
    out["served_vs_plain"] = round(best / out["plain_per_view_views_per_s"], 3)
    for L in ls:
        L.close()
    for r in rs:
        r.close()
    return out


def run_sort(args, stream, flush, n=1 << 26):
    """The stable radix sort alone on n random keys: 16-bit (2 passes, sl_sort_keys16) and 24-bit segmented-style
    32-bit keys (3 passes, sl_sort_keys32), device time per call (digit histograms + passes + scratch clears), against
    the library sort (torch.sort, stable: CUB's radix sort) on the same keys.  Bandwidth uses the algorithmic bytes
    per element 4 + 16 P (P passes; a key+value read and write per pass plus one key read for the histograms)."""
    import ctypes as C

    import torch
    from splatlight_gb300 import _native as N
    lib = N.lib()
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    k16 = torch.randint(0, 65536, (n,), device="cuda", dtype=torch.int32, generator=g)
    k16h = k16.to(torch.int16)    # the same values as u16 bits
    k24 = torch.randint(0, 1 << 24, (n,), device="cuda", dtype=torch.int32, generator=g)
    order = torch.empty(n, dtype=torch.int32, device="cuda")
    sc = stream.cuda_stream
    hbm, _, peak_kind = peaks()

    def timed(fn, reps):
        ts = []
        for _ in range(reps):
            with torch.cuda.stream(stream):
                flush.zero_()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            b.synchronize()
            ts.append(a.elapsed_time(b))
        return statistics.median(ts)

    def ours16():
        N.check(lib.sl_sort_keys16(k16h.data_ptr(), n, order.data_ptr(), C.c_void_p(sc)))

    def ours24():
        N.check(lib.sl_sort_keys32(k24.data_ptr(), n, 24, order.data_ptr(), C.c_void_p(sc)))

    def lib16():
        with torch.cuda.stream(stream):
            torch.sort(k16, stable=True)

    def lib24():
        with torch.cuda.stream(stream):
            torch.sort(k24, stable=True)

    res = {"n": n, "peak_gbs": hbm, "peak_kind": peak_kind,
           "library_note": "torch.sort(stable) on the same values as int32 keys (no bit-range control: all 32 bits)"}
    for name, fn, passes in (("ours_16bit", ours16, 2), ("ours_24bit", ours24, 3), ("library_16bit", lib16, 2),
                             ("library_24bit", lib24, 3)):
        for _ in range(3):
            fn()
        ms = timed(fn, 5)
        b = (4 + 16 * passes) * n
        res[name] = {"ms": round(ms, 4), "gbs": round(b / (ms * 1e-3) / 1e9, 1),
                     "frac": round(b / (ms * 1e-3) / 1e9 / hbm, 4), "bytes_per_elem": 4 + 16 * passes}
    return res


def run_lod(args, stream, flush, threshold_px: float = 2.0):
    """The headline workload (hill-like 1,048,576 Gaussians, 1920x1080, lit) with the reference's default screen-space
    LOD (2 px, projected-area rule) over a moment-matched tree of the scene (scene.lod_tree, built once, untimed):
    per frame the shading pass, the cut (sl_lod_select), the drawn nodes' colours (sl_lod_colour) and the frame,
    against the same frames without LOD (device time, L2 flushed between frames)."""
    import torch
    from splatlight_gb300 import scene as scn
    from splatlight_gb300.lighting import camera_forward, for_scene
    from splatlight_gb300.lod import DRAW, Lod, frame_lod
    from splatlight_gb300.renderer import SplatRenderer
    s = make_scene("hill")
    t0 = time.perf_counter()
    nodes, kids, parts = scn.lod_tree(s.gaussians, s.parts)
    t_tree = time.perf_counter() - t0
    s = scn.dataclasses.replace(s, parts=parts)
    r = SplatRenderer(s.gaussians, s.parts)
    L = for_scene(r, s)
    fwd = camera_forward(s)
    sc = stream.cuda_stream
    L.update(s.eye, fwd, stream=sc)
    t0 = time.perf_counter()
    lod = Lod(r, nodes, kids)
    t_create = time.perf_counter() - t0
    G, N = len(s.gaussians), len(nodes)
    f0 = frame_for(s, 3)
    f = frame_lod(f0.copy(), threshold_px, N - G)
    out = torch.empty((s.height, s.width, 4), dtype=torch.float32, device="cuda")
    ref = torch.empty_like(out)

    def with_lod():
        L.shade(s.eye, stream=sc)
        lod.select(f, stream=sc)
        lod.colour(f, stream=sc)
        r.render(f, out=out, stream=sc)

    def without():
        L.shade(s.eye, stream=sc)
        r.render(f0, out=ref, stream=sc)

    def timed(fn, steps):
        ts = []
        for _ in range(steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            b.synchronize()
            ts.append(a.elapsed_time(b))
        return statistics.median(ts)

    for _ in range(max(args.warmup, 3)):
        with_lod()
        without()
    torch.cuda.synchronize()
    steps = max(3, min(args.steps, 20))
    ms_l = timed(with_lod, steps)
    st = r.last_stats
    ms_p = timed(without, steps)

    def cut_only():
        lod.select(f, stream=sc)
        lod.colour(f, stream=sc)

    ms_cut = timed(cut_only, steps)
    flags = lod.read()[0]
    res = {"workload": "hill-like 1,048,576 Gaussians, 1920x1080, lit; screen-space LOD at "
                       f"{threshold_px:g} px (projected-area rule) over a {N - G:,}-node moment-matched tree",
           "lod_views_per_s": round(1000.0 / ms_l, 2), "lod_ms_per_frame": round(ms_l, 4),
           "plain_views_per_s": round(1000.0 / ms_p, 2), "plain_ms_per_frame": round(ms_p, 4),
           "speedup_vs_plain": round(ms_p / ms_l, 3), "select_colour_ms": round(ms_cut, 4),
           "drawn_leaves": int((flags[:G] == DRAW).sum()), "drawn_nodes": int((flags[G:] == DRAW).sum()),
           "visible": int(st.visible), "entries": int(st.entries),
           "mean_abs_diff_vs_plain": round(float((out - ref).abs().mean().item()), 6),
           "tree_build_s": round(t_tree, 2), "lod_create_s": round(t_create, 2)}
    lod.close()
    L.close()
    r.close()
    return res


def run_diff(args, stream, flush):
    """Inverse-rendering steps (forward + L2 loss + hand-written backward) on 500k hill-like Gaussians at 800x800
    against a target rendered from perturbed parameters; device time per step, L2 flushed between steps."""
    import torch
    from splatlight_gb300 import camera, scene
    from splatlight_gb300.diff import DiffRenderer, params_from_scene, perturb
    s = scene.hill(500_000, seed=1)
    params, lights = params_from_scene(s, n_lights=8)
    f = camera.make_frame(s.eye, s.target, s.up, s.fov_deg, 800, 800, s.count, far=s.far, view_mode=3, n_emit=0)
    D = DiffRenderer(s.count)
    Pt, Lt = D.to_device(perturb(params, np.random.default_rng(2)), lights)
    target = D.forward(Pt, Lt, f, s.eye)
    P, Lt = D.to_device(params, lights)
    sc = stream.cuda_stream
    for _ in range(max(args.warmup, 3)):
        with torch.cuda.stream(stream):
            D.step(P, Lt, f, s.eye, target, stream=sc)
    ts = []
    loss = 0.0
    for _ in range(max(3, min(args.steps, 10))):
        with torch.cuda.stream(stream):
            flush.zero_()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        loss, G, _ = D.step(P, Lt, f, s.eye, target, stream=sc)
        b.record(stream)
        b.synchronize()
        ts.append(a.elapsed_time(b))
    ms = statistics.median(ts)
    gnorm = {k: float(v.norm().item()) for k, v in G.items()}
    D.close()
    return {"workload": "500,000 hill-like Gaussians (seed 1), 800x800, 8 point lights; target from parameters "
                        "perturbed N(0,0.02) means / log-scales, N(0,0.1) opacity logits, N(0,0.05) albedo",
            "ms_per_step": round(ms, 3), "steps_per_s": round(1000.0 / ms, 2), "loss": loss,
            "grad_norms": {k: round(v, 6) for k, v in gnorm.items()}}


# bproject, scan and compaction of the visible keys, 3 depth-sort passes, binning (counts, offsets and entries in one
# pass), 2 tile-sort passes, runs (to ranges), coverage pass, shading list (one pass), bshade, bcomposite
BATCH_KERNELS = 14


def deferred_one_view(args, s, r, L, f, fwd, plain_out, flush, stream):
    """The same lit frame through the batch API as a batch of one view: projection, sort and binning first, then only
    the Gaussians the coverage pass marks are shaded (deferred shading) before the composite.  Device time per view,
    L2 flushed between views, and the largest image difference from the plain path's frame (same light state)."""
    import torch
    from splatlight_gb300.batch import BatchRenderer, View
    H, W = int(f["viewport"][1]), int(f["viewport"][0])
    B = BatchRenderer([r], [L], max_views=1)
    views = [View(0, f, s.eye)]
    out = torch.empty(4 * W * H, dtype=torch.float32, device="cuda")
    sc = stream.cuda_stream
    for _ in range(max(args.warmup, 3)):
        B.render_device(views, out=out, stream=sc)
    ts = []
    for _ in range(max(5, min(args.steps, 20))):
        with torch.cuda.stream(stream):
            flush.zero_()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        B.render_device(views, out=out, stream=sc)
        b.record(stream)
        b.synchronize()
        ts.append(a.elapsed_time(b))
    st = B.last_stats
    ms = statistics.median(ts)
    L.update(s.eye, fwd, stream=sc)
    r.render(f, out=plain_out, stream=sc)
    torch.cuda.synchronize()
    err = float((out.view(H, W, 4) - plain_out).abs().max().item())
    B.close()
    return {"workload": "the same frame as a batch of one view (sl_batch_render)", "views_per_s": round(1000.0 / ms, 2),
            "ms_per_view": round(ms, 4), "max_abs_err_vs_plain": err, "visible": int(st.visible),
            "shaded": int(st.shaded), "reshaded_views": int(st.reshaded_views)}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle
    oracle.build()
    s = make_scene(args.config)
    threads = os.cpu_count() or 1
    cache = cpu_cache(s, threads)
    t_warm = cpu_frame_seconds(s, cache, threads)
    # bounded: at most ~90 s of CPU frames whatever --steps asks (each step is one full frame)
    n_run = max(1, min(args.steps, int(90.0 / max(t_warm, 1e-3))))
    times = [cpu_frame_seconds(s, cache, threads) for _ in range(n_run)]
    ms = 1000.0 * sum(times) / len(times)
    v = 1000.0 / ms
    line = {"impl": "reference", "metric": "views/s", "value": round(v, 4), "unit": "views/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": workload_desc(s), "implementation": "CPU restatement of the reference pipeline "
                       "(the reference's WGSL needs WebGPU: unavailable on this box)"},
            "cpu_baseline": {"value": round(v, 4), "unit": "views/s", "cores": threads, "kind": "port",
                             "sample": f"{n_run} full frames of the workload (bounded to ~90 s)"},
            "e2e": {"value": round(v, 4), "unit": "views/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--config", default="hill", choices=["hill", "cornell"])
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the ragged-batch leg")
    ap.add_argument("--only-batch", action="store_true", help="the ragged-batch leg alone (its own JSON line)")
    ap.add_argument("--only-serve", action="store_true", help="the serving leg alone (its own JSON line)")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving leg")
    ap.add_argument("--only-diff", action="store_true", help="the differentiation leg alone (its own JSON line)")
    ap.add_argument("--only-sort", action="store_true", help="the sort leg alone (its own JSON line)")
    ap.add_argument("--only-lod", action="store_true", help="the screen-space LOD leg alone (its own JSON line)")
    ap.add_argument("--batch-views", type=int, default=64, help="views of the ragged batch (the config: 64)")
    ap.add_argument("--no-lod", action="store_true", help="skip the screen-space LOD leg")
    ap.add_argument("--sort-n", type=int, default=1 << 26, help="keys for the sort leg")
    ap.add_argument("--no-diff", action="store_true", help="skip the differentiation leg")
    ap.add_argument("--serve-seconds", type=float, default=4.0, help="arrival window per rate (the config: 60)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    args.warmup = max(args.warmup, 3)

    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    __import__("__graft_entry__").build()
    from splatlight_gb300.renderer import SplatRenderer

    if args.only_sort:
        stream = torch.cuda.Stream()
        flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
        res = run_sort(args, stream, flush, args.sort_n)
        if rank == 0:
            print(json.dumps({"metric": "sort GB/s", "value": res["ours_24bit"]["gbs"], "unit": "GB/s",
                              "n_gpus": world, "sort": res}))
        return
    if args.only_lod:
        stream = torch.cuda.Stream()
        flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
        res = run_lod(args, stream, flush)
        if rank == 0:
            print(json.dumps({"metric": "views/s", "value": res["lod_views_per_s"], "unit": "views/s",
                              "n_gpus": world, "lod": res}))
        return
    if args.only_diff:
        stream = torch.cuda.Stream()
        flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
        res = run_diff(args, stream, flush)
        if rank == 0:
            print(json.dumps({"metric": "inverse-rendering steps/s", "value": res["steps_per_s"], "unit": "steps/s",
                              "n_gpus": world, "differentiation": res}))
        return
    if args.only_serve:
        res = run_serving(args)
        if rank == 0:
            best = max(res["rates"], key=lambda x: x["views_per_s"])
            print(json.dumps({"metric": "views/s", "value": best["views_per_s"], "unit": "views/s",
                              "n_gpus": world, "serving": res}))
        return
    if args.only_batch:
        stream = torch.cuda.Stream()
        flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
        res = run_batch(args, stream, flush)
        if rank == 0:
            print(json.dumps({"metric": "views/s", "value": res["batched_views_per_s"], "unit": "views/s",
                              "n_gpus": world, "batched": res}))
        return

    from splatlight_gb300.lighting import camera_forward, for_scene

    s = make_scene(args.config)
    W, H = s.width, s.height
    f = frame_for(s, 3)
    r = SplatRenderer(s.gaussians, s.parts)
    L = for_scene(r, s)           # emitters, sun, sky; binds the radiance buffer the projection reads
    fwd = camera_forward(s)
    stream = torch.cuda.Stream()
    L.update(s.eye, fwd, stream=stream.cuda_stream)   # first update: iso_init + opacity maps (static scene)
    torch.cuda.synchronize()

    def step(out_buf):
        # one frame: the lighting pass (shade_emit + env_direct; the maps hold while nothing moves) and the render
        L.update(s.eye, fwd, stream=stream.cuda_stream)
        return r.render(f, out=out_buf, stream=stream.cuda_stream)

    out = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    # warm-up (also sizes the tile-entry buffers)
    for _ in range(args.warmup):
        step(out)

    # device-timed steps
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    barrier()
    with ClockSampler(local) as clk:
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                flush.zero_()
                starts[k].record(stream)
                step(out)
                ends[k].record(stream)
        torch.cuda.synchronize()
    barrier()
    step_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    ms = sum(step_ms) / len(step_ms)
    ms = max_over_ranks(ms, dist, "cuda")
    views_per_s = replicas_throughput(world, ms)
    stats = r.last_stats
    if not np.isfinite(out.sum().item()):
        raise RuntimeError("non-finite image")

    # per-stage device times (events inside the pipeline), for the rooflines
    r.set_timing(True)
    stage = {"lighting": [], "project": [], "sort": [], "bin": [], "composite": []}
    frags = []
    for _ in range(max(5, min(args.steps, 20))):
        with torch.cuda.stream(stream):
            flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        L.update(s.eye, fwd, stream=stream.cuda_stream)
        e1.record(stream)
        r.render(f, out=out, stream=stream.cuda_stream)
        stage["lighting"].append(e0.elapsed_time(e1))
        st = r.last_stats
        stage["project"].append(st.ms_project)
        stage["sort"].append(st.ms_sort)
        stage["bin"].append(st.ms_bin)
        stage["composite"].append(st.ms_composite)
        frags.append(st.fragments)
    r.set_timing(False)
    stage_ms = {k: statistics.median(v) for k, v in stage.items()}

    # the opacity maps rebuilt as when every part moved (light map A re-splatted, every sun layer re-splatted, then
    # the shading pass): the per-frame lighting cost of a scene whose parts all move
    all_parts = (1 << len(s.parts)) - 1
    maps = []
    for _ in range(5):
        with torch.cuda.stream(stream):
            flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        L.update(s.eye, fwd, moved_mask=all_parts, stream=stream.cuda_stream)
        e1.record(stream)
        e1.synchronize()
        maps.append(e0.elapsed_time(e1))
    L.update(s.eye, fwd, stream=stream.cuda_stream)
    deferred = deferred_one_view(args, s, r, L, f, fwd, out, flush, stream)
    lighting_maps = {"update_every_part_moved_ms": round(statistics.median(maps), 4),
                     "shading_pass_only_ms": round(stage_ms["lighting"], 4),
                     "maps": f"light map A {s.shadow_res}^2 per part ({len(s.parts)} parts), sun layers {s.sun_res}^2"}

    # end to end through the public API with host buffers: frame + parts up, image down (pinned), wall clock
    host_out = torch.empty((H, W, 4), dtype=torch.float32, pin_memory=True)
    host_out_np = host_out.numpy()
    parts = s.parts.copy()
    for _ in range(2):
        r.write_parts(parts)
        L.update(s.eye, fwd)
        r.render(f, out=host_out_np)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r.write_parts(parts)
        L.update(s.eye, fwd)
        r.render(f, out=host_out_np)
    e2e_s = (time.perf_counter() - t0) / args.steps
    e2e_s = max_over_ranks(e2e_s, dist, "cuda")
    h2d = f.nbytes + parts.nbytes
    d2h = W * H * 16

    hbm, sm_max_cfg, peak_kind = peaks()
    clocks = clk.summary()
    sm_mhz = clocks["sm_max_mhz"] or sm_max_cfg
    # sort: 2 onesweep passes over u16 keys + u32 values: (2 + 6) + (6 + 4) bytes per slot
    sort_bytes = 18.0 * stats.slots
    sort_gbs = sort_bytes / (stage_ms["sort"] * 1e-3) / 1e9
    # composite: 20 FP32 flops per blended fragment (local coordinates 4, q 2, tests 3, alpha 4, blend 7), nominal
    # FP32 issue peak = 152 SMs x 128 lanes x 2 flops x clock
    fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
    frag = statistics.median(frags)
    comp_tflops = 20.0 * frag / (stage_ms["composite"] * 1e-3) / 1e12
    roof_sort = {"bound": "hbm", "achieved": round(sort_gbs, 1), "peak": hbm, "unit": "GB/s",
                 "frac": round(sort_gbs / hbm, 4), "traffic": None, "peak_kind": peak_kind,
                 "algorithmic_bytes_per_launch": sort_bytes, "kernel": "onesweep_pass x2 (depth keys)"}
    roof_comp = {"bound": "fp32", "achieved": round(comp_tflops, 3), "peak": round(fp32_peak, 1), "unit": "TFLOP/s",
                 "frac": round(comp_tflops / fp32_peak, 4), "traffic": None,
                 "peak_kind": "nominal FP32 issue rate at the sampled max SM clock (no measured FP32 peak exists)",
                 "algorithmic_flops_per_launch": 20.0 * frag, "kernel": "composite_kernel<16>"}
    # shading pass (the lighting stage in steady state): 336 algorithmic bytes per Gaussian (record 64, leaf node 96,
    # V grid 128, lamp T 16, env T 16 in; radiance 16 out); its DRAM traffic per Gaussian from one ncu capture of the
    # kernel on this frame (487 MB for 1,048,576 Gaussians); it is issue-bound (same capture)
    shade_bytes = 336.0 * s.count
    shade_gbs = shade_bytes / (stage_ms["lighting"] * 1e-3) / 1e9
    roof_shade = {"bound": "hbm", "achieved": round(shade_gbs, 1), "peak": hbm, "unit": "GB/s",
                  "frac": round(shade_gbs / hbm, 4), "traffic": round(SHADE_DRAM_BYTES_PER_G * s.count),
                  "peak_kind": peak_kind, "algorithmic_bytes_per_launch": shade_bytes,
                  "kernel": "shade_kernel (issue-bound: 73% issue active, FMA pipe 51% in ncu; HBM 5%)"}
    dominant = max(stage_ms, key=stage_ms.get)
    roofline = {"composite": roof_comp, "lighting": roof_shade}.get(dominant, roof_sort)

    batch = None
    if not args.no_batch:
        batch = run_batch(args, stream, flush)
    serving = None
    if not args.no_serve:
        serving = run_serving(args)
    differentiation = None
    if not args.no_diff:
        differentiation = run_diff(args, stream, flush)
    sort_leg = run_sort(args, stream, flush)
    lod_leg = None
    if not args.no_lod:
        lod_leg = run_lod(args, stream, flush)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        sec = cpu_frame_seconds(s, cpu_cache(s, threads), threads)
        cpu = {"value": round(1.0 / sec, 4), "unit": "views/s", "cores": threads, "kind": "port",
               "sample": "1 full frame of the same workload (lighting pass, project, sort, bin, composite)"}

    if rank == 0:
        line = {"metric": "views/s", "value": round(views_per_s, 2), "unit": "views/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": workload_desc(s), "parallelism": f"replicas x{world}",
                           "l2": "flushed (256 MiB write) between timed frames", "tile": "16x16",
                           "slots": int(stats.slots), "visible": int(stats.visible), "entries": int(stats.entries)},
                "e2e": {"value": round(world / e2e_s, 2), "unit": "views/s", "h2d_bytes_per_step": int(h2d),
                        "d2h_bytes_per_step": int(d2h)},
                "gpu_launches": KERNELS_PER_FRAME * args.steps,
                "stage_ms": {k: round(v, 4) for k, v in stage_ms.items()},
                "roofline": roofline, "sort_roofline": roof_sort, "composite_roofline": roof_comp,
                "shade_roofline": roof_shade,
                "cpu_baseline": cpu, "clocks": clocks, "batched": batch, "serving": serving,
                "differentiation": differentiation, "sort": sort_leg, "lod": lod_leg, "lighting_maps": lighting_maps,
                "deferred_one_view": deferred}
        print(json.dumps(line))
    L.close()
    r.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
