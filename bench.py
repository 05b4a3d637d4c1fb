"""Benchmark of the GB300 splat pipeline: one JSON line on stdout (per-leg details as one JSON line on stderr).

Headline workload -- the ragged batch: 64 lit views over 4 resident scenes (cornell-like 100k and 400k Gaussians,
seed 0; hill-like 1M and 2M, seed 1), each view's resolution drawn from 256^2, 512^2, 1280x720 and 1920x1080, its
camera on a sphere of radius U[3, 6] around the scene centre.  A step is one batch of those 64 views through the
batched path (sl_batch_render: one CUDA graph of the fused chain over every view).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

value      views/s of the batched path over all ranks (replicas), device time: CUDA events around each batch on the
           render stream, the L2 flushed (a 256 MiB write) before every batch outside the timed region, the scenes,
           their lighting maps and the views' frames resident in HBM.
e2e        the same through the public C ABI with host buffers: the views' frames, eyes and light scales staged from
           the host and every image written into page-locked host memory, wall clock per batch.
batched    on the same 64 views: the plain per-view path (per view the shading pass over every Gaussian of its scene,
           then project/sort/bin/composite: the reference's order) and the per-view deferred path (each view as a
           one-view batch: deferred shading without batching), views/s from the summed per-view device times, the
           ratios, and the largest image difference between the batched and the plain images.
served     Poisson arrivals over 6 resident scenes (50k..3M Gaussians) at 100, 500 and 2000 requests/s: views/s and
           p50/p99 latency (lambda 500 over the configured 60 s window, the others over --serve-seconds-other).
plain      the single-frame forward of the hill-like 1,048,576-Gaussian scene at 1920x1080 (lit) on the plain path.
sort       the stable 16-bit key sort alone on 2^26 keys, GB/s against the measured HBM peak.
roofline   the batched chain's dominant stage against its bound (per-stage device times measured live).
cpu_baseline  the CPU restatement of the reference pipeline (oracle/, kind "port") on this host's cores, on one view
           of each scene of the same mix.
--impl reference  that CPU restatement alone on the same workload, each step one view of the mix, all host threads
           (the reference's own WGSL needs WebGPU: unavailable on this machine).
Replicas only on N > 1: every rank renders its own batches, no collective on the data path.
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
# the plain per-view frame: shade; project, 2 depth-sort passes, binning (counts, offsets and entries in one pass),
# 2 tile-sort passes, ranges, composite
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
           "seconds": {"500": args.serve_seconds, "100 and 2000": args.serve_seconds_other}, "rates": []}
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
        window = args.serve_seconds if lam == 500 else args.serve_seconds_other
        n = max(1, int(lam * window))
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
        out["rates"].append({"lambda": lam, "seconds": window, "requests": n, "refused_at_admission": refused,
                             "failed": fails,
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
    per element 4 + 16 P (P passes; a key+value read and write per pass plus one key read for the histograms).  The
    library bars: CUB's DeviceRadixSort over the keys' own bits, and torch.sort over all 32 bits."""
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

    # CUB's DeviceRadixSort::SortPairs over the keys' own bits (end_bit 16 / 24), values = indices, as ours
    from splatlight_gb300 import build as B
    cub = C.CDLL(str(B.build_library_bar()))
    for fn_name in ("cub_sort_pairs16", "cub_sort_pairs32"):
        getattr(cub, fn_name).restype = C.c_int
        getattr(cub, fn_name).argtypes = [C.c_void_p] * 4 + [C.c_uint32, C.c_int, C.c_void_p,
                                                             C.POINTER(C.c_size_t), C.c_void_p]
    idx = torch.arange(n, dtype=torch.int32, device="cuda")
    k16o = torch.empty_like(k16h)
    k24o = torch.empty_like(k24)
    vo = torch.empty_like(idx)
    tb = C.c_size_t(0)
    cub.cub_sort_pairs16(None, None, None, None, n, 16, None, C.byref(tb), None)
    tb24 = C.c_size_t(0)
    cub.cub_sort_pairs32(None, None, None, None, n, 24, None, C.byref(tb24), None)
    temp = torch.empty(max(tb.value, tb24.value) + 256, dtype=torch.uint8, device="cuda")

    def cub16():
        t = C.c_size_t(tb.value)
        rc = cub.cub_sort_pairs16(k16h.data_ptr(), k16o.data_ptr(), idx.data_ptr(), vo.data_ptr(), n, 16,
                                  temp.data_ptr(), C.byref(t), C.c_void_p(sc))
        assert rc == 0, rc

    def cub24():
        t = C.c_size_t(tb24.value)
        rc = cub.cub_sort_pairs32(k24.data_ptr(), k24o.data_ptr(), idx.data_ptr(), vo.data_ptr(), n, 24,
                                  temp.data_ptr(), C.byref(t), C.c_void_p(sc))
        assert rc == 0, rc

    res = {"n": n, "peak_gbs": hbm, "peak_kind": peak_kind,
           "library_note": "cub_*: CUB DeviceRadixSort::SortPairs (the toolkit's onesweep) over bits [0, 16) / "
                           "[0, 24), values = indices; torch_*: torch.sort(stable) on the same values as int32 keys "
                           "(all 32 bits)"}
    for name, fn, passes in (("ours_16bit", ours16, 2), ("ours_24bit", ours24, 3), ("cub_16bit", cub16, 2),
                             ("cub_24bit", cub24, 3), ("torch_16bit", lib16, 2), ("torch_24bit", lib24, 3)):
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
    from splatlight_gb300 import camera
    out = torch.empty((s.height, s.width, 4), dtype=torch.float32, device="cuda")
    ref = torch.empty_like(out)

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

    def measure(eye, far):
        """One camera: the lit frame with the LOD cut against the same frame without it."""
        f0 = camera.make_frame(eye, s.target, s.up, s.fov_deg, s.width, s.height, s.count, far=far, view_mode=3,
                               n_emit=len(s.emitters))
        f = frame_lod(f0.copy(), threshold_px, N - G)

        def with_lod():
            L.shade(eye, stream=sc)
            lod.select(f, stream=sc)
            lod.colour(f, stream=sc)
            r.render(f, out=out, stream=sc)

        def without():
            L.shade(eye, stream=sc)
            r.render(f0, out=ref, stream=sc)

        def cut_only():
            lod.select(f, stream=sc)
            lod.colour(f, stream=sc)

        for _ in range(max(args.warmup, 3)):
            with_lod()
            without()
        torch.cuda.synchronize()
        steps = max(3, min(args.steps, 20))
        ms_l = timed(with_lod, steps)
        st = r.last_stats
        ms_p = timed(without, steps)
        ms_cut = timed(cut_only, steps)
        flags = lod.read()[0]
        return {"lod_views_per_s": round(1000.0 / ms_l, 2), "lod_ms_per_frame": round(ms_l, 4),
                "plain_views_per_s": round(1000.0 / ms_p, 2), "plain_ms_per_frame": round(ms_p, 4),
                "speedup_vs_plain": round(ms_p / ms_l, 3), "select_colour_ms": round(ms_cut, 4),
                "drawn_leaves": int((flags[:G] == DRAW).sum()), "drawn_nodes": int((flags[G:] == DRAW).sum()),
                "visible": int(st.visible), "entries": int(st.entries),
                "mean_abs_diff_vs_plain": round(float((out - ref).abs().mean().item()), 6)}

    res = {"workload": "hill-like 1,048,576 Gaussians, 1920x1080, lit; screen-space LOD at "
                       f"{threshold_px:g} px (projected-area rule) over a {N - G:,}-node moment-matched tree; the "
                       "reference camera, and the same view from 4x the distance (where the 2 px rule closes subtrees)"}
    res.update(measure(s.eye, s.far))
    e = np.asarray(s.eye, np.float64)
    t = np.asarray(s.target, np.float64)
    eye_far = tuple(np.float32(t + 4.0 * (e - t)))
    far = max(float(s.far), 4.0 * float(np.linalg.norm(e - t)) + 40.0)
    res["distant_view"] = measure(eye_far, far)
    res["tree_build_s"] = round(t_tree, 2)
    res["lod_create_s"] = round(t_create, 2)
    lod.close()
    L.close()
    r.close()
    return res


def run_bounce(args, stream, flush):
    """The probe bounce (the reference's path without the sender cut) on the headline workload (hill-like 1,048,576
    Gaussians, its moment-matched tree, the 16 x 16 x 5 terrain lattice with its sky): device time of one bounce frame
    (an update of a still scene is the shading pass plus the bounce; the shading pass alone is timed beside it), and
    the lit 1920x1080 frame with the bounce added (bounce gain 1) against the frame without it."""
    import torch
    from splatlight_gb300 import camera
    from splatlight_gb300 import probes as PR
    from splatlight_gb300 import scene as scn
    from splatlight_gb300.lighting import camera_forward, for_scene
    from splatlight_gb300.renderer import SplatRenderer
    s = scn.dataclasses.replace(make_scene("hill"), sky_ambient=0.0)
    t0 = time.perf_counter()
    s, tree = scn.with_tree(s)
    t_tree = time.perf_counter() - t0
    r = SplatRenderer(s.gaussians, s.parts)
    L = for_scene(r, s)
    L.set_tree(*tree)
    L.set_sky(s.sky_sh)
    lay = PR.for_scene(s)
    L.set_probes(lay)
    fwd = camera_forward(s)
    sc = stream.cuda_stream
    out = torch.empty((s.height, s.width, 4), dtype=torch.float32, device="cuda")

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

    fb = camera.make_frame(s.eye, s.target, s.up, s.fov_deg, s.width, s.height, s.count, far=s.far, view_mode=3,
                           n_emit=len(s.emitters), bounce_gain=1.0)
    f0 = camera.make_frame(s.eye, s.target, s.up, s.fov_deg, s.width, s.height, s.count, far=s.far, view_mode=3,
                           n_emit=len(s.emitters), bounce_gain=0.0)
    for _ in range(max(args.warmup, 3) + 4):   # the first updates fill the maps and settle the quarter refresh
        L.update(s.eye, fwd, stream=sc)
    torch.cuda.synchronize()
    steps = max(3, min(args.steps, 20))
    ms_update = timed(lambda: L.update(s.eye, fwd, stream=sc), steps)
    ms_shade = timed(lambda: L.shade(s.eye, stream=sc), steps)
    ms_frame_b = timed(lambda: (L.update(s.eye, fwd, stream=sc), r.render(fb, out=out, stream=sc)), steps)
    ms_frame_0 = timed(lambda: (L.shade(s.eye, stream=sc), r.render(f0, out=out, stream=sc)), steps)
    st = L.read_bounce()
    # the sender cut (the reference's default senders): a frame that selects the cut again (as after a part moved),
    # then the steady frames between, where a quarter of the cut refreshes
    t0 = time.perf_counter()
    L.set_sender_cut(True)
    t_sc = time.perf_counter() - t0
    torch.cuda.synchronize()
    ms_sc_select = timed(lambda: L.update(s.eye, fwd, stream=sc), 1) - ms_shade   # the first frame selects
    for _ in range(8):
        L.update(s.eye, fwd, stream=sc)
    torch.cuda.synchronize()
    ms_sc = timed(lambda: L.update(s.eye, fwd, stream=sc), steps) - ms_shade
    sst = L.read_bounce()
    fl = sst["sc_flag"]
    res_sc = {"bounce_ms": round(ms_sc, 4), "reselect_frame_ms": round(ms_sc_select, 4),
              "cut_nodes": int((fl[s.count:] == 2).sum()), "cut_leaves": int((fl[:s.count] == 3).sum()),
              "open_nodes": int((fl[s.count:] == 1).sum()), "setup_s": round(t_sc, 2),
              "mean_bounce_rgb": [round(float(v), 5) for v in sst["lo_b"][:, 0, :3].mean(axis=0)]}
    res = {"workload": f"hill-like 1,048,576 Gaussians (seed 1), its {len(tree[0]) - s.count:,}-node moment-matched "
                       f"tree, terrain lattice {lay['dims'][0]}x{lay['dims'][1]}x{lay['dims'][2]} probes x 128 cells "
                       "(ray length {:.1f} m), the scene's sky SH; bounce frame = direct light toward the probes for a "
                       "quarter of the Gaussians, tree sums and SH2, gather, validity, probe SH2, bounce_sh".format(
                           lay["tmax"]),
           "bounce_ms": round(ms_update - ms_shade, 4), "update_ms": round(ms_update, 4),
           "shade_ms": round(ms_shade, 4), "lit_frame_with_bounce_ms": round(ms_frame_b, 4),
           "lit_frame_without_bounce_ms": round(ms_frame_0, 4),
           "lit_views_per_s_with_bounce": round(1000.0 / ms_frame_b, 2),
           "probes": L.probe_count, "lattice_probes": int(np.prod(lay["dims"])),
           "valid_probes": int((st["probe_data"][:, 0, 6] > 0).sum()),
           "mean_bounce_rgb": [round(float(v), 5) for v in st["lo_b"][:, 0, :3].mean(axis=0)],
           "tree_build_s": round(t_tree, 2), "sender_cut": res_sc}
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
    # per-Gaussian state held constant: the scene's V grids, transmittance and iso_norm read as arrays
    state = {"vgrid": s.vgrid, "lamp_T": np.ones(s.count, np.float32), "iso_norm": np.ones(s.count, np.float32)}
    Pt, Lt = D.to_device(perturb(params, np.random.default_rng(2)), lights, state)
    target = D.forward(Pt, Lt, f, s.eye)
    P, Lt = D.to_device(params, lights, state)
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
    return {"workload": "500,000 hill-like Gaussians (seed 1), 800x800, lit by 8 emissive Gaussian lights over the "
                        "emitter tree's light cut (V grids, transmittance and iso_norm held constant); target from parameters "
                        "perturbed N(0,0.02) means / log-scales, N(0,0.1) opacity logits, N(0,0.05) albedo",
            "ms_per_step": round(ms, 3), "steps_per_s": round(1000.0 / ms, 2), "loss": loss,
            "grad_norms": {k: round(v, 6) for k, v in gnorm.items()}}


# bproject, scan of the blocks' visible counts, compaction of the visible keys, 3 depth-sort passes, binning (counts,
# offsets and entries in one pass), 2 tile-sort passes, runs (to ranges), coverage pass, shading list (one pass),
# bshade, bcomposite
BATCH_KERNELS = 14
STAGES = ("project", "depth_sort", "bin", "coverage", "shade", "composite")


def timed_device(stream, flush, fn, steps):
    """Median device time (ms) of fn() over `steps` calls, events on `stream`, the L2 flushed before each call."""
    import torch
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


def batch_world(n_views):
    """The headline workload's scenes (renderers + lightings, maps at each scene's reference camera) and views."""
    import torch
    from splatlight_gb300.batch import View
    from splatlight_gb300.lighting import camera_forward, for_scene
    from splatlight_gb300.renderer import SplatRenderer
    scenes, mix = batch_mix(n_views=n_views)
    rs, ls = [], []
    for s in scenes:
        r = SplatRenderer(s.gaussians, s.parts)
        L = for_scene(r, s)
        L.update(s.eye, camera_forward(s))   # the resident light state: maps at the scene's reference camera
        rs.append(r)
        ls.append(L)
    torch.cuda.synchronize()
    return scenes, mix, rs, ls, [View(k, f, e) for k, f, e in mix]


def stage_rooflines(st, ms, peak_hbm, fp32_peak, peak_kind):
    """Per stage of the batched chain: algorithmic work / its device time against the stage's bound.  Bytes per unit
    (reads + writes of the algorithm, no re-reads): projection 64 B record in, 48 B splat + 4 B key + 8 B rectangle out
    per slot; depth sort 4 + 3 x 16 B per visible slot (3 onesweep passes over key + value); binning per visible slot
    56 B read, per tile entry 8 B written + 2 x 16 B sorted + 8 B read for the runs; shading 336 B per shaded
    Gaussian; compositing 20 FP32 flops per blended fragment; the coverage pass 12 FP32 flops per blended fragment
    (its walk without colour)."""
    vis, ent, slots = float(st.visible), float(st.entries), float(st.slots)
    work = {"project": (124.0 * slots, "GB/s", peak_hbm, "hbm"),
            "depth_sort": (52.0 * vis, "GB/s", peak_hbm, "hbm"),
            "bin": (56.0 * vis + 48.0 * ent, "GB/s", peak_hbm, "hbm"),
            "coverage": (12.0 * float(st.fragments), "TFLOP/s", fp32_peak, "fp32 issue"),
            "shade": (336.0 * float(st.shaded), "GB/s", peak_hbm, "instruction issue"),
            "composite": (20.0 * float(st.fragments), "TFLOP/s", fp32_peak, "fp32 issue")}
    out = {}
    for k, (w, unit, peak, bound) in work.items():
        t = ms[k] * 1e-3
        ach = w / t / (1e9 if unit == "GB/s" else 1e12) if t > 0 else 0.0
        out[k] = {"ms": round(ms[k], 4), "bound": bound, "achieved": round(ach, 3), "unit": unit,
                  "peak": round(peak, 1), "frac": round(ach / peak, 4) if peak else None,
                  "peak_kind": peak_kind if unit == "GB/s" else "nominal FP32 issue rate at the sampled max SM clock",
                  "algorithmic_per_launch": w}
        if bound == "instruction issue":
            # the shading pass's cost is its per-light arithmetic (the footprint integrals, the SGGX and ASG lobes:
            # issue-bound under ncu); its bytes are reported against HBM only for the survey's 336 B per Gaussian
            out[k]["frac_of"] = "HBM (not the kernel's bound)"
    return out


def run_headline(args, stream, flush, dist, world, local):
    """The batched path on the 64-view mix (the bench's value), with its plain and per-view deferred arms."""
    import torch
    from splatlight_gb300.batch import BatchRenderer
    scenes, mix, rs, ls, views = batch_world(args.batch_views)
    n = len(views)
    sizes = [(int(f["viewport"][1]), int(f["viewport"][0])) for _, f, _ in mix]
    pix = sum(h * w for h, w in sizes)
    B = BatchRenderer(rs, ls, max_views=n)
    out = torch.empty(4 * pix, dtype=torch.float32, device="cuda")
    tile, tune_ms = B.autotune(views, reps=2)
    blocks_per_sm = B.tuning()[1]
    sc = stream.cuda_stream

    def batched():
        return B.render_device(views, out=out, stream=sc)

    for _ in range(args.warmup):
        batched()
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            starts[k].record(stream)
            batched()
            ends[k].record(stream)
        torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    batch_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    ms = max_over_ranks(sum(batch_ms) / len(batch_ms), dist, "cuda")
    st = B.last_stats
    stats = {k: getattr(st, k) for k in ("slots", "visible", "entries", "fragments", "shaded", "reshaded_views",
                                         "max_radiance",
                                         "graph_replayed")}

    # per-stage device times (the same chain launched kernel by kernel with events between the stages)
    B.set_timing(2)
    per = {k: [] for k in STAGES}
    for _ in range(3):
        with torch.cuda.stream(stream):
            flush.zero_()
        batched()
        for k, v in zip(STAGES, B.last_stats.ms_stage):
            per[k].append(v)
    B.set_timing(0)
    stage_ms = {k: statistics.median(v) for k, v in per.items()}

    # the plain per-view path on the same views: the shading pass over every Gaussian of the view's scene at its eye,
    # then the frame; per-view device times summed (host gaps between views excluded), the L2 flushed per round
    plain_out = [torch.empty((h, w, 4), dtype=torch.float32, device="cuda") for h, w in sizes]

    def plain_round():
        evs = []
        with torch.cuda.stream(stream):
            flush.zero_()
        for (k, f, e), o in zip(mix, plain_out):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            ls[k].shade(e, stream=sc)
            rs[k].render(f, out=o, stream=sc)
            b.record(stream)
            evs.append((a, b))
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in evs)

    plain_round()
    plain_ms = statistics.median([plain_round() for _ in range(3)])
    # image difference, batched vs plain (the same light state)
    _, offs = batched()
    torch.cuda.synchronize()
    err = 0.0
    for (h, w), o, po in zip(sizes, offs, plain_out):
        err = max(err, float((out[int(o):int(o) + 4 * h * w].view(h, w, 4) - po).abs().max().item()))

    # the per-view deferred path: each view as a one-view batch
    B1 = BatchRenderer(rs, ls, max_views=1)
    B1.set_tile(*tile)
    one = [torch.empty(4 * h * w, dtype=torch.float32, device="cuda") for h, w in sizes]

    def deferred_round():
        evs = []
        with torch.cuda.stream(stream):
            flush.zero_()
        for v, o in zip(views, one):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            B1.render_device([v], out=o, stream=sc)
            b.record(stream)
            evs.append((a, b))
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in evs)

    deferred_round()
    deferred_ms = statistics.median([deferred_round() for _ in range(3)])
    B1.close()

    # end to end through the C ABI with host buffers: images written into page-locked host memory by the compositor
    host = torch.empty(4 * pix, dtype=torch.float32, pin_memory=True)
    for _ in range(2):
        B.render_device(views, out=host, stream=sc)
    if dist is not None:
        dist.barrier()
    t0 = time.perf_counter()
    e2e_steps = max(3, min(args.steps, 10))
    for _ in range(e2e_steps):
        B.render_device(views, out=host, stream=sc)
    e2e_s = max_over_ranks((time.perf_counter() - t0) / e2e_steps, dist, "cuda")
    e2e_err = float((host.to("cuda") - out).abs().max().item())
    h2d = n * (1200 + 4 + 12 + 4)         # per view: RenderFrame, scene index, eye, light scale
    d2h = 16 * pix
    del host
    B.close()
    for L in ls:
        L.close()
    for r in rs:
        r.close()
    return {"ms": ms, "views": n, "pixels": pix, "value": world * n * 1000.0 / ms, "clocks": clk.summary(),
            "stage_ms": stage_ms, "stats": stats, "tile": tile, "autotune_ms": tune_ms, "blocks_per_sm": blocks_per_sm,
            "plain_ms": plain_ms, "deferred_ms": deferred_ms, "max_abs_err_vs_plain": err,
            "e2e": {"value": round(world * n / e2e_s, 2), "unit": "views/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)}, "e2e_image_matches_device": e2e_err == 0.0,
            "scenes": scenes, "mix": mix}


def run_plain(args, stream, flush, dist, world):
    """The single-frame forward of the hill-like 1,048,576-Gaussian scene at 1920x1080, lit, on the plain per-view
    path: views/s (device time), e2e through the public API with a pinned host image, per-stage times, and the shading,
    sort and composite rooflines."""
    import torch
    from splatlight_gb300.lighting import camera_forward, for_scene
    from splatlight_gb300.renderer import SplatRenderer
    s = make_scene("hill")
    W, H = s.width, s.height
    f = frame_for(s, 3)
    r = SplatRenderer(s.gaussians, s.parts)
    L = for_scene(r, s)
    fwd = camera_forward(s)
    sc = stream.cuda_stream
    L.update(s.eye, fwd, stream=sc)
    out = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")

    def step():
        L.update(s.eye, fwd, stream=sc)    # the shading pass (the maps hold while nothing moves)
        r.render(f, out=out, stream=sc)

    for _ in range(args.warmup):
        step()
    ms = timed_device(stream, flush, step, max(5, min(args.steps, 20)))
    ms = max_over_ranks(ms, dist, "cuda")
    stats = r.last_stats
    r.set_timing(True)
    stage = {"lighting": [], "project": [], "sort": [], "bin": [], "composite": []}
    frags = []
    for _ in range(max(5, min(args.steps, 20))):
        with torch.cuda.stream(stream):
            flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        L.update(s.eye, fwd, stream=sc)
        e1.record(stream)
        r.render(f, out=out, stream=sc)
        stage["lighting"].append(e0.elapsed_time(e1))
        st = r.last_stats
        for k, v in (("project", st.ms_project), ("sort", st.ms_sort), ("bin", st.ms_bin),
                     ("composite", st.ms_composite)):
            stage[k].append(v)
        frags.append(st.fragments)
    r.set_timing(False)
    stage_ms = {k: statistics.median(v) for k, v in stage.items()}
    host_out = torch.empty((H, W, 4), dtype=torch.float32, pin_memory=True).numpy()
    parts = s.parts.copy()
    for _ in range(2):
        r.write_parts(parts)
        L.update(s.eye, fwd)
        r.render(f, out=host_out)
    t0 = time.perf_counter()
    n_e2e = max(5, min(args.steps, 20))
    for _ in range(n_e2e):
        r.write_parts(parts)
        L.update(s.eye, fwd)
        r.render(f, out=host_out)
    e2e_s = max_over_ranks((time.perf_counter() - t0) / n_e2e, dist, "cuda")
    all_parts = (1 << len(s.parts)) - 1
    maps = []
    for _ in range(5):
        with torch.cuda.stream(stream):
            flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        L.update(s.eye, fwd, moved_mask=all_parts, stream=sc)
        e1.record(stream)
        e1.synchronize()
        maps.append(e0.elapsed_time(e1))
    L.close()
    r.close()
    return {"s": s, "ms": ms, "views_per_s": world * 1000.0 / ms, "stage_ms": stage_ms,
            "fragments": statistics.median(frags), "slots": int(stats.slots), "visible": int(stats.visible),
            "entries": int(stats.entries), "e2e_views_per_s": world / e2e_s,
            "update_every_part_moved_ms": statistics.median(maps)}


def cpu_view_seconds(scenes, mix, caches, view, threads):
    """One view of the mix on the CPU restatement: the shading pass over every Gaussian of its scene at the view's eye
    (the scene's opacity maps from `caches`, as on the GPU) and the frame (project, sort, bin, composite)."""
    from oracle import oracle
    k, f, eye = mix[view]
    s = scenes[k]
    t0 = time.perf_counter()
    tgt = np.asarray(s.target, np.float64)
    colour, _, _, _ = oracle.lighting(s, eye=np.asarray(eye, np.float64), target=tgt, threads=threads,
                                      cached=caches[k])
    oracle.render(s.gaussians, s.parts, f, emitters=s.emitters, colour=colour, threads=threads, want_entries=False)
    return time.perf_counter() - t0


def cpu_caches(scenes, threads):
    """iso_init and every scene's opacity maps at its reference camera, computed once (untimed)."""
    return [cpu_cache(s, threads) for s in scenes]


def headline_desc(n_views):
    return (f"ragged batch: {n_views} lit views over 4 resident scenes (cornell-like 100k and 400k Gaussians, seed 0; "
            "hill-like 1,048,576 and 2,097,152, seed 1), resolutions from 256^2, 512^2, 1280x720, 1920x1080, cameras "
            "on radius U[3,6] spheres; one step = one batch through the batched path (one CUDA graph)")


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle
    oracle.build()
    threads = os.cpu_count() or 1
    scenes, mix = batch_mix(n_views=args.batch_views)
    caches = cpu_caches(scenes, threads)
    for k in range(args.warmup):
        cpu_view_seconds(scenes, mix, caches, k % len(mix), threads)
    times = [cpu_view_seconds(scenes, mix, caches, (args.warmup + k) % len(mix), threads) for k in range(args.steps)]
    ms = 1000.0 * sum(times) / len(times)
    v = 1000.0 / ms
    line = {"impl": "reference", "metric": "views/s", "value": round(v, 4), "unit": "views/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": headline_desc(args.batch_views),
                       "implementation": "CPU restatement of the reference pipeline in the reference's order (per "
                                         "view: the shading pass over the scene, then project, sort, bin, composite);"
                                         " the reference's WGSL needs WebGPU: unavailable on this box"},
            "cpu_baseline": {"value": round(v, 4), "unit": "views/s", "cores": threads, "kind": "port",
                             "sample": f"each step one view of the 64-view mix, in mix order ({args.steps} views)"},
            "e2e": {"value": round(v, 4), "unit": "views/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--batch-views", type=int, default=64, help="views of the ragged batch (the config: 64)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving leg")
    ap.add_argument("--no-plain", action="store_true", help="skip the single-frame plain leg")
    ap.add_argument("--no-lod", action="store_true", help="skip the screen-space LOD leg")
    ap.add_argument("--no-diff", action="store_true", help="skip the differentiation leg")
    ap.add_argument("--no-sort", action="store_true", help="skip the sort leg")
    ap.add_argument("--only-serve", action="store_true", help="the serving leg alone (its own JSON line)")
    ap.add_argument("--only-diff", action="store_true", help="the differentiation leg alone (its own JSON line)")
    ap.add_argument("--only-sort", action="store_true", help="the sort leg alone (its own JSON line)")
    ap.add_argument("--only-lod", action="store_true", help="the screen-space LOD leg alone (its own JSON line)")
    ap.add_argument("--only-plain", action="store_true", help="the single-frame plain leg alone (its own JSON line)")
    ap.add_argument("--only-bounce", action="store_true", help="the probe-bounce leg alone (its own JSON line)")
    ap.add_argument("--no-bounce", action="store_true", help="skip the probe-bounce leg")
    ap.add_argument("--sort-n", type=int, default=1 << 26, help="keys for the sort leg")
    ap.add_argument("--serve-seconds", type=float, default=60.0, help="arrival window at lambda 500 (the config: 60)")
    ap.add_argument("--serve-seconds-other", type=float, default=10.0, help="arrival window at lambda 100 and 2000")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        run_reference(args)
        return

    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    __import__("__graft_entry__").build()
    stream = torch.cuda.Stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    hbm, sm_max_cfg, peak_kind = peaks()

    def emit(line):
        if rank == 0:
            print(json.dumps(line), flush=True)

    if args.only_sort:
        res = run_sort(args, stream, flush, args.sort_n)
        emit({"metric": "sort GB/s", "value": res["ours_16bit"]["gbs"], "unit": "GB/s", "n_gpus": world, "sort": res})
        return
    if args.only_lod:
        res = run_lod(args, stream, flush)
        emit({"metric": "views/s", "value": res["lod_views_per_s"], "unit": "views/s", "n_gpus": world, "lod": res})
        return
    if args.only_bounce:
        res = run_bounce(args, stream, flush)
        emit({"metric": "bounce frame ms", "value": res["bounce_ms"], "unit": "ms", "higher_is_better": False,
              "n_gpus": world, "bounce": res})
        return
    if args.only_diff:
        res = run_diff(args, stream, flush)
        emit({"metric": "inverse-rendering steps/s", "value": res["steps_per_s"], "unit": "steps/s",
              "n_gpus": world, "differentiation": res})
        return
    if args.only_serve:
        res = run_serving(args)
        emit({"metric": "views/s", "value": max(x["views_per_s"] for x in res["rates"]), "unit": "views/s",
              "n_gpus": world, "serving": res})
        return
    if args.only_plain:
        res = run_plain(args, stream, flush, dist, world)
        res.pop("s")
        emit({"metric": "views/s", "value": round(res["views_per_s"], 2), "unit": "views/s", "n_gpus": world,
              "plain": {k: (round(v, 4) if isinstance(v, float) else v) for k, v in res.items()}})
        return

    hd = run_headline(args, stream, flush, dist, world, local)
    clocks = hd["clocks"]
    sm_mhz = clocks["sm_max_mhz"] or sm_max_cfg
    fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
    roofs = stage_rooflines(type("S", (), hd["stats"])(), hd["stage_ms"], hbm, fp32_peak, peak_kind)
    dom = max(hd["stage_ms"], key=hd["stage_ms"].get)
    kernel = {"project": "bproject_kernel", "depth_sort": "onesweep_pass x3 (depth keys)",
              "bin": "btile_bin_kernel + onesweep_pass x2 (tile ids) + btile_runs_kernel",
              "coverage": "bmark_kernel", "shade": "bshade_kernel", "composite": "bcomposite_kernel"}[dom]
    r = roofs[dom]
    roofline = {"bound": r["bound"], "achieved": r["achieved"], "peak": r["peak"], "unit": r["unit"],
                "frac": r["frac"], "traffic": None, "peak_kind": r["peak_kind"], "kernel": kernel,
                "algorithmic_per_launch": r["algorithmic_per_launch"]}
    n = hd["views"]
    plain_vps = world * n * 1000.0 / hd["plain_ms"]
    deferred_vps = world * n * 1000.0 / hd["deferred_ms"]
    batched = {"views_per_s": round(hd["value"], 2), "plain_views_per_s": round(plain_vps, 2),
               "x_vs_plain": round(hd["value"] / plain_vps, 3),
               "per_view_deferred_views_per_s": round(deferred_vps, 2),
               "x_vs_per_view_deferred": round(hd["value"] / deferred_vps, 3),
               "max_abs_err_vs_plain": round(hd["max_abs_err_vs_plain"], 6)}

    detail = {"headline": {"stage_ms": {k: round(v, 4) for k, v in hd["stage_ms"].items()}, "stage_rooflines": roofs,
                           "stats": hd["stats"], "tile": f"{hd['tile'][0]}x{hd['tile'][1]}",
                           "autotune_ms": {k: round(v, 3) for k, v in hd["autotune_ms"].items()},
                           "tuned_blocks_per_sm": hd["blocks_per_sm"],
                           "e2e_image_matches_device": hd["e2e_image_matches_device"]}}
    plain = None
    if not args.no_plain:
        p = run_plain(args, stream, flush, dist, world)
        sm = p["stage_ms"]
        comp_tf = 20.0 * p["fragments"] / (sm["composite"] * 1e-3) / 1e12
        sort_gbs = 18.0 * p["slots"] / (sm["sort"] * 1e-3) / 1e9
        plain = {"views_per_s": round(p["views_per_s"], 2), "e2e_views_per_s": round(p["e2e_views_per_s"], 2),
                 "lighting_ms": round(sm["lighting"], 4)}
        detail["plain"] = {"workload": workload_desc(p["s"]), "stage_ms": {k: round(v, 4) for k, v in sm.items()},
                           "slots": p["slots"], "visible": p["visible"], "entries": p["entries"],
                           "composite_tflops": round(comp_tf, 3), "composite_frac_fp32": round(comp_tf / fp32_peak, 4),
                           "depth_sort_gbs": round(sort_gbs, 1),
                           "update_every_part_moved_ms": round(p["update_every_part_moved_ms"], 4)}
    served = None
    if not args.no_serve:
        sv = run_serving(args)
        detail["serving"] = sv
        served = {str(x["lambda"]): {"views_per_s": x["views_per_s"], "p50_ms": x["p50_ms"], "p99_ms": x["p99_ms"],
                                     "s": x["seconds"]} for x in sv["rates"]}
        served["plain_views_per_s"] = sv["plain_per_view_views_per_s"]
        served["x_vs_plain"] = sv["served_vs_plain"]
    sort_c = None
    if not args.no_sort:
        so = run_sort(args, stream, flush, args.sort_n)
        detail["sort"] = so
        sort_c = {"gbs": so["ours_16bit"]["gbs"], "frac": so["ours_16bit"]["frac"], "n": so["n"]}
    if not args.no_lod:
        detail["lod"] = run_lod(args, stream, flush)
    if not args.no_diff:
        detail["differentiation"] = run_diff(args, stream, flush)
    if not args.no_bounce:
        detail["bounce"] = run_bounce(args, stream, flush)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        scenes, mix = hd["scenes"], hd["mix"]
        caches = cpu_caches(scenes, threads)
        pick = [next(v for v, (k, _, _) in enumerate(mix) if k == s) for s in range(len(scenes))]
        sec = sum(cpu_view_seconds(scenes, mix, caches, v, threads) for v in pick)
        cpu = {"value": round(len(pick) / sec, 4), "unit": "views/s", "cores": threads, "kind": "port",
               "sample": "the first view of each of the 4 scenes in the mix (per view: the shading pass over the "
                         "scene, then project, sort, bin, composite)"}

    if rank == 0:
        sys.stderr.write(json.dumps(detail, default=float) + "\n")
        line = {"metric": "views/s", "value": round(hd["value"], 2), "unit": "views/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(hd["ms"], 4),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded scene generators)",
                "config": {"workload": headline_desc(n), "parallelism": f"replicas x{world}",
                           "l2": "flushed (256 MiB write) before every timed batch",
                           "pixels_per_step": hd["pixels"], "tile": f"{hd['tile'][0]}x{hd['tile'][1]}"},
                "gpu_launches": BATCH_KERNELS * args.steps, "e2e": hd["e2e"], "roofline": roofline,
                "cpu_baseline": cpu, "clocks": clocks,
                "stage_ms": {k: round(v, 3) for k, v in hd["stage_ms"].items()},
                "plain_1m_1080p": plain, "sort": sort_c, "served": served, "batched": batched}
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
