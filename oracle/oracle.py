"""ctypes wrapper and build recipe of the CPU restatement (oracle/*.c).  TEST INFRASTRUCTURE: imported only by tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg, as the checker -- never by the product.

The C sources compile with gcc -O2 -ffp-contract=off (fp32 arithmetic in written order, no fused multiply-add except
where the source calls fmaf), -fopenmp for the multi-threaded baseline, into oracle/_build/liborc.so.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
BUILD = HERE / "_build"
LIB = BUILD / "liborc.so"
SOURCES = sorted(HERE.glob("*.c"))


def build(force: bool = False) -> Path:
    deps = SOURCES + list(HERE.glob("*.h")) + list((ROOT / "include").glob("*.h"))
    if not force and LIB.exists() and all(p.stat().st_mtime <= LIB.stat().st_mtime for p in deps):
        return LIB
    BUILD.mkdir(exist_ok=True)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
           "-I", str(ROOT / "include"), "-I", str(HERE), *map(str, SOURCES), "-o", str(tmp), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        P, U32, U64, I = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int
        L.orc_render.restype = C.c_int64
        L.orc_render.argtypes = [P, U32, P, U32, P, P, P, P, U32, U32, P, P, P, P, U64, C.POINTER(U64), P, P, I]
        L.orc_sort16.restype = None
        L.orc_sort16.argtypes = [P, U32, P]
        _lib = L
        for name, (res, args) in _EXTRA.items():
            fn = getattr(L, name, None)
            if fn is not None:
                fn.restype, fn.argtypes = res, args
    return _lib


SPLAT = np.dtype([("cx", "<f4"), ("cy", "<f4"), ("g0x", "<f4"), ("g0y", "<f4"), ("g1x", "<f4"), ("g1y", "<f4"),
                  ("r", "<f4"), ("qcut", "<f4"), ("tau0", "<f4"), ("rgb", "<f4", 3), ("ix0", "<i4"), ("iy0", "<i4"),
                  ("ix1", "<i4"), ("iy1", "<i4"), ("valid", "<u4")])

_EXTRA: dict = {
    "orc_project": (C.c_uint32, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p,
                                 C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_int]),
    "orc_logf_n": (None, [C.c_void_p, C.c_void_p, C.c_uint64]),
    "orc_expf_n": (None, [C.c_void_p, C.c_void_p, C.c_uint64]),
}


def _p(a):
    return None if a is None else a.ctypes.data


def render(gaussians, parts, frame, emitters=None, colour=None, lo_b=None, tile=(16, 16), threads: int = 1,
           want_entries: bool = True):
    """Runs the restated pipeline; returns dict(keys, order, ranges, entries, rgba, counts, visible)."""
    L = lib()
    f = np.ascontiguousarray(frame).reshape(())
    n_emit = int(f["palette"][3][1])
    n = len(gaussians) + 1 + n_emit
    W, H = int(f["viewport"][0]), int(f["viewport"][1])
    tw, th = tile
    tiles = ((W + tw - 1) // tw) * ((H + th - 1) // th)
    keys = np.empty(n, dtype=np.uint32)
    order = np.empty(n, dtype=np.uint32)
    ranges = np.empty((tiles, 2), dtype=np.uint32)
    rgba = np.empty((H, W, 4), dtype=np.float32)
    counts = np.empty((H, W), dtype=np.uint32)
    ne = C.c_uint64(0)
    g = np.ascontiguousarray(gaussians)
    p = np.ascontiguousarray(parts)
    e = np.ascontiguousarray(emitters) if emitters is not None and len(emitters) else None
    col = np.ascontiguousarray(colour, dtype=np.float32) if colour is not None else None
    lob = np.ascontiguousarray(lo_b, dtype=np.float32) if lo_b is not None else None
    cap = 0
    entries = None
    # first pass sizes the entries (the binning count is cheap)
    vis = L.orc_render(_p(g), len(g), _p(p), len(p), _p(e), _p(col), _p(lob), f.ctypes.data, tw, th,
                       _p(keys), _p(order), _p(ranges), None, 0, C.byref(ne), _p(rgba), _p(counts), threads)
    if vis < 0:
        raise RuntimeError(f"oracle render failed ({vis})")
    if want_entries:
        cap = int(ne.value)
        entries = np.empty(max(cap, 1), dtype=np.uint32)
        vis2 = L.orc_render(_p(g), len(g), _p(p), len(p), _p(e), _p(col), _p(lob), f.ctypes.data, tw, th,
                            None, None, None, entries.ctypes.data, cap, C.byref(ne), None, None, threads)
        if vis2 < 0:
            raise RuntimeError(f"oracle binning failed ({vis2})")
        entries = entries[:cap]
    return {"keys": keys, "order": order, "ranges": ranges, "entries": entries, "rgba": rgba, "counts": counts,
            "visible": int(vis), "n_entries": int(ne.value)}


def sort16(keys: np.ndarray) -> np.ndarray:
    k = np.ascontiguousarray(keys, dtype=np.uint32)
    o = np.empty(len(k), dtype=np.uint32)
    lib().orc_sort16(k.ctypes.data, len(k), o.ctypes.data)
    return o


def logf(x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.empty_like(x)
    lib().orc_logf_n(x.ctypes.data, y.ctypes.data, x.size)
    return y


def expf(x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.empty_like(x)
    lib().orc_expf_n(x.ctypes.data, y.ctypes.data, x.size)
    return y


def project(gaussians, parts, frame, emitters=None, colour=None, threads: int = 1):
    """project.wgsl restated: per slot the key (INVALID 0xFFFFFFFF) and the splat record (SPLAT dtype)."""
    f = np.ascontiguousarray(frame).reshape(())
    n = len(gaussians) + 1 + int(f["palette"][3][1])
    keys = np.empty(n, dtype=np.uint32)
    spl = np.zeros(n, dtype=SPLAT)
    g = np.ascontiguousarray(gaussians)
    p = np.ascontiguousarray(parts)
    e = np.ascontiguousarray(emitters) if emitters is not None and len(emitters) else None
    col = np.ascontiguousarray(colour, dtype=np.float32) if colour is not None else None
    vis = lib().orc_project(_p(g), len(g), _p(p), len(p), _p(e), _p(col), None, f.ctypes.data, n, keys.ctypes.data,
                            spl.ctypes.data, threads)
    return keys, spl, int(vis)
