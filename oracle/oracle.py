"""ctypes wrapper and build recipe of the CPU restatement (oracle/*.c).  TEST INFRASTRUCTURE: imported only by tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg, as the checker -- never by the product.  The reference (WGSL
on WebGPU) cannot run here and ships no golden vectors; the restatement is pinned on the reference's two shipped
assets (see sl_oracle.c).

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
    cmd = ["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
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
        L.orc_render_lod.restype = C.c_int64
        L.orc_render_lod.argtypes = [P, U32, P, U32, P, P, P, P, U32, U32, P, P, P, P, U64, C.POINTER(U64), P, P, I,
                                     P]
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
    "orc_atan2f_n": (None, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64]),
    "orc_asinf_n": (None, [C.c_void_p, C.c_void_p, C.c_uint64]),
    "orc_acosf_n": (None, [C.c_void_p, C.c_void_p, C.c_uint64]),
    "orc_row_tiles": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(C.c_uint32),
                                C.POINTER(C.c_uint32)]),
    "orc_bin": (C.c_int64, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                            C.c_void_p, C.c_void_p, C.c_uint64]),
    "orc_composite": (None, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p,
                             C.c_int]),
    "orc_lod_records": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]),
    "orc_lod_vgrids": (C.c_int, [C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]),
    "orc_lod_select": (None, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p,
                              C.c_uint32, C.c_uint32, C.c_float, C.c_void_p]),
    "orc_lod_colour": (None, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                              C.c_float, C.c_uint32, C.c_void_p]),
}


def _p(a):
    return None if a is None else a.ctypes.data


class LodCut(C.Structure):
    """orc_lod: a screen-space LOD cut as the restated projection reads it."""
    _fields_ = [("flags", C.c_void_p), ("nodes", C.c_void_p), ("colour", C.c_void_p), ("node_base", C.c_uint32),
                ("n_int", C.c_uint32)]


def render(gaussians, parts, frame, emitters=None, colour=None, lo_b=None, tile=(16, 16), threads: int = 1,
           want_entries: bool = True, lod=None):
    """Runs the restated pipeline; returns dict(keys, order, ranges, entries, rgba, counts, visible).  lod: None or
    (flags, node records, node colours) for a frame whose ``lod`` field is set (slots from frame.lod[1])."""
    L = lib()
    f = np.ascontiguousarray(frame).reshape(())
    n_emit = int(f["palette"][3][1])
    n = len(gaussians) + 1 + n_emit
    cut = None
    if lod is not None:
        flags, recs, ncol = (np.ascontiguousarray(x) for x in lod)
        ncol = np.ascontiguousarray(ncol, dtype=np.float32)
        cut = LodCut(flags.ctypes.data, recs.ctypes.data, ncol.ctypes.data, int(f["lod"][1]), int(f["lod"][2]))
        n = int(f["lod"][1]) + int(f["lod"][2])
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
    cref = C.byref(cut) if cut is not None else None
    vis = L.orc_render_lod(_p(g), len(g), _p(p), len(p), _p(e), _p(col), _p(lob), f.ctypes.data, tw, th,
                           _p(keys), _p(order), _p(ranges), None, 0, C.byref(ne), _p(rgba), _p(counts), threads, cref)
    if vis < 0:
        raise RuntimeError(f"oracle render failed ({vis})")
    if want_entries:
        cap = int(ne.value)
        entries = np.empty(max(cap, 1), dtype=np.uint32)
        vis2 = L.orc_render_lod(_p(g), len(g), _p(p), len(p), _p(e), _p(col), _p(lob), f.ctypes.data, tw, th,
                                None, None, None, entries.ctypes.data, cap, C.byref(ne), None, None, threads, cref)
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


def atan2f(y: np.ndarray, x: np.ndarray) -> np.ndarray:
    y = np.ascontiguousarray(y, dtype=np.float32)
    x = np.ascontiguousarray(x, dtype=np.float32)
    o = np.empty_like(x)
    lib().orc_atan2f_n(y.ctypes.data, x.ctypes.data, o.ctypes.data, x.size)
    return o


def asinf(x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.empty_like(x)
    lib().orc_asinf_n(x.ctypes.data, y.ctypes.data, x.size)
    return y


def acosf(x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.empty_like(x)
    lib().orc_acosf_n(x.ctypes.data, y.ctypes.data, x.size)
    return y


class EnvLight(C.Structure):
    _fields_ = [("dir", C.c_float * 3), ("std", C.c_float), ("irr", C.c_float * 3), ("shadows", C.c_int32)]


class LightSetup(C.Structure):
    _fields_ = [("emit_rec", C.c_void_p), ("n_emit", C.c_uint32), ("scale", C.c_float), ("theta", C.c_float),
                ("mode", C.c_uint32), ("asg", C.c_uint32), ("one_sided", C.c_uint32), ("normal", C.c_float * 3),
                ("edge_soft", C.c_float), ("skip_part", C.c_uint32), ("shadow_res", C.c_uint32),
                ("lights", C.c_void_p), ("n_lights", C.c_uint32), ("sun_res", C.c_uint32),
                ("sky_ambient", C.c_float), ("eye", C.c_float * 3), ("fwd", C.c_float * 3),
                ("shade_only", C.c_uint32), ("blur_shutter", C.c_float), ("tree_nodes", C.c_void_p),
                ("tree_parent", C.c_void_p), ("n_tree", C.c_uint32), ("cut_k", C.c_float)]


def node_parents(nodes, kids, G: int):
    """Every node's parent (src/lighting.js initNodeParents): internal nodes with a part own kids[child_lo:child_hi]."""
    parent = np.full(len(nodes), 0xFFFFFFFF, np.uint32)
    k = np.asarray(kids, np.uint32)
    for i in range(G, len(nodes)):
        if int(nodes["part"][i]) == 0xFFFFFFFF:
            continue
        parent[k[int(nodes["child_lo"][i]):int(nodes["child_hi"][i])]] = i
    return parent


def lighting(scene, eye=None, target=None, threads: int = 8, shadow_res=None, sun_res=None, mode: int = 1,
             asg: bool = True, cached=None, blur_shutter: float = 0.0, tree=None, cut_k: float = 1.0):
    """The restated lighting update on a splatlight_gb300.scene.Scene: returns (colour (G, 4), lamp_T (G,),
    env_T (G, 4), nodes with iso_norm).  Emitters are the scene's host emitter records.  cached: the (lamp_T,
    env_T, nodes) of an earlier call -- then only the shading pass runs (the maps of a static scene hold).
    blur_shutter > 0: the opacity maps draw moving parts (flags bit 1) stretched over the exposure; with tree = (nodes,
    kids) (the leaves, then the internal nodes) and cut_k > 0, a moving part splats the cut of its tree sized to its
    smear."""
    L = lib()
    L.orc_lighting.restype = C.c_int
    L.orc_lighting.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p,
                               C.c_uint32, C.POINTER(LightSetup), C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
    eye = np.asarray(scene.eye if eye is None else eye, np.float64)
    tgt = np.asarray(scene.target if target is None else target, np.float64)
    fwd = (tgt - eye) / np.linalg.norm(tgt - eye)
    rec = np.ascontiguousarray(scene.emitters).view(np.float32).reshape(-1, 16).copy()
    lights = (EnvLight * 4)()
    n_l = 0
    for d, std, irr, sh in scene.distant_lights()[:4]:
        lights[n_l].dir[:] = list(d)
        lights[n_l].std = std
        lights[n_l].irr[:] = list(irr)
        lights[n_l].shadows = 1 if sh else 0
        n_l += 1
    S = LightSetup()
    S.emit_rec = rec.ctypes.data if len(rec) else None
    S.n_emit = len(rec)
    S.scale = getattr(scene, "emit_scale", 1.0)
    S.theta = 4.0
    S.mode = mode
    S.asg = 1 if asg else 0
    S.one_sided = 1 if getattr(scene, "emit_one_sided", False) else 0
    S.normal[:] = list(getattr(scene, "emit_normal", (0.0, 0.0, 1.0)))
    S.edge_soft = 0.2
    S.skip_part = getattr(scene, "emit_skip_part", 0xFFFFFFFF)
    S.shadow_res = scene.shadow_res if shadow_res is None else shadow_res
    S.lights = C.addressof(lights)
    S.n_lights = n_l
    S.sun_res = scene.sun_res if sun_res is None else sun_res
    S.sky_ambient = scene.sky_ambient
    S.blur_shutter = float(blur_shutter)
    keep = []
    if tree is not None:
        tn = np.ascontiguousarray(tree[0])
        tp = node_parents(tn, tree[1], len(scene.gaussians))
        keep = [tn, tp]
        S.tree_nodes = tn.ctypes.data
        S.tree_parent = tp.ctypes.data
        S.n_tree = len(tn)
        S.cut_k = float(cut_k)
    S.eye[:] = eye.tolist()
    S.fwd[:] = fwd.tolist()
    g = np.ascontiguousarray(scene.gaussians)
    p = np.ascontiguousarray(scene.parts)
    nodes = np.ascontiguousarray(scene.nodes).copy()
    vg = np.ascontiguousarray(scene.vgrid)
    m = np.ascontiguousarray(scene.materials)
    n = len(g)
    colour = np.zeros((n, 4), np.float32)
    lamp_t = np.ones(n, np.float32)
    env_t = np.ones((n, 4), np.float32)
    if cached is not None:
        lamp_t, env_t, nodes = (np.ascontiguousarray(c).copy() for c in cached)
        S.shade_only = 1
    rc = L.orc_lighting(g.ctypes.data, n, p.ctypes.data, len(p), nodes.ctypes.data, vg.ctypes.data, m.ctypes.data,
                        len(m), C.byref(S), colour.ctypes.data, lamp_t.ctypes.data, env_t.ctypes.data, threads)
    if rc != 0:
        raise RuntimeError(f"oracle lighting failed ({rc})")
    return colour, lamp_t, env_t, nodes


def emitter_tree(rec: np.ndarray):
    """buildEmitterTree restated: (nodes (2n-1, 24) float32, root, root widened covariance)."""
    L = lib()
    L.orc_emitter_tree.restype = C.c_uint32
    L.orc_emitter_tree.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]
    r = np.ascontiguousarray(rec, np.float32).reshape(-1, 16)
    out = np.zeros((2 * len(r) - 1, 24), np.float32)
    cov = np.zeros(6, np.float32)
    root = L.orc_emitter_tree(r.ctypes.data, len(r), out.ctypes.data, cov.ctypes.data)
    return out, int(root), cov


def blur_record(parts, shutter: float, gaussian, node):
    """motion_blur.wgsl blur_records for one leaf: (Gaussian, node) stretched along its part's motion."""
    from splatlight_gb300.structs import GAUSSIAN, NODE
    p = np.ascontiguousarray(parts)
    g = np.ascontiguousarray(np.asarray(gaussian, dtype=GAUSSIAN).reshape(1))
    n = np.ascontiguousarray(np.asarray(node, dtype=NODE).reshape(1))
    go, no = np.zeros(1, GAUSSIAN), np.zeros(1, NODE)
    lib().orc_blur_record(p.ctypes.data, C.c_uint32(len(p)), C.c_float(shutter), g.ctypes.data, n.ctypes.data,
                          go.ctypes.data, no.ctypes.data)
    return go[0], no[0]


def emitter_tree_d(rec: np.ndarray, le_scale=None):
    """The same tree in float64 with each emitter's Le scaled by le_scale: (nodes (2n-1, 16): mu, radius, M xx yy zz
    xy xz yz, Le rgb, child_lo, child_hi (-1 for none), 0; root)."""
    L = lib()
    L.orc_emitter_tree_d.restype = C.c_uint32
    L.orc_emitter_tree_d.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]
    r = np.ascontiguousarray(rec, np.float32).reshape(-1, 16)
    sc = None if le_scale is None else np.ascontiguousarray(le_scale, np.float64)
    out = np.zeros((2 * len(r) - 1, 16), np.float64)
    root = L.orc_emitter_tree_d(r.ctypes.data, len(r), _p(sc), out.ctypes.data)
    return out, int(root)


def row_tiles(splat, ty: int, tile=(16, 16)):
    """sl_row_tiles of one SPLAT record: (t0, t1) tile columns of tile row ty, or None when the row holds none."""
    rec = np.ascontiguousarray(np.asarray(splat, dtype=SPLAT).reshape(1))
    a, b = C.c_uint32(), C.c_uint32()
    ok = lib().orc_row_tiles(rec.ctypes.data, ty, tile[0], tile[1], C.byref(a), C.byref(b))
    return (a.value, b.value) if ok else None


def diff_render(params: dict, lights: dict, frame, eye, order, target=None, threads: int = 1, state=None):
    """The differentiable path's forward in FP64, dense compositor (sl_oracle_diff.c).  params: means (n,3),
    log_scales (n,3), quats (n,4), opacity_logits (n,), albedo (n,3), roughness (n,) as float64; lights: rec (L
    emissive GAUSSIAN records), scale (L,), ambient, ks; state (optional): vgrid (n x 32 u32), lamp_T (n,),
    iso_norm (n,), held constant.  order: the depth order (far to near).  Returns (image H x W x 4, loss)."""
    L = lib()
    fn = L.orc_diff_render
    fn.restype = C.c_double
    fn.argtypes = [C.c_void_p] * 6 + [C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint32, C.c_double, C.c_double] + \
        [C.c_void_p] * 3 + [C.c_void_p] * 3 + [C.c_float] * 3 + \
        [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_int]
    f = np.asarray(frame).reshape(())
    W, H = int(f["viewport"][0]), int(f["viewport"][1])
    P = {k: np.ascontiguousarray(params[k], dtype=np.float64) for k in
         ("means", "log_scales", "quats", "opacity_logits", "albedo", "roughness")}
    rec = np.ascontiguousarray(lights["rec"])
    ls = np.ascontiguousarray(lights["scale"], dtype=np.float64)
    assert len(rec) == len(ls)
    st = state or {}
    vg = None if st.get("vgrid") is None else np.ascontiguousarray(st["vgrid"]).view(np.uint32)
    lt = None if st.get("lamp_T") is None else np.ascontiguousarray(st["lamp_T"], dtype=np.float64)
    iso = None if st.get("iso_norm") is None else np.ascontiguousarray(st["iso_norm"], dtype=np.float64)
    view = np.ascontiguousarray(f["view"], dtype=np.float32)
    focal = np.ascontiguousarray(f["focal"], dtype=np.float32)
    vp = np.ascontiguousarray(f["viewport"], dtype=np.float32)
    e = np.ascontiguousarray(eye, dtype=np.float64)
    o = np.ascontiguousarray(order, dtype=np.uint32)
    t = None if target is None else np.ascontiguousarray(target, dtype=np.float32)
    img = np.zeros((H, W, 4), np.float64)
    loss = fn(_p(P["means"]), _p(P["log_scales"]), _p(P["quats"]), _p(P["opacity_logits"]), _p(P["albedo"]),
              _p(P["roughness"]), len(P["roughness"]), rec.ctypes.data if len(rec) else None, _p(ls), len(ls),
              float(lights["ambient"]), float(lights["ks"]), _p(vg), _p(lt), _p(iso), _p(view), _p(focal), _p(vp),
              float(f["near"]), float(f["far"]), float(f["lowpass_px2"]), _p(e), _p(o), len(o), _p(t), _p(img),
              threads)
    return img, loss


def display(img, exposure: float = 1.0, tone: int = 0, view_mode: int = 3):
    """Display resolve (sl_oracle_display.c): H x W x 4 float -> H x W x 4 uint8."""
    L = lib()
    fn = L.orc_display
    fn.restype = None
    fn.argtypes = [C.c_void_p, C.c_uint32, C.c_float, C.c_uint32, C.c_uint32, C.c_void_p]
    a = np.ascontiguousarray(img, dtype=np.float32)
    out = np.empty(a.shape[:-1] + (4,), np.uint8)
    fn(a.ctypes.data, a.size // 4, exposure, tone, view_mode, out.ctypes.data)
    return out


def display_env(img, frame, sky):
    """Display resolve with the environment behind the splats (orc_display_env, FP64): H x W x 4 float -> uint8."""
    L = lib()
    fn = L.orc_display_env
    fn.restype = None
    fn.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_float, C.c_uint32, C.c_uint32, C.c_void_p, C.c_float,
                   C.c_float, C.c_float, C.c_float, C.c_void_p, C.c_void_p]
    a = np.ascontiguousarray(img, dtype=np.float32)
    f = np.asarray(frame).reshape(())
    view = np.ascontiguousarray(f["view"], np.float32)
    out = np.empty(a.shape[:-1] + (4,), np.uint8)
    fn(a.ctypes.data, a.shape[1], a.shape[0], float(f["exposure"]), int(f["tone"][0]), int(f["view_mode"]),
       view.ctypes.data, float(f["viewport"][0]), float(f["viewport"][1]), float(f["focal"][0]),
       float(f["focal"][1]), C.byref(sky) if sky is not None else None, out.ctypes.data)
    return out


def lod_records(gaussians, nodes, kids):
    """src/lod.js nodeGaussians restated (sl_oracle_lod.c): the internal nodes' Gaussian records."""
    from splatlight_gb300.structs import GAUSSIAN
    g = np.ascontiguousarray(gaussians)
    nd = np.ascontiguousarray(nodes)
    k = np.ascontiguousarray(kids, dtype=np.uint32)
    out = np.zeros(max(len(nd) - len(g), 1), dtype=GAUSSIAN)
    rc = lib().orc_lod_records(g.ctypes.data, len(g), nd.ctypes.data, len(nd), k.ctypes.data, out.ctypes.data)
    if rc != 0:
        raise RuntimeError("orc_lod_records failed")
    return out[:len(nd) - len(g)]


def lod_vgrids(nodes, G, kids, vgrid):
    """src/lod.js nodeGaussians' node V grids restated (sl_oracle_lod.c): (N - G) records of 128 cells."""
    from splatlight_gb300.structs import VGRID
    nd = np.ascontiguousarray(nodes)
    k = np.ascontiguousarray(kids, dtype=np.uint32)
    v = np.ascontiguousarray(vgrid)
    out = np.zeros(max(len(nd) - G, 1), dtype=VGRID)
    if lib().orc_lod_vgrids(G, nd.ctypes.data, len(nd), k.ctypes.data, v.ctypes.data, out.ctypes.data) != 0:
        raise RuntimeError("orc_lod_vgrids failed")
    return out[:len(nd) - G]


def lod_select(nodes, G, kids, parts, frame, flags, emit_part=0xFFFFFFFF, size_rule=1, blur_lod=0.0):
    """lod.wgsl lod_select restated: updates ``flags`` (N u32, the previous frame's cut) in place."""
    nd = np.ascontiguousarray(nodes)
    k = np.ascontiguousarray(kids, dtype=np.uint32)
    p = np.ascontiguousarray(parts)
    f = np.ascontiguousarray(frame).reshape(())
    assert flags.dtype == np.uint32 and flags.flags.c_contiguous
    lib().orc_lod_select(nd.ctypes.data, len(nd), G, k.ctypes.data, p.ctypes.data, len(p), f.ctypes.data, emit_part,
                         size_rule, blur_lod, flags.ctypes.data)
    return flags


def lod_colour(nodes, G, kids, flags, colour, lo_b=None, gain=0.0, colour_all=False):
    """lod.wgsl lod_colour restated: (N - G, 4) node colours from the leaves' colours (G, 4)."""
    nd = np.ascontiguousarray(nodes)
    k = np.ascontiguousarray(kids, dtype=np.uint32)
    fl = np.ascontiguousarray(flags, dtype=np.uint32)
    col = np.ascontiguousarray(colour, dtype=np.float32) if colour is not None else None
    lob = np.ascontiguousarray(lo_b, dtype=np.float32) if lo_b is not None else None
    out = np.zeros((max(len(nd) - G, 1), 4), np.float32)
    lib().orc_lod_colour(nd.ctypes.data, len(nd), G, k.ctypes.data, fl.ctypes.data, _p(col), _p(lob), gain,
                         1 if colour_all else 0, out.ctypes.data)
    return out[:len(nd) - G]


def render_given_order(gaussians, parts, frame, order, emitters=None, colour=None, lo_b=None, tile=(16, 16),
                       threads: int = 1):
    """The restated projection, then binning and compositing in a given order of the visible slots (the counting
    sort's order on the GPU, whose ties land in arbitrary order): dict(keys, ranges, entries, rgba, counts, visible)."""
    L = lib()
    f = np.ascontiguousarray(frame).reshape(())
    n = len(gaussians) + 1 + int(f["palette"][3][1])
    W, H = int(f["viewport"][0]), int(f["viewport"][1])
    tw, th = tile
    tiles = ((W + tw - 1) // tw) * ((H + th - 1) // th)
    g, p = np.ascontiguousarray(gaussians), np.ascontiguousarray(parts)
    e = np.ascontiguousarray(emitters) if emitters is not None and len(emitters) else None
    col = np.ascontiguousarray(colour, dtype=np.float32) if colour is not None else None
    lob = np.ascontiguousarray(lo_b, dtype=np.float32) if lo_b is not None else None
    keys = np.empty(n, np.uint32)
    splats = np.zeros(n, SPLAT)
    vis = int(L.orc_project(_p(g), len(g), _p(p), len(p), _p(e), _p(col), _p(lob), f.ctypes.data, n, keys.ctypes.data,
                            splats.ctypes.data, threads))
    o = np.ascontiguousarray(order[:vis], dtype=np.uint32)
    ranges = np.empty((tiles, 2), np.uint32)
    total = int(L.orc_bin(splats.ctypes.data, o.ctypes.data, vis, W, H, tw, th, ranges.ctypes.data, None, 0))
    entries = np.empty(max(total, 1), np.uint32)
    L.orc_bin(splats.ctypes.data, o.ctypes.data, vis, W, H, tw, th, None, entries.ctypes.data, total)
    rgba = np.empty((H, W, 4), np.float32)
    counts = np.empty((H, W), np.uint32)
    L.orc_composite(splats.ctypes.data, o.ctypes.data, vis, W, H, rgba.ctypes.data, counts.ctypes.data, threads)
    return {"keys": keys, "ranges": ranges, "entries": entries[:total], "rgba": rgba, "counts": counts,
            "visible": vis}


class ProbeLayoutC(C.Structure):
    _fields_ = [("dims", C.c_uint32 * 3), ("terrain", C.c_uint32), ("lo", C.c_float * 3), ("step", C.c_float * 3),
                ("levels", C.c_float * 16), ("ground", C.c_void_p), ("tmax", C.c_float), ("part_probes", C.c_uint32),
                ("n_vols", C.c_uint32), ("vols", (C.c_uint32 * 4) * 32)]


def probe_count(layout, part_count: int) -> int:
    """The lattice, 8 probes per part, then the static volumes' grids."""
    n = int(np.prod(layout["dims"])) + 8 * part_count
    for _, nx, ny, nz in layout.get("vols", []):
        n += nx * ny * nz
    return n


class BounceIn(C.Structure):
    _fields_ = [("gs", C.c_void_p), ("count", C.c_uint32), ("parts", C.c_void_p), ("part_count", C.c_uint32),
                ("nodes", C.c_void_p), ("n_nodes", C.c_uint32), ("kids", C.c_void_p), ("vgrid", C.c_void_p),
                ("mats", C.c_void_p), ("mat_count", C.c_uint32), ("tree", C.c_void_p), ("tree_root", C.c_uint32),
                ("n_emit", C.c_uint32), ("emit_mode", C.c_uint32), ("one_sided", C.c_uint32),
                ("emit_theta", C.c_float), ("emit_scale", C.c_float), ("edge_soft", C.c_float),
                ("normal", C.c_float * 3), ("lamp_T", C.c_void_p), ("env_T", C.c_void_p), ("lights", C.c_void_p),
                ("n_lights", C.c_uint32), ("sky_sh", C.c_void_p), ("lay", ProbeLayoutC), ("max_depth", C.c_uint32),
                ("eye", C.c_float * 3), ("alpha", C.c_float), ("frame", C.c_uint32), ("force", C.c_uint32),
                ("moved_mask", C.c_uint32), ("dark_part", C.c_uint32), ("asg_cells", C.c_uint32),
                ("sender_cut", C.c_uint32), ("sc_reselect", C.c_uint32), ("node_gs", C.c_void_p),
                ("node_vg", C.c_void_p)]


class BounceState(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("probe_data", "probe_sh", "xfer", "lo_dir", "lo_b", "node_acc", "node_sh",
                                          "probe_hist", "sc_flag", "sc_X", "sc_T", "sc_envT")]


def bounce_tables():
    """(D14 (14, 3), pinv (9, 14)) restated."""
    L = lib()
    L.orc_bounce_tables.restype = None
    L.orc_bounce_tables.argtypes = [C.c_void_p, C.c_void_p]
    d = np.zeros((14, 3), np.float32)
    p = np.zeros((9, 14), np.float32)
    L.orc_bounce_tables(d.ctypes.data, p.ctypes.data)
    return d, p


def f32_to_f16(x: np.ndarray) -> np.ndarray:
    """The restatement's round-to-nearest-even f32 -> f16 bits, elementwise."""
    L = lib()
    L.orc_f32_to_f16.restype = C.c_uint32
    L.orc_f32_to_f16.argtypes = [C.c_float]
    return np.array([L.orc_f32_to_f16(float(v)) for v in np.asarray(x, np.float32).ravel()], np.uint32)


class Bounce:
    """The probe bounce restated (sl_oracle_light.c orc_bounce_frame), stateful over frames.  scene: a Scene whose
    parts carry their tree roots; tree = (nodes, kids) (the leaves, then the internal nodes); lit = the (colour,
    lamp_T, env_T, nodes) of oracle.lighting on the scene (the leaves' iso_norm and the maps' transmittance);
    layout: a probes.* layout dict; sky_sh: (16, 3) or None; sender_cut: the reference's default level of detail
    for the senders (bounce.wgsl sc_select), re-selected on the first frame and whenever a part moved."""

    def __init__(self, scene, tree, lit, layout, sky_sh=None, max_depth: int = 0, blend: float = 1.0,
                 emitters_dark: bool = True, asg: bool = True, sender_cut: bool = False):
        self.scene = scene
        G = scene.count
        tn = np.ascontiguousarray(tree[0]).copy()
        tn["pad0"][:G] = lit[3]["pad0"]
        tn["pad1"][:G] = lit[3]["pad1"]
        self.nodes = tn
        self.kids = np.ascontiguousarray(tree[1], np.uint32)
        if max_depth == 0:
            max_depth = int(tn["depth"][G:].max()) + 1 if len(tn) > G else 1
        self.max_depth = max_depth
        self.blend = blend
        self.asg = asg
        self.dark_part = int(getattr(scene, "emit_skip_part", 0xFFFFFFFF)) if emitters_dark else 0xFFFFFFFF
        self.lamp_T = np.ascontiguousarray(lit[1], np.float32)
        self.env_T = np.ascontiguousarray(lit[2], np.float32)
        rec = np.ascontiguousarray(scene.emitters).view(np.float32).reshape(-1, 16).copy()
        if len(rec):
            self.tree, self.root, _ = emitter_tree(rec)
        else:
            self.tree, self.root = np.zeros((1, 24), np.float32), 0
        self.n_emit = len(rec)
        self.lights = (EnvLight * 4)()
        self.n_lights = 0
        for d, std, irr, sh in scene.distant_lights()[:4]:
            self.lights[self.n_lights].dir[:] = list(d)
            self.lights[self.n_lights].std = std
            self.lights[self.n_lights].irr[:] = list(irr)
            self.lights[self.n_lights].shadows = 1 if sh else 0
            self.n_lights += 1
        self.sky = None if sky_sh is None else np.ascontiguousarray(sky_sh, np.float32).reshape(16, 3)
        self.layout = layout
        self.ground = None if layout.get("ground") is None else np.ascontiguousarray(layout["ground"], np.float32)
        NP = probe_count(layout, len(scene.parts))
        N = len(tn)
        self.state = {"probe_data": np.zeros((NP, 128, 8), np.float32), "probe_sh": np.zeros((NP, 9, 4), np.float32),
                      "xfer": np.zeros((G, 12), np.float32), "lo_dir": np.zeros((G, 4), np.float32),
                      "lo_b": np.zeros((G, 3, 4), np.float32), "node_acc": np.zeros((N, 14, 4), np.float32),
                      "node_sh": np.zeros((N, 14), np.uint32), "probe_hist": np.zeros((NP, 128, 16), np.float32),
                      "sc_flag": np.zeros(N, np.uint32), "sc_X": np.zeros((max(N - G, 1), 8, 4), np.float32),
                      "sc_T": np.zeros(max(N - G, 1), np.float32), "sc_envT": np.zeros((max(N - G, 1), 4), np.float32)}
        self.sender_cut = sender_cut
        if sender_cut:
            self.node_gs = np.ascontiguousarray(lod_records(scene.gaussians, tn, self.kids))
            self.node_vg = np.ascontiguousarray(lod_vgrids(tn, G, self.kids, scene.vgrid))
        self.frame = 0
        self.first = True

    def step(self, eye, moved_mask: int = 0, threads: int = 8):
        """One frame (the GPU's sl_lighting_update after the shading); returns the state dict."""
        L = lib()
        L.orc_bounce_frame.restype = C.c_int
        L.orc_bounce_frame.argtypes = [C.POINTER(BounceIn), C.POINTER(BounceState), C.c_int]
        s = self.scene
        g = np.ascontiguousarray(s.gaussians)
        p = np.ascontiguousarray(s.parts)
        vg = np.ascontiguousarray(s.vgrid)
        m = np.ascontiguousarray(s.materials)
        B = BounceIn()
        B.gs, B.count = g.ctypes.data, len(g)
        B.parts, B.part_count = p.ctypes.data, len(p)
        B.nodes, B.n_nodes = self.nodes.ctypes.data, len(self.nodes)
        B.kids = self.kids.ctypes.data if len(self.kids) else None
        B.vgrid = vg.ctypes.data
        B.mats, B.mat_count = m.ctypes.data, len(m)
        B.tree, B.tree_root, B.n_emit = self.tree.ctypes.data, self.root, self.n_emit
        B.emit_mode, B.emit_theta, B.emit_scale = 1, 4.0, getattr(s, "emit_scale", 1.0)
        B.one_sided = 1 if getattr(s, "emit_one_sided", False) else 0
        B.normal[:] = list(getattr(s, "emit_normal", (0.0, 0.0, 1.0)))
        B.edge_soft = 0.2
        B.lamp_T, B.env_T = self.lamp_T.ctypes.data, self.env_T.ctypes.data
        B.lights, B.n_lights = C.addressof(self.lights), self.n_lights
        B.sky_sh = self.sky.ctypes.data if self.sky is not None else None
        lay = self.layout
        B.lay.dims[:] = [int(v) for v in lay["dims"]]
        B.lay.terrain = 1 if lay["terrain"] else 0
        B.lay.lo[:] = [float(v) for v in lay["lo"]]
        B.lay.step[:] = [float(v) for v in lay["step"]]
        B.lay.levels[:] = [float(v) for v in list(lay["levels"]) + [0.0] * (16 - len(lay["levels"]))]
        B.lay.ground = self.ground.ctypes.data if self.ground is not None else None
        B.lay.tmax = float(lay["tmax"])
        B.lay.part_probes = 1
        vols = list(lay.get("vols", []))[:32]
        B.lay.n_vols = len(vols)
        for i, v in enumerate(vols):
            B.lay.vols[i][:] = [int(x) for x in v]
        B.max_depth = self.max_depth
        B.eye[:] = [float(v) for v in eye]
        B.alpha = 1.0 if self.first else self.blend
        B.frame = self.frame
        B.force = 1 if self.first else 0
        B.moved_mask = moved_mask
        B.dark_part = self.dark_part
        B.asg_cells = 1 if self.asg else 0
        B.sender_cut = 1 if self.sender_cut else 0
        B.sc_reselect = 1 if (self.first or moved_mask) else 0
        if self.sender_cut:
            B.node_gs, B.node_vg = self.node_gs.ctypes.data, self.node_vg.ctypes.data
        st = BounceState(**{k: v.ctypes.data for k, v in self.state.items()})
        rc = L.orc_bounce_frame(C.byref(B), C.byref(st), threads)
        if rc != 0:
            raise RuntimeError(f"oracle bounce failed ({rc})")
        self.first = False
        self.frame += 1
        return self.state
