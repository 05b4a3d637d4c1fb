"""The gs-runtime asset format: asset.json plus raw little-endian .bin buffers, read as the reference's loader reads
them (src/asset.js: checkHeader :18-30, checkBuffer :32-38, readLamps :41-49, loadAsset :51-78, fingerprint
:83-88), and the scene an asset sets up for the lit path: the asset's own emissive part as the light set
(setAssetEmitters, src/lighting.js:690-721, with the lamp position main.js gives it, src/main.js:178-179, 197 and
the lamp part's translation in writeParts, src/main.js:656-659), its environment's distant lights (parseEnvironment
and Environment.write, src/environment.js:23-41, 49-56, 111-129), its camera (OrbitCamera.setView,
src/camera.js:21-29) and far plane (src/main.js:488).

The layout checks themselves run in libsplatlight (sl_asset_check_header / sl_asset_check_buffer /
sl_asset_check_bytes), so every host -- this one, an N-API addon, a C++ engine -- applies the same rules and gets
the reference's messages.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import json
import math
from pathlib import Path

import numpy as np

from . import _native as N
from .scene import Scene, Sun
from .structs import GAUSSIAN, MATERIAL, NODE, PART, VGRID

# The buffers loadAsset reads, in its order (src/asset.js:64), and their record types.
BUFFERS = ("gaussians", "parts", "lamps", "materials", "nodes", "kids", "vgrid")
LAMP = np.dtype([("center", "<f4", 3), ("kind", "<u4"), ("e1", "<f4", 3), ("radius", "<f4"), ("e2", "<f4", 3),
                 ("range", "<f4"), ("normal", "<f4", 3), ("flags", "<u4"), ("radiance", "<f4", 3), ("pad", "<u4"),
                 ("center_prev", "<f4", 3), ("pad2", "<u4")])
DTYPES = {"gaussians": GAUSSIAN, "parts": PART, "lamps": LAMP, "materials": MATERIAL, "nodes": NODE,
          "kids": np.dtype("<u4"), "vgrid": VGRID}
assert LAMP.itemsize == 96
DEG = math.pi / 180.0
# Ein(3) = int_0^3 (1 - e^-x) / x dx by the reference's 3000-step midpoint sum (src/lighting.js:55-56)
EIN3 = sum((1.0 - math.exp(-((i + 0.5) * 0.001))) / ((i + 0.5) * 0.001) * 0.001 for i in range(3000))


class AssetError(N.SplatlightError):
    """A layout check failed (SL_ERR_LAYOUT) or a file could not be read."""


def _check(rc: int) -> None:
    if rc != 0:
        raise AssetError(rc, N.last_error())


def check_header(header: dict) -> None:
    """checkHeader (src/asset.js:18-30): format and major version, then every buffer the kernels read: present,
    stride, field offsets, 0 < count <= 2^24.  Raises AssetError with the reference's message."""
    lib = N.lib()
    fmt = header.get("format")
    ver = header.get("version")
    _check(lib.sl_asset_check_header(None if fmt is None else str(fmt).encode(),
                                     None if ver is None else _js_string(ver).encode()))
    bufs = header.get("buffers") or {}
    for name in ("gaussians", "parts", "lamps", "materials", "nodes", "kids", "vgrid"):   # EXPECT's order
        b = bufs.get(name)
        if not b:
            raise AssetError(-2, f"Asset has no {name} buffer")
        fields = b.get("fields") or {}
        names = [k.encode() for k in fields]
        offs = [v.get("offset") if isinstance(v, dict) else None for v in fields.values()]
        offs = [o if isinstance(o, int) and not isinstance(o, bool) and 0 <= o < 0xFFFFFFFF else 0xFFFFFFFF
                for o in offs]
        stride = b.get("stride")
        stride = stride if isinstance(stride, int) and not isinstance(stride, bool) and 0 <= stride < 2 ** 32 \
            else 0xFFFFFFFF
        count = b.get("count")
        if not (isinstance(count, int) and not isinstance(count, bool)) or not 0 < count <= (1 << 24):
            # stride and fields are checked first (the reference's order); a bad count then reports its value
            _check(lib.sl_asset_check_buffer(name.encode(), stride, 1, (C.c_char_p * max(len(names), 1))(*names),
                                             (C.c_uint32 * max(len(offs), 1))(*offs), len(names)))
            raise AssetError(-2, f"Bad {name} count {_js_string(count)}")
        _check(lib.sl_asset_check_buffer(name.encode(), stride, count, (C.c_char_p * max(len(names), 1))(*names),
                                         (C.c_uint32 * max(len(offs), 1))(*offs), len(names)))


def check_buffer(header: dict, name: str, data: bytes) -> bytes:
    """checkBuffer (src/asset.js:32-38): the file holds exactly count x stride bytes."""
    b = header["buffers"][name]
    if N.lib().sl_asset_check_bytes(len(data), b["count"], b["stride"]) != 0:
        raise AssetError(-2, f"{b['file']} is {len(data)} B, expected {b['count']} x {b['stride']} B")
    return data


def read_lamps(header: dict, data: bytes) -> list[dict]:
    """readLamps (src/asset.js:41-49): the lamp records as plain values."""
    rec = np.frombuffer(data, dtype=LAMP, count=header["buffers"]["lamps"]["count"])
    return [{"center": [float(v) for v in r["center"]], "kind": int(r["kind"]), "e1": [float(v) for v in r["e1"]],
             "radius": float(r["radius"]), "e2": [float(v) for v in r["e2"]],
             "normal": [float(v) for v in r["normal"]], "radiance": [float(v) for v in r["radiance"]]}
            for r in rec]


def fingerprint(header: dict, gaussians: bytes) -> dict:
    """fingerprint (src/asset.js:83-88): Gaussian count, part ranges, byte length and
    sum_i w_i (i 2654435761 + 1) mod 2^32 over the u32 words of gaussians.bin."""
    w = np.frombuffer(gaussians, dtype="<u4").astype(np.uint64)
    i = np.arange(len(w), dtype=np.uint64)
    h = int(((w * ((i * np.uint64(2654435761) + np.uint64(1)) & np.uint64(0xFFFFFFFF))) & np.uint64(0xFFFFFFFF))
            .sum() & 0xFFFFFFFF)
    return {"count": header["buffers"]["gaussians"]["count"], "parts": [p["gaussians"] for p in header["parts"]],
            "bytes": len(gaussians), "hash": h}


@dataclasses.dataclass
class Asset:
    header: dict
    raw: dict              # buffer name -> numpy records (read-only views of the files' bytes)
    lamps: list
    count: int
    part_count: int
    fingerprint: dict
    base: Path

    @property
    def gaussians(self) -> np.ndarray:
        return self.raw["gaussians"]

    @property
    def parts(self) -> np.ndarray:
        return self.raw["parts"]


def load_asset(base) -> Asset:
    """loadAsset (src/asset.js:51-78): asset.json, checkHeader, then the seven buffers, each checked by size."""
    base = Path(base)
    try:
        header = json.loads((base / "asset.json").read_text())
    except OSError as e:
        raise AssetError(-2, f"Could not load {base}/asset.json ({e.strerror})") from None
    check_header(header)
    raw = {}
    for name in BUFFERS:
        f = base / header["buffers"][name]["file"]
        try:
            data = f.read_bytes()
        except OSError as e:
            raise AssetError(-2, f"Could not load {f} ({e.strerror})") from None
        check_buffer(header, name, data)
        raw[name] = np.frombuffer(data, dtype=DTYPES[name])
    # optional own-part blockers (64 B per Gaussian), kept only when they match (src/asset.js:66-75)
    raw["blockers"] = None
    bk = header.get("blockers") or {}
    if bk.get("file") and bk.get("stride") == 64 and bk.get("count") == header["buffers"]["gaussians"]["count"]:
        p = base / bk["file"]
        if p.exists() and p.stat().st_size == bk["count"] * 64:
            raw["blockers"] = np.frombuffer(p.read_bytes(), dtype=np.uint8).reshape(-1, 64)
    g_bytes = raw["gaussians"].tobytes()
    return Asset(header=header, raw=raw, lamps=read_lamps(header, raw["lamps"].tobytes()),
                 count=header["buffers"]["gaussians"]["count"], part_count=header["buffers"]["parts"]["count"],
                 fingerprint=fingerprint(header, g_bytes), base=base)


def _js_string(v) -> str:
    """String(v) for the JSON values a header holds (numbers print without a trailing .0, as JavaScript does)."""
    if isinstance(v, bool):
        return "true" if v else "false"
    if isinstance(v, float) and v.is_integer():
        return str(int(v))
    if v is None:
        return "null"
    return str(v)


def _normalize(v):
    v = [float(x) for x in v]
    n = math.hypot(*v) or 1.0
    return [x / n for x in v]


def sun_dir(az: float, el: float) -> list:
    """sunDir (src/environment.js:49-52): unit direction toward the light from azimuth and elevation in degrees."""
    a, e = az * DEG, el * DEG
    return [-math.sin(a) * math.cos(e), math.cos(a) * math.cos(e), math.sin(e)]


def sun_angles(d) -> list:
    """sunAngles (src/environment.js:53-55)."""
    return [math.atan2(-d[0], d[1]) / DEG, math.asin(max(-1.0, min(1.0, d[2]))) / DEG]


def environment_lights(env: dict | None, light_gain: float = 1.0) -> list:
    """The distant lights Environment.write sends to the shaders for an asset.json environment block
    (parseEnvironment, src/environment.js:23-41, then write :111-129 with the panel at its start state: the first
    light's direction through sunDir(sunAngles(dir)), the others' as given unless they follow the sun).  Returns
    [(direction, angular std in radians, irradiance rgb, casts shadows)]."""
    if not env:
        return []
    lights = []
    parsed = [{"dir": _normalize(L["dir"]), "irr": list(L.get("irradiance_rgb", [1.0, 1.0, 1.0])),
               "std": float(L.get("angular_std_deg", 0.27)) * DEG, "shadows": bool(L.get("casts_shadows", True)),
               "follow": bool(L.get("follows_sun", False))} for L in (env.get("lights") or [])[:4]]
    if not parsed:
        return []
    sun = sun_angles(parsed[0]["dir"])
    for k, L in enumerate(parsed):
        d = sun_dir(*sun) if k == 0 or L["follow"] else L["dir"]
        lights.append((tuple(d), L["std"], tuple(v * light_gain for v in L["irr"]), L["shadows"]))
    return lights


def asset_emitters(asset: Asset, center) -> dict:
    """setAssetEmitters(center) (src/lighting.js:690-721): the emissive part's Gaussians, moved so their rest
    centroid sits at `center`, with the asset's emission as Le, are the light set; EmitParams.scale is the overlap
    correction (the panel area spanned by the emitter grid over the emitters' summed footprint), the normal the first
    emitter's short axis, one-sided from the emissive material's flag bit 2, skip part = the emissive part."""
    em = asset.header["emitters"]
    part = int(em["part"])
    g0, g1 = asset.header["parts"][part]["gaussians"]
    n = g1 - g0
    rec = asset.gaussians[g0:g1].copy()
    mu = rec["mu"].astype(np.float64)
    c0 = [float(sum(mu[i, k] for i in range(n)) / n) for k in range(3)]      # sequential sums, as the reference
    for k in range(3):
        rec["mu"][:, k] = (mu[:, k] + (float(center[k]) - c0[k])).astype(np.float32)
    rec["albedo"] = np.asarray(em["emission"], np.float32)
    x, y, z, w = (float(v) for v in rec["quat"][0])
    nrm = (1 - 2 * (y * y + z * z), 2 * (x * y + w * z), 2 * (x * z - w * y))
    ax = [(2 * (x * y - w * z), 1 - 2 * (x * x + z * z), 2 * (y * z + w * x)),
          (2 * (x * z + w * y), 2 * (y * z - w * x), 1 - 2 * (x * x + y * y))]
    P = rec["mu"].astype(np.float64)
    extent = []
    for a in ax:
        vals = [a[0] * P[i, 0] + a[1] * P[i, 1] + a[2] * P[i, 2] for i in range(n)]
        lo, hi = min(vals), max(vals)
        cols = len({_js_round((v - lo) / (hi - lo + 1e-9) * 1000) for v in vals})
        extent.append((hi - lo) * cols / max(cols - 1, 1))
    foot = 0.0
    for i in range(n):
        foot += 2 * math.pi * float(rec["scale"][i, 1]) * float(rec["scale"][i, 2]) * EIN3
    mflags = int(asset.raw["materials"][int(em["material"])]["flags"])
    return {"records": rec, "scale": extent[0] * extent[1] / foot, "normal": nrm, "one_sided": (mflags & 4) != 0,
            "skip_part": part}


def _js_round(x: float) -> int:
    """Math.round: halves round up."""
    return math.floor(x + 0.5)


def lamp_home(asset: Asset) -> list:
    """main.js's lamp position at start (src/main.js:178-179, 197): lamps[0].center, z = 1.97 unless the asset's
    emitters stay at rest (emitters.home 'rest')."""
    home = asset.lamps[0]["center"] if asset.lamps else [0.0, 1.0, 1.9]
    em = asset.header.get("emitters") or {}
    return [home[0], home[1], home[2] if em.get("home") == "rest" else 1.97]


def asset_scene(asset: Asset, width: int | None = None, height: int | None = None, lamp=None, view: str | None = None,
                shadow_res: int = 512, sun_res: int = 512) -> Scene:
    """The scene an asset sets up, as the reference's page does on load: Gaussians, parts, the leaf nodes (the first
    `count` records of nodes.bin, in Gaussian order), V grids and materials as stored; the asset's emitters at
    `lamp` (default: main.js's start position; the lamp part translated by lamp - lamps[0].center, settled: xf_prev =
    xf); the environment's distant lights (no sky term: the reference's sky reaches Gaussians only through its probe
    bounce); the asset camera (or one of asset.json's named views) at its resolution; map resolutions at the
    reference's defaults (512, src/light_shadow.js:18, src/sun_map.js:54)."""
    h = asset.header
    parts = asset.parts.copy()
    emit = None
    if h.get("emitters"):
        home = asset.lamps[0]["center"] if asset.lamps else [0.0, 1.0, 1.9]
        center = lamp_home(asset) if lamp is None else [float(v) for v in lamp]
        emit = asset_emitters(asset, center)
        p = int(h["emitters"]["part"])
        t = [center[k] - home[k] for k in range(3)]
        xf = np.array([1, 0, 0, t[0], 0, 1, 0, t[1], 0, 0, 1, t[2]], np.float32)
        parts[p]["xf"] = xf
        parts[p]["xf_prev"] = xf
    cam = h["camera"]
    eye, target, fov = cam["eye"], cam["look_at"], float(cam["fov_deg"])
    if view is not None:
        v = h["views"][view]
        eye, target = v["eye"], v["look_at"]
    W, H = cam.get("resolution", [512, 512])
    if view is not None and "hfov_deg" in h["views"][view]:
        W = width or W
        H = height or H
        fov = 2 * math.degrees(math.atan(math.tan(math.radians(h["views"][view]["hfov_deg"]) / 2) * H / W))
    b = h.get("bounds")
    far = max(50.0, 1.5 * math.hypot(*[b["hi"][k] - b["lo"][k] for k in range(3)])) if b else 50.0
    lights = environment_lights(h.get("environment"))
    sun = Sun(direction=lights[0][0], irradiance=lights[0][2], angular_std=lights[0][1],
              casts_shadows=lights[0][3]) if lights else None
    empty = np.zeros(0, dtype=GAUSSIAN)
    s = Scene(name=h.get("name", asset.base.name), gaussians=asset.gaussians.copy(), parts=parts,
              nodes=asset.raw["nodes"][:asset.count].copy(), vgrid=asset.raw["vgrid"].copy(),
              materials=asset.raw["materials"].copy(), emitters=emit["records"] if emit else empty,
              eye=tuple(float(v) for v in eye), target=tuple(float(v) for v in target),
              up=tuple(float(v) for v in cam.get("up", [0, 0, 1])), fov_deg=fov, width=int(width or W),
              height=int(height or H), far=far, sun=sun, sky_ambient=0.0, shadow_res=shadow_res, sun_res=sun_res)
    return dataclasses.replace(
        s, extra_lights=tuple(lights[1:]), emit_scale=emit["scale"] if emit else 1.0,
        emit_one_sided=emit["one_sided"] if emit else False,
        emit_normal=tuple(emit["normal"]) if emit else (0.0, 0.0, 1.0),
        emit_skip_part=emit["skip_part"] if emit else 0xFFFFFFFF,
        emit_drawn=False,          # the emitters are scene Gaussians: drawn with the scene, not in extra slots
        tree_nodes=asset.raw["nodes"], kids=asset.raw["kids"], sky_sh=environment_sky(h.get("environment")),
        probes=probe_layout(asset))


def display_sky(env: dict | None):
    """The environment as the display draws it (Environment.write, src/environment.js:111-150, with its start state:
    sky and light gains 1): an sl_display_sky with the lighting sky, the distant lights with their visible discs'
    std (display_std_deg), and -- when sky.background_sh_rgb is given -- the background SH, the horizon ring
    (along_deg 25, across_deg 8 by default) with the ground below it (a 1 degree blend) and the glow round the sun
    (angular_std_deg 12 by default; toward the first light unless it has its own direction and does not follow the
    sun).  None without an environment."""
    from . import display as D
    if not env:
        return None
    lights = environment_lights(env)
    raw = (env.get("lights") or [])[:4]
    lights = [tuple(L) + (float(raw[k].get("display_std_deg", 0.0)) * DEG,) for k, L in enumerate(lights)]
    sk = env.get("sky") or {}
    bg = None
    if sk.get("background_sh_rgb"):
        bg = {"sh": sk["background_sh_rgb"][:81]}
        hz, ground = sk.get("horizon"), sk.get("ground_rgb")
        if hz and ground:
            along = float(hz.get("along_deg", 25)) * DEG
            across = float(hz.get("across_deg", 8)) * DEG
            bg.update(ring=hz["rgb"][:8], ring_par=(1.0 / (2.0 * along * along), 1.0 / (2.0 * across * across)),
                      ground=ground, ground_blend=math.sin(1.0 * DEG))
        g = sk.get("glow")
        if g:
            follow = bool(g.get("follows_sun", True))
            d = sun_dir(*sun_angles(lights[0][0])) if (follow or not g.get("dir")) and lights else \
                _normalize(g.get("dir") or [0.0, 0.0, 1.0])
            bg.update(glow=g["irradiance_rgb"], glow_std=float(g.get("angular_std_deg", 12)) * DEG, glow_dir=d)
    return D.sky(environment_sky(env), lights, bg)


def environment_sky(env: dict | None):
    """The sky the probes see (parseEnvironment's sh, Environment.write with the sky gain at 1,
    src/environment.js:25, 116-124): environment.sky.sh_rgb, up to 16 coefficients, (16, 3) float32; None without
    an environment or a sky."""
    sh = ((env or {}).get("sky") or {}).get("sh_rgb") or []
    if not sh:
        return None
    out = np.zeros((16, 3), np.float32)
    out[:min(16, len(sh))] = np.asarray(sh[:16], np.float64)
    return out


def probe_layout(asset: Asset) -> dict:
    """probeLayout (src/lighting.js:220-286) on the asset's header: the room layout for an asset with `room`, else
    the terrain layout over `bounds` (probes.layout may force either); probes.dims / heights_m / terrain_parts as
    given; the static probe volumes (probes.volumes, else probeVolumes's rule, :289-314)."""
    from . import probes as PR
    h = asset.header
    pr = h.get("probes") or {}
    terrain = pr.get("layout") == "terrain" or (not h.get("room") and bool(h.get("bounds")) and
                                                pr.get("layout") != "room")
    if h.get("room"):
        box = tuple((float(h["room"][k][0]), float(h["room"][k][1])) for k in "xyz")
    elif h.get("bounds"):
        b = h["bounds"]
        box = tuple((float(b["lo"][k]), float(b["hi"][k])) for k in range(3))
    else:
        raise ValueError("asset.json has neither room nor bounds (probe lattice)")
    env = bool(h.get("environment"))
    if not terrain:
        return PR.room_layout(box, environment=env)
    names = [p.get("name") for p in h["parts"]]
    tp = [names.index(n) for n in pr.get("terrain_parts", []) if n in names]
    named = None
    if pr.get("volumes"):
        named = [(names.index(v["part"]), v["dims"]) for v in pr["volumes"] if v.get("part") in names]
    return PR.terrain_layout(asset.gaussians, asset.parts, box, dims=tuple(pr.get("dims", (16, 16, 5))[:2]),
                             heights=tuple(pr.get("heights_m", (0.3, 1.0, 3.0, 8.0, 20.0))), terrain_parts=tp,
                             environment=env, volumes=named)
