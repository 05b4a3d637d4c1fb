"""Probe lattice layouts for the probe bounce (Lighting.set_probes), as the reference lays them out from an asset's
header (src/lighting.js probeLayout :215-286; runtime SPEC 2.7): float64 on the host, rounded to float32 where the
device reads them."""
from __future__ import annotations

import math

import numpy as np

PROBES_AXIS = 8      # room lattice: 8^3 (lighting.js:177)
TMAX = 6.0           # probe ray length without an environment (lighting.js:177)
ROOM_INSET = 0.125   # the room lattice's inset from the walls (lighting.js:228)


def _tmax(box, environment: bool) -> float:
    """Rays reach TMAX, or across the whole scene when it has an environment (rays that leave it see the sky)."""
    return max(TMAX, math.hypot(*[b - a for a, b in box])) if environment else TMAX


def room_layout(box, environment: bool = False) -> dict:
    """The room layout: an 8^3 lattice inset 0.125 m from the walls of box ((x0, x1), (y0, y1), (z0, z1)), ground 0
    and evenly spaced levels (lighting.js:227-233)."""
    n = PROBES_AXIS
    cen = [(a + b) / 2 for a, b in box]
    half = [(b - a) / 2 - ROOM_INSET for a, b in box]
    lo = [c - h for c, h in zip(cen, half)]
    step = [2 * h / (n - 1) for h in half]
    levels = [lo[2] + k * step[2] for k in range(n)]
    return {"terrain": False, "dims": [n, n, n], "lo": lo, "step": step, "levels": levels, "ground": None,
            "tmax": _tmax(box, environment), "vols": []}


def terrain_layout(gaussians: np.ndarray, parts: np.ndarray, box, dims=(16, 16, 5),
                   heights=(0.3, 1.0, 3.0, 8.0, 20.0), terrain_parts=None, environment: bool = True,
                   volumes=None) -> dict:
    """The terrain layout (lighting.js:234-286): dims[0] x dims[1] columns over box's x, y, each with one probe per
    height above the terrain under it -- the highest Gaussian centre of the terrain parts in the column's cell, empty
    cells taking their filled neighbours' mean ring by ring, else the box floor.  The terrain parts are the named
    ones, else the static part (flags bit 0) with the widest x-y footprint of its Gaussian centres (sampled every
    max(1, n >> 12)).  volumes: the asset's named (part, dims) volumes, else probe_volumes picks them."""
    dims = [int(dims[0]), int(dims[1]), len(heights)]
    if dims[0] * dims[1] > 1024 or dims[2] > 16:
        raise ValueError("probe terrain layout: at most 1024 columns and 16 levels")
    step = [(box[k][1] - box[k][0]) / dims[k] for k in (0, 1)]
    lo = [box[0][0] + step[0] / 2, box[1][0] + step[1] / 2, 0.0]
    mu = gaussians["mu"].astype(np.float64)
    tp = list(terrain_parts or [])
    if not tp:
        best, best_a = -1, -1.0
        for i, p in enumerate(parts):
            if (int(p["flags"]) & 1) == 0:   # movable
                continue
            g0, g1 = int(p["g_lo"]), int(p["g_hi"])
            if g1 <= g0:
                continue
            s = mu[g0:g1:max(1, (g1 - g0) >> 12)]
            a = (s[:, 0].max() - s[:, 0].min()) * (s[:, 1].max() - s[:, 1].min())
            if a > best_a:
                best, best_a = i, a
        tp = [best] if best >= 0 else []
    ground = np.full(dims[0] * dims[1], -np.inf)
    for i in tp:
        g0, g1 = int(parts[i]["g_lo"]), int(parts[i]["g_hi"])
        x, y, z = mu[g0:g1, 0], mu[g0:g1, 1], mu[g0:g1, 2]
        ci = np.floor((x - box[0][0]) / step[0]).astype(np.int64)
        cj = np.floor((y - box[1][0]) / step[1]).astype(np.int64)
        ok = (ci >= 0) & (cj >= 0) & (ci < dims[0]) & (cj < dims[1])
        np.maximum.at(ground, ci[ok] * dims[1] + cj[ok], z[ok])
    for _ in range(dims[0] + dims[1]):
        if not np.isinf(ground).any():
            break
        prev = ground.copy()
        for i in range(dims[0]):
            for j in range(dims[1]):
                if prev[i * dims[1] + j] != -np.inf:
                    continue
                s, c = 0.0, 0
                for di, dj in ((1, 0), (-1, 0), (0, 1), (0, -1)):
                    a, b = i + di, j + dj
                    if a < 0 or b < 0 or a >= dims[0] or b >= dims[1] or prev[a * dims[1] + b] == -np.inf:
                        continue
                    s += prev[a * dims[1] + b]
                    c += 1
                if c:
                    ground[i * dims[1] + j] = s / c
    ground[np.isinf(ground)] = box[2][0]
    return {"terrain": True, "dims": dims, "lo": lo, "step": [step[0], step[1], 0.0], "levels": list(heights),
            "ground": ground.astype(np.float32), "tmax": _tmax(box, environment),
            "vols": probe_volumes(parts, box, tp, volumes)}


def probe_volumes(parts: np.ndarray, box, terrain_parts, named=None) -> list:
    """probeVolumes (lighting.js:289-314): the named (part, dims) volumes, else every static part but the terrain
    whose bounding radius is 1 m to a quarter of the scene's half-diagonal (a tree, a rock, a house; not the ground or
    a carpet of grass), a grid of about 1.2 m spacing, 2-6 per axis.  Parts 0-31 only."""
    if named is not None:
        return [(int(q), *[int(v) for v in d]) for q, d in named if q < 32]
    half = 0.5 * math.hypot(*[b - a for a, b in box])
    out = []
    for q, p in enumerate(parts):
        if q >= 32 or q in terrain_parts or (int(p["flags"]) & 1) == 0:
            continue
        R = float(p["bound"][3])
        if R < 1.0 or R > 0.25 * half:
            continue
        n = max(2, min(6, math.floor(R / 1.2 + 0.5)))   # Math.round
        out.append((q, n, n, n))
    return out


def for_scene(scene) -> dict:
    """The layout of one of splatlight_gb300.scene's synthetic scenes: the Cornell-like room's walls are the box
    [-1, 1]^3; the hill-like scene is terrain over its Gaussians' bounds, with an environment (its sky)."""
    if scene.name.startswith("cornell"):
        return room_layout(((-1.0, 1.0), (-1.0, 1.0), (-1.0, 1.0)), environment=scene.sky_sh is not None)
    mu = scene.gaussians["mu"].astype(np.float64)
    box = tuple((float(mu[:, k].min()), float(mu[:, k].max())) for k in range(3))
    return terrain_layout(scene.gaussians, scene.parts, box, environment=scene.sky_sh is not None)
