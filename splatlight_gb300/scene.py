"""Seeded synthetic scenes in the gs-runtime layout (Gaussians, parts, leaf nodes, V grids, materials) plus host
emitter records and a camera.  They stand in for the reference's shipped assets at the sizes and value distributions
of the benchmark configurations:

* ``cornell``: a Cornell-box-like room: 70% of the Gaussians on five walls of [-1, 1]^3 (normal jitter N(0, 0.01)),
  30% inside two axis-aligned boxes; log-scales N(-4, 0.5); 8 emissive Gaussians (Le ~ U[1, 10]) under the ceiling.
* ``hill``: 80% on the heightfield z = 0.3 sin(x) cos(y) over [-10, 10]^2, 20% on a trunk cylinder (r 0.3, h 3) and in
  an ellipsoidal canopy (radii 2, 2, 1.5); log-scales N(-3.5, 0.6); a sun along (0.3, 0.2, 0.93); 32 emitters.

Common to both: unit quaternions uniform on S^3; opacity o = sigmoid(N(0, 1.5)) mapped to the reference's extinction
scale kappa = -ln(1 - o) / (sqrt(2 pi) s_x), so a face-on view along the short axis peaks at alpha = o
(shaders/project.wgsl:237-261 tau0 = kappa sqrt(2 pi / q)); albedo U[0, 1]^3; 32 materials with roughness U[0.1, 1]
(flake (1, r^2, r^2), src/lighting.js:1170-1178) and specular weight k = 0.25 so roughness matters.
Leaf nodes follow runtime/wgsl/common.wgsl:12-19 (mean, radius 3 max(s), rest-frame C^-1, kappa, smax, the SGGX
S-hat R diag(1, (sx/sy)^2, (sx/sz)^2) R^T, part); V grids are all 255 (no own-part occlusion).
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from .structs import GAUSSIAN, MATERIAL, NODE, PART, VGRID


@dataclasses.dataclass
class Sun:
    direction: tuple
    irradiance: tuple
    angular_std: float  # radians
    casts_shadows: bool = True


@dataclasses.dataclass
class Scene:
    name: str
    gaussians: np.ndarray      # GAUSSIAN records, part rest frame
    parts: np.ndarray          # PART records
    nodes: np.ndarray          # NODE leaves, one per Gaussian
    vgrid: np.ndarray          # VGRID per Gaussian
    materials: np.ndarray      # MATERIAL (32)
    emitters: np.ndarray       # GAUSSIAN records in world space, albedo = Le
    eye: tuple
    target: tuple
    up: tuple
    fov_deg: float
    width: int
    height: int
    far: float = 50.0
    sun: Sun | None = None
    sky_ambient: float = 0.0
    shadow_res: int = 1024     # emitter-light shadow map resolution
    sun_res: int = 2048        # sun map resolution
    extra_lights: tuple = ()   # distant lights after the sun: (direction, angular std, irradiance, casts shadows)
    # the emitter set's EmitParams (src/lighting.js:657-673): overlap scale, one-sided emission about `normal`, the
    # part whose Gaussians are the emitters (shadow lookups skip it), and whether the emitter records are drawn in
    # slots after the scene (host emitters) or are the scene's own Gaussians (an asset's emissive part)
    emit_scale: float = 1.0
    emit_one_sided: bool = False
    emit_normal: tuple = (0.0, 0.0, 1.0)
    emit_skip_part: int = 0xFFFFFFFF
    emit_drawn: bool = True
    tree_nodes: np.ndarray | None = None   # an asset's whole tree (leaves first) and its children lists, for LOD
    kids: np.ndarray | None = None
    sky_sh: np.ndarray | None = None       # the environment's sky, 16 real SH coefficients (bands 0-3) x rgb
    probes: dict | None = None             # an asset's probe lattice (probes.room_layout / terrain_layout)

    @property
    def count(self) -> int:
        return len(self.gaussians)

    @property
    def n_drawn_emitters(self) -> int:
        """The emitter count a RenderFrame carries (palette[3].y): the host emitters drawn after the scene."""
        return len(self.emitters) if self.emit_drawn else 0

    def distant_lights(self) -> list:
        """[(direction, angular std, irradiance, casts shadows)]: the sun, then any further distant lights."""
        out = []
        if self.sun is not None:
            out.append((self.sun.direction, self.sun.angular_std, self.sun.irradiance, self.sun.casts_shadows))
        return out + list(self.extra_lights)


def _quats(rng, n):
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    return q


def quat_rot(q):
    """Rotation matrices (n, 3, 3), M[:, r, c], of unit quaternions (x, y, z, w) (shaders/common.wgsl:83-89)."""
    x, y, z, w = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    R = np.empty((len(q), 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z)
    R[:, 1, 0] = 2 * (x * y + w * z)
    R[:, 2, 0] = 2 * (x * z - w * y)
    R[:, 0, 1] = 2 * (x * y - w * z)
    R[:, 1, 1] = 1 - 2 * (x * x + z * z)
    R[:, 2, 1] = 2 * (y * z + w * x)
    R[:, 0, 2] = 2 * (x * z + w * y)
    R[:, 1, 2] = 2 * (y * z - w * x)
    R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return R


def _records(rng, mu, log_mean, log_std, part, n_materials=32):
    n = len(mu)
    g = np.zeros(n, dtype=GAUSSIAN)
    s = np.sort(np.exp(rng.normal(log_mean, log_std, (n, 3))), axis=1)
    o = 1.0 / (1.0 + np.exp(-rng.normal(0.0, 1.5, n)))
    o = np.clip(o, 1e-4, 0.999)
    g["mu"] = mu
    g["quat"] = _quats(rng, n)
    g["scale"] = s
    g["kappa"] = -np.log1p(-o) / (math.sqrt(2 * math.pi) * s[:, 0])
    g["part_surface"] = part
    g["albedo"] = rng.uniform(0.0, 1.0, (n, 3))
    g["flags"] = rng.integers(0, n_materials, n)
    return g


def _materials(rng, n=32, shine=0.25):
    m = np.zeros(n, dtype=MATERIAL)
    r = rng.uniform(0.1, 1.0, n)
    a = np.maximum(r * r, 1e-4)
    m["flake"] = np.stack([np.ones(n), a, a], axis=1)
    m["phase_samples"] = np.where(r <= 0.011, 0, 8)
    m["vfloor"] = 0.02
    m["flags"] = 8 if shine > 0 else 0
    m["pad0"] = np.float16(shine).view(np.uint16)
    return m


def leaf_nodes(g: np.ndarray) -> np.ndarray:
    """Leaf Node records of Gaussians (runtime/wgsl/common.wgsl:12-19), float64 maths."""
    n = len(g)
    nd = np.zeros(n, dtype=NODE)
    R = quat_rot(g["quat"].astype(np.float64))
    s = g["scale"].astype(np.float64)
    C = np.einsum("nij,nj,nkj->nik", R, s * s, R)
    Ci = np.linalg.inv(C)
    sn = np.einsum("nij,nj,nkj->nik", R, np.stack([np.ones(n), (s[:, 0] / s[:, 1]) ** 2,
                                                     (s[:, 0] / s[:, 2]) ** 2], axis=1), R)
    nd["mean"] = g["mu"]
    nd["radius"] = 3.0 * s.max(axis=1)
    nd["cinv_diag"] = np.stack([Ci[:, 0, 0], Ci[:, 1, 1], Ci[:, 2, 2]], axis=1)
    nd["cinv_off"] = np.stack([Ci[:, 0, 1], Ci[:, 0, 2], Ci[:, 1, 2]], axis=1)
    nd["kappa"] = g["kappa"]
    nd["smax"] = s.max(axis=1)
    nd["sn_diag"] = np.stack([sn[:, 0, 0], sn[:, 1, 1], sn[:, 2, 2]], axis=1)
    nd["sn_off"] = np.stack([sn[:, 0, 1], sn[:, 0, 2], sn[:, 1, 2]], axis=1)
    nd["part"] = g["part_surface"] & 0xFFFF
    return nd


def _morton30(u: np.ndarray) -> np.ndarray:
    """30-bit Morton codes of points in [0, 1)^3 (n, 3)."""
    q = np.clip((u * 1024.0).astype(np.int64), 0, 1023)

    def spread(v):
        v = (v | (v << 16)) & 0x030000FF
        v = (v | (v << 8)) & 0x0300F00F
        v = (v | (v << 4)) & 0x030C30C3
        v = (v | (v << 2)) & 0x09249249
        return v
    return (spread(q[:, 0]) << 2) | (spread(q[:, 1]) << 1) | spread(q[:, 2])


def lod_tree(g: np.ndarray, parts: np.ndarray):
    """The scene's tree for screen-space LOD: one binary tree per part over its Gaussians, moment-matched (the tool that
    bakes the reference's asset trees is not part of the reference; this builds the same kind of tree for synthetic
    scenes).  Leaves are leaf_nodes(g), taken in Morton order of their means within the part; each level pairs
    neighbours (an odd one out moves up a level unchanged).  An internal node's mass (kappa sqrt(det C)) is its
    children's sum, its mean and covariance their mass-weighted moments, its radius bounds their spheres
    (|mu_child - mu| + R_child), float64.  Returns (nodes: G leaves then the internal nodes, kids, parts with
    ``root`` set; empty parts get root 0xFFFFFFFF)."""
    G = len(g)
    leaves = leaf_nodes(g)
    R = quat_rot(g["quat"].astype(np.float64))
    sc = g["scale"].astype(np.float64)
    cap = max(2 * G, 1)
    cov = np.zeros((cap, 3, 3))
    mean = np.zeros((cap, 3))
    mass = np.zeros(cap)
    rad = np.zeros(cap)
    part_of = np.zeros(cap, np.int64)
    cov[:G] = np.einsum("nij,nj,nkj->nik", R, sc * sc, R)
    mean[:G] = g["mu"]
    mass[:G] = g["kappa"].astype(np.float64) * np.sqrt(np.linalg.det(cov[:G]))
    rad[:G] = leaves["radius"]
    part_of[:G] = g["part_surface"] & 0xFFFF
    # the SGGX S-hat of an internal node: its children's, mass-weighted (the shadow splats of the motion-blur cut read
    # it; the reference's asset trees carry one baked by a tool outside the reference)
    sn = np.zeros((cap, 6))
    sn[:G, :3] = leaves["sn_diag"]
    sn[:G, 3:] = leaves["sn_off"]
    kids_a, kids_b = [], []
    next_id = G
    parts = parts.copy()
    for p in range(len(parts)):
        idx = np.nonzero(part_of[:G] == p)[0]
        if len(idx) == 0:
            parts[p]["root"] = 0xFFFFFFFF
            continue
        mu = mean[idx]
        lo, hi = mu.min(axis=0), mu.max(axis=0)
        cur = idx[np.argsort(_morton30((mu - lo) / np.maximum(hi - lo, 1e-12) * 0.999999), kind="stable")]
        while len(cur) > 1:
            a, b = cur[0:len(cur) - 1:2], cur[1::2]
            ma, mb = mass[a], mass[b]
            m = ma + mb
            mu_n = (ma[:, None] * mean[a] + mb[:, None] * mean[b]) / m[:, None]
            da, db = mean[a] - mu_n, mean[b] - mu_n
            ids = np.arange(next_id, next_id + len(a))
            next_id += len(a)
            cov[ids] = (ma[:, None, None] * (cov[a] + da[:, :, None] * da[:, None, :]) +
                        mb[:, None, None] * (cov[b] + db[:, :, None] * db[:, None, :])) / m[:, None, None]
            rad[ids] = np.maximum(np.linalg.norm(da, axis=1) + rad[a], np.linalg.norm(db, axis=1) + rad[b])
            mass[ids] = m
            mean[ids] = mu_n
            sn[ids] = (ma[:, None] * sn[a] + mb[:, None] * sn[b]) / m[:, None]
            part_of[ids] = p
            kids_a.append(a)
            kids_b.append(b)
            cur = np.concatenate([ids, cur[-1:]]) if len(cur) % 2 else ids
        parts[p]["root"] = int(cur[0])
    n_int = next_id - G
    N = G + n_int
    nodes = np.zeros(N, dtype=NODE)
    nodes[:G] = leaves
    if n_int:
        c_i = cov[G:N]
        ci = np.linalg.inv(c_i)
        nodes["mean"][G:] = mean[G:N]
        nodes["radius"][G:] = rad[G:N]
        nodes["cinv_diag"][G:] = np.stack([ci[:, 0, 0], ci[:, 1, 1], ci[:, 2, 2]], axis=1)
        nodes["cinv_off"][G:] = np.stack([ci[:, 0, 1], ci[:, 0, 2], ci[:, 1, 2]], axis=1)
        nodes["kappa"][G:] = mass[G:N] / np.sqrt(np.linalg.det(c_i))
        nodes["smax"][G:] = np.sqrt(np.linalg.eigvalsh(c_i)[:, 2])
        nodes["part"][G:] = part_of[G:N]
        nodes["sn_diag"][G:] = sn[G:N, :3]
        nodes["sn_off"][G:] = sn[G:N, 3:]
        k = np.arange(n_int, dtype=np.uint32)
        nodes["child_lo"][G:] = 2 * k
        nodes["child_hi"][G:] = 2 * k + 2
    kids = np.empty(2 * n_int, np.uint32)
    if n_int:
        kids[0::2] = np.concatenate(kids_a)
        kids[1::2] = np.concatenate(kids_b)
    # depths, top-down: parents are made after their children
    depth = np.zeros(N, np.int64)
    parent = np.full(N, -1, np.int64)
    if n_int:
        parent[kids[0::2]] = np.arange(G, N)
        parent[kids[1::2]] = np.arange(G, N)
    # a node's depth = its parent's + 1; parents have larger ids, so sweep ids downward level by level
    pending = np.nonzero(parent >= 0)[0]
    while len(pending):
        depth[pending] = depth[parent[pending]] + 1
        # re-sweep until stable (each pass fixes at least one more level)
        changed = depth[pending] != depth[parent[pending]] + 1
        pending = pending[changed] if changed.any() else pending[:0]
    nodes["depth"] = depth
    return nodes, kids, parts


def _parts(g: np.ndarray, n_parts: int) -> np.ndarray:
    p = np.zeros(n_parts, dtype=PART)
    ident = np.array([1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0], dtype=np.float32)
    part = g["part_surface"] & 0xFFFF
    for k in range(n_parts):
        idx = np.nonzero(part == k)[0]
        p[k]["xf"] = ident
        p[k]["xf_prev"] = ident
        p[k]["flags"] = 1  # static
        if len(idx):
            mu = g["mu"][idx].astype(np.float64)
            c = mu.mean(axis=0)
            rad = np.sqrt(((mu - c) ** 2).sum(axis=1)).max() + 3 * float(g["scale"][idx].max())
            p[k]["bound"] = [*c, rad]
            p[k]["g_lo"], p[k]["g_hi"] = idx.min(), idx.max() + 1
    return p


def _emitters(rng, pos, log_mean=-3.0, log_std=0.2):
    n = len(pos)
    e = np.zeros(n, dtype=GAUSSIAN)
    s = np.sort(np.exp(rng.normal(log_mean, log_std, (n, 3))), axis=1)
    e["mu"] = pos
    e["quat"] = _quats(rng, n)
    e["scale"] = s
    e["kappa"] = 3.0 / (math.sqrt(2 * math.pi) * s[:, 0])   # optical depth 3 along the short axis
    e["albedo"] = rng.uniform(1.0, 10.0, n)[:, None] * np.ones(3)
    e["part_surface"] = 0xFFFF
    e["flags"] = 254
    return e


def _finish(name, g, n_parts, rng, emitters, **kw) -> Scene:
    order = np.argsort(g["part_surface"] & 0xFFFF, kind="stable")
    g = g[order]
    vg = np.zeros(len(g), dtype=VGRID)
    vg["w"] = 0xFFFFFFFF
    return Scene(name=name, gaussians=g, parts=_parts(g, n_parts), nodes=leaf_nodes(g), vgrid=vg,
                 materials=_materials(rng), emitters=emitters, **kw)


def cornell(n: int = 65536, seed: int = 0, width: int = 512, height: int = 512, n_emit: int = 8) -> Scene:
    rng = np.random.default_rng(seed)
    n_wall = int(round(0.7 * n))
    n_box = n - n_wall
    # walls (camera looks down -z into the open +z face): back z=-1, floor y=-1, ceiling y=+1, left x=-1, right x=+1
    wall = rng.integers(0, 5, n_wall)
    uv = rng.uniform(-1, 1, (n_wall, 2))
    jit = rng.normal(0, 0.01, n_wall)
    mu_w = np.zeros((n_wall, 3))
    axis = np.array([2, 1, 1, 0, 0])[wall]
    sign = np.array([-1, -1, 1, -1, 1])[wall]
    other = np.array([[0, 1], [0, 2], [0, 2], [1, 2], [1, 2]])[wall]
    mu_w[np.arange(n_wall), other[:, 0]] = uv[:, 0]
    mu_w[np.arange(n_wall), other[:, 1]] = uv[:, 1]
    mu_w[np.arange(n_wall), axis] = sign + jit
    # two axis-aligned boxes on the floor
    which = rng.integers(0, 2, n_box)
    centre = np.array([[-0.35, -0.7, -0.3], [0.35, -0.4, -0.55]])[which]
    half = np.array([[0.3, 0.3, 0.3], [0.28, 0.6, 0.28]])[which]
    mu_b = centre + rng.uniform(-1, 1, (n_box, 3)) * half
    g_w = _records(rng, mu_w, -4.0, 0.5, wall)
    g_b = _records(rng, mu_b, -4.0, 0.5, 5 + which)
    g = np.concatenate([g_w, g_b])
    epos = np.stack([rng.uniform(-0.5, 0.5, n_emit), rng.uniform(0.85, 0.95, n_emit), rng.uniform(-0.5, 0.5, n_emit)], 1)
    em = _emitters(rng, epos)
    return _finish("cornell", g, 7, rng, em, eye=(0.0, 0.0, 3.5), target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0),
                   fov_deg=60.0, width=width, height=height, far=50.0, shadow_res=1024)


# the hill-like scene's sky for the probe bounce (real SH bands 0-3, rgb): a blue sky brighter toward the zenith and
# toward the sun's side, dim below the horizon (radiance ~0.35 at the zenith, ~0.1 at the horizon)
HILL_SKY = np.zeros((16, 3), np.float32)
HILL_SKY[0] = (0.55, 0.65, 0.85)
HILL_SKY[2] = (0.30, 0.34, 0.42)     # z
HILL_SKY[1] = (0.03, 0.03, 0.02)     # y
HILL_SKY[3] = (0.05, 0.045, 0.03)    # x
HILL_SKY[6] = (0.06, 0.07, 0.09)     # 3 z^2 - 1


def hill(n: int = 1048576, seed: int = 1, width: int = 1920, height: int = 1080, n_emit: int = 32) -> Scene:
    rng = np.random.default_rng(seed)
    n_ground = int(round(0.8 * n))
    n_trunk = int(round(0.05 * n))
    n_canopy = n - n_ground - n_trunk
    xy = rng.uniform(-10, 10, (n_ground, 2))
    z = 0.3 * np.sin(xy[:, 0]) * np.cos(xy[:, 1]) + rng.normal(0, 0.005, n_ground)
    mu_g = np.column_stack([xy, z])
    ang = rng.uniform(0, 2 * math.pi, n_trunk)
    mu_t = np.column_stack([0.3 * np.cos(ang), 0.3 * np.sin(ang), rng.uniform(0, 3, n_trunk)])
    # canopy: uniform in the ellipsoid (radii 2, 2, 1.5) centred above the trunk
    d = rng.standard_normal((n_canopy, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rad = rng.uniform(0, 1, n_canopy) ** (1 / 3)
    mu_c = d * rad[:, None] * np.array([2.0, 2.0, 1.5]) + np.array([0.0, 0.0, 4.0])
    g = np.concatenate([_records(rng, mu_g, -3.5, 0.6, 0), _records(rng, mu_t, -3.5, 0.6, 1),
                        _records(rng, mu_c, -3.5, 0.6, 2)])
    exy = rng.uniform(-8, 8, (n_emit, 2))
    ez = 0.3 * np.sin(exy[:, 0]) * np.cos(exy[:, 1]) + rng.uniform(0.3, 2.0, n_emit)
    em = _emitters(rng, np.column_stack([exy, ez]), log_mean=-2.5)
    sd = np.array([0.3, 0.2, 0.93])
    sd /= np.linalg.norm(sd)
    return _finish("hill", g, 3, rng, em, eye=(0.0, -14.0, 5.0), target=(0.0, 0.0, 1.5), up=(0.0, 0.0, 1.0),
                   fov_deg=50.0, width=width, height=height, far=100.0,
                   sun=Sun(tuple(sd), (3.0, 2.9, 2.7), 0.5 * math.pi / 180.0), sky_ambient=0.2,
                   shadow_res=1024, sun_res=2048, sky_sh=HILL_SKY.copy())


def with_tree(scene: Scene):
    """(scene, (nodes, kids)): the scene with its parts' tree roots set and its tree -- an asset's own, else
    lod_tree's -- for the probe gather and the motion-blur cut."""
    if scene.tree_nodes is not None and scene.kids is not None:
        return scene, (scene.tree_nodes, scene.kids)
    nodes, kids, parts = lod_tree(scene.gaussians, scene.parts)
    return dataclasses.replace(scene, parts=parts), (nodes, kids)


def subset(scene: Scene, n: int, seed: int = 123) -> Scene:
    """A random subset of n Gaussians (parity cases at oracle-friendly sizes); parts and nodes follow."""
    rng = np.random.default_rng(seed)
    idx = np.sort(rng.choice(scene.count, size=min(n, scene.count), replace=False))
    g = scene.gaussians[idx]
    return dataclasses.replace(scene, gaussians=g, parts=_parts(g, len(scene.parts)), nodes=scene.nodes[idx],
                               vgrid=scene.vgrid[idx])
