"""The probe bounce's CPU side: the restatement's tables and half rounding, the probe layouts (src/lighting.js
probeLayout), properties of the restated bounce that hold whatever the scene (no light and no sky: no bounce;
an open sky: the upward probe rays carry the sky's radiance times their transmittance; the same bits on any thread
count), and the sender cut's (its marks down the tree and against every lattice probe's gather rule, the node V
grids, the per-leaf path when nothing can be cut, and how close it sends to every leaf, on the reference's assets
too)."""
import dataclasses
import math
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

from splatlight_gb300 import probes as PR  # noqa: E402
from splatlight_gb300 import scene as S  # noqa: E402


@pytest.fixture(scope="module")
def orc():
    from oracle import oracle as O
    O.build()
    return O


def test_half_rounding_matches_ieee(orc):
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.normal(0, 1, 3000), rng.normal(0, 1e4, 1000), 2.0 ** rng.uniform(-30, -10, 1000),
                        [0.0, -0.0, 65504.0, 65519.0, 65520.0, 1e9, np.inf, -np.inf, 2 ** -25, 2 ** -24, 3 * 2 ** -26]])
    x = x.astype(np.float32)
    with np.errstate(over="ignore"):
        ref = x.astype(np.float16).view(np.uint16).astype(np.uint32)
    assert np.array_equal(orc.f32_to_f16(x), ref)


def test_sh2_fit_is_a_left_inverse(orc):
    d, p = orc.bounce_tables()
    assert np.allclose(np.linalg.norm(d.astype(np.float64), axis=1), 1.0, atol=1e-6)
    x, y, z = (d[:, k].astype(np.float64) for k in range(3))
    A = np.stack([np.full(14, 0.282095), 0.488603 * y, 0.488603 * z, 0.488603 * x, 1.092548 * x * y,
                  1.092548 * y * z, 0.315392 * (3 * z * z - 1), 1.092548 * x * z, 0.546274 * (x * x - y * y)], 1)
    assert np.abs(p.astype(np.float64) @ A - np.eye(9)).max() < 1e-6


def test_room_layout():
    lay = PR.room_layout(((-1.0, 1.0), (0.0, 2.0), (0.0, 2.0)))
    assert lay["dims"] == [8, 8, 8] and not lay["terrain"] and lay["tmax"] == 6.0
    assert np.allclose(lay["lo"], [-0.875, 0.125, 0.125])
    assert np.allclose(lay["step"], [1.75 / 7] * 3)
    assert np.allclose(lay["levels"], 0.125 + np.arange(8) * 1.75 / 7)
    env = PR.room_layout(((-1.0, 1.0), (0.0, 2.0), (0.0, 2.0)), environment=True)
    assert env["tmax"] == 6.0   # the diagonal (3.46 m) is shorter than TMAX


def test_terrain_layout_ground_and_fill():
    g = np.zeros(3, dtype=S.GAUSSIAN)
    g["mu"] = [[0.1, 0.1, 1.0], [0.2, 0.3, 2.0], [3.5, 3.5, 5.0]]
    parts = np.zeros(1, dtype=S.PART)
    parts[0]["g_lo"], parts[0]["g_hi"], parts[0]["flags"] = 0, 3, 1
    box = ((0.0, 4.0), (0.0, 4.0), (-1.0, 6.0))
    lay = PR.terrain_layout(g, parts, box, dims=(4, 4), heights=(0.5, 2.0))
    gr = lay["ground"].reshape(4, 4)
    assert lay["dims"] == [4, 4, 2] and lay["terrain"]
    assert gr[0, 0] == 2.0 and gr[3, 3] == 5.0       # the highest centre in each filled cell
    assert gr[0, 1] == 2.0 and gr[1, 0] == 2.0       # first ring: the filled neighbours' mean
    assert gr[2, 3] == 5.0 and gr[3, 2] == 5.0
    assert np.isfinite(gr).all()
    assert np.isclose(lay["tmax"], max(6.0, math.hypot(4.0, 4.0, 7.0)))
    assert lay["lo"] == [0.5, 0.5, 0.0] and lay["step"] == [1.0, 1.0, 0.0]


def _small_hill(**kw):
    s = S.hill(6000, seed=4, width=64, height=64, n_emit=4)
    s = dataclasses.replace(s, sky_ambient=0.0, shadow_res=64, sun_res=64, **kw)
    return S.with_tree(s)


def test_no_light_no_sky_no_bounce(orc):
    s, tree = _small_hill(emitters=np.zeros(0, dtype=S.GAUSSIAN), sun=None)
    lit = orc.lighting(s, threads=4)
    b = orc.Bounce(s, tree, lit, PR.for_scene(s), sky_sh=None)
    for _ in range(3):
        st = b.step(s.eye, threads=4)
    assert not st["lo_b"].any() and not st["probe_sh"].any() and not st["lo_dir"].any()


def test_open_sky_reaches_the_probes(orc):
    """A constant sky of radiance L (band 0 only): the upward rays of the probes above the hill leave the scene, and
    each carries L times what it crossed (exactly L where it crossed nothing)."""
    s, tree = _small_hill(emitters=np.zeros(0, dtype=S.GAUSSIAN), sun=None)
    sky = np.zeros((16, 3), np.float32)
    L = np.array([0.3, 0.5, 0.7], np.float32)
    sky[0] = L / np.float32(0.282095)
    b = orc.Bounce(s, tree, orc.lighting(s, threads=4), PR.for_scene(s), sky_sh=sky)
    st = b.step(s.eye, threads=4)
    pd = st["probe_data"]
    up = pd[:, :16, :]                     # the top elevation row of cells: straight up, above the scene
    open_rays = up[..., 3] < 0             # no hit took the transmittance below 1/2
    assert open_rays.mean() > 0.5
    col = up[..., :3][open_rays]
    assert np.all(col <= L * (1 + 1e-5))   # the sky times the ray's transmittance (<= 1)
    assert np.allclose(col.max(axis=0), L, rtol=1e-5)


def test_probe_volumes_rule():
    """probeVolumes (lighting.js:289-314): static non-terrain parts with a bounding radius of 1 m to a quarter of the
    scene's half-diagonal get a grid of about 1.2 m spacing, 2-6 per axis (Math.round); named volumes win."""
    parts = np.zeros(5, dtype=S.PART)
    parts["flags"] = [1, 1, 1, 0, 1]
    parts["bound"][:, 3] = [30.0, 2.9, 0.5, 3.0, 7.8]
    box = ((-50.0, 50.0), (-50.0, 50.0), (0.0, 10.0))     # half-diagonal 71: the quarter is 17.8 m
    vols = PR.probe_volumes(parts, box, terrain_parts=[0])
    assert vols == [(1, 2, 2, 2), (4, 6, 6, 6)]              # 2.9 / 1.2 rounds to 2; 7.8 / 1.2 = 6.5 -> 7, capped at 6
    assert PR.probe_volumes(parts, box, [0], named=[(2, (3, 4, 5))]) == [(2, 3, 4, 5)]


# ---- the sender cut (bounce.wgsl sc_select .. node_cut; the reference's default level of detail for the senders)

def _node_vgrids_numpy(nodes, G, kids, vgrid):
    """src/lod.js nodeGaussians' V grids in numpy: masses in float64, each cell kept as float32, half up, <= 255."""
    N = len(nodes)
    a = nodes["cinv_diag"].astype(np.float64)
    o = nodes["cinv_off"].astype(np.float64)
    det = (a[:, 0] * (a[:, 1] * a[:, 2] - o[:, 2] * o[:, 2]) - o[:, 0] * (o[:, 0] * a[:, 2] - o[:, 2] * o[:, 1])
           + o[:, 1] * (o[:, 0] * o[:, 2] - a[:, 1] * o[:, 1]))
    mass = np.zeros(N)
    mass[:G] = nodes["kappa"][:G].astype(np.float64) / np.sqrt(np.maximum(det[:G], 1e-30))
    V = np.zeros((N, 128), np.float32)
    V[:G] = np.ascontiguousarray(vgrid).view(np.uint8).reshape(G, 128)
    order = sorted(range(G, N), key=lambda n: -int(nodes["depth"][n]))   # stable: index order within a depth
    for n in order:
        ch = kids[nodes["child_lo"][n]:nodes["child_hi"][n]]
        m = 0.0
        for c in ch:
            m += mass[c]
        mass[n] = m
        for c in ch:
            V[n] = (V[n].astype(np.float64) + (mass[c] / max(m, 1e-30)) * V[c].astype(np.float64)).astype(np.float32)
    return np.minimum(255.0, np.floor(V[G:].astype(np.float64) + 0.5)).astype(np.uint8)


def test_node_vgrids_match_numpy(orc):
    s, tree = S.with_tree(S.subset(S.cornell(), 1500))
    nodes, kids = tree
    got = orc.lod_vgrids(nodes, s.count, kids, s.vgrid).view(np.uint8).reshape(-1, 128)
    ref = _node_vgrids_numpy(nodes, s.count, kids, s.vgrid)
    assert got.shape == ref.shape and np.array_equal(got, ref)
    assert got.max() <= 255 and got.astype(np.int64).sum() > 0


def _cut_scene(name):
    if name == "hill":
        s = S.hill(6000, seed=4, width=64, height=64, n_emit=4)
    else:
        s = S.subset(S.cornell(), 8000)
    s = dataclasses.replace(s, shadow_res=64, sun_res=64)
    return S.with_tree(s)


@pytest.mark.parametrize("name", ["hill", "cornell"])
def test_sender_cut_marks(orc, name):
    """Under an OPEN node every child is marked, under any other mark none is; every lattice probe's gather uses each
    cut node whole (distance from its gather centre less the block margin above theta smax)."""
    s, tree = _cut_scene(name)
    lit = orc.lighting(s, threads=4)
    lay = PR.for_scene(s)
    b = orc.Bounce(s, tree, lit, lay, sky_sh=s.sky_sh, sender_cut=True)
    st = b.step(s.eye, threads=4)
    fl, tn, kids, G = st["sc_flag"], b.nodes, b.kids, s.count
    counts = np.bincount(fl, minlength=4)
    assert counts[2] > 0 and counts[3] > 0 and counts[1] > 0     # cut nodes, cut leaves, open nodes
    assert (fl[:G] != 2).all() and (fl[G:] != 3).all()           # leaves are never NODE, internal nodes never LEAF
    for n in range(G, len(tn)):
        ch = kids[tn["child_lo"][n]:tn["child_hi"][n]]
        assert ((fl[ch] != 0) if fl[n] == 1 else (fl[ch] == 0)).all()
    d, lo, step = lay["dims"], np.array(lay["lo"]), np.array(lay["step"])
    ii, jj, kk = np.meshgrid(np.arange(d[0]), np.arange(d[1]), np.arange(d[2]), indexing="ij")
    if lay["terrain"]:
        cen = np.stack([lo[0] + step[0] * ii, lo[1] + step[1] * jj,
                        lay["ground"].reshape(d[0], d[1])[ii, jj] + np.array(lay["levels"])[kk]], -1)
        brad = 0.0
    else:
        cen = lo + step * (2 * (np.stack([ii, jj, kk], -1) // 2) + 0.5)
        brad = 0.5 * np.linalg.norm(step)
    cen = cen.reshape(-1, 3)
    cut = np.nonzero(fl == 2)[0]
    dmin = np.array([np.linalg.norm(cen - m, axis=1).min() for m in tn["mean"][cut].astype(np.float64)]) - brad
    assert (dmin > 4.0 * tn["smax"][cut]).all()


def test_sender_cut_with_nothing_to_cut_is_the_exact_path(orc):
    """With every node too large for any probe to use whole, the cut is every leaf under open nodes and the frame
    equals the per-leaf path bit for bit."""
    s, (nodes, kids) = _cut_scene("hill")
    nodes = nodes.copy()
    nodes["smax"][s.count:] = 1e9
    lit = orc.lighting(s, threads=4)
    lay = PR.for_scene(s)
    ex = orc.Bounce(s, (nodes, kids), lit, lay, sky_sh=s.sky_sh)
    sc = orc.Bounce(s, (nodes, kids), lit, lay, sky_sh=s.sky_sh, sender_cut=True)
    for f in range(3):
        a, b = ex.step(s.eye, threads=4), sc.step(s.eye, threads=4)
    assert np.bincount(b["sc_flag"], minlength=4)[2] == 0
    for k in ("probe_data", "probe_sh", "lo_dir", "lo_b", "node_sh"):
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("name", ["hill", "cornell"])
def test_sender_cut_is_close_to_the_exact_path(orc, name):
    """The cut approximates what the leaves send: after a few frames the bounce toward the eye is within 3% of the
    per-leaf path in the mean and 10% of its largest value anywhere."""
    s, tree = _cut_scene(name)
    lit = orc.lighting(s, threads=4)
    lay = PR.for_scene(s)
    ex = orc.Bounce(s, tree, lit, lay, sky_sh=s.sky_sh)
    sc = orc.Bounce(s, tree, lit, lay, sky_sh=s.sky_sh, sender_cut=True)
    for f in range(4):
        a, b = ex.step(s.eye, threads=4)["lo_b"][:, 0, :3].copy(), sc.step(s.eye, threads=4)["lo_b"][:, 0, :3]
    assert a.mean() > 0
    assert (np.abs(b.mean(0) - a.mean(0)) <= 0.03 * a.mean(0)).all()
    assert np.abs(b - a).max() <= 0.1 * a.max()


@pytest.mark.parametrize("name", ["cornell_sdf_room_plain_bin", "hill_lite_bin"])
def test_sender_cut_on_the_reference_assets(orc, name):
    """With the reference's own baked trees and V grids the cut sends what the leaves send: once the probes have
    settled (8 frames) the mean bounce toward the eye is within 2% of the per-leaf path, per channel."""
    p = ROOT / "tests" / "golden" / "assets" / name
    if not (p / "asset.json").exists():
        pytest.skip("reference assets not copied (tests/golden/copy_assets.py)")
    from splatlight_gb300 import asset as A
    s = A.asset_scene(A.load_asset(p), width=64, height=64)
    s, tree = S.with_tree(s)
    lit = orc.lighting(s, threads=8)
    ex = orc.Bounce(s, tree, lit, s.probes, sky_sh=s.sky_sh)
    sc = orc.Bounce(s, tree, lit, s.probes, sky_sh=s.sky_sh, sender_cut=True)
    for f in range(8):
        a, b = ex.step(s.eye, threads=8)["lo_b"][:, 0, :3].copy(), sc.step(s.eye, threads=8)["lo_b"][:, 0, :3]
    assert (np.bincount(sc.state["sc_flag"], minlength=4)[2:] > 0).all()
    assert (np.abs(b.mean(0) - a.mean(0)) <= 0.02 * a.mean(0)).all()


@pytest.mark.parametrize("cut", [False, True])
def test_restated_bounce_is_independent_of_the_thread_count(orc, cut):
    """The restatement's parallel loops write disjoint outputs in a fixed order: one thread and four give the same
    bits, with and without the sender cut."""
    s, tree = _cut_scene("cornell")
    lit = orc.lighting(s, threads=4)
    lay = PR.for_scene(s)
    a = orc.Bounce(s, tree, lit, lay, sky_sh=s.sky_sh, sender_cut=cut)
    b = orc.Bounce(s, tree, lit, lay, sky_sh=s.sky_sh, sender_cut=cut)
    for f in range(2):
        x, y = a.step(s.eye, threads=1), b.step(s.eye, threads=4)
    for k in x:
        assert np.array_equal(x[k], y[k]), k
