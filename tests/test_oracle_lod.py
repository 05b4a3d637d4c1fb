"""The restated screen-space LOD (oracle/sl_oracle_lod.c; src/lod.js, runtime/wgsl/lod.wgsl) on CPU: the synthetic
tree covers every leaf once; the internal nodes' records reproduce their covariance; the cut covers every leaf
exactly once at any threshold and camera; node colours are the leaves' mass-weighted means; a cut of leaves only
renders exactly what the plain restated pipeline renders."""
import numpy as np
import pytest

from oracle import oracle
from splatlight_gb300 import camera, scene
from splatlight_gb300.lod import DRAW, frame_lod
from splatlight_gb300.scene import quat_rot
from splatlight_gb300.structs import VIEW_FLAT


@pytest.fixture(scope="module")
def tree():
    s = scene.subset(scene.hill(), 8000, seed=3)
    nodes, kids, parts = scene.lod_tree(s.gaussians, s.parts)
    s = scene.dataclasses.replace(s, parts=parts)
    return s, nodes, kids


def _leaves_under(nodes, kids, G, n):
    out, st = [], [n]
    while st:
        k = st.pop()
        if k < G:
            out.append(k)
        else:
            st.extend(int(kids[j]) for j in range(nodes["child_lo"][k], nodes["child_hi"][k]))
    return out


def test_tree_covers_every_leaf_once(tree):
    s, nodes, kids = tree
    G = len(s.gaussians)
    seen = np.zeros(G, int)
    for r in s.parts["root"]:
        if r != 0xFFFFFFFF:
            for leaf in _leaves_under(nodes, kids, G, int(r)):
                seen[leaf] += 1
    assert (seen == 1).all()


def test_node_records_reproduce_covariance(tree):
    s, nodes, kids = tree
    G = len(s.gaussians)
    recs = oracle.lod_records(s.gaussians, nodes, kids)
    assert len(recs) == len(nodes) - G
    R = quat_rot(recs["quat"].astype(np.float64))
    sc = recs["scale"].astype(np.float64)
    C = np.einsum("nij,nj,nkj->nik", R, sc * sc, R)
    nd = nodes[G:]
    ci = np.zeros((len(nd), 3, 3))
    ci[:, 0, 0], ci[:, 1, 1], ci[:, 2, 2] = nd["cinv_diag"].T
    ci[:, 0, 1] = ci[:, 1, 0] = nd["cinv_off"][:, 0]
    ci[:, 0, 2] = ci[:, 2, 0] = nd["cinv_off"][:, 1]
    ci[:, 1, 2] = ci[:, 2, 1] = nd["cinv_off"][:, 2]
    ref = np.linalg.inv(ci)
    err = np.abs(C - ref).max(axis=(1, 2)) / np.abs(ref).max(axis=(1, 2))
    assert err.max() < 1e-4
    assert np.all(np.diff(sc, axis=1) >= 0)              # scales ascending
    assert np.allclose(np.linalg.norm(recs["quat"], axis=1), 1.0, atol=1e-6)
    assert np.array_equal(recs["part_surface"], nd["part"] & 0xFFFF)


def _frame(s, eye, W=320, H=240):
    return camera.make_frame(eye, s.target, s.up, s.fov_deg, W, H, s.count, far=s.far, view_mode=VIEW_FLAT,
                             n_emit=len(s.emitters))


@pytest.mark.parametrize("thr", [0.5, 2.0, 8.0, 64.0])
@pytest.mark.parametrize("rule", [0, 1])
def test_cut_covers_every_leaf_once(tree, thr, rule):
    s, nodes, kids = tree
    G, N = len(s.gaussians), len(nodes)
    flags = np.zeros(N, np.uint32)
    for eye in ((0.0, -9.0, 4.0), (3.0, 2.0, 2.5)):       # the second frame starts from the first's flags
        f = frame_lod(_frame(s, eye), thr, N - G)
        oracle.lod_select(nodes, G, kids, s.parts, f, flags, size_rule=rule)
        drawn = np.nonzero(flags == DRAW)[0]
        cover = np.zeros(G, int)
        for n in drawn:
            for leaf in _leaves_under(nodes, kids, G, int(n)):
                cover[leaf] += 1
        assert (cover == 1).all(), (thr, rule, np.bincount(cover))


def test_threshold_extremes(tree):
    s, nodes, kids = tree
    G, N = len(s.gaussians), len(nodes)
    flags = np.zeros(N, np.uint32)
    oracle.lod_select(nodes, G, kids, s.parts, frame_lod(_frame(s, (0.0, -9.0, 4.0)), 1e-30, N - G), flags)
    assert (flags[:G] == DRAW).all() and not (flags[G:] == DRAW).any()
    oracle.lod_select(nodes, G, kids, s.parts, frame_lod(_frame(s, (0.0, -9.0, 4.0)), 1e30, N - G), flags)
    roots = {int(r) for r in s.parts["root"] if r != 0xFFFFFFFF}
    assert set(np.nonzero(flags == DRAW)[0].tolist()) == roots


def test_node_colour_is_mass_weighted_mean(tree):
    s, nodes, kids = tree
    G, N = len(s.gaussians), len(nodes)
    flags = np.zeros(N, np.uint32)
    oracle.lod_select(nodes, G, kids, s.parts, frame_lod(_frame(s, (0.0, -9.0, 4.0)), 4.0, N - G), flags)
    rng = np.random.default_rng(1)
    col = rng.uniform(0, 2, (G, 4)).astype(np.float32)
    nc = oracle.lod_colour(nodes, G, kids, flags, col, colour_all=True)
    d = nodes.astype(nodes.dtype)

    def mass(n):
        a, o = d["cinv_diag"][n].astype(np.float64), d["cinv_off"][n].astype(np.float64)
        det = a[0] * (a[1] * a[2] - o[2] ** 2) - o[0] * (o[0] * a[2] - o[2] * o[1]) + o[1] * (o[0] * o[2] - a[1] * o[1])
        return d["kappa"][n] / np.sqrt(max(det, 1e-30))
    for n in range(G, N, max(1, (N - G) // 50)):
        leaves = _leaves_under(nodes, kids, G, n)
        # the recursive mean of means weights each leaf by its mass (node mass = its children's sum, to rounding)
        w = np.array([mass(k) for k in leaves])
        ref = (w[:, None] * col[leaves, :3].astype(np.float64)).sum(0) / w.sum()
        assert np.allclose(nc[n - G, :3], ref, rtol=2e-3), n


def test_leaf_cut_renders_as_plain(tree):
    s, nodes, kids = tree
    G, N = len(s.gaussians), len(nodes)
    f = frame_lod(_frame(s, (0.0, -9.0, 4.0)), 1e-30, N - G)
    flags = np.zeros(N, np.uint32)
    oracle.lod_select(nodes, G, kids, s.parts, f, flags)
    recs = oracle.lod_records(s.gaussians, nodes, kids)
    ncol = np.zeros((N - G, 4), np.float32)
    a = oracle.render(s.gaussians, s.parts, f, emitters=s.emitters, lod=(flags, recs, ncol))
    f0 = f.copy()
    f0["lod"] = 0
    b = oracle.render(s.gaussians, s.parts, f0, emitters=s.emitters)
    assert np.array_equal(a["rgba"], b["rgba"]) and np.array_equal(a["ranges"], b["ranges"])
    assert np.array_equal(a["entries"], b["entries"])


def test_render_given_the_stable_order_is_render():
    """render_given_order (the counting sort's check) with the stable order reproduces the whole restated frame."""
    s = scene.subset(scene.cornell(), 5000)
    f = _frame(s, (0.3, 0.2, 3.2), W=160, H=120)
    a = oracle.render(s.gaussians, s.parts, f, emitters=s.emitters)
    b = oracle.render_given_order(s.gaussians, s.parts, f, a["order"], emitters=s.emitters)
    assert np.array_equal(a["rgba"], b["rgba"]) and np.array_equal(a["entries"], b["entries"])
    assert np.array_equal(a["ranges"], b["ranges"]) and np.array_equal(a["counts"], b["counts"])
