"""The CPU restatement (oracle/) against its committed golden fixtures and against independent float64 brute-force
checks: every kept fragment lies in a binned tile, the contributor counts equal a dense per-pixel evaluation of the
same keep test, the composite equals a float64 back-to-front "over" of the kept fragments, and the permutation is
the stable order of the 16-bit keys.  The reference ships no tests or vectors to pin against (parity unpinned)."""
from pathlib import Path

import numpy as np
import pytest

from splatlight_gb300 import camera, scene
from splatlight_gb300.structs import VIEW_FLAT, VIEW_OVERDRAW

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("name", sorted(p.stem for p in GOLDEN.glob("*.npz")))
def test_golden(orc, name):
    z = np.load(GOLDEN / f"{name}.npz")
    col = z["colour"] if len(z["colour"]) else None
    r = orc.render(z["gaussians"], z["parts"], z["frame"][0], emitters=z["emitters"], colour=col,
                   tile=tuple(z["tile"]), threads=2)
    for k in ("keys", "order", "ranges", "entries", "counts"):
        assert np.array_equal(r[k], z[k]), k
    assert np.abs(r["rgba"] - z["rgba"]).max() <= 1e-6


def test_sort16_stable(orc):
    rng = np.random.default_rng(0)
    k = rng.integers(0, 50, 20000).astype(np.uint32)
    k[rng.random(20000) < 0.1] = 0xFFFFFFFF
    o = orc.sort16(k)
    assert np.array_equal(o, np.argsort(k & 0xFFFF, kind="stable"))


def _dense(spl, order, visible, W, H):
    """float64 evaluation of every splat at every pixel, back to front."""
    ys, xs = np.mgrid[0:H, 0:W]
    px, py = xs + 0.5, ys + 0.5
    cnt = np.zeros((H, W), np.int64)
    rgb = np.zeros((H, W, 3))
    a = np.zeros((H, W))
    q_margin = np.zeros((H, W), bool)
    for p in range(visible):
        s = spl[order[p]]
        dx, dy = px - float(s["cx"]), py - float(s["cy"])
        lx = dx * float(s["g0x"]) + dy * float(s["g0y"])
        ly = dx * float(s["g1x"]) + dy * float(s["g1y"])
        q = lx * lx + ly * ly
        keep = q <= s["qcut"]
        near = np.abs(q - float(s["qcut"])) <= 1e-4 * max(float(s["qcut"]), 1.0)
        q_margin |= near
        cnt += keep
        al = np.where(keep, 1 - np.exp(-float(s["tau0"]) * np.exp(-0.5 * q)), 0.0)
        rgb = rgb * (1 - al[..., None]) + al[..., None] * np.asarray(s["rgb"], np.float64)
        a = a * (1 - al) + al
    return cnt, rgb, a, q_margin


@pytest.mark.parametrize("which", ["cornell", "hill"])
def test_binning_and_composite_against_dense(orc, which):
    s = scene.subset(scene.cornell() if which == "cornell" else scene.hill(n=65536), 700, seed=11)
    W, H = 80, 60
    f = camera.make_frame(s.eye, s.target, s.up, s.fov_deg, W, H, s.count, far=s.far, view_mode=VIEW_FLAT,
                          n_emit=len(s.emitters))
    keys, spl, vis = orc.project(s.gaussians, s.parts, f, emitters=s.emitters)
    r = orc.render(s.gaussians, s.parts, f, emitters=s.emitters, threads=1)
    order = r["order"]
    assert vis == r["visible"] and np.array_equal(keys, r["keys"])
    cnt, rgb, a, margin = _dense(spl, order, vis, W, H)
    # counts: identical away from fragments whose q sits on the keep boundary
    mism = (cnt != r["counts"]) & ~margin
    assert not mism.any()
    assert np.abs(rgb - r["rgba"][..., :3]).max() < 2e-4
    assert np.abs(a - r["rgba"][..., 3]).max() < 2e-4
    # every splat kept at a pixel is in that pixel's tile list
    ent, rg = r["entries"], r["ranges"]
    tiles_x = (W + 15) // 16
    ys, xs = np.nonzero(r["counts"])
    for y, x in zip(ys[:200], xs[:200]):
        t = (y // 16) * tiles_x + x // 16
        lst = set(ent[rg[t, 0]:rg[t, 1]].tolist())
        for p in range(vis):
            s_ = spl[order[p]]
            dx, dy = x + 0.5 - s_["cx"], y + 0.5 - s_["cy"]
            lx = dx * s_["g0x"] + dy * s_["g0y"]
            ly = dx * s_["g1x"] + dy * s_["g1y"]
            if lx * lx + ly * ly < 0.999 * s_["qcut"]:
                assert int(order[p]) in lst


def test_overdraw_counts_equal_kept_fragments(orc):
    s = scene.subset(scene.cornell(), 3000, seed=4)
    f = camera.make_frame(s.eye, s.target, s.up, s.fov_deg, 120, 90, s.count, far=s.far, view_mode=VIEW_OVERDRAW,
                          n_emit=len(s.emitters))
    r1 = orc.render(s.gaussians, s.parts, f, emitters=s.emitters, threads=1)
    r4 = orc.render(s.gaussians, s.parts, f, emitters=s.emitters, threads=4)
    assert np.array_equal(r1["counts"], r4["counts"]) and np.array_equal(r1["rgba"], r4["rgba"])
    # each tile list has the splats of its tile in sort order
    pos = np.empty(len(r1["order"]), np.int64)
    pos[r1["order"]] = np.arange(len(r1["order"]))
    for t0, t1 in r1["ranges"]:
        seg = pos[r1["entries"][t0:t1]]
        assert np.all(np.diff(seg) > 0)


def test_blur_centres_the_smear_mid_exposure(orc):
    """A translated part with shutter 1: every splat of it sits half way between its previous and current
    projections, and its footprint grows along the motion."""
    import numpy as np
    from splatlight_gb300 import camera, scene
    s = scene.subset(scene.cornell(), 3000)
    parts = s.parts.copy()
    parts["xf_prev"][5] = parts["xf"][5]
    parts["xf"][5][3] += 0.2
    parts["flags"][5] |= 2
    f = camera.make_frame(s.eye, s.target, s.up, s.fov_deg, 128, 128, s.count, far=s.far, view_mode=0, n_emit=0)
    keys_now, now, _ = orc.project(s.gaussians, parts, f)
    p_prev = s.parts.copy()
    keys_prev, prev, _ = orc.project(s.gaussians, p_prev, f)
    f["palette"][3][2] = 1.0
    keys_b, blur, _ = orc.project(s.gaussians, parts, f)
    sel = np.nonzero((s.gaussians["part_surface"] & 0xFFFF) == 5)[0]
    sel = sel[(keys_now[sel] != 0xFFFFFFFF) & (keys_prev[sel] != 0xFFFFFFFF) & (keys_b[sel] != 0xFFFFFFFF)]
    assert len(sel) > 20
    mid = 0.5 * (now["cx"][sel] + prev["cx"][sel])
    assert np.abs(blur["cx"][sel] - mid).max() < 0.2          # pixels (perspective makes it inexact)
    # the smear lengthens the splat: its candidate rectangle spans more pixels than the sharp one's
    w_now = (now["ix1"] - now["ix0"])[sel]
    w_blur = (blur["ix1"] - blur["ix0"])[sel]
    assert np.median(w_blur - w_now) > 0
