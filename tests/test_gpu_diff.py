"""The hand-written backward of the differentiable splat path against FP64 central finite differences (h = 1e-4) of a
naive dense FP64 compositor (oracle/sl_oracle_diff.c), on a 1,024-Gaussian subset of the 500k-Gaussian hill-like
scene lit by the product lighting: 8 emissive Gaussian lights over their emitter tree's light cut, with V grids
(random cells), opacity-map transmittance and iso_norm from the restated lighting update held constant.  Gradients
with respect to means, log-scales, quaternions, opacity logits, albedo, roughness (128 sampled Gaussians, every
component) and the 8 light intensities, each parameter group within 2e-2 relative (L2 over the sample).  The forward
image and loss agree with the dense FP64 forward as well."""
import dataclasses

import numpy as np
import pytest

from splatlight_gb300 import camera, scene
from splatlight_gb300.diff import PARAMS, DiffRenderer, params_from_scene, perturb

pytestmark = pytest.mark.gpu

H_FD = 1e-4


def _subset_problem(orc, n=1024, res=96):
    s = scene.hill(500_000, seed=1)
    params, lights = params_from_scene(s, n_lights=8)
    mu = params["means"]
    high = mu[mu[:, 2] > 1.0]
    centre = np.median(high, axis=0)
    idx = np.argsort(np.linalg.norm(mu - centre, axis=1))[:n]
    idx.sort()
    sub = {k: np.ascontiguousarray(v[idx]) for k, v in params.items()}
    eye = tuple(np.float32(centre + np.array([0.0, -3.0, 0.8])))
    frame = camera.make_frame(eye, tuple(centre), s.up, 50.0, res, res, n, far=100.0, view_mode=3, n_emit=0)
    # the emissive lights around the subset, so every light shades it, at intensities away from 1
    rng = np.random.default_rng(4)
    ang = np.linspace(0, 2 * np.pi, 8, endpoint=False)
    rec = lights["rec"].copy()
    rec["mu"] = (centre + np.stack([2.0 * np.cos(ang), 2.0 * np.sin(ang), 1.0 + 0.5 * rng.random(8)], 1))
    rec["albedo"] *= 25.0                               # lit radiance well above the ambient term
    lights["rec"] = rec
    lights["scale"] = rng.uniform(0.7, 1.4, 8).astype(np.float32)
    # per-Gaussian state held constant: V grids with every cell in [96, 255], and the lamp transmittance and
    # iso_norm of the restated lighting update of the subset under these lights (the subset split into three
    # interleaved parts, since a part casts no shadow on itself in the lamp's opacity map)
    g = s.gaussians[idx].copy()
    g["part_surface"] = (g["part_surface"] & 0xFFFF0000) | (3 * np.arange(n) // n).astype(np.uint32)
    vg = np.zeros(n, dtype=s.vgrid.dtype)
    vg["w"] = rng.integers(96, 256, (n, 128), dtype=np.uint8).view(np.uint32)
    sub_scene = dataclasses.replace(s, gaussians=g, parts=scene._parts(g, len(s.parts)), nodes=scene.leaf_nodes(g),
                                    vgrid=vg, emitters=rec, sun=None, shadow_res=256, emit_drawn=False)
    _, lamp_T, _, nodes = orc.lighting(sub_scene, eye=eye, target=tuple(centre), threads=16)
    iso = nodes["pad0"].view(np.float32)[:n]
    assert (lamp_T > 0).all() and (lamp_T < 1).any() and np.isfinite(iso).all() and (iso > 0).all()
    state = {"vgrid": vg, "lamp_T": lamp_T.astype(np.float64), "iso_norm": iso.astype(np.float64)}
    return sub, lights, frame, eye, state


def _fd(orc, base, lights, frame, eye, order, target, key, i, c, threads, state):
    p = {k: v.astype(np.float64) for k, v in base.items()}
    L = dict(lights, scale=np.asarray(lights["scale"], np.float64).copy())
    if key == "light_scale":
        a = L["scale"].reshape(-1, 1)
    else:
        a = p[key].reshape(len(p[key]), -1)
    a[i, c] += H_FD
    _, lp = orc.diff_render(p, L, frame, eye, order, target, threads, state)
    a[i, c] -= 2 * H_FD
    _, lm = orc.diff_render(p, L, frame, eye, order, target, threads, state)
    return (lp - lm) / (2 * H_FD)


def test_gradients_against_fp64_finite_differences(cuda, orc):
    base, lights, frame, eye, state = _subset_problem(orc)
    rng = np.random.default_rng(0)
    tgt_params = perturb(base, rng)
    with DiffRenderer(len(base["means"])) as D:
        Pt, Lt = D.to_device(tgt_params, lights, state)
        target = D.forward(Pt, Lt, frame, eye)
        P, Lt = D.to_device(base, lights, state)
        loss, G, img = D.step(P, Lt, frame, eye, target)
        order = D.order()
    G = {k: v.cpu().numpy().astype(np.float64) for k, v in G.items()}
    tgt = target.cpu().numpy()
    # the forward against the dense FP64 compositor (same order)
    ref_img, ref_loss = orc.diff_render({k: v.astype(np.float64) for k, v in base.items()}, lights, frame, eye, order,
                                        tgt, 16, state)
    assert float(np.abs(img.cpu().numpy() - ref_img).max()) < 1e-3
    assert abs(loss - ref_loss) <= 1e-3 * ref_loss + 1e-6, (loss, ref_loss)
    # the lights matter: the lit radiance is well above the ambient term
    assert ref_img[..., :3].max() > 2.0 * lights["ambient"] * base["albedo"].max()
    # finite differences on a sample of Gaussians that the image sees, every parameter, and every light
    vis = np.unique(order)
    sample = rng.choice(vis, size=min(128, len(vis)), replace=False)
    report = {}
    for key in PARAMS:
        width = base[key].reshape(len(base[key]), -1).shape[1]
        fd, gp = [], []
        for i in sample:
            for c in range(width):
                fd.append(_fd(orc, base, lights, frame, eye, order, tgt, key, int(i), c, 16, state))
                gp.append(G[key].reshape(len(base[key]), -1)[i, c])
        fd, gp = np.array(fd), np.array(gp)
        report[key] = np.linalg.norm(gp - fd) / max(np.linalg.norm(fd), 1e-12)
    fd = np.array([_fd(orc, base, lights, frame, eye, order, tgt, "light_scale", l, 0, 16, state) for l in range(8)])
    report["light_scale"] = np.linalg.norm(G["light_scale"] - fd) / max(np.linalg.norm(fd), 1e-12)
    print(report)
    for key, rel in report.items():
        assert rel < 2e-2, (key, rel, report)
