"""The hand-written backward of the differentiable splat path against FP64 central finite differences (h = 1e-4) of a
naive dense FP64 compositor (oracle/sl_oracle_diff.c), on a 1,024-Gaussian subset of the 500k-Gaussian hill-like
scene: gradients with respect to means, log-scales, quaternions, opacity logits, albedo, roughness and 8 light
intensities.  The forward image and loss agree with the dense FP64 forward as well."""
import numpy as np
import pytest

from splatlight_gb300 import camera, scene
from splatlight_gb300.diff import PARAMS, DiffRenderer, params_from_scene, perturb

pytestmark = pytest.mark.gpu

H_FD = 1e-4


def _subset_problem(n=1024, res=96):
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
    # lights around the subset so every light shades it
    rng = np.random.default_rng(4)
    ang = np.linspace(0, 2 * np.pi, 8, endpoint=False)
    lights["pos"] = (centre + np.stack([2.0 * np.cos(ang), 2.0 * np.sin(ang), 1.0 + 0.5 * rng.random(8)], 1)
                     ).astype(np.float32)
    return sub, lights, frame, eye


def _fd(orc, base, lights, frame, eye, order, target, key, i, c, threads):
    p = {k: v.astype(np.float64) for k, v in base.items()}
    L = {k: (np.asarray(v, np.float64) if not np.isscalar(v) else v) for k, v in lights.items()}
    if key == "light_scale":
        L["scale"] = L["scale"].copy()
        L["scale"][i] += H_FD
        _, lp = orc.diff_render(p, L, frame, eye, order, target, threads)
        L["scale"][i] -= 2 * H_FD
        _, lm = orc.diff_render(p, L, frame, eye, order, target, threads)
    else:
        a = p[key].reshape(len(p[key]), -1)
        a[i, c] += H_FD
        _, lp = orc.diff_render(p, L, frame, eye, order, target, threads)
        a[i, c] -= 2 * H_FD
        _, lm = orc.diff_render(p, L, frame, eye, order, target, threads)
    return (lp - lm) / (2 * H_FD)


def test_gradients_against_fp64_finite_differences(cuda, orc):
    torch = cuda
    base, lights, frame, eye = _subset_problem()
    rng = np.random.default_rng(0)
    tgt_params = perturb(base, rng)
    with DiffRenderer(len(base["means"])) as D:
        Pt, Lt = D.to_device(tgt_params, lights)
        target = D.forward(Pt, Lt, frame, eye)
        P, Lt = D.to_device(base, lights)
        loss, G, img = D.step(P, Lt, frame, eye, target)
        order = D.order()
    G = {k: v.cpu().numpy().astype(np.float64) for k, v in G.items()}
    tgt = target.cpu().numpy()
    # the forward against the dense FP64 compositor (same order)
    ref_img, ref_loss = orc.diff_render({k: v.astype(np.float64) for k, v in base.items()}, lights, frame, eye, order,
                                        tgt, 16)
    assert float(np.abs(img.cpu().numpy() - ref_img).max()) < 1e-3
    assert abs(loss - ref_loss) <= 1e-3 * ref_loss + 1e-6, (loss, ref_loss)
    # finite differences on a sample of Gaussians that the image sees, every parameter, and every light
    vis = np.unique(order)
    sample = rng.choice(vis, size=min(24, len(vis)), replace=False)
    report = {}
    for key in PARAMS:
        width = base[key].reshape(len(base[key]), -1).shape[1]
        fd, gp = [], []
        for i in sample:
            for c in range(width):
                fd.append(_fd(orc, base, lights, frame, eye, order, tgt, key, int(i), c, 16))
                gp.append(G[key].reshape(len(base[key]), -1)[i, c])
        fd, gp = np.array(fd), np.array(gp)
        rel = np.linalg.norm(gp - fd) / max(np.linalg.norm(fd), 1e-12)
        report[key] = rel
    fd = np.array([_fd(orc, base, lights, frame, eye, order, tgt, "light_scale", l, 0, 16) for l in range(8)])
    report["light_scale"] = np.linalg.norm(G["light_scale"] - fd) / max(np.linalg.norm(fd), 1e-12)
    print(report)
    for key, rel in report.items():
        assert rel < 2e-2, (key, rel, report)
