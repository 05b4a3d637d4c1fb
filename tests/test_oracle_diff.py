"""The dense FP64 forward of the differentiable path (oracle/sl_oracle_diff.c) on cases with known answers: a Gaussian
seen along its short axis without the low-pass dilation peaks at alpha = sigmoid(opacity logit) (the splat path's
kappa convention), and the radiance is linear in the light intensities (two emissive Gaussian lights over their
emitter tree)."""
import numpy as np

from splatlight_gb300 import camera
from splatlight_gb300.structs import GAUSSIAN


def _lights():
    rec = np.zeros(2, GAUSSIAN)
    rec["mu"] = [[1.0, 1.0, 3.0], [-1.0, 0.5, 2.0]]
    rec["quat"] = [0.0, 0.0, 0.0, 1.0]
    rec["scale"] = [0.05, 0.06, 0.07]
    rec["kappa"] = 3.0 / (np.sqrt(2 * np.pi) * 0.05)
    rec["albedo"] = [[2.0, 2.0, 2.0], [1.0, 3.0, 1.0]]
    return rec


def _one(logit=0.3, lowpass=0.0, scale=(0.05, 0.2, 0.3)):
    params = {"means": np.zeros((1, 3)), "log_scales": np.log(np.array([scale])),
              "quats": np.array([[0.0, -np.sqrt(0.5), 0.0, np.sqrt(0.5)]]),   # axis 0 along z, towards the camera
              "opacity_logits": np.array([logit]), "albedo": np.array([[0.5, 0.25, 1.0]]),
              "roughness": np.array([0.4])}
    lights = {"rec": _lights(), "scale": np.array([1.0, 1.0]), "ambient": 0.0, "ks": 0.25}
    f = camera.make_frame((0.0, 0.0, 5.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 50.0, 65, 65, 1, far=100.0,
                          view_mode=3, n_emit=0, lowpass_px2=lowpass)
    return params, lights, f


def test_peak_alpha_is_the_opacity(orc):
    params, lights, f = _one()
    img, _ = orc.diff_render(params, lights, f, (0.0, 0.0, 5.0), np.array([0], np.uint32))
    a = img[32, 32, 3]
    assert abs(a - 1.0 / (1.0 + np.exp(-0.3))) < 1e-9, a
    assert img[..., 3].max() == a


def test_radiance_linear_in_light_intensities(orc):
    params, lights, f = _one()
    img1, _ = orc.diff_render(params, lights, f, (0.0, 0.0, 5.0), np.array([0], np.uint32))
    lights2 = dict(lights, scale=np.array([2.0, 2.0]))
    img2, _ = orc.diff_render(params, lights2, f, (0.0, 0.0, 5.0), np.array([0], np.uint32))
    assert np.allclose(img2[..., :3], 2.0 * img1[..., :3], rtol=1e-12, atol=1e-15)
    assert img1[..., :3].max() > 0.0
