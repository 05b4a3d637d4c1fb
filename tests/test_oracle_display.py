"""The display restatement (oracle/sl_oracle_display.c) on known answers: the sRGB transfer function, the tone
curves' fixed points, the overdraw heat ramp's ends."""
import numpy as np


def _px(orc, rgb, tone=0, view_mode=3, exposure=1.0):
    img = np.zeros((1, 1, 4), np.float32)
    img[0, 0, :3] = rgb
    return orc.display(img, exposure, tone, view_mode)[0, 0]


def test_srgb_and_clamp(orc):
    assert list(_px(orc, (0.0, 0.5, 1.0))[:3]) == [0, 188, 255]
    assert list(_px(orc, (-1.0, 2.0, 0.0031308))[:3]) == [0, 255, 10]
    assert _px(orc, (0.1, 0.2, 0.3))[3] == 255


def test_exposure_scales_before_the_curve(orc):
    assert list(_px(orc, (0.25, 0.25, 0.25), exposure=2.0)[:3]) == list(_px(orc, (0.5, 0.5, 0.5))[:3])


def test_tone_curves_fixed_points(orc):
    for tone in range(6):
        assert list(_px(orc, (0.0, 0.0, 0.0), tone=tone)[:3]) == [0, 0, 0] or tone == 1
        hi = _px(orc, (1e4, 1e4, 1e4), tone=tone)[:3]
        assert min(hi) >= 250, (tone, hi)


def test_heat_ramp_ends(orc):
    assert list(_px(orc, (0.0, 0.0, 0.0), view_mode=2)[:3]) == [0, 0, 0]
    assert list(_px(orc, (127.0, 0.0, 0.0), view_mode=2)[:3]) == [255, 0, 0]
