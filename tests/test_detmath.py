"""The deterministic log/exp shared by the CPU restatement and the GPU kernels (include/sl_detmath.h): accuracy
against float64 (<= 2 ulp over the pipeline's ranges) and special values."""
import numpy as np
import pytest


def _ulp_err(y, t):
    tf = t.astype(np.float32)
    ulp = np.spacing(np.abs(tf)).astype(np.float64)
    return np.abs(y.astype(np.float64) - t) / ulp


def test_logf_accuracy(orc):
    rng = np.random.default_rng(0)
    x = np.concatenate([np.exp(rng.uniform(-80, 80, 200000)), rng.uniform(0.5, 2.0, 200000),
                        np.float32([1.0, 2.0, 0.5, 1e-38, 3.4e38])]).astype(np.float32)
    y = orc.logf(x)
    t = np.log(x.astype(np.float64))
    ok = np.abs(t) > 0
    assert _ulp_err(y[ok], t[ok]).max() <= 2.0
    assert orc.logf(np.float32([1.0]))[0] == 0.0


def test_logf_special(orc):
    y = orc.logf(np.float32([0.0, -1.0, np.inf, np.nan, 1e-45]))
    assert y[0] == -np.inf and np.isnan(y[1]) and y[2] == np.inf and np.isnan(y[3])
    assert abs(y[4] - np.log(1.401298464324817e-45)) < 1e-5


def test_expf_accuracy(orc):
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.uniform(-87, 88, 400000), rng.uniform(-1, 1, 100000)]).astype(np.float32)
    y = orc.expf(x)
    t = np.exp(x.astype(np.float64))
    assert _ulp_err(y, t).max() <= 2.0
    # gradual underflow and the ends
    y2 = orc.expf(np.float32([-100.0, -104.5, 89.0, 0.0]))
    assert 0 < y2[0] < 1.2e-38 and y2[1] == 0.0 and y2[2] == np.inf and y2[3] == 1.0


def test_atan2_asin_acos_accuracy(orc):
    rng = np.random.default_rng(2)
    ang = rng.uniform(-np.pi, np.pi, 300000)
    r = np.exp(rng.uniform(-20, 20, 300000))
    y = (r * np.sin(ang)).astype(np.float32)
    x = (r * np.cos(ang)).astype(np.float32)
    got = orc.atan2f(y, x).astype(np.float64)
    want = np.arctan2(y.astype(np.float64), x.astype(np.float64))
    assert np.abs(got - want).max() < 4e-7
    assert orc.atan2f(np.float32([0, 1, -1, 0]), np.float32([0, 0, 0, -1])).tolist() == \
        pytest.approx([0.0, np.pi / 2, -np.pi / 2, np.pi], abs=1e-7)
    u = rng.uniform(-1, 1, 300000).astype(np.float32)
    assert np.abs(orc.asinf(u) - np.arcsin(u.astype(np.float64))).max() < 5e-7
    assert np.abs(orc.acosf(u) - np.arccos(u.astype(np.float64))).max() < 5e-7
    assert orc.acosf(np.float32([1.0]))[0] == 0.0 and orc.asinf(np.float32([0.0]))[0] == 0.0
