"""The oracle's restatement of motion_blur.wgsl blur_records (the records the opacity-map splats draw for a moving
part): a still part's records are copied unchanged; a moving part's leaf becomes the box-shutter average of its
motion -- covariance C + d d^T / 12 centred mid-exposure, the node's inverse covariance its Sherman-Morrison
update, mass kept (kappa sqrt(det C) unchanged), a unit right-handed quaternion with ascending scales."""
import numpy as np

from splatlight_gb300 import scene


def _cov(g):
    x, y, z, w = (float(v) for v in g["quat"])
    R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                  [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                  [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
    s2 = np.asarray(g["scale"], np.float64) ** 2
    return R @ np.diag(s2) @ R.T, R


def test_blur_record_moving_and_still(orc):
    s = scene.subset(scene.cornell(), 2000)
    parts = s.parts.copy()
    moving = 5
    parts["flags"][moving] |= 2
    parts["xf_prev"][moving] = parts["xf"][moving]
    parts["xf_prev"][moving][3] -= 0.3           # moved +0.3 in x and +0.1 in z over the frame
    parts["xf_prev"][moving][11] -= 0.1
    shutter = 0.5
    d_world = shutter * np.array([0.3, 0.0, 0.1])
    n_moving = 0
    for i in range(len(s.gaussians)):
        g, nd = s.gaussians[i], s.nodes[i]
        go, no = orc.blur_record(parts, shutter, g, nd)
        if int(g["part_surface"]) & 0xFFFF != moving:
            assert go.tobytes() == g.tobytes() and no.tobytes() == nd.tobytes()
            continue
        n_moving += 1
        # the rest frame of the moving part is the identity rotation, so d is the world displacement
        d = d_world
        assert np.allclose(go["mu"], g["mu"] - 0.5 * d, atol=1e-6)
        assert np.allclose(no["mean"], nd["mean"] - 0.5 * d, atol=1e-6)
        C, _ = _cov(g)
        Cs = C + np.outer(d, d) / 12.0
        Cb, R = _cov(go)
        assert np.allclose(Cb, Cs, rtol=2e-4, atol=1e-9 + 2e-4 * np.abs(Cs).max())
        assert abs(np.linalg.norm(np.asarray(go["quat"], np.float64)) - 1.0) < 1e-5
        assert np.linalg.det(R) > 0.999
        sc = np.asarray(go["scale"], np.float64)
        assert sc[0] <= sc[1] * (1 + 1e-6) and sc[1] <= sc[2] * (1 + 1e-6)
        ci = np.array([[no["cinv_diag"][0], no["cinv_off"][0], no["cinv_off"][1]],
                       [no["cinv_off"][0], no["cinv_diag"][1], no["cinv_off"][2]],
                       [no["cinv_off"][1], no["cinv_off"][2], no["cinv_diag"][2]]], np.float64)
        assert np.allclose(ci @ Cs, np.eye(3), atol=2e-3)
        mass = float(g["kappa"]) * np.sqrt(np.linalg.det(C))
        assert abs(float(go["kappa"]) * np.sqrt(np.linalg.det(Cs)) / mass - 1.0) < 1e-4
        assert float(go["kappa"]) == float(no["kappa"])
    assert n_moving > 50
    # no shutter: every record unchanged
    g, nd = s.gaussians[-1], s.nodes[-1]
    go, no = orc.blur_record(parts, 0.0, g, nd)
    assert go.tobytes() == g.tobytes() and no.tobytes() == nd.tobytes()
