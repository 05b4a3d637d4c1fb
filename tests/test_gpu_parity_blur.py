"""Motion blur in the projection (shaders/project.wgsl:138-146, 207-272): a part moving over the exposure, its
Gaussians stretched by the box-shutter average (covariance + v v^T / 12, Sherman-Morrison q, mass-keeping kappa,
coverage cap), bit-exact keys, permutation, tile lists and contributor counts and RGB within 1e-3 against the CPU
restatement, in the flat, overdraw and lit views."""
import numpy as np
import pytest

from splatlight_gb300 import camera, scene
from splatlight_gb300.renderer import SplatRenderer
from splatlight_gb300.structs import VIEW_FLAT, VIEW_LIT, VIEW_OVERDRAW

pytestmark = pytest.mark.gpu


def _moving(s, part=5, shift=(0.12, 0.05, -0.03)):
    parts = s.parts.copy()
    parts["xf_prev"][part] = parts["xf"][part]
    xf = parts["xf"][part].reshape(3, 4).copy()
    xf[:, 3] += np.asarray(shift, np.float32)
    c, sn = np.cos(0.2), np.sin(0.2)               # and a turn about z
    xf[:, :3] = np.array([[c, -sn, 0], [sn, c, 0], [0, 0, 1]], np.float32) @ xf[:, :3]
    parts["xf"][part] = xf.reshape(12)
    parts["flags"][part] |= 2
    return parts


@pytest.mark.parametrize("mode", [VIEW_FLAT, VIEW_OVERDRAW])
@pytest.mark.parametrize("cov_cap", [0.0, 1.0])
def test_blur_parity(cuda, orc, mode, cov_cap):
    s = scene.subset(scene.cornell(), 20000)
    parts = _moving(s)
    f = camera.make_frame(s.eye, s.target, s.up, s.fov_deg, 192, 160, s.count, far=s.far, view_mode=mode,
                          n_emit=len(s.emitters))
    f["palette"][3][2] = 0.5
    f["palette"][3][3] = cov_cap
    with SplatRenderer(s.gaussians, parts) as r:
        r.set_emitters(s.emitters)
        img = r.render(f)
        dbg = r.read_debug()
        ref = orc.render(s.gaussians, parts, f, emitters=s.emitters, threads=8)
        assert np.array_equal(dbg["keys"], ref["keys"])
        assert np.array_equal(dbg["order"], ref["order"])
        assert np.array_equal(dbg["ranges"], ref["ranges"])
        assert np.array_equal(dbg["entries"], ref["entries"])
        if mode == VIEW_OVERDRAW:
            assert np.array_equal(r.read_counts(192, 160), ref["counts"])
        else:
            assert float(np.abs(img - ref["rgba"]).max()) <= 1e-3
        # the blur changes the picture (the moving part is smeared)
        f0 = f.copy()
        f0["palette"][3][2] = 0.0
        assert not np.array_equal(r.render(f0), img)


def test_lit_view_of_a_blurred_moving_part(cuda, orc):
    """The lit view of a moving part with the blur in the projection only (the reference's ?blurlight=0: the lighting
    shades and shadows every Gaussian at its pose, the projection smears the display): the lighting, then the
    frame's keys, permutation, tile lists bit-exact and RGB within 1e-3 against the CPU restatement."""
    from splatlight_gb300.lighting import camera_forward, for_scene
    s = scene.subset(scene.cornell(), 20000)
    s = scene.dataclasses.replace(s, parts=_moving(s))
    f = camera.make_frame(s.eye, s.target, s.up, s.fov_deg, 192, 160, s.count, far=s.far, view_mode=VIEW_LIT,
                          n_emit=len(s.emitters))
    f["palette"][3][2] = 0.5
    f["palette"][3][3] = 1.0
    with SplatRenderer(s.gaussians, s.parts) as r:
        L = for_scene(r, s)
        L.update(s.eye, camera_forward(s))
        col, _, _, _ = L.read()
        ocol, _, _, _ = orc.lighting(s, threads=8)
        assert np.allclose(col, ocol, rtol=1e-3, atol=1e-5), np.abs(col - ocol).max()
        img = r.render(f)
        dbg = r.read_debug()
        ref = orc.render(s.gaussians, s.parts, f, emitters=s.emitters, colour=ocol, threads=8)
        assert np.array_equal(dbg["keys"], ref["keys"])
        assert np.array_equal(dbg["order"], ref["order"])
        assert np.array_equal(dbg["ranges"], ref["ranges"])
        assert np.array_equal(dbg["entries"], ref["entries"])
        assert float(np.abs(img - ref["rgba"]).max()) <= 1e-3
        f0 = f.copy()
        f0["palette"][3][2] = 0.0
        assert not np.array_equal(r.render(f0), img)
        L.close()
