"""GPU lighting (iso_init, emitter tree + light cut, emitter-light opacity maps, sun maps, shade_emit + env_direct)
against the CPU restatement, and the lit frame end to end: linear RGB within 1e-3."""
import numpy as np
import pytest

from splatlight_gb300 import camera, scene
from splatlight_gb300.lighting import camera_forward, for_scene
from splatlight_gb300.renderer import SplatRenderer
from splatlight_gb300.structs import VIEW_LIT

pytestmark = pytest.mark.gpu

RGB_TOL = 1e-3


def _compare(cuda, orc, s, check_render=True, mode=1, asg=True, W=None, H=None, eye=None, target=None):
    W = W or s.width
    H = H or s.height
    eye = s.eye if eye is None else eye
    target = s.target if target is None else target
    fwd = camera_forward(s, eye, target)
    with SplatRenderer(s.gaussians, s.parts) as r:
        L = for_scene(r, s)
        L.set_options(shadow_res=s.shadow_res, sun_res=s.sun_res, mode=mode, asg=asg)
        L.update(eye, fwd)
        col, lt, et, nodes = L.read()
        ocol, olt, oet, onodes = orc.lighting(s, eye=eye, target=target, threads=16, mode=mode, asg=asg)
        iso_g = nodes["pad0"].view(np.float32)
        iso_o = onodes["pad0"].view(np.float32)
        assert np.allclose(iso_g, iso_o, rtol=1e-6, atol=0), np.abs(iso_g - iso_o).max()
        assert np.allclose(lt, olt, rtol=1e-5, atol=1e-6), np.abs(lt - olt).max()
        assert np.allclose(et, oet, rtol=1e-5, atol=1e-6), np.abs(et - oet).max()
        # the shading pass runs with fast division / square root: ~1e-6 relative typically, up to ~1e-4 where the
        # ASG lobe's acos is ill-conditioned; the linear-RGB check below is the bar
        assert np.allclose(col, ocol, rtol=1e-3, atol=1e-5), np.abs(col - ocol).max()
        if check_render:
            f = camera.make_frame(eye, target, s.up, s.fov_deg, W, H, s.count, far=s.far, view_mode=VIEW_LIT,
                                  n_emit=len(s.emitters))
            img = r.render(f)
            ref = orc.render(s.gaussians, s.parts, f, emitters=s.emitters, colour=ocol, threads=16)
            err = float(np.abs(img - ref["rgba"]).max())
            assert err <= RGB_TOL, err
        L.close()
        return col, ocol


def test_cornell_lighting_and_lit_frame(cuda, orc):
    col, ocol = _compare(cuda, orc, scene.cornell())
    rel = np.abs(col - ocol)[:, :3] / np.maximum(np.abs(ocol[:, :3]), 1e-6)
    assert np.median(rel) < 1e-5


@pytest.mark.parametrize("mode,asg", [(0, True), (1, False)])
def test_cornell_cut_modes(cuda, orc, mode, asg):
    _compare(cuda, orc, scene.subset(scene.cornell(), 20000), mode=mode, asg=asg, W=256, H=256)


def test_hill_subset_sun_and_emitters(cuda, orc):
    s = scene.subset(scene.hill(), 150000)
    s = scene.dataclasses.replace(s, shadow_res=512, sun_res=1024)
    _compare(cuda, orc, s, W=640, H=360)


def test_hill_full_config_lit_frame(cuda, orc):
    """1,048,576 Gaussians, 32 emitters with a 1024^2 emitter-light map, the sun with 2048^2 maps, 1920x1080."""
    _compare(cuda, orc, scene.hill())


def test_update_after_moving_a_part(cuda, orc):
    """A moved part re-splats its layers only; the result equals a fresh update with the new pose."""
    s = scene.subset(scene.cornell(), 20000)
    fwd = camera_forward(s)
    parts = s.parts.copy()
    parts["xf"][5][3] += 0.1        # shift the short box along x
    with SplatRenderer(s.gaussians, s.parts) as r:
        L = for_scene(r, s)
        L.update(s.eye, fwd)
        r.write_parts(parts)
        L.update(s.eye, fwd, moved_mask=1 << 5)
        col, lt, et, _ = L.read()
        L.close()
    s2 = scene.dataclasses.replace(s, parts=parts)
    ocol, olt, oet, _ = orc.lighting(s2, threads=16)
    assert np.allclose(lt, olt, rtol=1e-5, atol=1e-6)
    assert np.allclose(col, ocol, rtol=1e-3, atol=1e-5)
