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


@pytest.mark.parametrize("which,cut", [("cornell", 0.0), ("hill", 0.0), ("cornell", 1.0), ("hill", 1.0)])
def test_motion_blur_in_the_lighting(cuda, orc, which, cut):
    """motion_blur.wgsl blur_records: a moving part (flags bit 1, xf_prev behind xf) draws stretched records into the
    opacity maps (light map A on the Cornell room, the sun maps on the hill) while every receiver keeps its rest
    record; with the scene's tree and cut factor 1 (the reference's default ?blurcut) the moving part splats the cut of
    its tree sized to its smear, each node keeping its rest coverage.  Lamp and env transmittance within 1e-5 of the
    restatement with the same blur, measurably unlike the unblurred maps, and the lit frame within 1e-3; back to the
    unblurred maps once the part stops."""
    if which == "cornell":
        s = scene.subset(scene.cornell(), 20000)
        moving, shift = 5, (0.25, 0.0, 0.1)
    else:
        s = scene.dataclasses.replace(scene.subset(scene.hill(), 150000), shadow_res=512, sun_res=1024)
        moving, shift = 2, (0.6, 0.3, 0.0)        # the canopy
    tree = None
    if cut > 0.0:
        nodes, kids, rooted = scene.lod_tree(s.gaussians, s.parts)
        s = scene.dataclasses.replace(s, parts=rooted)
        tree = (nodes, kids)
    parts = s.parts.copy()
    parts["xf_prev"][moving] = parts["xf"][moving]
    for k, v in zip((3, 7, 11), shift):
        parts["xf"][moving][k] += v
    parts["flags"][moving] |= 2
    s2 = scene.dataclasses.replace(s, parts=parts)
    fwd = camera_forward(s2)
    with SplatRenderer(s.gaussians, s.parts) as r:
        L = for_scene(r, s)
        L.set_options(shadow_res=s.shadow_res, sun_res=s.sun_res)
        if tree is not None:
            L.set_tree(*tree)
        L.set_blur(0.5, cut)
        L.update(s.eye, fwd)
        r.write_parts(parts)
        L.update(s.eye, fwd, moved_mask=1 << moving)
        col, lt, et, _ = L.read()
        ocol, olt, oet, _ = orc.lighting(s2, threads=16, blur_shutter=0.5, tree=tree, cut_k=cut)
        assert np.allclose(lt, olt, rtol=1e-5, atol=1e-6), np.abs(lt - olt).max()
        assert np.allclose(et, oet, rtol=1e-5, atol=1e-6), np.abs(et - oet).max()
        assert np.allclose(col, ocol, rtol=1e-3, atol=1e-5)
        _, plt, pet, _ = orc.lighting(s2, threads=16)
        changed = np.abs(lt - plt).max() if which == "cornell" else np.abs(et - pet).max()
        assert changed > 1e-3, changed
        f = camera.make_frame(s.eye, s.target, s.up, s.fov_deg, 320, 240, s.count, far=s.far, view_mode=VIEW_LIT,
                              n_emit=len(s.emitters))
        img = r.render(f)
        ref = orc.render(s.gaussians, parts, f, emitters=s.emitters, colour=ocol, threads=16)
        assert float(np.abs(img - ref["rgba"]).max()) <= RGB_TOL
        # the part stops (flags bit 1 cleared, xf_prev = xf): its copies go back to rest in the next update
        parts2 = parts.copy()
        parts2["flags"][moving] &= ~np.uint32(2)
        parts2["xf_prev"][moving] = parts2["xf"][moving]
        r.write_parts(parts2)
        L.update(s.eye, fwd, moved_mask=0)
        _, lt2, et2, _ = L.read()
        _, olt2, oet2, _ = orc.lighting(scene.dataclasses.replace(s, parts=parts2), threads=16, blur_shutter=0.5,
                                        tree=tree, cut_k=cut)
        assert np.allclose(lt2, olt2, rtol=1e-5, atol=1e-6) and np.allclose(et2, oet2, rtol=1e-5, atol=1e-6)
        L.close()
