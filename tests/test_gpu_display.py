"""The display resolve on the GPU against the restatement: every tone curve and the overdraw ramp on random HDR
values (negative, tiny, huge) and on a rendered frame, 8-bit channels within one step."""
import numpy as np
import pytest

from splatlight_gb300 import camera, scene
from splatlight_gb300.display import to_srgb8
from splatlight_gb300.renderer import SplatRenderer
from splatlight_gb300.structs import VIEW_FLAT, VIEW_OVERDRAW

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("tone", range(6))
def test_tones_random_hdr(cuda, orc, tone):
    torch = cuda
    rng = np.random.default_rng(tone)
    img = np.exp(rng.normal(-1.0, 2.0, (64, 96, 4))).astype(np.float32)
    img[rng.random((64, 96)) < 0.05, :3] *= -1.0
    from splatlight_gb300.structs import FRAME
    f = np.zeros((), dtype=FRAME)
    f["exposure"] = 1.3
    f["tone"][0] = tone
    f["view_mode"] = 3
    got = to_srgb8(torch.from_numpy(img).cuda(), f)
    ref = orc.display(img, 1.3, tone, 3)
    d = np.abs(got.astype(np.int32) - ref.astype(np.int32))
    assert d.max() <= 1, (tone, d.max())
    assert (d == 0).mean() > 0.99


def test_rendered_frames(cuda, orc):
    torch = cuda
    s = scene.subset(scene.cornell(), 8000)
    with SplatRenderer(s.gaussians, s.parts) as r:
        r.set_emitters(s.emitters)
        for mode in (VIEW_FLAT, VIEW_OVERDRAW):
            f = camera.make_frame(s.eye, s.target, s.up, s.fov_deg, 128, 96, s.count, far=s.far, view_mode=mode,
                                  n_emit=len(s.emitters))
            f["exposure"] = 1.0
            f["tone"][0] = 1
            img = torch.empty((96, 128, 4), dtype=torch.float32, device="cuda")
            r.render(f, out=img)
            got = to_srgb8(img, f)
            ref = orc.display(img.cpu().numpy(), 1.0, 1, mode)
            assert np.abs(got.astype(np.int32) - ref.astype(np.int32)).max() <= 1


def test_sky_behind_the_splats_hill_lite(cuda, orc):
    """The reference's hill_lite at its camera, lit, with its environment behind the splats (display.wgsl:22-133):
    where the splats leave the sky showing, the background SH to band 8, the horizon ring and ground, the glow round the
    sun and the sun's disc; 8-bit channels within one step of the FP64 restatement, and the sky visibly there."""
    from pathlib import Path
    torch = cuda
    p = Path(__file__).resolve().parent / "golden" / "assets" / "hill_lite_bin"
    if not (p / "asset.json").exists():
        pytest.skip("reference assets not copied (tests/golden/copy_assets.py)")
    from splatlight_gb300 import asset as A
    from splatlight_gb300.lighting import camera_forward, for_scene
    from splatlight_gb300.structs import VIEW_LIT
    a = A.load_asset(p)
    s = A.asset_scene(a, width=320, height=180)
    sky = A.display_sky(a.header.get("environment"))
    assert sky.bg_count == 81 and sky.ring_count > 0
    with SplatRenderer(s.gaussians, s.parts) as r:
        L = for_scene(r, s)
        L.update(s.eye, camera_forward(s))
        f = camera.make_frame(s.eye, s.target, s.up, s.fov_deg, s.width, s.height, s.count, far=s.far,
                              view_mode=VIEW_LIT, n_emit=s.n_drawn_emitters)
        for tone in (0, 1):
            f["exposure"] = 1.0
            f["tone"][0] = tone
            img = torch.empty((s.height, s.width, 4), dtype=torch.float32, device="cuda")
            r.render(f, out=img)
            got = to_srgb8(img, f, sky_env=sky)
            host = img.cpu().numpy()
            ref = orc.display_env(host, f, sky)
            d = np.abs(got.astype(np.int32) - ref.astype(np.int32))
            assert d.max() <= 1, (tone, d.max())
            bare = host[..., 3] < 0.5
            assert bare.mean() > 0.05                  # the camera sees sky
            plain = orc.display(host, 1.0, tone, 3)
            assert (got[bare, :3].astype(np.int32) - plain[bare, :3].astype(np.int32)).mean() > 10   # and it is drawn
        L.close()


def test_lighting_sky_and_sun_disc(cuda, orc):
    """Without a background of its own the display draws the lighting sky (16 coefficients) and the sun's disc:
    the synthetic hill from a low camera looking up past its canopy."""
    from splatlight_gb300 import display as D
    torch = cuda
    s = scene.subset(scene.hill(), 20000)
    lights = s.distant_lights()
    sky = D.sky(s.sky_sh, lights)
    eye, target = (0.0, -9.0, 0.6), (0.0, 0.0, 4.0)
    f = camera.make_frame(eye, target, s.up, 70.0, 160, 120, s.count, far=s.far, view_mode=3, n_emit=0)
    rng = np.random.default_rng(3)
    img = rng.uniform(0.0, 1.0, (120, 160, 4)).astype(np.float32)
    img[..., 3] = np.where(rng.random((120, 160)) < 0.5, 0.0, img[..., 3])   # half the pixels bare
    got = to_srgb8(torch.from_numpy(img).cuda(), f, sky_env=sky)
    ref = orc.display_env(img, f, sky)
    assert np.abs(got.astype(np.int32) - ref.astype(np.int32)).max() <= 1
