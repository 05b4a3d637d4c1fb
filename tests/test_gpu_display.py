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
