"""The probe bounce (runtime/wgsl/bounce.wgsl, the reference's path without the sender cut), GPU against the CPU
restatement over several frames: the transfer SH2, the light toward the probes, the tree's sums and SH2, the probes'
gather (colour, depth moments, first-hit part and near flags), validity and SH2, and the Gaussians' bounce lo_b.
The restatement takes the GPU's own lighting state (iso_norm, lamp and sun transmittance), so the bounce alone is
compared; those inputs have their own parity tests.  The geometry (first-hit parts, near flags, validity, depth
moments, transfer) is exact or within a few float32 ulps: both sides run the same float32 arithmetic in the same
order.  The light toward the probes comes from a kernel compiled for speed (as the shading pass, and to the same
1e-3); through the half-precision node SH2 (a flip of one half step is 5e-4 of a coefficient) and the frames'
feedback, the radiance downstream agrees within 2e-3 (of the largest value, where a value is near zero).

Scenes: the hill-like scene (terrain lattice, its sky), the Cornell-like room (room lattice, no sky), and, when the
assets are copied, the reference's Cornell room (room layout) and hill_lite (terrain layout, its environment's sky),
each with its baked tree (kids.bin) and real V grids."""
import dataclasses
from pathlib import Path

import numpy as np
import pytest

from splatlight_gb300 import camera
from splatlight_gb300 import probes as PR
from splatlight_gb300 import scene as S
from splatlight_gb300.lighting import camera_forward, for_scene
from splatlight_gb300.renderer import SplatRenderer
from splatlight_gb300.structs import VIEW_LIT

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
ASSETS = ROOT / "tests" / "golden" / "assets"
FRAMES = 5
RTOL, ATOL = 1e-5, 1e-7          # geometry: depth moments, transfer
RAD_RTOL, RAD_ATOL = 2e-3, 1e-6  # radiance downstream of the light toward the probes


def _close(name, a, b, rtol=RTOL, atol=ATOL, frac=0.0, scaled=False):
    """a within rtol/atol of b everywhere, or outside it on at most a fraction `frac` of the entries; scaled: atol is
    also at least rtol x the largest |b| (radiance: half steps of the node SH2 move a value near zero by that much)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if scaled and b.size:
        atol = max(atol, rtol * float(np.abs(b).max()))
    bad = ~np.isclose(a, b, rtol=rtol, atol=atol)
    n = int(bad.sum())
    worst = float(np.max(np.abs(a - b))) if a.size else 0.0
    assert n <= frac * a.size, f"{name}: {n} of {a.size} differ (max abs {worst:.3e})"


def _run(s, tree, layout, frames=FRAMES, gain=1.0, moves=None, blend=1.0, sender_cut=False):
    """frames bounce frames on GPU and restatement side by side; moves: {frame: (parts, moved_mask)} written before
    that frame's update (the maps re-splat; both sides take the GPU's transmittance of that frame).  sender_cut: the
    reference's default senders; its marks are exact, the cut nodes' transfer within RTOL, their shadow T exact up to
    float32 sums, their direct light (a kernel compiled for speed) within 1e-3."""
    import torch
    from oracle import oracle as O
    r = SplatRenderer(s.gaussians, s.parts)
    L = for_scene(r, s)
    L.set_tree(*tree)
    L.set_sky(s.sky_sh)
    L.set_probes(layout, blend=blend)
    if sender_cut:
        L.set_sender_cut(True)
    fwd = camera_forward(s)
    b = None
    for f in range(frames):
        mask = 0
        if moves and f in moves:
            parts, mask = moves[f]
            r.write_parts(parts)
        L.update(s.eye, fwd, moved_mask=mask)
        torch.cuda.synchronize()
        col, lamp_t, env_t, nodes = L.read()
        if b is None:
            b = O.Bounce(s, tree, (col, lamp_t, env_t, nodes), layout, sky_sh=s.sky_sh, blend=blend,
                         sender_cut=sender_cut)
        if moves and f in moves:
            b.scene = dataclasses.replace(b.scene, parts=moves[f][0])
        b.lamp_T = np.ascontiguousarray(lamp_t, np.float32)
        b.env_T = np.ascontiguousarray(env_t, np.float32)
        ost = b.step(s.eye, moved_mask=mask, threads=16)
        gst = L.read_bounce()
        if sender_cut:
            assert np.array_equal(gst["sc_flag"], ost["sc_flag"]), f"frame {f}: sender-cut marks differ"
            cut = gst["sc_flag"][s.count:] == 2
            assert cut.any()
            _close(f"frame {f} cut transfer", gst["sc_X"][cut, :6], ost["sc_X"][cut, :6])
            _close(f"frame {f} cut shadow T", gst["sc_T"][cut], ost["sc_T"][cut])
            _close(f"frame {f} cut distant T", gst["sc_envT"][cut], ost["sc_envT"][cut])
            _close(f"frame {f} cut direct light", gst["sc_X"][cut, 6:], ost["sc_X"][cut, 6:], rtol=1e-3,
                   atol=RAD_ATOL, scaled=True)
        pd, opd = gst["probe_data"], ost["probe_data"]
        # discrete fields exactly: first-hit part (.w of the colour record), near / backface flags, validity
        assert np.array_equal(pd[:, :, 3], opd[:, :, 3]), f"frame {f}: first-hit parts differ"
        assert np.array_equal(pd[:, :, 7], opd[:, :, 7]), f"frame {f}: near flags differ"
        assert np.array_equal(pd[:, 0, 6], opd[:, 0, 6]), f"frame {f}: probe validity differs"
        _close(f"frame {f} probe moments", pd[:, :, 4:6], opd[:, :, 4:6])
        _close(f"frame {f} transfer", gst["xfer"], ost["xfer"])
        _close(f"frame {f} light toward the probes", gst["lo_dir"], ost["lo_dir"], rtol=1e-3 if f == 0 else RAD_RTOL,
               atol=RAD_ATOL, scaled=True)
        _close(f"frame {f} node sums", gst["node_acc"], ost["node_acc"], rtol=RAD_RTOL, atol=RAD_ATOL, scaled=True)
        gh = gst["node_sh"].view(np.float16).astype(np.float64)
        oh = ost["node_sh"].view(np.float16).astype(np.float64)
        _close(f"frame {f} node SH2", gh, oh, rtol=RAD_RTOL, atol=1e-4 * max(1.0, float(np.abs(oh).max())))
        _close(f"frame {f} probe colour", pd[:, :, :3], opd[:, :, :3], rtol=RAD_RTOL, atol=RAD_ATOL, scaled=True)
        _close(f"frame {f} probe SH2", gst["probe_sh"], ost["probe_sh"], rtol=RAD_RTOL, atol=RAD_ATOL, scaled=True)
        _close(f"frame {f} bounce", gst["lo_b"], ost["lo_b"], rtol=RAD_RTOL, atol=RAD_ATOL, scaled=True)
    return r, L, gst


def _bounce_lit(s):
    return dataclasses.replace(s, sky_ambient=0.0)


def test_bounce_hill_terrain_sky():
    s = _bounce_lit(S.hill(40000, seed=3, width=320, height=240, n_emit=8))
    s = dataclasses.replace(s, shadow_res=256, sun_res=256)
    s, tree = S.with_tree(s)
    _, _, st = _run(s, tree, PR.for_scene(s))
    # the sky reaches the ground through the probes: a positive bounce on most Gaussians
    assert (st["lo_b"][:, 0, :3].sum(axis=1) > 0).mean() > 0.9


@pytest.mark.parametrize("blend", [0.5, -1.0])
def test_bounce_history_blends(blend):
    """The probes' history blends after the first gather: the EMA (?probeblend=ema, weight 0.5) and the tapered blend
    of the last three gathers (?probeblend=fir)."""
    s = _bounce_lit(S.hill(20000, seed=6, width=160, height=120, n_emit=4))
    s = dataclasses.replace(s, shadow_res=128, sun_res=128)
    s, tree = S.with_tree(s)
    _run(s, tree, PR.for_scene(s), frames=4, blend=blend)


def test_bounce_near_mirror_materials():
    """bounce_dirs: a quarter of the hill's materials made near-mirror (roughness 0.05: a flake lobe below 0.1 rad)
    take the per-cell path -- the probes' per-cell radiance through their transfer and specular lobe, the cells near
    the eye's mirror direction as lights with a size -- the rest bounce_sh's."""
    s = _bounce_lit(S.hill(20000, seed=7, width=160, height=120, n_emit=4))
    m = s.materials.copy()
    m["flake"][:8] = (1.0, 0.0025, 0.0025)
    s = dataclasses.replace(s, shadow_res=128, sun_res=128, materials=m)
    s, tree = S.with_tree(s)
    mirror = (s.gaussians["flags"] & 0xFFFF) < 8
    assert 0.1 < mirror.mean() < 0.5
    _, _, st = _run(s, tree, PR.for_scene(s), frames=3)
    assert (st["lo_b"][mirror, 0, :3].sum(axis=1) > 0).mean() > 0.5


def test_bounce_cornell_room():
    s = _bounce_lit(S.cornell(20000, seed=2, width=256, height=256, n_emit=4))
    s = dataclasses.replace(s, shadow_res=256)
    s, tree = S.with_tree(s)
    _run(s, tree, PR.for_scene(s))


def test_bounce_cornell_asset():
    p = ASSETS / "cornell_sdf_room_plain_bin"
    if not (p / "asset.json").exists():
        pytest.skip("reference assets not copied (tests/golden/copy_assets.py)")
    from splatlight_gb300 import asset as A
    s = A.asset_scene(A.load_asset(p), width=256, height=256)
    s, tree = S.with_tree(s)
    _run(s, tree, s.probes, frames=4)


def test_bounce_moving_part():
    """The Cornell room's short box (a movable part, with its 8 riding probes) moves between frames: the transfer of
    the Gaussians near it refreshes, its probes follow it, the light maps re-splat; then it rests again."""
    p = ASSETS / "cornell_sdf_room_plain_bin"
    if not (p / "asset.json").exists():
        pytest.skip("reference assets not copied (tests/golden/copy_assets.py)")
    from splatlight_gb300 import asset as A
    s = A.asset_scene(A.load_asset(p), width=256, height=256)
    s, tree = S.with_tree(s)
    q = next(i for i in range(len(s.parts)) if (int(s.parts["flags"][i]) & 1) == 0)   # the first movable part
    moved = s.parts.copy()
    moved["xf_prev"][q] = moved["xf"][q]
    moved["xf"][q][3] += 0.08
    moved["xf"][q][7] += 0.05
    rest = moved.copy()
    rest["xf_prev"][q] = rest["xf"][q]
    _run(s, tree, s.probes, frames=4, moves={1: (moved, 1 << q), 2: (rest, 0)})


def test_bounce_hill_lite_asset():
    """The reference's hill_lite: its baked tree, real V grids, the terrain lattice over its bounds and the
    environment's own sky SH (asset.json environment.sky.sh_rgb), lit by its sun."""
    p = ASSETS / "hill_lite_bin"
    if not (p / "asset.json").exists():
        pytest.skip("reference assets not copied (tests/golden/copy_assets.py)")
    from splatlight_gb300 import asset as A
    s = A.asset_scene(A.load_asset(p), width=256, height=256)
    assert s.sky_sh is not None and s.probes["terrain"]
    s, tree = S.with_tree(s)
    _run(s, tree, s.probes, frames=3)


def test_bounce_in_the_lit_frame():
    """The projection adds gain x lo_b (toward the eye) to the lit colour (shaders/project.wgsl:321-326): the frame
    with the bounce equals the restatement's render of the same colour and bounce."""
    import torch
    from oracle import oracle as O
    s = _bounce_lit(S.hill(30000, seed=5, width=256, height=192, n_emit=8))
    s = dataclasses.replace(s, shadow_res=256, sun_res=256)
    s, tree = S.with_tree(s)
    r, L, st = _run(s, tree, PR.for_scene(s), frames=3)
    col = L.read()[0]
    gain = 0.8
    f = camera.make_frame(s.eye, s.target, s.up, s.fov_deg, s.width, s.height, s.count, far=s.far,
                          view_mode=VIEW_LIT, n_emit=s.n_drawn_emitters, bounce_gain=gain)
    img = r.render(f)
    torch.cuda.synchronize()
    ref = O.render(s.gaussians, s.parts, f, emitters=s.emitters, colour=col, lo_b=st["lo_b"].reshape(-1, 4),
                   threads=8)["rgba"]
    assert np.abs(img - ref).max() <= 1e-3
    f0 = camera.make_frame(s.eye, s.target, s.up, s.fov_deg, s.width, s.height, s.count, far=s.far,
                           view_mode=VIEW_LIT, n_emit=s.n_drawn_emitters, bounce_gain=0.0)
    img0 = r.render(f0)
    assert img.sum() > img0.sum()   # the bounce brightens the frame


# ---- the sender cut (the reference's default senders: bounce.wgsl sc_select .. node_sh2_sc)

def test_sender_cut_hill_terrain_sky():
    """The hill's terrain lattice with its sky: the cut's marks, its nodes' transfer, sampled shadow and direct light,
    and everything downstream against the restatement over 5 frames (the cut nodes refresh a quarter a frame)."""
    s = _bounce_lit(S.hill(40000, seed=3, width=320, height=240, n_emit=8))
    s = dataclasses.replace(s, shadow_res=256, sun_res=256)
    s, tree = S.with_tree(s)
    _, L, st = _run(s, tree, PR.for_scene(s), sender_cut=True)
    fl = st["sc_flag"]
    assert (fl[s.count:] == 2).sum() > 0 and (fl[:s.count] == 3).sum() > 0
    assert (st["lo_b"][:, 0, :3].sum(axis=1) > 0).mean() > 0.9


def test_sender_cut_cornell_room():
    s = _bounce_lit(S.cornell(20000, seed=2, width=256, height=256, n_emit=4))
    s = dataclasses.replace(s, shadow_res=256)
    s, tree = S.with_tree(s)
    _run(s, tree, PR.for_scene(s), frames=4, sender_cut=True)


def test_sender_cut_moving_part():
    """The reference's Cornell room with the cut: the short box moves (the cut is selected again around its riding
    probes), then rests."""
    p = ASSETS / "cornell_sdf_room_plain_bin"
    if not (p / "asset.json").exists():
        pytest.skip("reference assets not copied (tests/golden/copy_assets.py)")
    from splatlight_gb300 import asset as A
    s = A.asset_scene(A.load_asset(p), width=256, height=256)
    s, tree = S.with_tree(s)
    q = next(i for i in range(len(s.parts)) if (int(s.parts["flags"][i]) & 1) == 0)
    moved = s.parts.copy()
    moved["xf_prev"][q] = moved["xf"][q]
    moved["xf"][q][3] += 0.08
    moved["xf"][q][7] += 0.05
    rest = moved.copy()
    rest["xf_prev"][q] = rest["xf"][q]
    _run(s, tree, s.probes, frames=4, moves={1: (moved, 1 << q), 2: (rest, 0)}, sender_cut=True)


def test_sender_cut_hill_lite_asset():
    p = ASSETS / "hill_lite_bin"
    if not (p / "asset.json").exists():
        pytest.skip("reference assets not copied (tests/golden/copy_assets.py)")
    from splatlight_gb300 import asset as A
    s = A.asset_scene(A.load_asset(p), width=256, height=256)
    s, tree = S.with_tree(s)
    _run(s, tree, s.probes, frames=3, sender_cut=True)

