"""GPU parity of the plain per-view path against the CPU restatement (oracle/): sort keys, the stable permutation, the
per-tile ranges and lists and the per-pixel contributor counts bit-exact; linear RGBA within 1e-3 max abs."""
import numpy as np
import pytest

from splatlight_gb300 import camera, scene
from splatlight_gb300.renderer import SplatRenderer
from splatlight_gb300.structs import VIEW_DEPTH, VIEW_FLAT, VIEW_LIT, VIEW_OVERDRAW

pytestmark = pytest.mark.gpu

RGB_TOL = 1e-3   # max abs, linear RGBA


def _frame(s, W, H, mode, **kw):
    return camera.make_frame(kw.pop("eye", s.eye), kw.pop("target", s.target), s.up, s.fov_deg, W, H, s.count,
                             far=s.far, view_mode=mode, n_emit=kw.pop("n_emit", len(s.emitters)), **kw)


def _check(r, s, f, orc, tile, colour_host=None, check_rgb=True):
    W, H = int(f["viewport"][0]), int(f["viewport"][1])
    img = r.render(f)
    dbg = r.read_debug()
    ref = orc.render(s.gaussians, s.parts, f, emitters=s.emitters, colour=colour_host, tile=tile, threads=8)
    assert r.last_stats.visible == ref["visible"]
    assert np.array_equal(dbg["keys"], ref["keys"])
    assert np.array_equal(dbg["order"], ref["order"])
    assert np.array_equal(dbg["ranges"], ref["ranges"])
    assert np.array_equal(dbg["entries"], ref["entries"])
    if int(f["view_mode"]) == VIEW_OVERDRAW:
        assert np.array_equal(r.read_counts(W, H), ref["counts"])
        assert np.array_equal(img[..., 0], ref["counts"].astype(np.float32))
    elif check_rgb:
        err = float(np.abs(img - ref["rgba"]).max())
        assert err <= RGB_TOL, err
    return img, ref


@pytest.mark.parametrize("mode", [VIEW_FLAT, VIEW_OVERDRAW, VIEW_DEPTH])
@pytest.mark.parametrize("tile", [(16, 16), (8, 32), (32, 8)])
def test_cornell_small(cuda, orc, mode, tile):
    s = scene.subset(scene.cornell(), 6000)
    with SplatRenderer(s.gaussians, s.parts) as r:
        r.set_emitters(s.emitters)
        r.set_options(tile_w=tile[0], tile_h=tile[1])
        _check(r, s, _frame(s, 160, 120, mode), orc, tile)


def test_cornell_lit_bound_colour(cuda, orc):
    torch = cuda
    s = scene.cornell()
    rng = np.random.default_rng(5)
    colour = rng.uniform(0, 3, (s.count, 4)).astype(np.float32)
    dev = torch.from_numpy(colour).cuda()
    with SplatRenderer(s.gaussians, s.parts) as r:
        r.set_emitters(s.emitters)
        r.bind_colour(dev)
        _check(r, s, _frame(s, s.width, s.height, VIEW_LIT), orc, (16, 16), colour_host=colour)


@pytest.mark.parametrize("mode", [VIEW_FLAT, VIEW_OVERDRAW])
def test_cornell_full_config(cuda, orc, mode):
    s = scene.cornell()
    with SplatRenderer(s.gaussians, s.parts) as r:
        r.set_emitters(s.emitters)
        _check(r, s, _frame(s, s.width, s.height, mode), orc, (16, 16))


def test_hill_subset_views(cuda, orc):
    s = scene.subset(scene.hill(), 120000)
    with SplatRenderer(s.gaussians, s.parts) as r:
        r.set_emitters(s.emitters)
        for k, (yaw, pitch, rad) in enumerate([(0.3, 0.4, 12.0), (2.0, 0.15, 6.0), (4.0, 0.9, 20.0)]):
            eye = camera.orbit_eye((0.0, 0.0, 1.0), rad, yaw, pitch)
            for mode in (VIEW_FLAT, VIEW_OVERDRAW):
                _check(r, s, _frame(s, 480, 270, mode, eye=eye, target=(0.0, 0.0, 1.0)), orc, (16, 16))


def test_hill_full_config(cuda, orc):
    """The benchmark's configuration at full size: 1,048,576 Gaussians at 1920x1080."""
    s = scene.hill()
    with SplatRenderer(s.gaussians, s.parts) as r:
        r.set_emitters(s.emitters)
        _check(r, s, _frame(s, s.width, s.height, VIEW_OVERDRAW), orc, (16, 16))
        img, ref = _check(r, s, _frame(s, s.width, s.height, VIEW_FLAT), orc, (16, 16))
        assert r.last_stats.entries == ref["n_entries"]


def test_tile_entry_overflow_grows_and_renders_again(cuda, orc):
    """A tile-entry capacity far below the frame's entries: the one-pass binning writes none past it, flags the
    overflow and reports the exact total; the renderer grows to it and renders again, with lists and image equal to
    the restatement's and to a render that never overflowed."""
    s = scene.subset(scene.cornell(), 20000)
    f = _frame(s, 256, 192, VIEW_FLAT)
    with SplatRenderer(s.gaussians, s.parts) as r0:
        r0.set_emitters(s.emitters)
        want = r0.render(f)
    with SplatRenderer(s.gaussians, s.parts) as r:
        r.set_emitters(s.emitters)
        r.set_options(entry_capacity=64)
        img, ref = _check(r, s, f, orc, (16, 16))
        assert ref["n_entries"] > 64
        assert np.array_equal(img, want)


def test_empty_view(cuda, orc):
    """Camera looking away from everything: no valid key, no entry, a transparent image."""
    s = scene.subset(scene.cornell(), 2000)
    with SplatRenderer(s.gaussians, s.parts) as r:
        r.set_emitters(s.emitters)
        f = _frame(s, 64, 64, VIEW_FLAT, eye=(0.0, 0.0, 3.5), target=(0.0, 0.0, 10.0))
        img, ref = _check(r, s, f, orc, (16, 16))
        assert r.last_stats.visible == 0 and r.last_stats.entries == 0
        assert not img.any()


def test_hidden_parts_and_fade(cuda, orc):
    s = scene.subset(scene.cornell(), 5000)
    parts = s.parts.copy()
    parts["flags"][2] |= 4            # hidden (shaders/common.wgsl:40)
    with SplatRenderer(s.gaussians, parts) as r:
        r.set_emitters(s.emitters)
        f = _frame(s, 128, 128, VIEW_FLAT)
        f["part_fade"][3] = 0.5
        f["part_fade"][4] = 1.0
        s2 = scene.dataclasses.replace(s, parts=parts)
        _check(r, s2, f, orc, (16, 16))


def test_equal_keys_keep_index_order(cuda, orc):
    """Thousands of Gaussians at one depth share a key: the stable sort keeps them in slot order."""
    s = scene.subset(scene.cornell(), 3000)
    g = s.gaussians.copy()
    g["mu"][:, 2] = -1.0                     # all on the back wall plane, facing the camera
    g["mu"][:, :2] *= 0.5
    s2 = scene.dataclasses.replace(s, gaussians=g)
    with SplatRenderer(g, s.parts) as r:
        r.set_emitters(s.emitters)
        f = _frame(s2, 128, 128, VIEW_OVERDRAW, n_emit=0)
        _check(r, s2, f, orc, (16, 16))
        dbg = r.read_debug()
        k = dbg["keys"][dbg["order"]]
        v = r.last_stats.visible
        same = k[1:v] == k[: v - 1]
        assert same.sum() > 1000
        assert np.all(dbg["order"][1:v][same] > dbg["order"][: v - 1][same])


def test_unsupported_frame_features(cuda):
    from splatlight_gb300._native import SplatlightError
    s = scene.subset(scene.cornell(), 500)
    with SplatRenderer(s.gaussians, s.parts) as r:
        r.set_emitters(s.emitters)
        for field, idx, val in [("lod", 0, 1), ("explode_k", 2, 1.0), ("lamp", 3, 1.0), ("lamp_color", 3, 1.0)]:
            f = _frame(s, 32, 32, VIEW_FLAT)
            f[field][idx] = val
            with pytest.raises(SplatlightError) as e:
                r.render(f)
            assert e.value.code == -6
        f = _frame(s, 32, 32, VIEW_FLAT, n_emit=len(s.emitters) + 1)
        with pytest.raises(SplatlightError) as e:
            r.render(f)
        assert e.value.code == -1


def test_device_output_and_stream(cuda, orc):
    torch = cuda
    s = scene.subset(scene.cornell(), 3000)
    with SplatRenderer(s.gaussians, s.parts) as r:
        r.set_emitters(s.emitters)
        f = _frame(s, 96, 64, VIEW_FLAT)
        out = torch.empty((64, 96, 4), dtype=torch.float32, device="cuda")
        st = torch.cuda.Stream()
        r.render(f, out=out, stream=st.cuda_stream)
        ref = orc.render(s.gaussians, s.parts, f, emitters=s.emitters)
        assert float(np.abs(out.cpu().numpy() - ref["rgba"]).max()) <= RGB_TOL


@pytest.mark.parametrize("mode", [VIEW_FLAT, VIEW_OVERDRAW])
def test_counting_sort(cuda, orc, mode):
    """The counting-sort placement (scan.wgsl + scatter.wgsl; sort_mode 2): the order holds every valid slot once, in
    key order, each key's slots the same set as the stable sort's (ties land in arbitrary order, as the reference
    says); given that order, the tile lists are bit-exact, the contributor counts bit-exact and RGB within 1e-3."""
    s = scene.subset(scene.cornell(), 30000)
    with SplatRenderer(s.gaussians, s.parts) as r:
        r.set_emitters(s.emitters)
        f = _frame(s, 256, 192, mode)
        r.set_options(sort_mode=1)
        r.render(f)
        stable = r.read_debug()
        r.set_options(sort_mode=2)
        img = r.render(f)
        dbg = r.read_debug()
        vis = r.last_stats.visible
        order = dbg["order"][:vis]
        assert np.array_equal(np.sort(order), np.sort(stable["order"][:vis]))
        k = dbg["keys"][order]
        assert np.all(np.diff(k.astype(np.int64)) >= 0)
        assert np.array_equal(np.sort(order.astype(np.uint64) + (k.astype(np.uint64) << 32)),
                              np.sort(stable["order"][:vis].astype(np.uint64) +
                                      (dbg["keys"][stable["order"][:vis]].astype(np.uint64) << 32)))
        ref = orc.render_given_order(s.gaussians, s.parts, f, order, emitters=s.emitters)
        assert np.array_equal(dbg["keys"], ref["keys"])
        assert np.array_equal(dbg["ranges"], ref["ranges"])
        assert np.array_equal(dbg["entries"], ref["entries"])
        if mode == VIEW_OVERDRAW:
            assert np.array_equal(img[..., 0].astype(np.uint32), ref["counts"])
        else:
            assert float(np.abs(img - ref["rgba"]).max()) <= RGB_TOL
        r.set_options(sort_mode=1)


def test_pinned_host_image_written_in_place(cuda):
    """A page-locked host image is written by the compositor in place (no staging copy): the same pixels as a
    pageable host image and as a device image."""
    torch = cuda
    s = scene.subset(scene.cornell(), 20000)
    with SplatRenderer(s.gaussians, s.parts) as r:
        r.set_emitters(s.emitters)
        for mode in (VIEW_FLAT, VIEW_OVERDRAW):
            f = _frame(s, 200, 150, mode)
            pageable = r.render(f)
            pinned = torch.empty((150, 200, 4), dtype=torch.float32, pin_memory=True).numpy()
            r.render(f, out=pinned)
            dev = torch.empty((150, 200, 4), dtype=torch.float32, device="cuda")
            r.render(f, out=dev)
            assert np.array_equal(pinned, pageable) and np.array_equal(dev.cpu().numpy(), pageable)
