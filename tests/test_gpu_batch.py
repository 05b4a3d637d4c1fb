"""The batched path (sl_batch_*): a ragged batch of views over several resident scenes equals, view by view, the
per-view path (itself pinned to the CPU restatement by test_gpu_parity_plain / test_gpu_lighting): the stable
permutation, the per-tile ranges and lists bit-exact, the images identical; a view alone and in a mix of others give
the same result; the captured graph replays for later batches that fit; capacities grow on demand."""
import numpy as np
import pytest

from splatlight_gb300 import camera, scene
from splatlight_gb300.batch import BatchRenderer, View
from splatlight_gb300.lighting import camera_forward, for_scene
from splatlight_gb300.renderer import SplatRenderer
from splatlight_gb300.structs import VIEW_DEPTH, VIEW_FLAT, VIEW_LIT, VIEW_OVERDRAW

pytestmark = pytest.mark.gpu

RGB_TOL = 1e-3


def _frame(s, W, H, mode, eye=None, target=None):
    return camera.make_frame(s.eye if eye is None else eye, s.target if target is None else target, s.up, s.fov_deg,
                             W, H, s.count, far=s.far, view_mode=mode, n_emit=len(s.emitters))


def _plain(r, f, tile):
    r.set_options(tile_w=tile[0], tile_h=tile[1])
    img = r.render(f)
    return img, r.read_debug()


def _assert_view(B, k, view, r, tile, exact=True):
    f = np.asarray(view.frame).reshape(())
    img_b = view._img
    img_p, dbg = _plain(r, f, tile)
    order, ranges, entries = B.read_view(k, r.last_stats.slots, r.last_stats.tiles)
    assert np.array_equal(order, dbg["order"]), k
    assert np.array_equal(ranges, dbg["ranges"]), k
    assert np.array_equal(entries, dbg["entries"]), k
    if exact:
        assert np.array_equal(img_b, img_p), (k, float(np.abs(img_b - img_p).max()))
    else:
        assert float(np.abs(img_b - img_p).max()) <= RGB_TOL


def _scenes():
    a = scene.subset(scene.cornell(), 20000)
    b = scene.subset(scene.hill(), 60000)
    return a, b


def _views(a, b):
    """A ragged mix: two scenes, five resolutions, three view modes, several cameras."""
    hill_eye = lambda yaw, pitch, rad: camera.orbit_eye((0.0, 0.0, 1.0), rad, yaw, pitch)
    vs = [
        View(0, _frame(a, 160, 120, VIEW_FLAT), a.eye),
        View(1, _frame(b, 320, 180, VIEW_FLAT, eye=hill_eye(0.3, 0.4, 12.0), target=(0, 0, 1)), hill_eye(0.3, 0.4, 12.0)),
        View(0, _frame(a, 97, 61, VIEW_OVERDRAW, eye=(0.4, 0.2, 3.2)), (0.4, 0.2, 3.2)),
        View(1, _frame(b, 255, 257, VIEW_DEPTH, eye=hill_eye(2.0, 0.15, 6.0), target=(0, 0, 1)), hill_eye(2.0, 0.15, 6.0)),
        View(1, _frame(b, 480, 270, VIEW_OVERDRAW, eye=hill_eye(4.0, 0.9, 20.0), target=(0, 0, 1)), hill_eye(4.0, 0.9, 20.0)),
        View(0, _frame(a, 33, 200, VIEW_FLAT, eye=(-0.5, 0.3, 2.5)), (-0.5, 0.3, 2.5)),
    ]
    return vs


def _render(B, views):
    imgs = B.render(views)
    for v, im in zip(views, imgs):
        v._img = im
    return imgs


@pytest.mark.parametrize("tile", [(16, 16), (8, 32), (32, 8)])
def test_ragged_mix_equals_per_view(cuda, tile):
    a, b = _scenes()
    with SplatRenderer(a.gaussians, a.parts) as ra, SplatRenderer(b.gaussians, b.parts) as rb:
        ra.set_emitters(a.emitters)
        rb.set_emitters(b.emitters)
        with BatchRenderer([ra, rb], max_views=16, tile=tile) as B:
            views = _views(a, b)
            _render(B, views)
            assert B.last_stats.views == len(views)
            for k, v in enumerate(views):
                _assert_view(B, k, v, [ra, rb][v.scene], tile)


def test_view_with_nothing_visible(cuda):
    """A camera turned away from its scene: no visible splat, so the binning emits no entry (every block of the
    one-pass binning is past the visible count and the entry total stays 0); alone and between other views it gives
    the per-view path's empty image, lists and ranges."""
    a, b = _scenes()
    away = tuple(2.0 * np.asarray(a.eye, np.float64) - np.asarray(a.target, np.float64))
    with SplatRenderer(a.gaussians, a.parts) as ra, SplatRenderer(b.gaussians, b.parts) as rb:
        ra.set_emitters(a.emitters)
        rb.set_emitters(b.emitters)
        with BatchRenderer([ra, rb], max_views=16) as B:
            empty = View(0, _frame(a, 200, 150, VIEW_FLAT, target=away), a.eye)
            img = _render(B, [empty])[0]
            assert B.last_stats.entries == 0
            assert not img.any()
            _assert_view(B, 0, empty, ra, (16, 16))
            views = _views(a, b)
            mix = views[:3] + [empty] + views[3:]
            _render(B, mix)
            assert B.last_stats.entries > 0
            for k, v in enumerate(mix):
                _assert_view(B, k, v, [ra, rb][v.scene], (16, 16))


def test_alone_and_in_mix(cuda):
    a, b = _scenes()
    with SplatRenderer(a.gaussians, a.parts) as ra, SplatRenderer(b.gaussians, b.parts) as rb:
        ra.set_emitters(a.emitters)
        rb.set_emitters(b.emitters)
        with BatchRenderer([ra, rb], max_views=16) as B:
            views = _views(a, b)
            mix = [im.copy() for im in _render(B, views)]
            for k, v in enumerate(views):
                alone = B.render([v])[0]
                assert np.array_equal(alone, mix[k]), k
            # reversed order: every view still the same
            rev = B.render(views[::-1])
            for k, im in enumerate(rev[::-1]):
                assert np.array_equal(im, mix[k]), k


def test_graph_replay_and_growth(cuda):
    a, b = _scenes()
    with SplatRenderer(a.gaussians, a.parts) as ra, SplatRenderer(b.gaussians, b.parts) as rb:
        ra.set_emitters(a.emitters)
        rb.set_emitters(b.emitters)
        # tiny capacities: the first batch grows slots, tiles and (through the overflow retry) tile entries
        with BatchRenderer([ra, rb], max_views=8, max_slots=256, max_tiles=8, max_entries=64) as B:
            views = _views(a, b)[:4]
            first = [im.copy() for im in _render(B, views)]
            for k, v in enumerate(views):
                _assert_view(B, k, v, [ra, rb][v.scene], (16, 16))
            again = B.render(views)
            assert B.last_stats.graph_replayed == 1
            for x, y in zip(first, again):
                assert np.array_equal(x, y)
            fewer = views[1:3]
            _render(B, fewer)
            assert B.last_stats.graph_replayed == 1
            for k, v in enumerate(fewer):
                _assert_view(B, k, v, [ra, rb][v.scene], (16, 16))


def test_capacity_classes(cuda):
    """A small batch runs the graph of a small capacity class (1/16 or 1/4 of the capacity); when its tile entries
    outgrow the class it runs again in the class that holds them.  Every class gives the same images, bit for bit,
    as a batch sized exactly for the views."""
    a, b = _scenes()
    with SplatRenderer(a.gaussians, a.parts) as ra, SplatRenderer(b.gaussians, b.parts) as rb:
        ra.set_emitters(a.emitters)
        rb.set_emitters(b.emitters)
        views = _views(a, b)[:2]
        with BatchRenderer([ra, rb], max_views=8) as exact:
            ref = [im.copy() for im in _render(exact, views)]
            entries = exact.last_stats.entries
        # slots for 64 such batches; entries for 8x these views: class 0 holds 1/16 of that, fewer than the views need
        with BatchRenderer([ra, rb], max_views=8, max_slots=64 * exact.last_stats.slots,
                           max_entries=8 * entries) as big:
            assert 8 * entries // 16 < entries
            got = [im.copy() for im in _render(big, views)]
            for x, y in zip(ref, got):
                assert np.array_equal(x, y)
            for k, v in enumerate(views):
                _assert_view(big, k, v, [ra, rb][v.scene], (16, 16))
            again = big.render(views)          # the class that held them, replayed
            assert big.last_stats.graph_replayed == 1
            for x, y in zip(ref, again):
                assert np.array_equal(x, y)


def test_no_graph_matches_graph(cuda):
    a, b = _scenes()
    with SplatRenderer(a.gaussians, a.parts) as ra, SplatRenderer(b.gaussians, b.parts) as rb:
        ra.set_emitters(a.emitters)
        rb.set_emitters(b.emitters)
        views = _views(a, b)
        with BatchRenderer([ra, rb], graph=True) as B1, BatchRenderer([ra, rb], graph=False) as B2:
            x = [im.copy() for im in B1.render(views)]
            y = B2.render(views)
            for p, q in zip(x, y):
                assert np.array_equal(p, q)


def test_lit_views_two_scenes(cuda):
    """Lit views: each scene's lighting updated at that view's camera; the batched shading pass gives the same
    radiance as the lighting's own pass (RGB within 1e-3; ordering and lists exact)."""
    a, b = _scenes()
    b = scene.dataclasses.replace(b, shadow_res=256, sun_res=512)
    with SplatRenderer(a.gaussians, a.parts) as ra, SplatRenderer(b.gaussians, b.parts) as rb:
        La = for_scene(ra, a)
        Lb = for_scene(rb, b)
        La.update(a.eye, camera_forward(a))
        Lb.update(b.eye, camera_forward(b))
        views = [View(0, _frame(a, 200, 150, VIEW_LIT), a.eye),
                 View(1, _frame(b, 320, 180, VIEW_LIT), b.eye),
                 View(0, _frame(a, 64, 64, VIEW_FLAT, eye=(0.2, 0.1, 3.0)), (0.2, 0.1, 3.0)),
                 View(1, _frame(b, 160, 90, VIEW_LIT), b.eye)]
        with BatchRenderer([ra, rb], [La, Lb]) as B:
            _render(B, views)
            for k, v in enumerate(views):
                _assert_view(B, k, v, [ra, rb][v.scene], (16, 16), exact=False)
        La.close()
        Lb.close()


def test_lit_views_many_eyes(cuda):
    """Several lit views of one scene from different cameras: the batch shades each view at its own eye with the
    scene's maps; the per-view path gives the same with the maps kept and the shading pass re-run at that eye."""
    a, _ = _scenes()
    with SplatRenderer(a.gaussians, a.parts) as ra:
        La = for_scene(ra, a)
        La.update(a.eye, camera_forward(a))
        eyes = [(0.0, 0.0, 3.5), (0.6, 0.3, 3.0), (-0.8, -0.2, 2.6), (0.1, 0.7, 3.9)]
        views = [View(0, _frame(a, 128 + 32 * k, 96 + 16 * k, VIEW_LIT, eye=e), e) for k, e in enumerate(eyes)]
        with BatchRenderer([ra], [La]) as B:
            _render(B, views)
            for k, v in enumerate(views):
                La.shade(v.eye)
                _assert_view(B, k, v, ra, (16, 16), exact=False)
        La.close()


def test_light_scale_matches_plain(cuda):
    """A request's light-intensity scale: the batched view equals the per-view path with every light's intensity
    (emitters and sun) scaled through the lighting setters (RGB within 1e-3)."""
    _, b = _scenes()
    b = scene.dataclasses.replace(b, shadow_res=256, sun_res=512)
    k = 1.7
    with SplatRenderer(b.gaussians, b.parts) as rb:
        Lb = for_scene(rb, b)
        Lb.update(b.eye, camera_forward(b))
        views = [View(0, _frame(b, 320, 180, VIEW_LIT), b.eye, light_scale=k),
                 View(0, _frame(b, 160, 90, VIEW_LIT), b.eye, light_scale=1.0)]
        with BatchRenderer([rb], [Lb]) as B:
            imgs = [im.copy() for im in B.render(views)]
            base = rb.render(views[1].frame)
            assert float(np.abs(imgs[1] - base).max()) <= RGB_TOL
            Lb.set_emitters(b.emitters, scale=k)
            sun = b.sun
            Lb.set_environment([(sun.direction, sun.angular_std, tuple(np.float32(sun.irradiance) * np.float32(k)),
                                 sun.casts_shadows)], b.sky_ambient)
            Lb.update(b.eye, camera_forward(b))
            scaled = rb.render(views[0].frame)
            assert float(np.abs(imgs[0] - scaled).max()) <= RGB_TOL
            assert float(imgs[0][..., :3].max()) > 0.0   # the lit image is not empty
        Lb.close()


def test_coverage_pass_and_bright_views(cuda):
    """Deferred shading: the batch shades only the Gaussians its coverage pass marks (fewer than the visible ones); a
    view whose shaded radiance passes the coverage pass's allowance (here: a scene whose lights are 500x brighter, at
    request light scale 1; the allowance already grows with the request's own scale) runs again with every blended
    splat shaded, and each view's image is the same alone as in the mix (bit for bit) -- the decision depends on the
    view alone."""
    a, b = _scenes()
    b = scene.dataclasses.replace(b, shadow_res=256, sun_res=512)
    with SplatRenderer(a.gaussians, a.parts) as ra, SplatRenderer(b.gaussians, b.parts) as rb:
        La = for_scene(ra, a)
        La.update(a.eye, camera_forward(a))
        Lb = for_scene(rb, b)
        k = 500.0
        Lb.set_emitters(b.emitters, scale=k)
        sun = b.sun
        Lb.set_environment([(sun.direction, sun.angular_std, tuple(np.float32(sun.irradiance) * np.float32(k)),
                             sun.casts_shadows)], b.sky_ambient)
        Lb.update(b.eye, camera_forward(b))
        normal = View(0, _frame(a, 200, 150, VIEW_LIT), a.eye)
        bright = View(1, _frame(b, 256, 144, VIEW_LIT), b.eye)
        with BatchRenderer([ra, rb], [La, Lb]) as B:
            alone_n = B.render([normal])[0].copy()
            st = B.last_stats
            assert 0 < st.shaded < st.visible and st.reshaded_views == 0
            alone_b = B.render([bright])[0].copy()
            assert B.last_stats.reshaded_views == 1
            mix = [im.copy() for im in B.render([bright, normal])]
            assert B.last_stats.reshaded_views == 1
            assert np.array_equal(mix[0], alone_b) and np.array_equal(mix[1], alone_n)
            assert float(alone_b[..., :3].max()) > 32.0
        La.close()
        Lb.close()


def test_autotune_keeps_results(cuda):
    a, b = _scenes()
    with SplatRenderer(a.gaussians, a.parts) as ra, SplatRenderer(b.gaussians, b.parts) as rb:
        ra.set_emitters(a.emitters)
        rb.set_emitters(b.emitters)
        views = _views(a, b)
        with BatchRenderer([ra, rb]) as B:
            tile, ms = B.autotune(views, reps=2)
            assert tile in ((16, 16), (8, 32), (32, 8))
            assert all(t > 0 for t in ms.values())
            _render(B, views)
            for k, v in enumerate(views):
                _assert_view(B, k, v, [ra, rb][v.scene], tile)


def test_block_size_variants_agree(cuda):
    """Every block-size variant of bproject, btile_bin, bshade and bcomposite (the autotuner's choices) renders a lit
    ragged batch identically, bit for bit; the autotuner's pick is one of them and is reported."""
    a, b = _scenes()
    b = scene.dataclasses.replace(b, shadow_res=256, sun_res=512)
    with SplatRenderer(a.gaussians, a.parts) as ra, SplatRenderer(b.gaussians, b.parts) as rb:
        La = for_scene(ra, a)
        Lb = for_scene(rb, b)
        La.update(a.eye, camera_forward(a))
        Lb.update(b.eye, camera_forward(b))
        views = [View(0, _frame(a, 200, 150, VIEW_LIT), a.eye),
                 View(1, _frame(b, 320, 180, VIEW_LIT), b.eye),
                 View(0, _frame(a, 64, 64, VIEW_OVERDRAW, eye=(0.2, 0.1, 3.0)), (0.2, 0.1, 3.0)),
                 View(1, _frame(b, 160, 90, VIEW_LIT, eye=(3.0, -6.0, 4.0)), (3.0, -6.0, 4.0))]
        choices = {"bproject": (4, 3), "btile_bin": (4, 5), "bshade": (4, 3, 5), "bcomposite": (6, 5)}
        with BatchRenderer([ra, rb], [La, Lb]) as B:
            base = {k: v[0] for k, v in choices.items()}
            B.set_tuning(base)
            ref = [x.copy() for x in B.render(views)]
            for k, vals in choices.items():
                for mb in vals[1:]:
                    B.set_tuning(dict(base, **{k: mb}))
                    assert B.tuning()[1][k] == mb
                    for i, img in enumerate(B.render(views)):
                        assert np.array_equal(img, ref[i]), (k, mb, i)
            tile, _ = B.autotune(views, reps=1)
            got = B.tuning()
            assert got[0] == tile and all(got[1][k] in v for k, v in choices.items())
            from splatlight_gb300._native import SplatlightError
            with pytest.raises(SplatlightError):
                B.set_tuning(dict(base, bshade=7))
        La.close()
        Lb.close()


def test_bad_arguments(cuda):
    a, _ = _scenes()
    from splatlight_gb300._native import SplatlightError
    with SplatRenderer(a.gaussians, a.parts) as ra:
        ra.set_emitters(a.emitters)
        with BatchRenderer([ra], max_views=2) as B:
            v = View(0, _frame(a, 64, 64, VIEW_FLAT), a.eye)
            with pytest.raises(SplatlightError):
                B.render([v, v, v])                    # more than max_views
            with pytest.raises(SplatlightError):
                B.render([View(3, v.frame, a.eye)])    # no such scene
            with pytest.raises(SplatlightError):
                B.set_tile(16, 8)
            assert np.isfinite(B.render([v])[0]).all()


def test_full_size_lit_batch(cuda):
    """Config 2 at full size on its two largest scenes: the 1,048,576- and 2,097,152-Gaussian hill scenes lit (emitter
    light map, sun maps), two 1920x1080 views of each from different cameras in one batch; every view's permutation,
    ranges and lists equal the per-view path's, its image within 1e-3, with the per-view shading pass re-run at that
    view's eye."""
    s1 = scene.hill(1048576, seed=1)
    s2 = scene.hill(2097152, seed=1)
    eyes = {0: [s1.eye, camera.orbit_eye((0.0, 0.0, 1.5), 9.0, 1.2, 0.35)],
            1: [s2.eye, camera.orbit_eye((0.0, 0.0, 1.5), 7.0, 3.9, 0.55)]}
    with SplatRenderer(s1.gaussians, s1.parts) as r1, SplatRenderer(s2.gaussians, s2.parts) as r2:
        L1 = for_scene(r1, s1)
        L2 = for_scene(r2, s2)
        L1.update(s1.eye, camera_forward(s1))
        L2.update(s2.eye, camera_forward(s2))
        ss, rr, LL = [s1, s2], [r1, r2], [L1, L2]
        views = [View(k, _frame(ss[k], 1920, 1080, VIEW_LIT, eye=e, target=ss[k].target), e)
                 for k in (0, 1) for e in eyes[k]]
        with BatchRenderer(rr, LL, max_views=len(views)) as B:
            _render(B, views)
            for k, v in enumerate(views):
                LL[v.scene].shade(v.eye)
                _assert_view(B, k, v, rr[v.scene], (16, 16), exact=False)
        L1.close()
        L2.close()
