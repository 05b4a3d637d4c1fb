"""The request server (sl_server_*): continuous batching over resident scenes.  Every served image equals the same
request rendered alone by the batched path (bit for bit) and, at light scale 1, the per-view path (RGB within 1e-3);
admission refuses what can never fit and bad requests without disturbing the others; batches overlap on the device;
shutdown never waits on result slots the caller keeps."""
import time

import numpy as np
import pytest

from splatlight_gb300 import camera, scene
from splatlight_gb300._native import SplatlightError
from splatlight_gb300.batch import BatchRenderer, View
from splatlight_gb300.lighting import camera_forward, for_scene
from splatlight_gb300.renderer import SplatRenderer
from splatlight_gb300.server import RenderServer
from splatlight_gb300.structs import VIEW_FLAT, VIEW_LIT

pytestmark = pytest.mark.gpu

RGB_TOL = 1e-3


def _frame(s, W, H, mode, eye):
    return camera.make_frame(eye, s.target, s.up, s.fov_deg, W, H, s.count, far=s.far, view_mode=mode,
                             n_emit=len(s.emitters))


@pytest.fixture(scope="module")
def world(cuda):
    a = scene.subset(scene.cornell(), 20000)
    b = scene.dataclasses.replace(scene.subset(scene.hill(), 60000), shadow_res=256, sun_res=512)
    rs = [SplatRenderer(a.gaussians, a.parts), SplatRenderer(b.gaussians, b.parts)]
    ls = [for_scene(rs[0], a), for_scene(rs[1], b)]
    for L, s in zip(ls, (a, b)):
        L.update(s.eye, camera_forward(s))
    yield (a, b), rs, ls
    for L in ls:
        L.close()
    for r in rs:
        r.close()


def _requests(scenes, n, seed=0):
    rng = np.random.default_rng(seed)
    res = [(64, 64), (160, 120), (320, 180), (97, 53)]
    out = []
    for k in range(n):
        si = int(rng.integers(2))
        s = scenes[si]
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        eye = tuple(np.float32(np.asarray(s.target) + rng.uniform(3.0, 6.0) * d))
        W, H = res[int(rng.integers(len(res)))]
        mode = VIEW_LIT if rng.random() < 0.75 else VIEW_FLAT
        ls = float(np.float32(rng.uniform(0.5, 2.0)))
        out.append((si, _frame(s, W, H, mode, eye), eye, ls))
    return out


def _drain(srv, n, timeout=60.0):
    got = {}
    t0 = time.time()
    while len(got) < n and time.time() - t0 < timeout:
        for r in srv.poll(wait_us=20000):
            got[r.tag] = r
    assert len(got) == n, (len(got), n)
    return got


def test_served_equals_alone(world):
    scenes, rs, ls = world
    reqs = _requests(scenes, 40)
    with RenderServer(rs, ls, max_views=16, pipelines=2, max_view_pixels=320 * 180) as srv:
        for k, (si, f, eye, lsc) in enumerate(reqs):
            srv.submit(si, f, eye, lsc, tag=k)
        got = _drain(srv, len(reqs))
        st = srv.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["batches"] >= 3          # batched, and more than one batch
    with BatchRenderer(rs, ls, max_views=4) as B:
        for k, (si, f, eye, lsc) in enumerate(reqs):
            r = got[k]
            assert r.status == 0
            alone = B.render([View(si, f, eye, lsc)])[0]
            assert np.array_equal(r.image, alone), k


def test_served_equals_per_view_path(world):
    scenes, rs, ls = world
    reqs = [q for q in _requests(scenes, 12, seed=3)]
    reqs = [(si, f, eye, 1.0) for si, f, eye, _ in reqs]
    with RenderServer(rs, ls, max_views=8, pipelines=2, max_view_pixels=320 * 180) as srv:
        for k, (si, f, eye, lsc) in enumerate(reqs):
            srv.submit(si, f, eye, lsc, tag=k)
        got = _drain(srv, len(reqs))
    for k, (si, f, eye, _) in enumerate(reqs):
        ls[si].shade(eye)
        ref = rs[si].render(f)
        err = float(np.abs(got[k].image - ref).max())
        assert err <= RGB_TOL, (k, err)


def test_bright_request_reruns_and_completes(world):
    """A request of a scene bright enough to pass the coverage pass's radiance allowance is re-run with every blended
    splat shaded (inside the same batch's retry): it completes, and every request equals its image rendered alone."""
    scenes, rs, ls = world
    b = scenes[1]
    a = scenes[0]
    with SplatRenderer(b.gaussians, b.parts) as rb:
        Lb = for_scene(rb, b)
        k = 500.0
        Lb.set_emitters(b.emitters, scale=k)
        sun = b.sun
        Lb.set_environment([(sun.direction, sun.angular_std, tuple(np.float32(sun.irradiance) * np.float32(k)),
                             sun.casts_shadows)], b.sky_ambient)
        Lb.update(b.eye, camera_forward(b))
        R, L = [rs[0], rb], [ls[0], Lb]
        reqs = [(1, _frame(b, 160, 120, VIEW_LIT, b.eye), b.eye, 1.0),
                (0, _frame(a, 96, 64, VIEW_LIT, a.eye), a.eye, 1.0),
                (0, _frame(a, 64, 64, VIEW_FLAT, a.eye), a.eye, 1.0)]
        with RenderServer(R, L, max_views=8, pipelines=1, max_view_pixels=160 * 120) as srv:
            for t, (si, f, eye, lsc) in enumerate(reqs):
                srv.submit(si, f, eye, lsc, tag=t)
            got = _drain(srv, len(reqs))
            st = srv.stats()
            assert st["failed"] == 0 and st["reshaded_views"] >= 1
            assert st["relaunches"] >= 1  # the re-shade runs the batch again
        with BatchRenderer(R, L, max_views=4) as B:
            for t, (si, f, eye, lsc) in enumerate(reqs):
                assert got[t].status == 0
                assert np.array_equal(got[t].image, B.render([View(si, f, eye, lsc)])[0]), t
        Lb.close()


def test_admission_and_bad_requests(world):
    scenes, rs, ls = world
    a = scenes[0]
    with RenderServer(rs, ls, max_views=8, max_view_pixels=128 * 128) as srv:
        with pytest.raises(SplatlightError) as e:
            srv.submit(0, _frame(a, 256, 256, VIEW_FLAT, a.eye), a.eye)   # larger than a result slot
        assert e.value.code == -7
        with pytest.raises(SplatlightError):
            srv.submit(5, _frame(a, 64, 64, VIEW_FLAT, a.eye), a.eye)     # no such scene
        bad = _frame(a, 64, 64, VIEW_FLAT, a.eye)
        bad["count"] = 7
        with pytest.raises(SplatlightError):
            srv.submit(0, bad, a.eye)                                      # frame of another asset
        srv.submit(0, _frame(a, 64, 64, VIEW_FLAT, a.eye), a.eye, tag=1)  # the good ones still run
        srv.submit(1, _frame(scenes[1], 96, 64, VIEW_LIT, scenes[1].eye), scenes[1].eye, tag=2)
        got = _drain(srv, 2)
        assert got[1].status == 0 and got[2].status == 0
        st = srv.stats()
        assert st["rejected"] == 1


def test_batches_overlap_with_two_pipelines(world):
    scenes, rs, ls = world
    reqs = _requests(scenes, 96, seed=5)
    with RenderServer(rs, ls, max_views=8, pipelines=2, max_view_pixels=320 * 180, result_slots=96) as srv:
        for k, (si, f, eye, lsc) in enumerate(reqs):
            srv.submit(si, f, eye, lsc, tag=k)
        got = _drain(srv, len(reqs))
    spans = sorted({(r.t_start, r.t_done) for r in got.values()})
    overlaps = sum(1 for (s0, e0), (s1, e1) in zip(spans, spans[1:]) if s1 < e0)
    assert overlaps >= 1, spans[:8]


def test_shutdown_with_unreleased_slots(world):
    scenes, rs, ls = world
    a = scenes[0]
    srv = RenderServer(rs, ls, max_views=2, pipelines=1, max_view_pixels=64 * 64, result_slots=2)
    for k in range(6):
        srv.submit(0, _frame(a, 64, 64, VIEW_FLAT, a.eye), a.eye, tag=k)
    time.sleep(0.5)          # two requests run; the rest wait for result slots that are never released
    t0 = time.time()
    srv.close()
    assert time.time() - t0 < 10.0


def test_bounded_pending_queue(world):
    """With max_pending set, a request beyond the queue bound is refused at submit (SL_ERR_ADMISSION); what was
    admitted still completes."""
    scenes, rs, ls = world
    a = scenes[0]
    f = _frame(a, 64, 64, VIEW_FLAT, a.eye)
    with RenderServer(rs, ls, max_views=1, pipelines=1, max_view_pixels=64 * 64, result_slots=1,
                      max_pending=2) as srv:
        srv.submit(0, f, a.eye, tag=0)
        time.sleep(0.3)                       # request 0 holds the only result slot until it is polled
        srv.submit(0, f, a.eye, tag=1)
        srv.submit(0, f, a.eye, tag=2)
        with pytest.raises(SplatlightError) as e:
            srv.submit(0, f, a.eye, tag=3)
        assert e.value.code == -7
        got = _drain(srv, 3)
        assert all(r.status == 0 for r in got.values())
        assert srv.stats()["rejected"] == 1


def test_release_only_delivered_slots(world):
    """sl_server_release accepts only a slot that sl_server_poll handed out: a slot a batch may still be writing, one
    never handed out, and one already released are refused, so two views can never share a result slot."""
    scenes, rs, ls = world
    a = scenes[0]
    from splatlight_gb300 import _native as N
    lib = N.lib()
    with RenderServer(rs, ls, max_views=1, pipelines=1, max_view_pixels=64 * 64, result_slots=2) as srv:
        assert lib.sl_server_release(srv._h, 0) == -1          # never handed out
        srv.submit(0, _frame(a, 64, 64, VIEW_FLAT, a.eye), a.eye, tag=0)
        got = []
        for _ in range(200):
            got = srv.poll(wait_us=50_000, copy=False)       # poll(copy=False) releases what it delivers
            if got:
                break
        assert got and got[0].status == 0
        assert lib.sl_server_release(srv._h, 1) == -1          # the other slot was never used
        assert "released twice" in N.last_error()
        # a delivered slot, released by hand exactly once
        srv.submit(0, _frame(a, 64, 64, VIEW_FLAT, a.eye), a.eye, tag=1)
        n = N.C.c_uint32()
        for _ in range(200):
            N.check(lib.sl_server_poll(srv._h, srv._res, len(srv._res), N.C.byref(n), 50_000))
            if n.value:
                break
        assert n.value == 1 and srv._res[0].status == 0
        slot = int(srv._res[0].result_slot)
        assert lib.sl_server_release(srv._h, slot) == 0
        assert lib.sl_server_release(srv._h, slot) == -1
