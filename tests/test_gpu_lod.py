"""Screen-space LOD on the GPU (sl_lod_*; src/lod.js, runtime/wgsl/lod.wgsl) against the restatement: the internal
nodes' records, the cut's flags over successive frames (both size rules, several thresholds), the node colours, and
frames drawn with the cut -- keys, permutation, tile ranges and lists bit-exact, RGB within 1e-3."""
import numpy as np
import pytest

from oracle import oracle
from splatlight_gb300 import camera, scene
from splatlight_gb300._native import SplatlightError
from splatlight_gb300.batch import BatchRenderer, View
from splatlight_gb300.lod import DRAW, Lod, frame_lod
from splatlight_gb300.renderer import SplatRenderer
from splatlight_gb300.structs import VIEW_FLAT, VIEW_LIT, VIEW_OVERDRAW

pytestmark = pytest.mark.gpu

RGB_TOL = 1e-3


@pytest.fixture(scope="module")
def world(cuda):
    s = scene.subset(scene.hill(), 40000, seed=5)
    nodes, kids, parts = scene.lod_tree(s.gaussians, s.parts)
    s = scene.dataclasses.replace(s, parts=parts)
    r = SplatRenderer(s.gaussians, s.parts)
    r.set_emitters(s.emitters)
    lod = Lod(r, nodes, kids)
    yield s, nodes, kids, r, lod
    lod.close()
    r.close()


def _frame(s, eye, mode=VIEW_FLAT, W=320, H=240):
    return camera.make_frame(eye, s.target, s.up, s.fov_deg, W, H, s.count, far=s.far, view_mode=mode,
                             n_emit=len(s.emitters))


def test_node_records_match(world):
    s, nodes, kids, r, lod = world
    _, _, recs = lod.read()
    ref = oracle.lod_records(s.gaussians, nodes, kids)
    assert recs.tobytes() == ref.tobytes()


@pytest.mark.parametrize("rule", [1, 0])
def test_flags_match_over_frames(world, rule):
    s, nodes, kids, r, lod = world
    G, N = len(s.gaussians), len(nodes)
    ref = lod.read()[0].copy()           # continue from whatever cut the LOD holds
    for eye, thr in (((0.0, -9.0, 4.0), 2.0), ((4.0, 1.0, 2.0), 2.0), ((4.0, 1.0, 2.0), 12.0), ((-6, 6, 8), 0.7)):
        f = frame_lod(_frame(s, eye), thr, N - G)
        lod.select(f, size_rule=rule)
        oracle.lod_select(nodes, G, kids, s.parts, f, ref, size_rule=rule)
        got = lod.read()[0]
        assert np.array_equal(got, ref), (eye, thr, int((got != ref).sum()))
        assert (got == DRAW).sum() > 0


def test_flags_with_blur_and_emitter_part(world):
    """The emitters' part always opens to its leaves; with the shutter open a moving part opens only nodes larger than
    blur_lod x its smear (motion blur variant D): both bit-exact against the restatement."""
    s, nodes, kids, r, lod = world
    G, N = len(s.gaussians), len(nodes)
    parts = s.parts.copy()
    parts[1]["flags"] |= 2                                   # part 1 moves this frame
    parts[1]["xf_prev"] = parts[1]["xf"]
    parts[1]["xf_prev"][3] -= 0.4                            # from 0.4 m to the left
    r.write_parts(parts)
    try:
        ref = lod.read()[0].copy()
        for emit_part, blur in ((0, 0.0), (0xFFFFFFFF, 3.0), (2, 8.0)):
            f = frame_lod(_frame(s, (1.0, -8.0, 4.0)), 2.0, N - G)
            f["palette"][3][2] = 0.5                         # shutter
            lod.select(f, emit_part=emit_part, blur_lod=blur)
            oracle.lod_select(nodes, G, kids, parts, f, ref, emit_part=emit_part, blur_lod=blur)
            assert np.array_equal(lod.read()[0], ref), (emit_part, blur)
    finally:
        r.write_parts(s.parts)


@pytest.mark.parametrize("mode", [VIEW_FLAT, VIEW_OVERDRAW])
def test_frame_with_cut_matches(world, mode):
    s, nodes, kids, r, lod = world
    G, N = len(s.gaussians), len(nodes)
    f = frame_lod(_frame(s, (3.0, -5.0, 3.0), mode), 3.0, N - G)
    lod.select(f)
    img = r.render(f)
    dbg = r.read_debug()
    flags, ncol, recs = lod.read()
    assert (flags[G:] == DRAW).any()     # some internal nodes are drawn
    ref = oracle.render(s.gaussians, s.parts, f, emitters=s.emitters, lod=(flags, recs, ncol))
    assert np.array_equal(dbg["keys"], ref["keys"])
    assert np.array_equal(dbg["order"], ref["order"])
    assert np.array_equal(dbg["ranges"], ref["ranges"])
    assert np.array_equal(dbg["entries"], ref["entries"])
    if mode == VIEW_OVERDRAW:
        assert np.array_equal(img[..., 0].astype(np.uint32), ref["counts"])
    else:
        assert float(np.abs(img - ref["rgba"]).max()) <= RGB_TOL


def test_lit_cut_colours_and_frame(world):
    torch = pytest.importorskip("torch")
    s, nodes, kids, r, lod = world
    G, N = len(s.gaussians), len(nodes)
    rng = np.random.default_rng(7)
    col = rng.uniform(0, 2, (G, 4)).astype(np.float32)
    r.bind_colour(torch.from_numpy(col).cuda())
    f = frame_lod(_frame(s, (0.0, -7.0, 3.5), VIEW_LIT), 2.5, N - G)
    lod.select(f)
    lod.colour(f)
    img = r.render(f)
    flags, ncol, recs = lod.read()
    ref_col = oracle.lod_colour(nodes, G, kids, flags, col)
    drawn_or_under = (flags[G:] == DRAW) | (flags[G:] == 4)
    assert np.array_equal(ncol[drawn_or_under], ref_col[drawn_or_under])
    ref = oracle.render(s.gaussians, s.parts, f, emitters=s.emitters, colour=col, lod=(flags, recs, ncol))
    assert np.array_equal(r.read_debug()["keys"], ref["keys"])
    assert float(np.abs(img - ref["rgba"]).max()) <= RGB_TOL
    # every node colour, on request
    lod.colour(f, colour_all=True)
    assert np.array_equal(lod.read()[1], oracle.lod_colour(nodes, G, kids, flags, col, colour_all=True))


def test_bad_lod_frames(world):
    s, nodes, kids, r, lod = world
    G, N = len(s.gaussians), len(nodes)
    f = frame_lod(_frame(s, (0.0, -9.0, 4.0)), 2.0, N - G + 1)       # wrong node count
    with pytest.raises(SplatlightError) as e:
        r.render(f)
    assert e.value.code == -1
    f = frame_lod(_frame(s, (0.0, -9.0, 4.0)), 2.0, N - G, node_base=s.count)   # overlaps the emitter slots
    with pytest.raises(SplatlightError):
        r.render(f)
    with BatchRenderer([r]) as B:                                   # batches draw every leaf: LOD frames refused
        with pytest.raises(SplatlightError) as e:
            B.render([View(0, frame_lod(_frame(s, (0.0, -9.0, 4.0)), 2.0, N - G), (0.0, -9.0, 4.0))])
        assert e.value.code == -6
