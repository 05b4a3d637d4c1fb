"""The gs-runtime loader (splatlight_gb300/asset.py over sl_asset_check_*) on the reference's two shipped assets, and
checkHeader's rejections with the reference's messages (src/asset.js:18-38).  The assets are copied from the reference
checkout by tests/golden/copy_assets.py; without them these tests skip."""
import copy
import json
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
ASSETS = ROOT / "tests" / "golden" / "assets"
NAMES = ("cornell_sdf_room_plain_bin", "hill_lite_bin")


@pytest.fixture(scope="module")
def A():
    from splatlight_gb300 import build
    build.build()
    from splatlight_gb300 import asset
    return asset


def _need(name):
    p = ASSETS / name
    if not (p / "asset.json").exists():
        pytest.skip("reference assets not copied (tests/golden/copy_assets.py)")
    return p


@pytest.mark.parametrize("name", NAMES)
def test_shipped_assets_load(A, name):
    a = A.load_asset(_need(name))
    h = a.header
    assert a.count == h["buffers"]["gaussians"]["count"] == len(a.gaussians)
    assert a.part_count == len(a.parts) == len(h["parts"])
    nodes = a.raw["nodes"]
    assert len(nodes) == h["buffers"]["nodes"]["count"] and len(a.raw["kids"]) == h["buffers"]["kids"]["count"]
    # the leaves are the first `count` nodes, in Gaussian order (runtime/wgsl/common.wgsl:12-19)
    assert np.array_equal(nodes["mean"][:a.count], a.gaussians["mu"])
    assert np.array_equal(nodes["kappa"][:a.count], a.gaussians["kappa"])
    assert (nodes["child_lo"][:a.count] == 0).all() and (nodes["child_hi"][:a.count] == 0).all()
    # every part's root is an internal node of that part, over exactly its Gaussian range
    for k, p in enumerate(h["parts"]):
        assert int(a.parts[k]["root"]) == p["root"] and nodes["part"][p["root"]] == k
        g0, g1 = p["gaussians"]
        assert ((a.gaussians["part_surface"][g0:g1] & 0xFFFF) == k).all()
    # real V grids: the own-part visibility the synthetic scenes never exercise
    assert np.mean(~np.all(a.raw["vgrid"]["w"] == 0xFFFFFFFF, axis=1)) > 0.9
    fp = a.fingerprint
    assert fp["count"] == a.count and fp["bytes"] == 64 * a.count and 0 <= fp["hash"] < 2 ** 32


def test_cornell_scene_setup(A):
    a = A.load_asset(_need(NAMES[0]))
    s = A.asset_scene(a)
    em = a.header["emitters"]
    assert len(s.emitters) == em["gaussians"] == 320 and not s.emit_drawn and s.n_drawn_emitters == 0
    assert s.emit_one_sided and s.emit_skip_part == em["part"]
    assert np.allclose(s.emitters["albedo"], em["emission"])
    # the lamp moves to main.js's start position (z 1.97): the records' centroid and the part's translation agree
    c = s.emitters["mu"].astype(np.float64).mean(axis=0)
    assert np.allclose(c, [a.lamps[0]["center"][0], a.lamps[0]["center"][1], 1.97], atol=1e-5)
    xf = s.parts[em["part"]]["xf"]
    assert np.isclose(xf[11], 1.97 - a.lamps[0]["center"][2], atol=1e-6) and np.array_equal(xf, s.parts[em["part"]]["xf_prev"])
    assert np.allclose(np.linalg.norm(s.emit_normal), 1.0, atol=1e-6) and 0.0 < s.emit_scale < 10.0
    assert (s.width, s.height) == tuple(a.header["camera"]["resolution"])


def test_hill_scene_setup(A):
    a = A.load_asset(_need(NAMES[1]))
    s = A.asset_scene(a)
    assert len(s.emitters) == 0 and s.sun is not None and s.sky_ambient == 0.0
    d = np.asarray(s.sun.direction)
    want = np.asarray(a.header["environment"]["lights"][0]["dir"], np.float64)
    assert np.allclose(d, want / np.linalg.norm(want), atol=1e-6)
    assert np.isclose(s.sun.angular_std, 1.1 * np.pi / 180)
    assert s.far > 200.0                                   # past the scene's bounds (src/main.js:488)


def _header():
    return json.loads((_need(NAMES[0]) / "asset.json").read_text())


def _raises(A, h, text):
    with pytest.raises(A.AssetError) as e:
        A.check_header(h)
    assert e.value.code == -2
    assert text in str(e.value), str(e.value)


def test_check_header_rejects_like_the_reference(A):
    h = _header()
    A.check_header(h)
    h2 = copy.deepcopy(h); h2["format"] = "gs-other"
    _raises(A, h2, "Unknown asset format gs-other")
    h2 = copy.deepcopy(h); del h2["format"]
    _raises(A, h2, "Unknown asset format undefined")
    h2 = copy.deepcopy(h); h2["version"] = "1.0"
    _raises(A, h2, "Unsupported asset version 1.0")
    h2 = copy.deepcopy(h); h2["version"] = 0.3
    A.check_header(h2)                                     # String(0.3).split('.')[0] === '0'
    h2 = copy.deepcopy(h); h2["version"] = 1
    _raises(A, h2, "Unsupported asset version 1")
    h2 = copy.deepcopy(h); del h2["buffers"]["vgrid"]
    _raises(A, h2, "Asset has no vgrid buffer")
    h2 = copy.deepcopy(h); h2["buffers"]["gaussians"]["stride"] = 48
    _raises(A, h2, "gaussians stride 48, renderer expects 64")
    h2 = copy.deepcopy(h); h2["buffers"]["parts"]["fields"]["root"]["offset"] = 116
    _raises(A, h2, "parts.root at 116, renderer expects 112")
    h2 = copy.deepcopy(h); del h2["buffers"]["lamps"]["fields"]["radiance"]
    _raises(A, h2, "lamps.radiance at undefined, renderer expects 64")
    for bad in (0, (1 << 24) + 1, 1.5, "7"):
        h2 = copy.deepcopy(h); h2["buffers"]["kids"]["count"] = bad
        _raises(A, h2, "Bad kids count")
    h2 = copy.deepcopy(h); h2["buffers"]["kids"]["count"] = 1 << 24
    A.check_header(h2)


def test_check_buffer_size(A):
    h = _header()
    n, st = h["buffers"]["materials"]["count"], h["buffers"]["materials"]["stride"]
    A.check_buffer(h, "materials", bytes(n * st))
    with pytest.raises(A.AssetError) as e:
        A.check_buffer(h, "materials", bytes(n * st + 4))
    assert f"is {n * st + 4} B, expected {n} x {st} B" in str(e.value)


def test_missing_asset_folder(A, tmp_path):
    with pytest.raises(A.AssetError) as e:
        A.load_asset(tmp_path / "nothing_here")
    assert "Could not load" in str(e.value)


def test_probe_layouts_from_the_headers(A):
    """probeLayout (src/lighting.js:220-286) on the shipped headers: the Cornell room's 8^3 lattice inset 0.125 m from
    its `room` walls (no environment: rays of 6 m); hill_lite's 16 x 16 x 5 terrain lattice over its `bounds` (cell
    centres, the default heights, rays across the whole scene for its environment), its ground inside the bounds, and
    the one static volume probeVolumes picks (its tree part, 4 per axis); hill_lite's sky SH for the probes."""
    a = A.load_asset(_need(NAMES[0]))
    lay = A.probe_layout(a)
    room = a.header["room"]
    box = [(float(room[k][0]), float(room[k][1])) for k in "xyz"]
    half = [(b - c) / 2 - 0.125 for c, b in box]
    assert not lay["terrain"] and lay["dims"] == [8, 8, 8] and lay["tmax"] == 6.0 and lay["vols"] == []
    assert np.allclose(lay["lo"], [(c + b) / 2 - h for (c, b), h in zip(box, half)])
    assert np.allclose(lay["step"], [2 * h / 7 for h in half])
    assert A.environment_sky(a.header.get("environment")) is None
    a = A.load_asset(_need(NAMES[1]))
    lay = A.probe_layout(a)
    lo, hi = (np.asarray(a.header["bounds"][k], np.float64) for k in ("lo", "hi"))
    step = (hi - lo)[:2] / 16
    assert lay["terrain"] and lay["dims"] == [16, 16, 5] and list(lay["levels"]) == [0.3, 1.0, 3.0, 8.0, 20.0]
    assert np.allclose(lay["step"][:2], step) and np.allclose(lay["lo"][:2], lo[:2] + step / 2)
    assert np.isclose(lay["tmax"], max(6.0, float(np.linalg.norm(hi - lo))))
    g = np.asarray(lay["ground"])
    assert g.shape == (256,) and np.isfinite(g).all() and (g >= lo[2] - 1e-4).all() and (g <= hi[2] + 1e-4).all()
    assert [tuple(v) for v in lay["vols"]] == [(2, 4, 4, 4)]
    sky = A.environment_sky(a.header["environment"])
    assert sky.shape == (16, 3)
    assert np.allclose(sky, np.asarray(a.header["environment"]["sky"]["sh_rgb"][:16], np.float64))
