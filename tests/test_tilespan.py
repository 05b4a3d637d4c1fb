"""The row spans of the tile binning (include/sl_tilespan.h) never drop a pixel the compositor keeps: for random
ellipses -- round, thin, tilted, tiny, huge, off-screen centres -- every pixel centre inside the ellipse (q computed in
float64, with 1e-5 relative slack over the cutoff) lies in a tile of its row's span."""
import numpy as np
import pytest

from oracle import oracle


def _splat(rng, W, H):
    s = np.zeros((), dtype=oracle.SPLAT)
    kind = rng.integers(4)
    scale = {0: 1.0, 1: 6.0, 2: 40.0, 3: 300.0}[int(kind)]
    sx = scale * rng.uniform(0.3, 1.5)
    sy = sx * (rng.uniform(0.02, 1.0) if rng.random() < 0.6 else 1.0)
    th = rng.uniform(0, np.pi)
    # g0, g1: rows of R(-th) / sigma: local = (d.g0, d.g1)
    c, s_ = np.cos(th), np.sin(th)
    g0 = np.array([c, s_]) / sx
    g1 = np.array([-s_, c]) / sy
    s["cx"], s["cy"] = rng.uniform(-0.2 * W, 1.2 * W), rng.uniform(-0.2 * H, 1.2 * H)
    s["g0x"], s["g0y"], s["g1x"], s["g1y"] = np.float32(g0[0]), np.float32(g0[1]), np.float32(g1[0]), np.float32(g1[1])
    s["qcut"] = np.float32(rng.uniform(1.0, 12.0))
    # candidate rectangle: the exact bounding box of the ellipse plus one pixel, clipped (as the projection does)
    M = np.outer(g0, g0) + np.outer(g1, g1)
    Mi = np.linalg.inv(M)
    hx = np.sqrt(float(s["qcut"]) * Mi[0, 0]) + 1.0
    hy = np.sqrt(float(s["qcut"]) * Mi[1, 1]) + 1.0
    ix0 = max(int(np.ceil(s["cx"] - hx - 0.5)), 0)
    ix1 = min(int(np.floor(s["cx"] + hx - 0.5)), W - 1)
    iy0 = max(int(np.ceil(s["cy"] - hy - 0.5)), 0)
    iy1 = min(int(np.floor(s["cy"] + hy - 0.5)), H - 1)
    s["ix0"], s["ix1"], s["iy0"], s["iy1"] = ix0, ix1, iy0, iy1
    return s


@pytest.mark.parametrize("tile", [(16, 16), (8, 32), (32, 8)])
def test_row_spans_are_conservative(tile):
    rng = np.random.default_rng(11)
    W, H = 640, 480
    tw, th = tile
    checked = saved = full = 0
    for _ in range(400):
        s = _splat(rng, W, H)
        if s["ix0"] > s["ix1"] or s["iy0"] > s["iy1"]:
            continue
        xs = np.arange(int(s["ix0"]), int(s["ix1"]) + 1)
        ys = np.arange(int(s["iy0"]), int(s["iy1"]) + 1)
        X, Y = np.meshgrid(xs + 0.5, ys + 0.5)
        dx, dy = X - float(s["cx"]), Y - float(s["cy"])
        lx = dx * float(s["g0x"]) + dy * float(s["g0y"])
        ly = dx * float(s["g1x"]) + dy * float(s["g1y"])
        kept = (lx * lx + ly * ly) <= float(s["qcut"]) * (1 + 1e-5)
        for ty in range(int(s["iy0"]) // th, int(s["iy1"]) // th + 1):
            span = oracle.row_tiles(s, ty, tile)
            rows = (ys >= ty * th) & (ys < ty * th + th)
            cols = xs[kept[rows].any(axis=0)] if rows.any() else xs[:0]
            full += int(s["ix1"]) // tw - int(s["ix0"]) // tw + 1
            if cols.size == 0:
                if span is not None:
                    saved += int(s["ix1"]) // tw - int(s["ix0"]) // tw + 1 - (span[1] - span[0] + 1)
                else:
                    saved += int(s["ix1"]) // tw - int(s["ix0"]) // tw + 1
                continue
            assert span is not None, (s, ty)
            assert span[0] <= cols.min() // tw and cols.max() // tw <= span[1], (s, ty, span, cols.min(), cols.max())
            assert int(s["ix0"]) // tw <= span[0] <= span[1] <= int(s["ix1"]) // tw
            saved += int(s["ix1"]) // tw - int(s["ix0"]) // tw - (span[1] - span[0])
            checked += 1
    assert checked > 200
    assert saved > 0.1 * full   # the spans are tighter than the rectangle rows
