"""Generates the committed golden fixtures of the CPU restatement (tests/golden/*.npz): small seeded scenes with
their inputs (Gaussians, parts, emitters, RenderFrame) and outputs (keys, permutation, tile ranges and lists,
contributor counts, linear RGBA).  The restatement is deterministic (no libm in its hot path), so the same fixtures
hold on x86-64 and aarch64 hosts.  Run from the repository root: python tests/golden/make_golden.py"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import oracle  # noqa: E402
from splatlight_gb300 import camera, scene  # noqa: E402
from splatlight_gb300.structs import VIEW_FLAT, VIEW_LIT, VIEW_OVERDRAW  # noqa: E402

HERE = Path(__file__).resolve().parent


def cases():
    c = scene.subset(scene.cornell(), 1500, seed=7)
    h = scene.subset(scene.hill(n=65536), 2500, seed=8)
    yield "cornell_flat", c, camera.make_frame(c.eye, c.target, c.up, c.fov_deg, 64, 48, c.count, far=c.far,
                                               view_mode=VIEW_FLAT, n_emit=len(c.emitters)), (16, 16), None
    yield "cornell_overdraw_8x32", c, camera.make_frame(c.eye, c.target, c.up, c.fov_deg, 64, 48, c.count,
                                                        far=c.far, view_mode=VIEW_OVERDRAW,
                                                        n_emit=len(c.emitters)), (8, 32), None
    rng = np.random.default_rng(3)
    col = rng.uniform(0, 2, (h.count, 4)).astype(np.float32)
    yield "hill_lit_32x8", h, camera.make_frame(h.eye, h.target, h.up, h.fov_deg, 96, 54, h.count, far=h.far,
                                                view_mode=VIEW_LIT, n_emit=len(h.emitters)), (32, 8), col


def main():
    for name, s, f, tile, col in cases():
        r = oracle.render(s.gaussians, s.parts, f, emitters=s.emitters, colour=col, tile=tile, threads=1)
        np.savez_compressed(HERE / f"{name}.npz", gaussians=s.gaussians, parts=s.parts, emitters=s.emitters,
                            frame=np.asarray(f).reshape(1), tile=np.array(tile), colour=col if col is not None else
                            np.zeros((0, 4), np.float32), keys=r["keys"], order=r["order"], ranges=r["ranges"],
                            entries=r["entries"], counts=r["counts"], rgba=r["rgba"])
        print(name, r["visible"], r["n_entries"])


if __name__ == "__main__":
    main()
