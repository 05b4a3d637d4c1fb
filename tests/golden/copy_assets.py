"""Copies the reference's two shipped gs-runtime assets -- the only scene data the reference holds -- into
tests/golden/assets/ (git-ignored: about 180 MB of little-endian buffers), so the GPU parity tests can render them
where the reference checkout is absent.  Only the files loadAsset reads are copied: asset.json and the seven buffers
(src/asset.js:51-78).  Run here, where the reference checkout exists (__graft_entry__.build() calls it); a copy that
is already complete is left as it is.

    python tests/golden/copy_assets.py [reference root]
"""
from __future__ import annotations

import json
import shutil
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
DEST = HERE / "assets"
NAMES = ("cornell_sdf_room_plain_bin", "hill_lite_bin")
BUFFERS = ("gaussians", "parts", "lamps", "materials", "nodes", "kids", "vgrid")


def _files(src: Path) -> list[str]:
    header = json.loads((src / "asset.json").read_text())
    return ["asset.json"] + [header["buffers"][b]["file"] for b in BUFFERS]


def ensure(reference: Path = Path("/root/reference")) -> list[Path]:
    """The asset folders under tests/golden/assets that are complete after the copy (none without a reference)."""
    out = []
    for name in NAMES:
        src = reference / "runtime" / "assets" / name
        dst = DEST / name
        if not (src / "asset.json").exists():
            if (dst / "asset.json").exists():
                out.append(dst)
            continue
        dst.mkdir(parents=True, exist_ok=True)
        for f in _files(src):
            s, d = src / f, dst / f
            if not d.exists() or d.stat().st_size != s.stat().st_size:
                shutil.copyfile(s, d)
        out.append(dst)
    return out


if __name__ == "__main__":
    for p in ensure(Path(sys.argv[1]) if len(sys.argv) > 1 else Path("/root/reference")):
        print(p)
