"""Builds libsplatlight.so (every CUDA kernel and the C ABI) in-tree for sm_103a with nvcc, and the sort leg's
library bar (library_bar/libcub_sort.so: CUB's radix sort, for comparison only).

Each translation unit compiles in parallel to an object under splatlight_gb300/_build/, then one shared library is
linked next to this file.  project.cu, lighting.cu, tiles.cu, batch.cu and lod.cu are compiled with --fmad=false:
their arithmetic must match the CPU restatement bit for bit (sort keys, tile rectangles and row spans, the fragment
keep bound, the opacity maps, the LOD cut).  shade.cu is compiled for speed (its output is checked to a tolerance).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libsplatlight.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# translation units whose arithmetic is part of the bit-parity contract
NO_FMAD = {"project.cu", "lighting.cu", "tiles.cu", "batch.cu", "lod.cu", "bounce.cu"}
# translation units compiled for speed: fused multiply-add, approximate division and square root
FAST = {"shade.cu", "bounce_direct.cu"}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build libsplatlight")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _compile(src: Path) -> Path:
    obj = BUILD / (src.stem + ".o")
    cmd = [nvcc(), *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
           "-Xcompiler", "-ffp-contract=off",
           "-I", str(ROOT / "include"), "-I", str(CSRC), "--expt-relaxed-constexpr", "-c", str(src), "-o", str(obj)]
    if src.name in NO_FMAD:
        cmd.insert(1, "--fmad=false")
    if src.name in FAST:
        cmd[1:1] = ["-prec-div=false", "-prec-sqrt=false"]
    if os.environ.get("SL_PTXAS_VERBOSE"):
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
    if os.environ.get("SL_PTXAS_VERBOSE"):
        sys.stderr.write(r.stderr)
    return obj


def needs_build() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = list(CSRC.glob("*")) + list((ROOT / "include").glob("*.h"))
    return any(p.stat().st_mtime > t for p in deps)


BAR_SRC = PKG / "library_bar" / "cub_sort.cu"
BAR_LIB = PKG / "library_bar" / "libcub_sort.so"


def build_library_bar(force: bool = False) -> Path:
    """The sort leg's library bar (CUB's DeviceRadixSort, a comparison baseline the pipeline never calls)."""
    if not force and BAR_LIB.exists() and BAR_LIB.stat().st_mtime >= BAR_SRC.stat().st_mtime:
        return BAR_LIB
    tmp = BAR_LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden", "-shared",
           str(BAR_SRC), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {BAR_SRC.name}:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, BAR_LIB)
    return BAR_LIB


def build(force: bool = False, jobs: int | None = None) -> Path:
    if not force and not needs_build():
        return LIB
    BUILD.mkdir(exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=jobs or min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, srcs))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
