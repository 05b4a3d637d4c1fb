"""The C-ABI library loads without a GPU and exports every entry point include/*.h declares; host-only entry points
work; device entry points fail with a clean status code when no sm_103 device is present."""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _declared():
    names = []
    for h in (ROOT / "include").glob("*.h"):
        names += re.findall(r"^SL_API\s+[\w\s\*]+?\b(sl_\w+)\s*\(", h.read_text(), flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def native():
    from splatlight_gb300 import build
    build.build()
    from splatlight_gb300 import _native
    return _native


def test_every_declared_symbol_is_exported(native):
    L = native.lib()
    declared = _declared()
    assert len(declared) >= 10
    for name in declared:
        assert hasattr(L, name), name
        assert name in native.PROTOTYPES, f"{name} has no ctypes prototype"


def test_asset_layout_checks(native):
    L = native.lib()
    names = (C.c_char_p * 7)(b"mu", b"kappa", b"quat", b"scale", b"part_surface", b"albedo", b"flags")
    offs = (C.c_uint32 * 7)(0, 12, 16, 32, 44, 48, 60)
    assert L.sl_asset_check_buffer(b"gaussians", 64, 1000, names, offs, 7) == 0
    assert L.sl_asset_check_buffer(b"gaussians", 48, 1000, names, offs, 7) == -2
    assert "stride 48" in native.last_error()
    offs[5] = 52
    assert L.sl_asset_check_buffer(b"gaussians", 64, 1000, names, offs, 7) == -2
    assert "albedo at 52" in native.last_error()
    offs[5] = 48
    assert L.sl_asset_check_buffer(b"gaussians", 64, 0, names, offs, 7) == -2
    assert L.sl_asset_check_buffer(b"gaussians", 64, (1 << 24) + 1, names, offs, 7) == -2
    assert L.sl_asset_check_buffer(b"blockers", 64, 10, None, None, 0) == -2
    assert L.sl_asset_check_buffer(b"kids", 4, 10, None, None, 0) == 0
    assert L.sl_asset_check_bytes(6400, 100, 64) == 0
    assert L.sl_asset_check_bytes(6401, 100, 64) == -2


def test_null_arguments_are_rejected(native):
    L = native.lib()
    h = C.c_void_p()
    assert L.sl_renderer_create(None, 10, None, 1, 0, C.byref(h)) == -1
    assert L.sl_render(None, None, None, 0, None, None) == -1
    assert L.sl_renderer_destroy(None) == 0


def test_device_calls_fail_cleanly_without_gpu(native):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import numpy as np
    from splatlight_gb300.structs import GAUSSIAN, PART
    g = np.zeros(4, dtype=GAUSSIAN)
    p = np.zeros(1, dtype=PART)
    h = C.c_void_p()
    rc = native.lib().sl_renderer_create(g.ctypes.data, 4, p.ctypes.data, 1, 0, C.byref(h))
    assert rc in (-4, -9) and not h.value
    assert native.last_error()
