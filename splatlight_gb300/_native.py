"""ctypes binding of libsplatlight.so (the C ABI in include/splatlight.h).

The library is built in-tree by splatlight_gb300.build (or __graft_entry__.build()).  There is no fallback: if the
shared library is missing or fails to load, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libsplatlight.so"

SL_OK = 0
ERRORS = {
    -1: "SL_ERR_INVALID_ARG", -2: "SL_ERR_LAYOUT", -3: "SL_ERR_OOM", -4: "SL_ERR_CUDA", -5: "SL_ERR_TIMEOUT",
    -6: "SL_ERR_UNSUPPORTED", -7: "SL_ERR_ADMISSION", -8: "SL_ERR_OVERFLOW", -9: "SL_ERR_NO_DEVICE",
    -10: "SL_ERR_CANCELLED",
}


class SplatlightError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class RenderStats(C.Structure):
    _fields_ = [("slots", C.c_uint32), ("visible", C.c_uint32), ("entries", C.c_uint32), ("tiles", C.c_uint32),
                ("fragments", C.c_uint32),
                ("ms_project", C.c_float), ("ms_sort", C.c_float), ("ms_bin", C.c_float),
                ("ms_composite", C.c_float), ("ms_total", C.c_float)]


class RenderOptions(C.Structure):
    _fields_ = [("tile_w", C.c_uint32), ("tile_h", C.c_uint32), ("t_stop", C.c_float),
                ("entry_capacity", C.c_uint32), ("sort_mode", C.c_uint32)]


class ProbeLayout(C.Structure):
    """sl_probe_layout (include/splatlight.h)."""
    _fields_ = [("dims", C.c_uint32 * 3), ("terrain", C.c_uint32), ("lo", C.c_float * 3), ("step", C.c_float * 3),
                ("levels", C.c_float * 16), ("ground", C.c_void_p), ("tmax", C.c_float), ("n_vols", C.c_uint32),
                ("vols", (C.c_uint32 * 4) * 32)]


class DisplaySky(C.Structure):
    """sl_display_sky (include/splatlight.h)."""
    _fields_ = [("has_sky", C.c_uint32), ("n_lights", C.c_uint32), ("sky_sh", (C.c_float * 3) * 16),
                ("light_dir", (C.c_float * 3) * 4), ("light_std", C.c_float * 4), ("light_irr", (C.c_float * 3) * 4),
                ("disc_std", C.c_float * 4), ("bg_count", C.c_uint32), ("ring_count", C.c_uint32),
                ("bg_sh", (C.c_float * 3) * 81), ("ring", (C.c_float * 3) * 8), ("ground", C.c_float * 3),
                ("ground_blend", C.c_float), ("ring_par", C.c_float * 2), ("glow", C.c_float * 3),
                ("glow_std", C.c_float), ("glow_dir", C.c_float * 3)]


class BatchOptions(C.Structure):
    _fields_ = [("max_views", C.c_uint32), ("max_tiles", C.c_uint32), ("max_slots", C.c_uint64),
                ("max_entries", C.c_uint64), ("tile_w", C.c_uint32), ("tile_h", C.c_uint32),
                ("no_graph", C.c_uint32), ("radiance_allowance", C.c_float)]


class BatchStats(C.Structure):
    _fields_ = [("views", C.c_uint32), ("slots", C.c_uint32), ("tiles", C.c_uint32), ("entries", C.c_uint32),
                ("visible", C.c_uint64), ("fragments", C.c_uint64), ("ms_total", C.c_float),
                ("graph_replayed", C.c_uint32), ("shaded", C.c_uint32), ("reshaded_views", C.c_uint32),
                ("max_radiance", C.c_float), ("ms_stage", C.c_float * 6)]


class ServerOptions(C.Structure):
    _fields_ = [("max_views", C.c_uint32), ("pipelines", C.c_uint32), ("max_slots", C.c_uint64),
                ("max_pixels", C.c_uint64), ("max_view_pixels", C.c_uint64), ("hbm_budget_bytes", C.c_uint64),
                ("max_tiles", C.c_uint32), ("result_slots", C.c_uint32), ("tile_w", C.c_uint32),
                ("tile_h", C.c_uint32), ("max_pending", C.c_uint32), ("pad", C.c_uint32)]


class ServerResult(C.Structure):
    _fields_ = [("tag", C.c_uint64), ("status", C.c_int32), ("batch_views", C.c_uint32), ("width", C.c_uint32),
                ("height", C.c_uint32), ("result_slot", C.c_uint32), ("pad", C.c_uint32), ("t_submit", C.c_double),
                ("t_start", C.c_double), ("t_done", C.c_double), ("image", C.POINTER(C.c_float))]


class ServerStats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("submitted", "completed", "rejected", "failed", "batches", "batch_views",
                                         "graph_replays", "pending", "device_bytes", "free_result_slots",
                                         "reshaded_views", "relaunches")]


class DiffScene(C.Structure):
    _fields_ = [("means", C.c_void_p), ("log_scales", C.c_void_p), ("quats", C.c_void_p),
                ("opacity_logits", C.c_void_p), ("albedo", C.c_void_p), ("roughness", C.c_void_p),
                ("n", C.c_uint32), ("n_lights", C.c_uint32), ("lights", C.c_void_p), ("light_scale", C.c_void_p),
                ("ambient", C.c_float), ("ks", C.c_float), ("vgrid", C.c_void_p), ("lamp_T", C.c_void_p),
                ("iso_norm", C.c_void_p)]


class DiffGrads(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("means", "log_scales", "quats", "opacity_logits", "albedo", "roughness",
                                         "light_scale")]


_P = C.c_void_p
_U32 = C.c_uint32
_U64 = C.c_uint64
_I = C.c_int

# name -> (restype, argtypes); every symbol include/splatlight.h declares
PROTOTYPES: dict[str, tuple] = {
    "sl_last_error": (C.c_size_t, [C.c_char_p, C.c_size_t]),
    "sl_version": (_I, []),
    "sl_asset_check_buffer": (_I, [C.c_char_p, _U32, _U32, C.POINTER(C.c_char_p), C.POINTER(_U32), _U32]),
    "sl_asset_check_bytes": (_I, [_U64, _U32, _U32]),
    "sl_renderer_create": (_I, [_P, _U32, _P, _U32, _U32, C.POINTER(_P)]),
    "sl_renderer_destroy": (_I, [_P]),
    "sl_renderer_set_parts": (_I, [_P, _P, _U32]),
    "sl_renderer_set_emitters": (_I, [_P, _P, _U32]),
    "sl_renderer_bind_colour": (_I, [_P, _P, _P]),
    "sl_renderer_set_options": (_I, [_P, C.POINTER(RenderOptions)]),
    "sl_renderer_set_timing": (_I, [_P, _I]),
    "sl_render": (_I, [_P, _P, _P, _I, C.POINTER(RenderStats), _P]),
    "sl_renderer_read_debug": (_I, [_P, _P, _P, _P, _P]),
    "sl_renderer_read_entries": (_I, [_P, _P, _U64]),
    "sl_lighting_create": (_I, [_P, _P, _P, _P, _U32, C.POINTER(_P)]),
    "sl_lighting_destroy": (_I, [_P]),
    "sl_lighting_set_emitters": (_I, [_P, _P, _U32, C.c_float, _I, _P, _U32]),
    "sl_emitter_tree": (_I, [_P, _U32, _P, _P, _P, C.POINTER(_U32)]),
    "sl_lighting_set_environment": (_I, [_P, _P, _U32, C.c_float]),
    "sl_lighting_set_options": (_I, [_P, _U32, _U32, _U32, C.c_float, _I]),
    "sl_lighting_set_blur": (_I, [_P, C.c_float, C.c_float]),
    "sl_lighting_set_tree": (_I, [_P, _P, _U32, _P, _U32]),
    "sl_lighting_set_probes": (_I, [_P, _P, _U32, C.c_float, C.c_int]),
    "sl_lighting_set_sky": (_I, [_P, _P, _U32]),
    "sl_lighting_read_bounce": (_I, [_P, _U32, _P, C.c_size_t]),
    "sl_lighting_set_sender_cut": (_I, [_P, _U32]),
    "sl_lighting_update": (_I, [_P, _P, _P, _U32, _P]),
    "sl_lighting_shade": (_I, [_P, _P, _P]),
    "sl_lighting_read": (_I, [_P, _P, _P, _P, _P]),
    "sl_renderer_bind_lighting": (_I, [_P, _P]),
    "sl_display": (_I, [_P, _U32, _U32, _P, _P, _P]),
    "sl_display_env": (_I, [_P, _U32, _U32, _P, _P, _P, _P]),
    "sl_lod_create": (_I, [_P, _P, _U32, _P, _U32, C.POINTER(_P)]),
    "sl_lod_destroy": (_I, [_P]),
    "sl_lod_select": (_I, [_P, _P, _U32, _U32, C.c_float, _P]),
    "sl_lod_colour": (_I, [_P, _P, _U32, _P]),
    "sl_lod_read": (_I, [_P, _P, _P, _P]),
    "sl_sort_keys16": (_I, [_P, _U32, _P, _P]),
    "sl_asset_check_header": (_I, [C.c_char_p, C.c_char_p]),
    "sl_sort_keys16_noalloc": (_I, [_P, _U32, _P, _P]),
    "sl_sort_keys32": (_I, [_P, _U32, _U32, _P, _P]),
    "sl_batch_create": (_I, [_P, _P, _U32, C.POINTER(BatchOptions), C.POINTER(_P)]),
    "sl_batch_destroy": (_I, [_P]),
    "sl_batch_set_tile": (_I, [_P, _U32, _U32]),
    "sl_batch_set_timing": (_I, [_P, _I]),
    "sl_batch_render": (_I, [_P, _P, _P, _P, _P, _U32, _P, _U64, _P, C.POINTER(BatchStats), _P]),
    "sl_batch_read_view": (_I, [_P, _U32, _P, _P, _P, _U64, C.POINTER(_U64)]),
    "sl_diff_create": (_I, [_U32, C.POINTER(_P)]),
    "sl_diff_destroy": (_I, [_P]),
    "sl_diff_forward": (_I, [_P, C.POINTER(DiffScene), _P, _P, _P, _P]),
    "sl_diff_step": (_I, [_P, C.POINTER(DiffScene), _P, _P, _P, _P, C.POINTER(DiffGrads), C.POINTER(C.c_double), _P]),
    "sl_diff_read_order": (_I, [_P, _P, C.POINTER(_U32)]),
    "sl_server_create": (_I, [_P, _P, _U32, C.POINTER(ServerOptions), C.POINTER(_P)]),
    "sl_server_submit": (_I, [_P, _P, _U64]),
    "sl_server_poll": (_I, [_P, C.POINTER(ServerResult), _U32, C.POINTER(_U32), _U32]),
    "sl_server_release": (_I, [_P, _U32]),
    "sl_server_get_stats": (_I, [_P, C.POINTER(ServerStats)]),
    "sl_server_destroy": (_I, [_P]),
    "sl_batch_autotune": (_I, [_P, _P, _P, _P, _P, _U32, _P, _U64, _U32, C.POINTER(_U32), C.POINTER(_U32),
                               _P, _P]),
    "sl_batch_get_tuning": (_I, [_P, C.POINTER(_U32), C.POINTER(_U32), _P]),
    "sl_batch_set_tuning": (_I, [_P, _P]),
}

_lib: C.CDLL | None = None


def lib() -> C.CDLL:
    """Loads libsplatlight.so once; raises if it is missing (no CPU fallback exists)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH.name} is not built: run splatlight_gb300.build.build() (needs nvcc)")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in PROTOTYPES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def last_error() -> str:
    buf = C.create_string_buffer(1024)
    lib().sl_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def check(code: int) -> None:
    if code != SL_OK:
        raise SplatlightError(code, last_error())


def ptr(a) -> int | None:
    """Address of a numpy array, a torch tensor (host or device) or None."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data
