"""numpy record layouts of the gs-runtime buffers and the RenderFrame uniform (little-endian, byte-exact with
include/splatlight.h and the reference's WGSL structs: shaders/common.wgsl:5-77, runtime/wgsl/common.wgsl:4-65)."""
from __future__ import annotations

import numpy as np

GAUSSIAN = np.dtype([
    ("mu", "<f4", 3), ("kappa", "<f4"), ("quat", "<f4", 4), ("scale", "<f4", 3),
    ("part_surface", "<u4"), ("albedo", "<f4", 3), ("flags", "<u4"),
])
PART = np.dtype([
    ("xf", "<f4", 12), ("xf_prev", "<f4", 12), ("bound", "<f4", 4),
    ("root", "<u4"), ("g_lo", "<u4"), ("g_hi", "<u4"), ("flags", "<u4"),
])
NODE = np.dtype([
    ("mean", "<f4", 3), ("radius", "<f4"), ("cinv_diag", "<f4", 3), ("kappa", "<f4"),
    ("cinv_off", "<f4", 3), ("smax", "<f4"), ("sn_diag", "<f4", 3), ("part", "<u4"),
    ("sn_off", "<f4", 3), ("child_lo", "<u4"), ("child_hi", "<u4"), ("depth", "<u4"), ("pad0", "<u4"), ("pad1", "<u4"),
])
MATERIAL = np.dtype([
    ("flake", "<f4", 3), ("phase_samples", "<u4"), ("vfloor", "<f4"), ("flags", "<u4"), ("pad0", "<u4"), ("pad1", "<u4"),
])
VGRID = np.dtype([("w", "<u4", 32)])
# RenderFrame, 1200 B (src/renderer.js:9 FRAME_BYTES)
FRAME = np.dtype([
    ("view", "<f4", 16), ("proj", "<f4", 16), ("palette", "<f4", (4, 4)), ("part_material", "<u4", 16),
    ("lamp", "<f4", 4), ("lamp_color", "<f4", 4), ("viewport", "<f4", 2), ("focal", "<f4", 2),
    ("near", "<f4"), ("far", "<f4"), ("count", "<u4"), ("view_mode", "<u4"), ("albedo_scale", "<f4"),
    ("flake_roughness", "<f4"), ("exposure", "<f4"), ("lowpass_px2", "<f4"), ("palette_ext", "<f4", (4, 4)),
    ("mat_view", "<f4", (16, 4)), ("part_material_ext", "<u4", 16), ("lod", "<u4", 4), ("explode", "<f4", 4),
    ("explode_c", "<f4", 4), ("explode_k", "<f4", 4), ("mat_view_ext", "<f4", (16, 4)), ("tone", "<u4", 4),
    ("part_fade", "<f4", 32), ("particles", "<u4", 4),
])

assert GAUSSIAN.itemsize == 64 and PART.itemsize == 128 and NODE.itemsize == 96
assert MATERIAL.itemsize == 32 and VGRID.itemsize == 128 and FRAME.itemsize == 1200

VIEW_FLAT, VIEW_DEPTH, VIEW_OVERDRAW, VIEW_LIT = 0, 1, 2, 3
EMITTER_MATERIAL = 254
