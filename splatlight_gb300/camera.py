"""Camera maths and RenderFrame assembly, mirroring the reference host: lookAt/perspective (src/math.js:36-57) and
writeFrame (src/main.js:526-556)."""
from __future__ import annotations

import math

import numpy as np

from .structs import FRAME, VIEW_LIT


def _normalize(v):
    v = np.asarray(v, dtype=np.float64)
    return v / np.linalg.norm(v)


def look_at(eye, target, up) -> np.ndarray:
    """Column-major world->view matrix, views look down -z (src/math.js:36-46).  float64 maths, float32 result."""
    eye = np.asarray(eye, dtype=np.float64)
    z = _normalize(eye - np.asarray(target, dtype=np.float64))
    x = _normalize(np.cross(np.asarray(up, dtype=np.float64), z))
    y = np.cross(z, x)
    return np.array([x[0], y[0], z[0], 0, x[1], y[1], z[1], 0, x[2], y[2], z[2], 0,
                     -x @ eye, -y @ eye, -z @ eye, 1], dtype=np.float32)


def perspective(fovy: float, aspect: float, near: float, far: float) -> np.ndarray:
    """WebGPU clip-space projection (src/math.js:50-57); carried in the frame, unused by the splat path."""
    f = 1.0 / math.tan(fovy / 2)
    m = np.zeros(16, dtype=np.float32)
    m[0] = f / aspect
    m[5] = f
    m[10] = far / (near - far)
    m[11] = -1
    m[14] = near * far / (near - far)
    return m


def make_frame(eye, target, up, fov_deg: float, width: int, height: int, count: int, *, near: float = 0.02,
               far: float = 50.0, view_mode: int = VIEW_LIT, n_emit: int = 0, bounce_gain: float = 0.0,
               lowpass_px2: float = 0.3, albedo_scale: float = 1.0, part_material=None) -> np.ndarray:
    """One RenderFrame (1200 B) as writeFrame fills it for the plain lit path: focal = H / (2 tan(fovy/2)), near 0.02
    (src/main.js:527, 545), palette slots white (1, 1, 1) with w = 1 (lit view: chosen/asset albedo ratio 1)."""
    fovy = fov_deg * math.pi / 180.0
    f = np.zeros((), dtype=FRAME)
    f["view"] = look_at(eye, target, up)
    f["proj"] = perspective(fovy, width / height, near, far)
    f["palette"][:3] = [1.0, 1.0, 1.0, 1.0]
    f["palette"][3] = [bounce_gain, n_emit, 0.0, 1.0]
    focal = height / (2.0 * math.tan(fovy / 2.0))
    f["viewport"] = [width, height]
    f["focal"] = [focal, focal]
    f["near"] = near
    f["far"] = far
    f["count"] = count
    f["view_mode"] = view_mode
    f["albedo_scale"] = albedo_scale
    f["exposure"] = 1.0
    f["lowpass_px2"] = lowpass_px2
    if part_material is not None:
        pm = np.zeros(32, dtype=np.uint32)
        pm[: len(part_material)] = part_material
        f["part_material"] = pm[:16]
        f["part_material_ext"] = pm[16:]
    else:
        f["part_material"] = 8   # no palette slot: the asset's own albedo
        f["part_material_ext"] = 8
    return f


def orbit_eye(center, radius: float, yaw: float, pitch: float):
    """Eye on a sphere around `center` (the orbit camera's eye(), src/camera.js:55-62)."""
    c = math.cos(pitch)
    return [center[0] + radius * c * math.cos(yaw), center[1] + radius * c * math.sin(yaw),
            center[2] + radius * math.sin(pitch)]
