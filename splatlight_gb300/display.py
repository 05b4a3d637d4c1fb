"""Headless display resolve (sl_display / sl_display_env in include/splatlight.h): a frame's linear RGBA image on the
device to 8-bit sRGB with the frame's exposure and tone curve (shaders/display.wgsl:120-189), and with an environment
its sky and the distant lights' discs where the splats leave the sky showing (display.wgsl:22-133)."""
from __future__ import annotations

import math

import numpy as np

from . import _native as N
from .structs import FRAME

TONES = ("clamp", "agx", "aces", "reinhard", "neutral", "filmic")
DEG = math.pi / 180.0


def sky(sky_sh=None, lights=(), background=None) -> N.DisplaySky:
    """An sl_display_sky: sky_sh (16, 3) the lighting sky (None: no sky); lights [(direction, angular std, irradiance,
    casts shadows[, display std])]; background: None or a dict with "sh" (n <= 81, 3) and optionally "ring" (<= 8, 3),
    "ring_par" (2,), "ground" (3,), "ground_blend", "glow" (3,), "glow_std", "glow_dir" (3,)."""
    S = N.DisplaySky()
    if sky_sh is not None and len(sky_sh):
        S.has_sky = 1
        a = np.zeros((16, 3), np.float32)
        a[:min(16, len(sky_sh))] = np.asarray(sky_sh, np.float64)[:16]
        for k in range(16):
            S.sky_sh[k][:] = [float(v) for v in a[k]]
    S.n_lights = min(4, len(lights))
    for k, L in enumerate(list(lights)[:4]):
        S.light_dir[k][:] = [float(v) for v in L[0]]
        S.light_std[k] = float(L[1])
        S.light_irr[k][:] = [float(v) for v in L[2]]
        S.disc_std[k] = float(L[4]) if len(L) > 4 else 0.0
    if background is not None:
        bg = np.asarray(background["sh"], np.float64)[:81]
        S.bg_count = len(bg)
        for k in range(len(bg)):
            S.bg_sh[k][:] = [float(v) for v in bg[k]]
        ring = np.asarray(background.get("ring", np.zeros((0, 3))), np.float64)[:8]
        S.ring_count = len(ring)
        for k in range(len(ring)):
            S.ring[k][:] = [float(v) for v in ring[k]]
        S.ring_par[:] = [float(v) for v in background.get("ring_par", (0.0, 0.0))]
        S.ground[:] = [float(v) for v in background.get("ground", (0.0, 0.0, 0.0))]
        S.ground_blend = float(background.get("ground_blend", 1.0))
        S.glow[:] = [float(v) for v in background.get("glow", (0.0, 0.0, 0.0))]
        S.glow_std = float(background.get("glow_std", 0.0))
        S.glow_dir[:] = [float(v) for v in background.get("glow_dir", (0.0, 0.0, 1.0))]
    return S


def to_srgb8(image, frame, stream=None, sky_env: N.DisplaySky | None = None) -> np.ndarray:
    """image: CUDA tensor (H, W, 4) float32 (as SplatRenderer.render(out=...) leaves it); returns (H, W, 4) uint8.
    sky_env: the environment behind the splats (display.sky / asset.display_sky), or None (bare pixels black)."""
    import torch
    import ctypes as C
    f = np.ascontiguousarray(frame, dtype=FRAME).reshape(())
    H, W = int(image.shape[0]), int(image.shape[1])
    out = torch.empty((H, W, 4), dtype=torch.uint8, device=image.device)
    ptr = C.byref(sky_env) if sky_env is not None else None
    N.check(N.lib().sl_display_env(image.data_ptr(), W, H, f.ctypes.data, ptr, out.data_ptr(), stream))
    return out.cpu().numpy()
