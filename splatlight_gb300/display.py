"""Headless display resolve (sl_display in include/splatlight.h): a frame's linear RGBA image on the device to 8-bit
sRGB with the frame's exposure and tone curve (shaders/display.wgsl:120-189)."""
from __future__ import annotations

import numpy as np

from . import _native as N
from .structs import FRAME

TONES = ("clamp", "agx", "aces", "reinhard", "neutral", "filmic")


def to_srgb8(image, frame, stream=None) -> np.ndarray:
    """image: CUDA tensor (H, W, 4) float32 (as SplatRenderer.render(out=...) leaves it); returns (H, W, 4) uint8."""
    import torch
    f = np.ascontiguousarray(frame, dtype=FRAME).reshape(())
    H, W = int(image.shape[0]), int(image.shape[1])
    out = torch.empty((H, W, 4), dtype=torch.uint8, device=image.device)
    N.check(N.lib().sl_display(image.data_ptr(), W, H, f.ctypes.data, out.data_ptr(), stream))
    return out.cpu().numpy()
