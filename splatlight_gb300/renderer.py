"""SplatRenderer: the host object of the splat path, mirroring src/renderer.js (constructor :38-233, bindColour
:264-268, writeParts :407-409, encode :411-524) over the C ABI.  All device work happens in libsplatlight.so."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .structs import FRAME, GAUSSIAN, PART


class SplatRenderer:
    """Owns the device copy of a scene's Gaussians and parts and every per-view buffer.

    ``render(frame)`` runs project -> stable depth sort -> per-tile ranges -> composite and returns the W x H x 4
    linear RGBA image (row 0 at the top).  ``frame`` is a RenderFrame record (``structs.FRAME``), as writeFrame
    builds it (see ``camera.make_frame``).
    """

    def __init__(self, gaussians: np.ndarray, parts: np.ndarray, max_emitters: int = 16384):
        self._lib = N.lib()
        self._g = np.ascontiguousarray(gaussians, dtype=GAUSSIAN)
        self._p = np.ascontiguousarray(parts, dtype=PART)
        h = C.c_void_p()
        N.check(self._lib.sl_renderer_create(self._g.ctypes.data, len(self._g), self._p.ctypes.data, len(self._p),
                                             max_emitters, C.byref(h)))
        self._h = h
        self.count = len(self._g)
        self.part_count = len(self._p)
        self.last_stats = N.RenderStats()
        self._bound = None

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.sl_renderer_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    def write_parts(self, parts: np.ndarray) -> None:
        p = np.ascontiguousarray(parts, dtype=PART)
        N.check(self._lib.sl_renderer_set_parts(self._h, p.ctypes.data, len(p)))

    def set_emitters(self, emitters: np.ndarray) -> None:
        e = np.ascontiguousarray(emitters, dtype=GAUSSIAN)
        N.check(self._lib.sl_renderer_set_emitters(self._h, e.ctypes.data if len(e) else None, len(e)))

    def bind_colour(self, colour, lo_b=None) -> None:
        """colour: device tensor (count, 4) float32; lo_b: device tensor (count * 3, 4) or None.  Kept alive here."""
        self._bound = (colour, lo_b)
        N.check(self._lib.sl_renderer_bind_colour(self._h, N.ptr(colour), N.ptr(lo_b)))

    def set_options(self, tile_w: int = 0, tile_h: int = 0, t_stop: float = 0.0, entry_capacity: int = 0,
                    sort_mode: int = 0) -> None:
        """sort_mode: 0 keep, 1 stable radix sort (default), 2 counting sort (ties in arbitrary order)."""
        o = N.RenderOptions(tile_w, tile_h, t_stop, entry_capacity, sort_mode)
        N.check(self._lib.sl_renderer_set_options(self._h, C.byref(o)))

    def set_timing(self, on: bool) -> None:
        N.check(self._lib.sl_renderer_set_timing(self._h, 1 if on else 0))

    def render(self, frame: np.ndarray, out=None, stream=None) -> np.ndarray:
        """Renders one frame.  ``out``: None (a new host array), a host float32 array (H, W, 4), or a CUDA tensor of
        the same shape (the image stays on the device).  ``stream``: an int cudaStream_t or None."""
        f = np.ascontiguousarray(frame, dtype=FRAME).reshape(())
        W, H = int(f["viewport"][0]), int(f["viewport"][1])
        if out is None:
            out = np.empty((H, W, 4), dtype=np.float32)
        on_dev = 1 if getattr(out, "is_cuda", False) else 0
        N.check(self._lib.sl_render(self._h, f.ctypes.data, N.ptr(out), on_dev, C.byref(self.last_stats), stream))
        return out

    def read_debug(self) -> dict:
        """Of the last render: keys (u32 per slot, INVALID 0xFFFFFFFF), order (the stable permutation), ranges
        (tiles x 2, [start, end)) and entries (the per-tile slot lists, back to front within a tile)."""
        st = self.last_stats
        keys = np.empty(st.slots, dtype=np.uint32)
        order = np.empty(st.slots, dtype=np.uint32)
        ranges = np.empty((st.tiles, 2), dtype=np.uint32)
        N.check(self._lib.sl_renderer_read_debug(self._h, keys.ctypes.data, order.ctypes.data, ranges.ctypes.data,
                                                 None))
        ent = np.empty(max(st.entries, 1), dtype=np.uint32)
        N.check(self._lib.sl_renderer_read_entries(self._h, ent.ctypes.data, len(ent)))
        return {"keys": keys, "order": order, "ranges": ranges, "entries": ent[: st.entries]}

    def read_counts(self, width: int, height: int) -> np.ndarray:
        """Per-pixel contributor counts of the last render, which must have used the overdraw view (mode 2)."""
        cnt = np.empty((height, width), dtype=np.uint32)
        N.check(self._lib.sl_renderer_read_debug(self._h, None, None, None, cnt.ctypes.data))
        return cnt
