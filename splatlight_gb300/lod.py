"""Screen-space LOD (sl_lod_* in include/splatlight.h; src/lod.js Lod, runtime/wgsl/lod.wgsl): the scene's tree drawn
as a level of detail.  ``Lod(renderer, nodes, kids)`` makes the internal nodes' Gaussian records and attaches the LOD
to the renderer; per frame, ``select`` (the cut) and, for a lit view, ``colour`` (the drawn nodes' lit colours) run
before ``renderer.render`` of a frame whose ``lod`` field is set by ``frame_lod``."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .structs import FRAME, GAUSSIAN, NODE

NONE, OPEN, DRAW, CAND, UNDER = 0, 1, 2, 3, 4


def frame_lod(frame, threshold_px: float, n_internal: int, node_base: int | None = None):
    """Sets frame['lod'] = (threshold px as float bits, node slot base, internal node count, 0) in place; the base
    defaults to the first slot after the frame's emitters."""
    f = frame.reshape(()) if isinstance(frame, np.ndarray) else frame
    count = int(f["count"])
    n_emit = int(f["palette"][3][1])
    base = count + 1 + n_emit if node_base is None else node_base
    f["lod"] = [np.float32(threshold_px).view(np.uint32), base, n_internal, 0]
    return frame


class Lod:
    def __init__(self, renderer, nodes: np.ndarray, kids: np.ndarray):
        self._lib = N.lib()
        self._nodes = np.ascontiguousarray(nodes, dtype=NODE)
        self._kids = np.ascontiguousarray(kids, dtype=np.uint32)
        self.N = len(self._nodes)
        self.G = renderer.count
        self.n_internal = self.N - self.G
        h = C.c_void_p()
        N.check(self._lib.sl_lod_create(renderer.handle, self._nodes.ctypes.data, self.N, self._kids.ctypes.data,
                                        len(self._kids), C.byref(h)))
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.sl_lod_destroy(self._h)
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

    def select(self, frame, emit_part: int = 0xFFFFFFFF, size_rule: int = 1, blur_lod: float = 0.0,
               stream=None) -> None:
        f = np.ascontiguousarray(frame, dtype=FRAME).reshape(())
        N.check(self._lib.sl_lod_select(self._h, f.ctypes.data, emit_part, size_rule, blur_lod, stream))

    def colour(self, frame, colour_all: bool = False, stream=None) -> None:
        f = np.ascontiguousarray(frame, dtype=FRAME).reshape(())
        N.check(self._lib.sl_lod_colour(self._h, f.ctypes.data, 1 if colour_all else 0, stream))

    def read(self):
        """(flags (N,) u32, node colours (N - G, 4) f32, internal node records (N - G,) GAUSSIAN)."""
        flags = np.zeros(self.N, np.uint32)
        col = np.zeros((max(self.n_internal, 1), 4), np.float32)
        recs = np.zeros(max(self.n_internal, 1), GAUSSIAN)
        N.check(self._lib.sl_lod_read(self._h, flags.ctypes.data, col.ctypes.data, recs.ctypes.data))
        return flags, col[:self.n_internal], recs[:self.n_internal]
