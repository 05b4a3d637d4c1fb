"""RenderServer: continuous batching of render requests over resident scenes (sl_server_* in include/splatlight.h).

Requests (scene index, RenderFrame, eye, light-intensity scale) are submitted from any thread; a native worker thread
forms batches from the pending queue as pipelines and result slots free up, runs the batched chain, and returns each
image in a pinned result slot.  ``poll`` copies finished images out and releases their slots."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _native as N
from .structs import FRAME

# sl_server_request: u32 scene, f32 eye[3], f32 light_scale, u32 pad, then the 1200-byte RenderFrame
REQUEST = np.dtype([("scene", "<u4"), ("eye", "<f4", 3), ("light_scale", "<f4"), ("pad", "<u4"), ("frame", FRAME)])


@dataclass
class Result:
    tag: int
    status: int
    image: np.ndarray | None     # H x W x 4 (a copy; None on failure)
    batch_views: int
    t_submit: float
    t_start: float
    t_done: float

    @property
    def latency(self) -> float:
        return self.t_done - self.t_submit


class RenderServer:
    def __init__(self, renderers, lightings=None, max_views: int = 64, pipelines: int = 2, max_slots: int = 0,
                 max_pixels: int = 0, max_view_pixels: int = 0, max_tiles: int = 0, result_slots: int = 0,
                 hbm_budget_bytes: int = 0, tile=(16, 16), max_pending: int = 0):
        self._lib = N.lib()
        self._renderers = list(renderers)
        self._lightings = list(lightings) if lightings is not None else None
        rs = (C.c_void_p * len(self._renderers))(*[r.handle for r in self._renderers])
        ls = None
        if self._lightings is not None:
            ls = (C.c_void_p * len(self._lightings))(*[(l.handle if l is not None else None)
                                                        for l in self._lightings])
        o = N.ServerOptions(max_views, pipelines, max_slots, max_pixels, max_view_pixels, hbm_budget_bytes,
                            max_tiles, result_slots, tile[0], tile[1], max_pending, 0)
        h = C.c_void_p()
        N.check(self._lib.sl_server_create(rs, ls, len(self._renderers), C.byref(o), C.byref(h)))
        self._h = h
        self._res = (N.ServerResult * 256)()

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.sl_server_destroy(self._h)
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

    def submit(self, scene: int, frame, eye, light_scale: float = 1.0, tag: int = 0) -> None:
        """Queues one request; raises SplatlightError (SL_ERR_ADMISSION when it can never fit a batch)."""
        req = np.zeros((), dtype=REQUEST)
        req["scene"] = scene
        req["eye"] = np.asarray(eye, np.float32)
        req["light_scale"] = light_scale
        req["frame"] = np.asarray(frame, dtype=FRAME).reshape(())
        N.check(self._lib.sl_server_submit(self._h, req.ctypes.data, tag))

    def poll(self, wait_us: int = 0, copy: bool = True) -> list[Result]:
        """Finished requests (waiting up to wait_us for the first).  Images are copied out and their result slots
        released (copy=False: no image, slot released)."""
        n = C.c_uint32()
        N.check(self._lib.sl_server_poll(self._h, self._res, len(self._res), C.byref(n), wait_us))
        out = []
        for k in range(n.value):
            r = self._res[k]
            img = None
            if r.status == 0:
                if copy:
                    a = np.ctypeslib.as_array(r.image, shape=(r.height * r.width * 4,))
                    img = a.reshape(r.height, r.width, 4).copy()
                N.check(self._lib.sl_server_release(self._h, r.result_slot))
            out.append(Result(int(r.tag), int(r.status), img, int(r.batch_views), r.t_submit, r.t_start, r.t_done))
        return out

    def stats(self) -> dict:
        st = N.ServerStats()
        N.check(self._lib.sl_server_get_stats(self._h, C.byref(st)))
        return {name: int(getattr(st, name)) for name, _ in N.ServerStats._fields_}
