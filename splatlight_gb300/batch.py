"""BatchRenderer: a ragged batch of views over several resident scenes in one chain of kernels (sl_batch_* in
include/splatlight.h).  Every view's image, permutation and tile ranges equal those of SplatRenderer.render for that
frame alone with the same tile shape; the chain replays as one CUDA graph while the batch fits its capacity."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _native as N
from .structs import FRAME


@dataclass
class View:
    scene: int            # index into the batch's renderers
    frame: np.ndarray     # RenderFrame record (structs.FRAME)
    eye: tuple            # camera position (the lit radiance's view direction)
    light_scale: float = 1.0  # intensity scale of every light of the scene (the request's light state)


class BatchRenderer:
    def __init__(self, renderers, lightings=None, max_views: int = 64, tile=(16, 16), graph: bool = True,
                 max_slots: int = 0, max_tiles: int = 0, max_entries: int = 0, radiance_allowance: float = 0.0):
        self._lib = N.lib()
        self._renderers = list(renderers)
        self._lightings = list(lightings) if lightings is not None else None
        rs = (C.c_void_p * len(self._renderers))(*[r.handle for r in self._renderers])
        ls = None
        if self._lightings is not None:
            ls = (C.c_void_p * len(self._lightings))(*[(l.handle if l is not None else None)
                                                        for l in self._lightings])
        o = N.BatchOptions(max_views, max_tiles, max_slots, max_entries, tile[0], tile[1], 0 if graph else 1,
                           float(radiance_allowance))
        h = C.c_void_p()
        N.check(self._lib.sl_batch_create(rs, ls, len(self._renderers), C.byref(o), C.byref(h)))
        self._h = h
        self.max_views = max_views
        self.last_stats = N.BatchStats()
        self._out = None

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.sl_batch_destroy(self._h)
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

    def set_tile(self, tile_w: int, tile_h: int) -> None:
        N.check(self._lib.sl_batch_set_tile(self._h, tile_w, tile_h))

    def set_timing(self, on) -> None:
        """False/0 off, True/1 the whole chain (last_stats.ms_total), 2 also per stage (last_stats.ms_stage)."""
        N.check(self._lib.sl_batch_set_timing(self._h, int(on)))

    @staticmethod
    def _pack(views):
        n = len(views)
        frames = np.zeros(n, dtype=FRAME)
        scenes = np.zeros(n, dtype=np.uint32)
        eyes = np.zeros((n, 3), dtype=np.float32)
        scales = np.ones(n, dtype=np.float32)
        pix = 0
        for k, v in enumerate(views):
            frames[k] = np.asarray(v.frame, dtype=FRAME).reshape(())
            scenes[k] = v.scene
            eyes[k] = np.asarray(v.eye, dtype=np.float32)
            scales[k] = v.light_scale
            pix += int(frames[k]["viewport"][0]) * int(frames[k]["viewport"][1])
        return frames, scenes, eyes, scales, pix

    def _device_out(self, floats: int, out):
        import torch
        if out is not None:
            return out
        if self._out is None or self._out.numel() < floats:
            self._out = torch.empty(floats, dtype=torch.float32, device="cuda")
        return self._out

    def render_device(self, views, out=None, stream=None):
        """Renders the batch into a device float tensor (packed images); returns (tensor, offsets in floats)."""
        frames, scenes, eyes, scales, pix = self._pack(views)
        dev = self._device_out(4 * pix, out)
        offs = np.zeros(len(views), dtype=np.uint64)
        N.check(self._lib.sl_batch_render(self._h, scenes.ctypes.data, frames.ctypes.data, eyes.ctypes.data,
                                          scales.ctypes.data, len(views), dev.data_ptr(), dev.numel(), offs.ctypes.data,
                                          C.byref(self.last_stats), stream))
        self._keep = (frames, scenes, eyes, scales)
        return dev, offs

    def render(self, views, stream=None) -> list[np.ndarray]:
        """Renders the batch and returns each view's H x W x 4 image on the host."""
        dev, offs = self.render_device(views, stream=stream)
        sizes = []
        for v in views:
            f = np.asarray(v.frame, dtype=FRAME).reshape(())
            sizes.append((int(f["viewport"][1]), int(f["viewport"][0])))
        host = dev[: 4 * sum(h * w for h, w in sizes)].cpu().numpy()
        return [host[int(o):int(o) + 4 * h * w].reshape(h, w, 4) for o, (h, w) in zip(offs, sizes)]

    def tuning(self):
        """((tile_w, tile_h), {kernel: blocks per SM of its variant in use}) for bproject, btile_bin, bshade,
        bcomposite."""
        tw, th = C.c_uint32(), C.c_uint32()
        mb = np.zeros(4, dtype=np.uint32)
        N.check(self._lib.sl_batch_get_tuning(self._h, C.byref(tw), C.byref(th), mb.ctypes.data))
        names = ("bproject", "btile_bin", "bshade", "bcomposite")
        return (tw.value, th.value), {k: int(v) for k, v in zip(names, mb)}

    def set_tuning(self, blocks_per_sm: dict):
        """Sets each tunable kernel's block-size variant by its blocks per SM (keys as tuning() reports them)."""
        names = ("bproject", "btile_bin", "bshade", "bcomposite")
        mb = np.array([blocks_per_sm[k] for k in names], dtype=np.uint32)
        N.check(self._lib.sl_batch_set_tuning(self._h, mb.ctypes.data))

    def autotune(self, views, reps: int = 3):
        """Times the batch with each tile shape and keeps the fastest, then each tunable kernel's block-size variant
        by its stage's time; returns ((tile_w, tile_h), ms per shape)."""
        frames, scenes, eyes, scales, pix = self._pack(views)
        dev = self._device_out(4 * pix, None)
        tw, th = C.c_uint32(), C.c_uint32()
        ms = np.zeros(3, dtype=np.float32)
        N.check(self._lib.sl_batch_autotune(self._h, scenes.ctypes.data, frames.ctypes.data, eyes.ctypes.data,
                                            scales.ctypes.data, len(views), dev.data_ptr(), dev.numel(), reps, C.byref(tw),
                                            C.byref(th), ms.ctypes.data, None))
        return (tw.value, th.value), {"16x16": float(ms[0]), "8x32": float(ms[1]), "32x8": float(ms[2])}

    def read_view(self, view: int, n_slots: int, n_tiles: int):
        """Permutation, per-tile ranges and tile-list entries of one view of the last batch (the view's indices)."""
        order = np.empty(n_slots, dtype=np.uint32)
        ranges = np.empty((n_tiles, 2), dtype=np.uint32)
        ne = C.c_uint64()
        N.check(self._lib.sl_batch_read_view(self._h, view, order.ctypes.data, ranges.ctypes.data, None, 0,
                                             C.byref(ne)))
        entries = np.empty(ne.value, dtype=np.uint32)
        N.check(self._lib.sl_batch_read_view(self._h, view, None, None, entries.ctypes.data, ne.value, None))
        return order, ranges, entries
