"""Lighting: the per-Gaussian lighting the splat path composites, mirroring src/lighting.js (Lighting: setEmitters
:612, encode :1258), src/environment.js (Environment.set :106) and their shadow maps, over the C ABI."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .renderer import SplatRenderer
from .structs import GAUSSIAN, MATERIAL, NODE, VGRID


class EnvLight(C.Structure):
    _fields_ = [("dir", C.c_float * 3), ("std", C.c_float), ("irradiance", C.c_float * 3),
                ("casts_shadows", C.c_int32)]


class Lighting:
    """Radiance per Gaussian from emissive-Gaussian lights (light cut over a host emitter tree, per-part opacity map
    shadows) and distant lights (sun maps), bound to a SplatRenderer's scene."""

    def __init__(self, renderer: SplatRenderer, nodes: np.ndarray, vgrid: np.ndarray, materials: np.ndarray):
        self._lib = N.lib()
        self.renderer = renderer
        nd = np.ascontiguousarray(nodes, dtype=NODE)
        vg = np.ascontiguousarray(vgrid, dtype=VGRID)
        mt = np.ascontiguousarray(materials, dtype=MATERIAL)
        h = C.c_void_p()
        N.check(self._lib.sl_lighting_create(renderer.handle, nd.ctypes.data, vg.ctypes.data, mt.ctypes.data, len(mt),
                                             C.byref(h)))
        self._h = h
        self.count = renderer.count

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.sl_lighting_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def set_emitters(self, emitters: np.ndarray, scale: float = 1.0, one_sided: bool = False, normal=(0.0, 0.0, 1.0),
                     skip_part: int = 0xFFFFFFFF) -> None:
        e = np.ascontiguousarray(emitters, dtype=GAUSSIAN)
        nrm = (C.c_float * 3)(*normal)
        N.check(self._lib.sl_lighting_set_emitters(self._h, e.ctypes.data if len(e) else None, len(e), scale,
                                                   1 if one_sided else 0, nrm, skip_part))

    def set_environment(self, lights=(), sky_ambient: float = 0.0) -> None:
        """lights: iterable of (direction, angular std in radians, irradiance rgb, casts shadows)."""
        arr = (EnvLight * 4)()
        n = 0
        for d, std, irr, sh in lights:
            arr[n].dir[:] = list(d)
            arr[n].std = std
            arr[n].irradiance[:] = list(irr)
            arr[n].casts_shadows = 1 if sh else 0
            n += 1
        N.check(self._lib.sl_lighting_set_environment(self._h, C.addressof(arr) if n else None, n, sky_ambient))

    def set_options(self, shadow_res: int = 512, sun_res: int = 512, mode: int = 1, theta: float = 4.0,
                    asg: bool = True) -> None:
        N.check(self._lib.sl_lighting_set_options(self._h, shadow_res, sun_res, mode, theta, 1 if asg else 0))

    def set_blur(self, shutter: float, cut_k: float = 1.0) -> None:
        """Motion blur for the lighting: moving parts' records drawn stretched into the opacity maps (shutter 0 =
        off); with a tree (set_tree) and cut_k > 0 a moving part splats the cut of its tree sized to its smear."""
        N.check(self._lib.sl_lighting_set_blur(self._h, C.c_float(shutter), C.c_float(cut_k)))

    def set_tree(self, nodes, kids) -> None:
        """The scene's tree (leaves then internal nodes, NODE records; kids the children lists) for the blur cut."""
        nd = np.ascontiguousarray(nodes, dtype=NODE)
        k = np.ascontiguousarray(kids, dtype=np.uint32)
        N.check(self._lib.sl_lighting_set_tree(self._h, nd.ctypes.data, len(nd), k.ctypes.data if len(k) else None,
                                               len(k)))
        self.tree_count = len(nd)
        self.sender_cut = False   # a new tree turns the sender cut off

    def set_probes(self, layout: dict, max_depth: int = 0, blend: float = 1.0, emitters_dark: bool = True) -> None:
        """The probe bounce over a lattice (probes.room_layout / probes.terrain_layout); needs set_tree.  From the
        next update on, each update runs one bounce frame and the renderer adds gain x lo_b to the lit colour.
        emitters_dark: the emitters' own part sends nothing into the probes (the reference's emitBounceFix).
        blend: each gather's history weight after the first (1 as is; -1 the FIR blend of the last three)."""
        lay = N.ProbeLayout()
        lay.dims[:] = [int(v) for v in layout["dims"]]
        lay.terrain = 1 if layout["terrain"] else 0
        lay.lo[:] = [float(v) for v in layout["lo"]]
        lay.step[:] = [float(v) for v in layout["step"]]
        lv = list(layout["levels"]) + [0.0] * (16 - len(layout["levels"]))
        lay.levels[:] = [float(v) for v in lv]
        self._ground = np.ascontiguousarray(layout["ground"], np.float32) if layout.get("ground") is not None else None
        lay.ground = self._ground.ctypes.data if self._ground is not None else None
        lay.tmax = float(layout["tmax"])
        vols = list(layout.get("vols", []))[:32]
        lay.n_vols = len(vols)
        for i, v in enumerate(vols):
            lay.vols[i][:] = [int(x) for x in v]
        N.check(self._lib.sl_lighting_set_probes(self._h, C.byref(lay), int(max_depth), C.c_float(blend),
                                                 1 if emitters_dark else 0))
        self.probe_count = int(np.prod(layout["dims"])) + 8 * self.renderer.part_count + \
            sum(int(v[1]) * int(v[2]) * int(v[3]) for v in vols)

    def set_sender_cut(self, on: bool = True) -> None:
        """The sender cut (the reference's default level of detail for the probes' senders, bounce.wgsl sc_select):
        only the senders some probe resolves are lit, the rest of each part's tree as the nodes every probe uses whole.
        Needs set_probes; selected again on the next update and whenever a part moved."""
        N.check(self._lib.sl_lighting_set_sender_cut(self._h, 1 if on else 0))
        self.sender_cut = bool(on)

    def set_sky(self, sh_rgb) -> None:
        """The probes' sky: up to 16 real SH coefficients (bands 0-3), rgb; None or empty = no sky."""
        sh = np.ascontiguousarray(np.zeros((0, 3)) if sh_rgb is None else sh_rgb, np.float32).reshape(-1, 3)
        N.check(self._lib.sl_lighting_set_sky(self._h, sh.ctypes.data if len(sh) else None, len(sh)))

    def read_bounce(self):
        """The bounce state as a dict of host arrays: lo_b (G, 3, 4), lo_dir (G, 4), xfer (G, 12), probe_sh (NP, 9, 4),
        probe_data (NP, 128, 8), node_sh (N, 14) and node_acc (N, 14, 4); with the sender cut also sc_flag (N,),
        sc_X (N - G, 8, 4), sc_T (N - G,) and sc_envT (N - G, 4)."""
        G, NP, Nn = self.count, self.probe_count, self.tree_count
        shapes = [("lo_b", (G, 3, 4), np.float32), ("lo_dir", (G, 4), np.float32), ("xfer", (G, 12), np.float32),
                  ("probe_sh", (NP, 9, 4), np.float32), ("probe_data", (NP, 128, 8), np.float32),
                  ("node_sh", (Nn, 14), np.uint32), ("node_acc", (Nn, 14, 4), np.float32)]
        if getattr(self, "sender_cut", False):
            shapes += [("sc_flag", (Nn,), np.uint32), ("sc_X", (Nn - G, 8, 4), np.float32),
                       ("sc_T", (Nn - G,), np.float32), ("sc_envT", (Nn - G, 4), np.float32)]
        out = {}
        for k, (name, shape, dt) in enumerate(shapes):
            a = np.empty(shape, dt)
            N.check(self._lib.sl_lighting_read_bounce(self._h, k, a.ctypes.data, a.nbytes))
            out[name] = a
        return out

    def update(self, eye, forward=None, moved_mask: int = 0, stream=None) -> None:
        e = (C.c_float * 3)(*[float(v) for v in eye])
        f = (C.c_float * 3)(*[float(v) for v in forward]) if forward is not None else None
        N.check(self._lib.sl_lighting_update(self._h, e, f, moved_mask, stream))

    def shade(self, eye, stream=None) -> None:
        """The shading pass alone at a new eye; the maps stay as the last update left them."""
        e = (C.c_float * 3)(*[float(v) for v in eye])
        N.check(self._lib.sl_lighting_shade(self._h, e, stream))

    def bind(self) -> None:
        N.check(self._lib.sl_renderer_bind_lighting(self.renderer.handle, self._h))

    def read(self):
        """(colour (G, 4), lamp_T (G,), env_T (G, 4), nodes) from the device."""
        n = self.count
        col = np.empty((n, 4), np.float32)
        lt = np.empty(n, np.float32)
        et = np.empty((n, 4), np.float32)
        nd = np.empty(n, dtype=NODE)
        N.check(self._lib.sl_lighting_read(self._h, col.ctypes.data, lt.ctypes.data, et.ctypes.data, nd.ctypes.data))
        return col, lt, et, nd


def for_scene(renderer: SplatRenderer, scene) -> Lighting:
    """A Lighting set up from a splatlight_gb300.scene.Scene: its host emitters, its sun and sky, its map sizes."""
    L = Lighting(renderer, scene.nodes, scene.vgrid, scene.materials)
    L.set_options(shadow_res=scene.shadow_res, sun_res=scene.sun_res)
    L.set_emitters(scene.emitters, scale=scene.emit_scale, one_sided=scene.emit_one_sided, normal=scene.emit_normal,
                   skip_part=scene.emit_skip_part)
    L.set_environment(scene.distant_lights(), scene.sky_ambient)
    L.bind()
    return L


def camera_forward(scene, eye=None, target=None) -> np.ndarray:
    """Unit view direction as float32 (the value both the GPU path and the restatement receive)."""
    eye = np.asarray(scene.eye if eye is None else eye, np.float64)
    tgt = np.asarray(scene.target if target is None else target, np.float64)
    return ((tgt - eye) / np.linalg.norm(tgt - eye)).astype(np.float32)
