"""DiffRenderer: the differentiable splat path (sl_diff_* in include/splatlight.h) -- one inverse-rendering step
(forward, L2 loss against a target image, hand-written backward) over device tensors of free parameters.

``params_from_scene`` turns a generated scene (splatlight_gb300.scene) into those parameters: means, log-scales,
quaternions, opacity logits (kappa = softplus(logit) / (sqrt(2 pi) s0), the scene's own opacity), albedo, roughness
(the material's flake roughness), and its first emitters as the emissive Gaussian lights, each with an intensity
scale (the emitter tree over them is rebuilt at those intensities every step)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .structs import FRAME

PARAMS = ("means", "log_scales", "quats", "opacity_logits", "albedo", "roughness")
WIDTH = {"means": 3, "log_scales": 3, "quats": 4, "opacity_logits": 1, "albedo": 3, "roughness": 1}


def params_from_scene(s, n_lights: int = 8, ambient: float = 0.2, ks: float = 0.25):
    """(params, lights) as float32 numpy arrays from a Scene (part transforms applied to the means)."""
    g = s.gaussians
    part = (g["part_surface"] & 0xFFFF).astype(np.int64)
    part = np.minimum(part, len(s.parts) - 1)
    xf = s.parts["xf"][part].reshape(-1, 3, 4)
    mu = np.einsum("nij,nj->ni", xf[:, :, :3], g["mu"]) + xf[:, :, 3]
    s0 = g["scale"][:, 0].astype(np.float64)
    o = 1.0 - np.exp(-g["kappa"].astype(np.float64) * np.sqrt(2 * np.pi) * s0)
    o = np.clip(o, 1e-6, 1 - 1e-6)
    mats = s.materials[np.minimum(g["flags"] & 0xFFFF, len(s.materials) - 1)]
    rough = np.sqrt(np.maximum(mats["flake"][:, 1], 1e-4))
    params = {
        "means": mu.astype(np.float32),
        "log_scales": np.log(g["scale"]).astype(np.float32),
        "quats": g["quat"].astype(np.float32),
        "opacity_logits": np.log(o / (1 - o)).astype(np.float32),
        "albedo": g["albedo"].astype(np.float32),
        "roughness": rough.astype(np.float32),
    }
    e = np.ascontiguousarray(s.emitters[:n_lights])
    lights = {"rec": e, "scale": np.ones(len(e), np.float32), "ambient": ambient, "ks": ks}
    return params, lights


def perturb(params, rng, mean_std=0.02, log_scale_std=0.02, logit_std=0.1, albedo_std=0.05):
    """The target's parameters: N(0, 0.02) on means and log-scales, N(0, 0.1) on opacity logits, N(0, 0.05) on
    albedo."""
    p = {k: v.copy() for k, v in params.items()}
    p["means"] += rng.normal(0, mean_std, p["means"].shape).astype(np.float32)
    p["log_scales"] += rng.normal(0, log_scale_std, p["log_scales"].shape).astype(np.float32)
    p["opacity_logits"] += rng.normal(0, logit_std, p["opacity_logits"].shape).astype(np.float32)
    p["albedo"] += rng.normal(0, albedo_std, p["albedo"].shape).astype(np.float32)
    return p


class DiffRenderer:
    def __init__(self, n: int):
        self._lib = N.lib()
        h = C.c_void_p()
        N.check(self._lib.sl_diff_create(n, C.byref(h)))
        self._h = h
        self.n = n

    def close(self):
        if getattr(self, "_h", None):
            self._lib.sl_diff_destroy(self._h)
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

    @staticmethod
    def to_device(params, lights, state=None):
        """Parameters and light intensities as device tensors; the light records stay on the host.  state
        (optional): per-Gaussian vgrid (n VGRID records), lamp_T (n,) and iso_norm (n,), uploaded as constants."""
        import torch
        P = {k: torch.from_numpy(np.ascontiguousarray(params[k], np.float32)).cuda() for k in PARAMS}
        Lt = {"rec": np.ascontiguousarray(lights["rec"]),
              "scale": torch.from_numpy(np.ascontiguousarray(lights["scale"], np.float32)).cuda(),
              "ambient": float(lights["ambient"]), "ks": float(lights["ks"])}
        st = state or {}
        if st.get("vgrid") is not None:
            v = np.ascontiguousarray(st["vgrid"]).view(np.int32)
            Lt["vgrid"] = torch.from_numpy(v.copy()).cuda()
        for k in ("lamp_T", "iso_norm"):
            if st.get(k) is not None:
                Lt[k] = torch.from_numpy(np.ascontiguousarray(st[k], np.float32)).cuda()
        return P, Lt

    def _scene(self, P, Lt):
        def ptr(k):
            return Lt[k].data_ptr() if Lt.get(k) is not None else None
        rec = Lt["rec"]
        return N.DiffScene(P["means"].data_ptr(), P["log_scales"].data_ptr(), P["quats"].data_ptr(),
                           P["opacity_logits"].data_ptr(), P["albedo"].data_ptr(), P["roughness"].data_ptr(),
                           self.n, int(Lt["scale"].numel()), rec.ctypes.data if len(rec) else None,
                           Lt["scale"].data_ptr(), Lt["ambient"], Lt["ks"], ptr("vgrid"), ptr("lamp_T"),
                           ptr("iso_norm"))

    def forward(self, P, Lt, frame, eye, stream=None):
        import torch
        f = np.ascontiguousarray(frame, dtype=FRAME).reshape(())
        W, H = int(f["viewport"][0]), int(f["viewport"][1])
        img = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
        e = (C.c_float * 3)(*[float(v) for v in eye])
        sc = self._scene(P, Lt)
        N.check(self._lib.sl_diff_forward(self._h, C.byref(sc), f.ctypes.data, e, img.data_ptr(), stream))
        return img

    def step(self, P, Lt, frame, eye, target, stream=None):
        """Forward + backward against target (device H x W x 4).  Returns (loss, grads dict, image)."""
        import torch
        f = np.ascontiguousarray(frame, dtype=FRAME).reshape(())
        W, H = int(f["viewport"][0]), int(f["viewport"][1])
        img = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
        G = {k: torch.empty_like(P[k]) for k in PARAMS}
        G["light_scale"] = torch.empty_like(Lt["scale"])
        g = N.DiffGrads(*[G[k].data_ptr() for k in PARAMS], G["light_scale"].data_ptr())
        e = (C.c_float * 3)(*[float(v) for v in eye])
        sc = self._scene(P, Lt)
        loss = C.c_double()
        N.check(self._lib.sl_diff_step(self._h, C.byref(sc), f.ctypes.data, e, target.data_ptr(), img.data_ptr(),
                                       C.byref(g), C.byref(loss), stream))
        return loss.value, G, img

    def order(self) -> np.ndarray:
        nv = C.c_uint32()
        N.check(self._lib.sl_diff_read_order(self._h, None, C.byref(nv)))
        o = np.empty(nv.value, np.uint32)
        N.check(self._lib.sl_diff_read_order(self._h, o.ctypes.data, C.byref(nv)))
        return o
