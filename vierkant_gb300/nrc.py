"""Neural radiance cache through libvkg's C ABI (vkg_nrc_*): hash-grid + spherical-harmonics encoding,
fully-fused tensor-core MLP, relative-L2 loss, Adam. Feature records are [N, 13] fp32 CUDA tensors
(position, outgoing direction, normal, roughness, albedo); predictions are [N, 3] fp32."""
from __future__ import annotations

import ctypes as C

import torch

from ._lib import check, lib, vkg_nrc_config, vkg_nrc_info_t
from .raytracing import Context


class NeuralRadianceCache:
    @staticmethod
    def default_config() -> vkg_nrc_config:
        c = vkg_nrc_config()
        check(lib().vkg_nrc_config_default(C.byref(c)))
        return c

    def __init__(self, ctx: Context, config: vkg_nrc_config | None = None):
        self.ctx = ctx
        self.config = config if config is not None else self.default_config()
        h = C.c_void_p()
        check(lib().vkg_nrc_create(ctx.handle, C.byref(self.config), C.byref(h)), ctx.handle, "vkg_nrc_create")
        self.handle = h
        ctx.adopt(self)

    def info(self) -> vkg_nrc_info_t:
        i = vkg_nrc_info_t()
        check(lib().vkg_nrc_info(self.handle, C.byref(i)))
        return i

    def _s(self):
        return C.c_void_p(self.ctx.stream())

    def infer(self, feats: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        feats = feats.contiguous()
        n = feats.shape[0]
        if out is None:
            out = torch.empty((n, 3), dtype=torch.float32, device=feats.device)
        check(lib().vkg_nrc_infer(self.handle, C.c_void_p(feats.data_ptr()), n, C.c_void_p(out.data_ptr()), self._s()),
              self.ctx.handle, "vkg_nrc_infer")
        return out

    def backward(self, feats: torch.Tensor, targets: torch.Tensor):
        check(lib().vkg_nrc_backward(self.handle, C.c_void_p(feats.contiguous().data_ptr()),
                                     C.c_void_p(targets.contiguous().data_ptr()), feats.shape[0], self._s()),
              self.ctx.handle, "vkg_nrc_backward")

    def adam_step(self):
        check(lib().vkg_nrc_adam_step(self.handle, self._s()), self.ctx.handle, "vkg_nrc_adam_step")

    def train_step(self, feats: torch.Tensor, targets: torch.Tensor) -> float:
        loss = C.c_float()
        check(lib().vkg_nrc_train_step(self.handle, C.c_void_p(feats.contiguous().data_ptr()),
                                       C.c_void_p(targets.contiguous().data_ptr()), feats.shape[0], C.byref(loss),
                                       self._s()), self.ctx.handle, "vkg_nrc_train_step")
        return float(loss.value)

    def load_params(self, mlp: torch.Tensor | None = None, grid: torch.Tensor | None = None):
        check(lib().vkg_nrc_load_params(self.handle, C.c_void_p(mlp.data_ptr()) if mlp is not None else None,
                                        C.c_void_p(grid.data_ptr()) if grid is not None else None, self._s()),
              self.ctx.handle, "vkg_nrc_load_params")

    def save(self, path: str):
        """checkpoint: weights, grid, both Adam moments and the step count (vkg_nrc_save)"""
        check(lib().vkg_nrc_save(self.handle, str(path).encode(), self._s()), self.ctx.handle, "vkg_nrc_save")

    def load(self, path: str):
        """restore a checkpoint of a cache with the same grid layout (vkg_nrc_load)"""
        check(lib().vkg_nrc_load(self.handle, str(path).encode(), self._s()), self.ctx.handle, "vkg_nrc_load")

    def close(self):
        if getattr(self, "handle", None) and getattr(self.ctx, "handle", None):
            lib().vkg_nrc_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def cache_for_scene(ctx: Context, scene, config: vkg_nrc_config | None = None, margin: float = 1e-3):
    """a NeuralRadianceCache whose hash grid spans `scene`'s bounds (slightly enlarged)"""
    cfg = config if config is not None else NeuralRadianceCache.default_config()
    lo, hi = scene.bounds()
    for a in range(3):
        pad = margin * max(hi[a] - lo[a], 1e-6)
        cfg.scene_min[a] = lo[a] - pad
        cfg.scene_max[a] = hi[a] + pad
    return NeuralRadianceCache(ctx, cfg)
