"""GPU ray queries through libvkg's C ABI: context, BVH build, closest-hit / any-hit, camera rays.

Device buffers are torch tensors (torch provides device memory and the current CUDA stream; all
work runs in libvkg's own kernels). Ray batches are float32 tensors of shape [N, 8]
({origin.xyz, tmin, direction.xyz, tmax}, 32 B per ray); hits are int32 tensors [N, 4]
({prim, t, u, v} with t/u/v as float bits, 16 B per hit; prim == -1 (0xFFFFFFFF) on a miss).
"""
from __future__ import annotations

import ctypes as C
import weakref

import numpy as np
import torch

from ._lib import (RAY_COUNT_STATS, RAY_CULL_BACK_FACES, RAY_KEEP_ORDER, check, lib, vkg_bvh_build_options,
                   vkg_bvh_info, vkg_tlas_info, vkg_camera)

__all__ = ["Context", "BVH", "TLAS", "INSTANCE_DTYPE", "hits_view", "RAY_CULL_BACK_FACES", "RAY_COUNT_STATS",
           "RAY_KEEP_ORDER"]


def _stream_ptr(device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


class Context:
    """One libvkg context per host thread and device (vkg_ctx_create / vkg_ctx_destroy)."""

    def __init__(self, device: int = 0):
        if not torch.cuda.is_available():
            raise RuntimeError("vierkant_gb300.Context needs a CUDA device")
        self.device = device
        torch.cuda.init()
        h = C.c_void_p()
        check(lib().vkg_ctx_create(device, C.byref(h)), None, "vkg_ctx_create")
        self.handle = h
        self._children = weakref.WeakSet()

    def adopt(self, obj):
        """objects created on this context are released before it (the C API needs that order)"""
        self._children.add(obj)

    def close(self):
        if getattr(self, "handle", None):
            for child in list(self._children):
                try:
                    child.close()
                except Exception:
                    pass
            torch.cuda.synchronize(self.device)
            lib().vkg_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- helpers -------------------------------------------------------------------------
    def _check(self, status, what):
        check(status, self.handle, what)

    def stream(self) -> int:
        return _stream_ptr(self.device)

    def camera_rays(self, cam: vkg_camera, seed: int, stream_id: int, spp: int = 1, out: torch.Tensor | None = None):
        n = cam.width * cam.height * spp
        if out is None:
            out = torch.empty((n, 8), dtype=torch.float32, device=f"cuda:{self.device}")
        self._check(lib().vkg_camera_rays(self.handle, C.byref(cam), seed, stream_id, spp,
                                          C.c_void_p(out.data_ptr()), C.c_void_p(self.stream())), "vkg_camera_rays")
        return out

    def stats(self, reset: bool = True):
        v, t = C.c_uint64(), C.c_uint64()
        self._check(lib().vkg_ray_stats_get(self.handle, C.byref(v), C.byref(t), int(reset)), "vkg_ray_stats_get")
        return int(v.value), int(t.value)


class BVH:
    """8-wide quantised BVH built on the GPU from fp32 xyz vertices and uint32 triangle indices."""

    def __init__(self, ctx: Context, xyz: torch.Tensor, indices: torch.Tensor, leaf_max: int = 2):
        self.ctx = ctx
        dev = f"cuda:{ctx.device}"
        xyz = xyz.to(device=dev, dtype=torch.float32).contiguous()
        idx = indices.to(device=dev).contiguous()
        if idx.dtype != torch.int32:
            idx = idx.to(torch.int64).to(torch.int32)
        self._xyz, self._idx = xyz, idx  # keep alive for the build
        opts = vkg_bvh_build_options(leaf_max)
        h = C.c_void_p()
        ctx._check(lib().vkg_bvh_build(ctx.handle, C.c_void_p(xyz.data_ptr()), xyz.numel() // 3,
                                       C.c_void_p(idx.data_ptr()), idx.numel() // 3, C.byref(opts), C.byref(h),
                                       C.c_void_p(ctx.stream())), "vkg_bvh_build")
        self.handle = h
        ctx.adopt(self)

    def info(self) -> vkg_bvh_info:
        inf = vkg_bvh_info()
        check(lib().vkg_bvh_info_get(self.handle, C.byref(inf)))
        return inf

    def close(self):
        if getattr(self, "handle", None) and getattr(self.ctx, "handle", None):
            lib().vkg_bvh_destroy(self.ctx.handle, self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def closest_hit(self, rays: torch.Tensor, out: torch.Tensor | None = None, flags: int = 0) -> torch.Tensor:
        n = rays.shape[0]
        if out is None:
            out = torch.empty((n, 4), dtype=torch.int32, device=rays.device)
        self.ctx._check(lib().vkg_closest_hit(self.ctx.handle, self.handle, C.c_void_p(rays.data_ptr()), n,
                                              C.c_void_p(out.data_ptr()), flags, C.c_void_p(self.ctx.stream())),
                        "vkg_closest_hit")
        return out

    def any_hit(self, rays: torch.Tensor, out: torch.Tensor | None = None, flags: int = 0) -> torch.Tensor:
        n = rays.shape[0]
        if out is None:
            out = torch.empty((n,), dtype=torch.int32, device=rays.device)
        self.ctx._check(lib().vkg_any_hit(self.ctx.handle, self.handle, C.c_void_p(rays.data_ptr()), n,
                                          C.c_void_p(out.data_ptr()), flags, C.c_void_p(self.ctx.stream())),
                        "vkg_any_hit")
        return out

    def closest_hit_host(self, rays_host: torch.Tensor, hits_host: torch.Tensor, flags: int = 0) -> torch.Tensor:
        """Host buffers in, host buffers out (H2D copy, trace, D2H copy, synchronise)."""
        n = rays_host.shape[0]
        self.ctx._check(lib().vkg_closest_hit_host(self.ctx.handle, self.handle, C.c_void_p(rays_host.data_ptr()), n,
                                                   C.c_void_p(hits_host.data_ptr()), flags,
                                                   C.c_void_p(self.ctx.stream())), "vkg_closest_hit_host")
        return hits_host


INSTANCE_DTYPE = np.dtype([("transform", "<f4", 12), ("blas", "<u4"), ("material", "<u4"), ("pad", "<u4", 2)])


class TLAS:
    """Two-level BVH: instances (INSTANCE_DTYPE: object -> world 3x4 transform, BLAS index, material)
    over bottom-level BVHs, which must outlive it."""

    def __init__(self, ctx: Context, blas: list, instances, leaf_max: int = 4):
        self.ctx = ctx
        self.blas = list(blas)
        dev = f"cuda:{ctx.device}"
        inst = np.ascontiguousarray(instances, INSTANCE_DTYPE)
        self.num_instances = len(inst)
        self._inst = torch.from_numpy(inst.view(np.uint8).copy()).to(dev)
        arr = (C.c_void_p * max(1, len(self.blas)))(*[b.handle.value for b in self.blas])
        opts = vkg_bvh_build_options(leaf_max)
        h = C.c_void_p()
        ctx._check(lib().vkg_tlas_build(ctx.handle, arr, len(self.blas), C.c_void_p(self._inst.data_ptr()),
                                        len(inst), C.byref(opts), C.byref(h), C.c_void_p(ctx.stream())),
                   "vkg_tlas_build")
        self.handle = h
        ctx.adopt(self)

    def info(self) -> vkg_tlas_info:
        inf = vkg_tlas_info()
        check(lib().vkg_tlas_info_get(self.handle, C.byref(inf)))
        return inf

    def instance_records(self, by_id: bool = True) -> np.ndarray:
        """the device's 128-byte instance records as float32 [N, 32] (w2o = [:, 0:12], o2w = [:, 12:24])"""
        inf = self.info()
        n = inf.num_instances
        if n == 0:
            return np.zeros((0, 32), np.float32)
        t = torch.empty(n * 32, dtype=torch.float32, device=f"cuda:{self.ctx.device}")
        src = inf.d_instances_by_id if by_id else inf.d_instances
        torch.cuda.synchronize()
        rt = _cudart()
        rt.cudaMemcpy(C.c_void_p(t.data_ptr()), C.c_void_p(src), C.c_size_t(n * 128), 3)
        return t.cpu().numpy().reshape(n, 32)

    def close(self):
        if getattr(self, "handle", None) and getattr(self.ctx, "handle", None):
            lib().vkg_tlas_destroy(self.ctx.handle, self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def closest_hit(self, rays: torch.Tensor, out: torch.Tensor | None = None, flags: int = 0) -> torch.Tensor:
        """int32 [N, 8] = {prim, instance, t, u, v, pad x 3} (t, u, v as float bits)"""
        n = rays.shape[0]
        if out is None:
            out = torch.empty((n, 8), dtype=torch.int32, device=rays.device)
        self.ctx._check(lib().vkg_tlas_closest_hit(self.ctx.handle, self.handle, C.c_void_p(rays.data_ptr()), n,
                                                   C.c_void_p(out.data_ptr()), flags, C.c_void_p(self.ctx.stream())),
                        "vkg_tlas_closest_hit")
        return out

    def any_hit(self, rays: torch.Tensor, out: torch.Tensor | None = None, flags: int = 0) -> torch.Tensor:
        n = rays.shape[0]
        if out is None:
            out = torch.empty(n, dtype=torch.int32, device=rays.device)
        self.ctx._check(lib().vkg_tlas_any_hit(self.ctx.handle, self.handle, C.c_void_p(rays.data_ptr()), n,
                                               C.c_void_p(out.data_ptr()), flags, C.c_void_p(self.ctx.stream())),
                        "vkg_tlas_any_hit")
        return out


def _cudart():
    import glob
    for cand in ["libcudart.so.13", "libcudart.so"] + sorted(glob.glob("/usr/local/cuda/lib64/libcudart.so*")):
        try:
            rt = C.CDLL(cand)
            rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
            return rt
        except OSError:
            continue
    raise RuntimeError("libcudart not found")


def hits_view(hits):
    """Split a [N,4] int32 hit tensor / array into (prim uint32, t, u, v float32) numpy arrays."""
    import numpy as np
    h = hits.cpu().numpy() if isinstance(hits, torch.Tensor) else np.asarray(hits)
    h = np.ascontiguousarray(h).view(np.uint32).reshape(-1, 4)
    return h[:, 0].copy(), h[:, 1].view(np.float32).copy(), h[:, 2].view(np.float32).copy(), \
        h[:, 3].view(np.float32).copy()
