"""Batched uneven rendering through libvkg's C ABI (vkg_batch_*): many (scene, camera, settings) jobs
traced through one set of wavefront queues, one CUDA-graph launch per render, with an autotuner for
the queue kernels and wave size. Each job's image equals the single-scene PBRPathTracer's for the same
seed and settings."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import torch

from ._lib import check, lib, vkg_batch_job, vkg_batch_stats, vkg_batch_tuning, vkg_camera, vkg_settings
from .raytracing import Context


@dataclass
class BatchJob:
    scene: object           # pathtracer.Scene
    camera: vkg_camera
    settings: vkg_settings
    seed: int = 0


class BatchRenderer:
    @staticmethod
    def default_tuning() -> vkg_batch_tuning:
        t = vkg_batch_tuning()
        check(lib().vkg_batch_tuning_default(C.byref(t)))
        return t

    def __init__(self, ctx: Context, jobs: list[BatchJob], tuning: vkg_batch_tuning | None = None):
        self.ctx = ctx
        self.jobs = list(jobs)
        dev = f"cuda:{ctx.device}"
        self.images = []
        arr = (vkg_batch_job * len(jobs))()
        for k, jb in enumerate(jobs):
            s = jb.settings
            w, h = (s.crop[2], s.crop[3]) if s.crop[2] and s.crop[3] else (s.resolution[0], s.resolution[1])
            img = torch.zeros((h, w, 3), dtype=torch.float32, device=dev)
            self.images.append(img)
            arr[k] = vkg_batch_job(jb.scene.handle, jb.camera, s, jb.seed, 0, img.data_ptr())
        h = C.c_void_p()
        check(lib().vkg_batch_create(ctx.handle, arr, len(jobs), C.byref(tuning) if tuning is not None else None,
                                     C.byref(h)), ctx.handle, "vkg_batch_create")
        self.handle = h
        ctx.adopt(self)

    def autotune(self) -> vkg_batch_tuning:
        t = vkg_batch_tuning()
        check(lib().vkg_batch_autotune(self.handle, C.c_void_p(self.ctx.stream()), C.byref(t)), self.ctx.handle,
              "vkg_batch_autotune")
        return t

    def set_tuning(self, t: vkg_batch_tuning):
        check(lib().vkg_batch_set_tuning(self.handle, C.byref(t)), self.ctx.handle, "vkg_batch_set_tuning")

    def render(self) -> list[torch.Tensor]:
        """one batch of every job; returns the jobs' running-mean images (device tensors, updated in place)"""
        check(lib().vkg_batch_render(self.handle, C.c_void_p(self.ctx.stream())), self.ctx.handle, "vkg_batch_render")
        return self.images

    def reset_accumulator(self):
        check(lib().vkg_batch_reset_accumulator(self.handle), self.ctx.handle, "vkg_batch_reset_accumulator")

    def statistics(self) -> vkg_batch_stats:
        st = vkg_batch_stats()
        check(lib().vkg_batch_statistics(self.handle, C.byref(st)), self.ctx.handle, "vkg_batch_statistics")
        return st

    def close(self):
        if getattr(self, "handle", None) and getattr(self.ctx, "handle", None):
            lib().vkg_batch_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
