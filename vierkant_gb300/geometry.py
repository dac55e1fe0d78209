"""Geometry generators (host, deterministic), mirroring vierkant::Geometry and the benchmark scenes.

- icosphere(radius, tess): Geometry::IcoSphere (src/Geometry.cpp:566-613), unshared vertices
- cornell_scene(seed, stream, num_spheres, n): 5-quad Cornell box + PCG32-placed cube-spheres
- camera_lookat(...): pinhole camera basis for the ray generators
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from ._lib import check, lib, vkg_camera, vkg_material

MATERIAL_DTYPE = np.dtype([("base_color", "<f4", 3), ("roughness", "<f4"), ("metalness", "<f4"),
                           ("emission", "<f4", 3), ("twosided", "<u4"), ("pad", "<f4", 3)])
assert MATERIAL_DTYPE.itemsize == C.sizeof(vkg_material)


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def icosphere(radius: float = 1.0, tess: int = 5):
    L = lib()
    nv, nt = C.c_uint32(), C.c_uint32()
    check(L.vkg_geometry_icosphere_counts(tess, C.byref(nv), C.byref(nt)))
    xyz = np.zeros((nv.value, 3), np.float32)
    idx = np.zeros((nt.value, 3), np.uint32)
    check(L.vkg_geometry_icosphere(C.c_float(radius), tess, _p(xyz), _p(idx)))
    return xyz, idx


def cornell_scene(seed: int = 0x5EED, stream: int = 2, num_spheres: int = 64, n: int = 16):
    """Returns dict(xyz [V,3] f32, indices [T,3] u32, tri_material [T] u32, materials structured array)."""
    L = lib()
    nv, nt, nm = C.c_uint32(), C.c_uint32(), C.c_uint32()
    check(L.vkg_scene_cornell_counts(num_spheres, n, C.byref(nv), C.byref(nt), C.byref(nm)))
    xyz = np.zeros((nv.value, 3), np.float32)
    idx = np.zeros((nt.value, 3), np.uint32)
    tm = np.zeros(nt.value, np.uint32)
    mats = np.zeros(nm.value, MATERIAL_DTYPE)
    check(L.vkg_scene_cornell(seed, stream, num_spheres, n, _p(xyz), _p(idx), _p(tm), _p(mats)))
    return {"xyz": xyz, "indices": idx, "tri_material": tm, "materials": mats}


def camera_lookat(eye, target, up, fovy_deg: float, width: int, height: int) -> vkg_camera:
    """tan(fovy/2) is evaluated here in double precision and passed to the library as a float."""
    L = lib()
    e = np.asarray(eye, np.float32)
    t = np.asarray(target, np.float32)
    u = np.asarray(up, np.float32)
    cam = vkg_camera()
    tan_half = float(np.float32(math.tan(math.radians(fovy_deg) / 2.0)))
    check(L.vkg_camera_lookat(_p(e), _p(t), _p(u), C.c_float(tan_half), width, height, C.byref(cam)))
    return cam


class _Pcg32:
    """PCG32 (XSH-RR, O'Neill 2014) for host-side workload parameters; the same generator as the kernels'."""
    MULT = 6364136223846793005
    MASK = (1 << 64) - 1

    def __init__(self, initstate: int, initseq: int):
        self.state = 0
        self.inc = ((initseq << 1) | 1) & self.MASK
        self.next()
        self.state = (self.state + initstate) & self.MASK
        self.next()

    def next(self) -> int:
        old = self.state
        self.state = (old * self.MULT + self.inc) & self.MASK
        xorshifted = (((old >> 18) ^ old) >> 27) & 0xFFFFFFFF
        rot = old >> 59
        return ((xorshifted >> rot) | (xorshifted << ((-rot) & 31))) & 0xFFFFFFFF

    def uniform(self) -> float:
        return (self.next() >> 8) * (1.0 / (1 << 24))


BATCH_RESOLUTIONS = (256, 512, 768, 1024)
BATCH_SPP = (4, 16, 64)


def batch_scene_params(index: int, seed: int = 0x5EED, min_tris: int = 5_000, max_tris: int = 2_000_000):
    """Parameters of scene `index` of the batched uneven workload (PCG32 seed 0x5EED, stream 3 + index):
    triangle count log-uniform in [min_tris, max_tris] (a Cornell box plus that many 3,072-triangle
    cube-spheres as fit, at least one), square resolution from {256, 512, 768, 1024}, spp from {4, 16, 64}.
    Returns dict(stream, spheres, triangles, resolution, spp)."""
    g = _Pcg32(seed, 3 + index)
    u_tris, u_res, u_spp = g.uniform(), g.uniform(), g.uniform()
    target = math.exp(math.log(min_tris) + u_tris * (math.log(max_tris) - math.log(min_tris)))
    spheres = max(1, int(round((target - 10) / 3072)))
    return {"stream": 3 + index, "spheres": spheres, "triangles": 10 + 3072 * spheres,
            "resolution": BATCH_RESOLUTIONS[min(3, int(u_res * 4))], "spp": BATCH_SPP[min(2, int(u_spp * 3))]}
