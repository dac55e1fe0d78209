"""Scalar intersection API mirroring vierkant's include/vierkant/intersection.hpp.

Value types keep the reference's names (Ray, Triangle, AABB, OBB, Sphere, Plane) and results keep
``ray_intersection`` / ``ray_triangle_intersection`` semantics (type REJECT/INTERSECT/INSIDE,
distance, barycentrics u/v). Every call goes through libvkg's C ABI (host code, bit-identical to
vierkant::intersect in src/intersection.cpp).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from ._lib import INSIDE, INTERSECT, REJECT, check, lib, vkg_ray_intersection, vkg_ray_triangle_intersection

__all__ = ["REJECT", "INTERSECT", "INSIDE", "Ray", "Triangle", "AABB", "OBB", "Sphere", "Plane",
           "RayIntersection", "RayTriangleIntersection", "intersect"]


def _f32(v, n):
    a = np.ascontiguousarray(np.asarray(v, dtype=np.float32).reshape(n))
    return a, a.ctypes.data_as(C.c_void_p)


@dataclass
class Ray:
    """origin + direction (used as given: vierkant's Ray(o, d) constructor normalises d)."""
    origin: tuple
    direction: tuple

    @staticmethod
    def normalized(origin, direction) -> "Ray":
        d = np.asarray(direction, dtype=np.float32)
        inv = np.float32(1.0) / np.sqrt(np.float32(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]))
        return Ray(tuple(np.asarray(origin, np.float32)), tuple(d * inv))


@dataclass
class Triangle:
    v0: tuple
    v1: tuple
    v2: tuple


@dataclass
class AABB:
    min: tuple
    max: tuple


@dataclass
class OBB:
    center: tuple
    axes: tuple  # three unit column vectors
    half_lengths: tuple


@dataclass
class Sphere:
    center: tuple
    radius: float


@dataclass
class Plane:
    """Ax + By + Cz + D = 0, normalised like vierkant::Plane(a, b, c, d)."""
    coefficients: tuple


@dataclass
class RayIntersection:
    type: int
    distance: float

    def __bool__(self):
        return self.type != REJECT


@dataclass
class RayTriangleIntersection(RayIntersection):
    u: float = 0.0
    v: float = 0.0


def intersect(a, b):
    """vierkant::intersect overload set: (Triangle|AABB|OBB|Sphere|Plane, Ray) in either order,
    (Triangle, AABB) and (Triangle, Triangle)."""
    L = lib()
    if isinstance(a, Ray) and not isinstance(b, Ray):
        a, b = b, a
    if isinstance(b, Triangle) and isinstance(a, AABB):
        a, b = b, a
    if isinstance(b, Ray):
        o, po = _f32(b.origin, 3)
        d, pd = _f32(b.direction, 3)
        if isinstance(a, Triangle):
            t, pt = _f32([a.v0, a.v1, a.v2], 9)
            r = vkg_ray_triangle_intersection()
            check(L.vkg_intersect_ray_triangle(po, pd, pt, C.byref(r)))
            return RayTriangleIntersection(r.type, r.distance, r.u, r.v)
        r = vkg_ray_intersection()
        if isinstance(a, AABB):
            lo, plo = _f32(a.min, 3)
            hi, phi = _f32(a.max, 3)
            check(L.vkg_intersect_ray_aabb(po, pd, plo, phi, C.byref(r)))
        elif isinstance(a, OBB):
            c, pc = _f32(a.center, 3)
            ax, pax = _f32(a.axes, 9)
            h, ph = _f32(a.half_lengths, 3)
            check(L.vkg_intersect_ray_obb(po, pd, pc, pax, ph, C.byref(r)))
        elif isinstance(a, Sphere):
            c, pc = _f32(a.center, 3)
            check(L.vkg_intersect_ray_sphere(po, pd, pc, C.c_float(a.radius), C.byref(r)))
        elif isinstance(a, Plane):
            p, pp = _f32(a.coefficients, 4)
            check(L.vkg_intersect_ray_plane(po, pd, pp, C.byref(r)))
        else:
            raise TypeError(f"intersect({type(a).__name__}, Ray) is not defined")
        return RayIntersection(r.type, r.distance)
    if isinstance(a, Triangle) and isinstance(b, AABB):
        t, pt = _f32([a.v0, a.v1, a.v2], 9)
        lo, plo = _f32(b.min, 3)
        hi, phi = _f32(b.max, 3)
        out = C.c_uint32()
        check(L.vkg_intersect_triangle_aabb(pt, plo, phi, C.byref(out)))
        return int(out.value)
    if isinstance(a, Triangle) and isinstance(b, Triangle):
        t1, p1 = _f32([a.v0, a.v1, a.v2], 9)
        t2, p2 = _f32([b.v0, b.v1, b.v2], 9)
        out = C.c_uint32()
        check(L.vkg_intersect_triangle_triangle(p1, p2, C.byref(out)))
        return int(out.value)
    raise TypeError(f"intersect({type(a).__name__}, {type(b).__name__}) is not defined")
