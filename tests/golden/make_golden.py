"""Generate the committed golden fixtures from the reference's OWN code.

Runs where the reference checkout exists (it is compiled into oracle/_ref/libvkref.so by
oracle/Makefile from src/intersection.cpp + src/triangle_intersection.h, unmodified, against the
project-written glm/crocore shim). The GPU machine never runs this; it only reads the .npz files.

    python tests/golden/make_golden.py

Fixtures:
  ray_triangle.npz   intersect(Triangle, Ray)  (intersection.cpp:114-129)
  ray_aabb.npz       AABB::intersect(Ray)      (intersection.cpp:308-312 -> :152-184)
  ray_sphere.npz     intersect(Sphere, Ray)    (intersection.cpp:133-148)
  ray_plane.npz      intersect(Plane, Ray)     (intersection.cpp:10-21, Plane(a,b,c,d) :196-201)
  tri_box.npz        intersect(Triangle, AABB) (intersection.cpp:364-370 -> tri_box_overlap)
  tri_tri.npz        intersect(Triangle, Triangle) (intersection.cpp:374-378 -> tri_tri_overlap_test_3d)
  config1_hits.npz   closest hits of every 64th ray of the 1024x1024 icosphere workload, computed
                     by the reference's ray-triangle test over all triangles; plus SHA-256 of the
                     full vertex / index / ray buffers
  rng.npz            PCG32 (seed 0x5EED, stream 1) first 4096 draws and xxhash32 / lcg tables from
                     the CPU oracle (the reference has no PCG32; its shader RNG has no CPU code)
"""
from __future__ import annotations

import ctypes as C
import hashlib
import math
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
import oracle  # noqa: E402

OUT = Path(__file__).resolve().parent
P = oracle.ptr


def ray_triangle(R, rng, n=4096):
    o = rng.normal(size=(n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True).astype(np.float32)
    tri = rng.normal(size=(n, 9)).astype(np.float32)
    # aim half of the rays at a point inside their triangle so INTERSECT is well represented
    w = rng.dirichlet([1, 1, 1], size=n).astype(np.float32)
    target = (w[:, :1] * tri[:, 0:3] + w[:, 1:2] * tri[:, 3:6] + w[:, 2:3] * tri[:, 6:9]).astype(np.float32)
    aim = target - o
    aim /= np.linalg.norm(aim, axis=1, keepdims=True).astype(np.float32)
    d[: n // 2] = aim[: n // 2]
    # edge cases: grazing (det ~ 0), degenerate triangle, ray starting on the triangle
    tri[-1] = [0, 0, 0, 1, 0, 0, 2, 0, 0]
    o[-2] = tri[-2, 0:3]
    d[-3] = (tri[-3, 3:6] - tri[-3, 0:3]) / np.linalg.norm(tri[-3, 3:6] - tri[-3, 0:3])
    res = np.zeros((n, 4), np.float32)
    typ = np.zeros(n, np.int32)
    for i in range(n):
        out = np.zeros(3, np.float32)
        typ[i] = R.vkref_intersect_ray_triangle(P(o[i]), P(d[i]), P(tri[i]), P(out))
        res[i, :3] = out
    np.savez_compressed(OUT / "ray_triangle.npz", o=o, d=d, tri=tri, type=typ, tuv=res[:, :3])
    return typ.mean()


def ray_aabb(R, rng, n=4096):
    o = (rng.normal(size=(n, 3)) * 2).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True).astype(np.float32)
    c = rng.normal(size=(n, 3)).astype(np.float32)
    h = np.abs(rng.normal(size=(n, 3))).astype(np.float32) + 0.1
    lo, hi = (c - h).astype(np.float32), (c + h).astype(np.float32)
    d[::7, 0] = 0.0  # axis-parallel rays exercise the |f| <= 1e-10 branch
    o[::5] = c[::5]  # origin inside -> t_max
    typ = np.zeros(n, np.int32)
    t = np.zeros(n, np.float32)
    for i in range(n):
        tt = C.c_float()
        typ[i] = R.vkref_intersect_ray_aabb(P(o[i]), P(d[i]), P(lo[i]), P(hi[i]), C.byref(tt))
        t[i] = tt.value
    np.savez_compressed(OUT / "ray_aabb.npz", o=o, d=d, lo=lo, hi=hi, type=typ, t=t)
    return typ.mean()


def ray_sphere_plane(R, rng, n=2048):
    o = (rng.normal(size=(n, 3)) * 2).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True).astype(np.float32)
    c = rng.normal(size=(n, 3)).astype(np.float32)
    r = (np.abs(rng.normal(size=n)) + 0.2).astype(np.float32)
    typ = np.zeros(n, np.int32)
    t = np.zeros(n, np.float32)
    for i in range(n):
        tt = C.c_float()
        typ[i] = R.vkref_intersect_ray_sphere(P(o[i]), P(d[i]), P(c[i]), float(r[i]), C.byref(tt))
        t[i] = tt.value
    np.savez_compressed(OUT / "ray_sphere.npz", o=o, d=d, c=c, r=r, type=typ, t=t)
    pl = rng.normal(size=(n, 4)).astype(np.float32)
    typ2 = np.zeros(n, np.int32)
    t2 = np.zeros(n, np.float32)
    for i in range(n):
        tt = C.c_float()
        typ2[i] = R.vkref_intersect_ray_plane(P(o[i]), P(d[i]), P(pl[i]), C.byref(tt))
        t2[i] = tt.value
    np.savez_compressed(OUT / "ray_plane.npz", o=o, d=d, plane=pl, type=typ2, t=t2)
    return typ.mean(), typ2.mean()


def tri_box_tri_tri(R, rng, n=4096):
    tri = (rng.normal(size=(n, 9)) * 0.7).astype(np.float32)
    c = rng.normal(size=(n, 3)).astype(np.float32) * 0.5
    h = (np.abs(rng.normal(size=(n, 3))) * 0.4 + 0.05).astype(np.float32)
    lo, hi = (c - h).astype(np.float32), (c + h).astype(np.float32)
    res = np.array([R.vkref_triangle_aabb_overlap(P(tri[i]), P(lo[i]), P(hi[i])) for i in range(n)], np.uint32)
    np.savez_compressed(OUT / "tri_box.npz", tri=tri, lo=lo, hi=hi, overlap=res)
    a = (rng.normal(size=(n, 9)) * 0.7).astype(np.float32)
    b = (rng.normal(size=(n, 9)) * 0.7).astype(np.float32)
    # coplanar pairs (z = 0 plane) and shared-vertex pairs exercise the 2D branch and ties
    a[: n // 8, 2::3] = 0.0
    b[: n // 8, 2::3] = 0.0
    b[n // 8: n // 4, 0:3] = a[n // 8: n // 4, 0:3]
    res2 = np.array([R.vkref_triangle_triangle_overlap(P(a[i]), P(b[i])) for i in range(n)], np.uint32)
    np.savez_compressed(OUT / "tri_tri.npz", a=a, b=b, overlap=res2)
    return res.mean(), res2.mean()


def config1(R):
    xyz, idx = oracle.icosphere(1.0, 5)
    th = float(np.float32(math.tan(math.radians(60.0) / 2.0)))
    cam = oracle.camera((0, 0, 3), (0, 0, 0), (0, 1, 0), th, 1024, 1024)
    rays = oracle.camera_rays(cam, 0x5EED, 1, 1)
    sel = np.arange(0, len(rays), 64, dtype=np.int64)
    sub = np.ascontiguousarray(rays[sel])
    hits = np.zeros(len(sub), oracle.HIT_DTYPE)
    R.vkref_closest_hit_bruteforce(P(xyz), P(idx), idx.shape[0], P(sub), len(sub), P(hits), 0, 0)
    np.savez_compressed(OUT / "config1_hits.npz", ray_index=sel, rays=sub.view(np.float32).reshape(-1, 8),
                        hits=hits.view(np.uint32).reshape(-1, 4), tan_half_fovy=np.float32(th),
                        sha_xyz=hashlib.sha256(xyz.tobytes()).hexdigest(),
                        sha_idx=hashlib.sha256(idx.tobytes()).hexdigest(),
                        sha_rays=hashlib.sha256(rays.tobytes()).hexdigest())
    return (hits["prim"] != 0xFFFFFFFF).mean()


def rng_tables():
    L = oracle.orc()
    pcg = np.zeros(4096, np.uint32)
    L.orc_pcg32_fill(0x5EED, 1, 0, 4096, P(pcg))
    lhs = np.arange(64, dtype=np.uint32) * np.uint32(2654435761)
    rhs = np.arange(64, dtype=np.uint32)
    xx = np.array([L.orc_xxhash32(int(a), int(b)) for a, b in zip(lhs, rhs)], np.uint32)
    st = C.c_uint32(12345)
    lcg = np.array([L.orc_rnd(C.byref(st)) for _ in range(256)], np.float32)
    np.savez_compressed(OUT / "rng.npz", pcg32_5eed_1=pcg, xx_lhs=lhs, xx_rhs=rhs, xxhash32=xx, rnd_12345=lcg)


def main():
    oracle.build(ref=True)
    R = oracle.ref()
    if R is None:
        raise SystemExit("oracle/_ref/libvkref.so is missing: the reference checkout is needed")
    rng = np.random.default_rng(20261203)
    print("ray_triangle hit rate", ray_triangle(R, rng))
    print("ray_aabb hit rate", ray_aabb(R, rng))
    print("ray_sphere / plane hit rate", ray_sphere_plane(R, rng))
    print("tri_box / tri_tri overlap rate", tri_box_tri_tri(R, rng))
    print("config1 hit rate", config1(R))
    rng_tables()
    print("written to", OUT)


if __name__ == "__main__":
    main()
