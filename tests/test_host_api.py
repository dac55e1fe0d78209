"""The product's host-side API (libvkg scalar intersection functions and geometry generators) is
bit-identical to the reference (golden fixtures made from its own compiled code) and to the oracle."""
import ctypes as C

import numpy as np

import oracle
from vierkant_gb300 import _lib, geometry
from vierkant_gb300._lib import vkg_ray_intersection, vkg_ray_triangle_intersection


def P(a):
    return np.ascontiguousarray(a).ctypes.data_as(C.c_void_p)


def test_ray_triangle_golden(golden):
    g = golden("ray_triangle")
    L = _lib.lib()
    for i in range(len(g["type"])):
        r = vkg_ray_triangle_intersection()
        assert L.vkg_intersect_ray_triangle(P(g["o"][i]), P(g["d"][i]), P(g["tri"][i]), C.byref(r)) == 0
        assert r.type == g["type"][i], i
        if r.type:
            assert np.float32([r.distance, r.u, r.v]).tobytes() == g["tuv"][i].tobytes(), i


def test_ray_aabb_golden(golden):
    g = golden("ray_aabb")
    L = _lib.lib()
    for i in range(len(g["type"])):
        r = vkg_ray_intersection()
        L.vkg_intersect_ray_aabb(P(g["o"][i]), P(g["d"][i]), P(g["lo"][i]), P(g["hi"][i]), C.byref(r))
        assert r.type == g["type"][i]
        if r.type:
            assert np.float32(r.distance).tobytes() == g["t"][i].tobytes()


def test_ray_obb_identity_equals_aabb(golden):
    g = golden("ray_aabb")
    L = _lib.lib()
    axes = np.eye(3, dtype=np.float32).reshape(-1)
    for i in range(0, len(g["type"]), 3):
        c = ((g["lo"][i] + g["hi"][i]) / np.float32(2)).astype(np.float32)
        h = ((g["hi"][i] - g["lo"][i]) / np.float32(2)).astype(np.float32)
        r = vkg_ray_intersection()
        L.vkg_intersect_ray_obb(P(g["o"][i]), P(g["d"][i]), P(c), P(axes), P(h), C.byref(r))
        assert r.type == g["type"][i]
        if r.type:
            assert np.float32(r.distance).tobytes() == g["t"][i].tobytes()


def test_ray_sphere_plane_golden(golden):
    L = _lib.lib()
    g = golden("ray_sphere")
    for i in range(len(g["type"])):
        r = vkg_ray_intersection()
        L.vkg_intersect_ray_sphere(P(g["o"][i]), P(g["d"][i]), P(g["c"][i]), C.c_float(g["r"][i]), C.byref(r))
        assert r.type == g["type"][i]
        if r.type:
            assert np.float32(r.distance).tobytes() == g["t"][i].tobytes()
    g = golden("ray_plane")
    for i in range(len(g["type"])):
        r = vkg_ray_intersection()
        L.vkg_intersect_ray_plane(P(g["o"][i]), P(g["d"][i]), P(g["plane"][i]), C.byref(r))
        assert r.type == g["type"][i]
        if r.type:
            assert np.float32(r.distance).tobytes() == g["t"][i].tobytes()


def test_triangle_box_and_triangle_triangle_golden(golden):
    L = _lib.lib()
    g = golden("tri_box")
    out = C.c_uint32()
    for i in range(len(g["overlap"])):
        L.vkg_intersect_triangle_aabb(P(g["tri"][i]), P(g["lo"][i]), P(g["hi"][i]), C.byref(out))
        assert out.value == g["overlap"][i], i
    g = golden("tri_tri")
    for i in range(len(g["overlap"])):
        L.vkg_intersect_triangle_triangle(P(g["a"][i]), P(g["b"][i]), C.byref(out))
        assert out.value == g["overlap"][i], i


def test_live_reference_random_overlap():
    R = oracle.ref()
    if R is None:
        import pytest
        pytest.skip("reference checkout not present here (fixtures cover this case)")
    L = _lib.lib()
    rng = np.random.default_rng(11)
    out = C.c_uint32()
    for i in range(20000):
        a = (rng.normal(size=9) * 0.7).astype(np.float32)
        b = (rng.normal(size=9) * 0.7).astype(np.float32)
        if i % 5 == 0:
            a[2::3] = 0.0
            b[2::3] = 0.0
        L.vkg_intersect_triangle_triangle(P(a), P(b), C.byref(out))
        assert out.value == R.vkref_triangle_triangle_overlap(P(a), P(b))
        lo = (rng.normal(size=3) * 0.5).astype(np.float32)
        hi = (lo + np.abs(rng.normal(size=3)).astype(np.float32)).astype(np.float32)
        L.vkg_intersect_triangle_aabb(P(a), P(lo), P(hi), C.byref(out))
        assert out.value == R.vkref_triangle_aabb_overlap(P(a), P(lo), P(hi))


def test_python_intersect_dispatch():
    from vierkant_gb300.intersection import AABB, INTERSECT, Ray, Sphere, Triangle, intersect
    r = intersect(Triangle((0, 0, 0), (1, 0, 0), (0, 1, 0)), Ray((0.25, 0.25, 1), (0, 0, -1)))
    assert r.type == INTERSECT and r.distance == 1.0 and r.u == 0.25 and r.v == 0.25
    assert intersect(Ray((0, 0, -5), (0, 0, 1)), AABB((-1, -1, -1), (1, 1, 1))).distance == 4.0
    assert intersect(Sphere((0, 0, 0), 1.0), Ray((0, 0, -5), (0, 0, 1))).distance == 4.0
    assert intersect(Triangle((0, 0, 0), (1, 0, 0), (0, 1, 0)), AABB((0.1, 0.1, -1), (0.2, 0.2, 1))) == 1


def test_icosphere_matches_oracle():
    a = geometry.icosphere(1.0, 5)
    b = oracle.icosphere(1.0, 5)
    assert a[0].tobytes() == b[0].tobytes() and a[1].tobytes() == b[1].tobytes()
    for tess in range(0, 4):
        a = geometry.icosphere(0.5, tess)
        b = oracle.icosphere(0.5, tess)
        assert a[0].tobytes() == b[0].tobytes() and a[1].tobytes() == b[1].tobytes()


def test_cornell_scene_matches_oracle():
    a = geometry.cornell_scene(0x5EED, 2, 64, 16)
    b = oracle.cornell_scene(0x5EED, 2, 64, 16)
    assert a["xyz"].shape == (110996, 3) and a["indices"].shape == (196618, 3)
    assert a["xyz"].tobytes() == b["xyz"].tobytes()
    assert a["indices"].tobytes() == b["indices"].tobytes()
    assert a["tri_material"].tobytes() == b["tri_material"].tobytes()
    sp = b["spheres"]
    for s in range(64):
        m = a["materials"][3 + s]
        assert np.float32(m["roughness"]) == np.float32(sp[s].roughness)
        assert np.float32(m["metalness"]) == np.float32(sp[s].metalness)
        assert np.array_equal(m["base_color"], np.float32(list(sp[s].base)))
        assert 0.1 <= sp[s].radius <= 0.4


def test_camera_lookat_matches_oracle():
    import math
    th = float(np.float32(math.tan(math.radians(45.0) / 2.0)))
    a = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, 1280, 720)
    b = oracle.camera((0, 0, 3.4), (0, 0, 0), (0, 1, 0), th, 1280, 720)
    assert bytes(a) == bytes(b)
