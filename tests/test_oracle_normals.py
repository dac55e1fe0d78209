"""Vertex normals in the radiance oracle (CPU only): with each vertex carrying its triangle's face
normal the FP64 oracle renders the flat-shaded image (the plumbing interpolates, moves and turns the
normal like the face normal), and sphere normals pointing away from the centres change the image."""
import math

import numpy as np

import oracle
from vierkant_gb300.geometry import cornell_vertex_normals

SUN = np.array([0.2962, 0.5, 0.8138], np.float32)


def _scene():
    sc = oracle.cornell_scene(0x5EED, 2, 8, 8)
    mats = oracle.cornell_materials(0x5EED, 2, 8)
    th = float(np.float32(math.tan(math.radians(45.0) / 2.0)))
    cam = oracle.camera((0, 0, 3.4), (0, 0, 0), (0, 1, 0), th, 320, 180)
    env = oracle.env_procedural(256, 128, SUN)
    return sc, mats, cam, env


def test_face_normals_as_vertex_normals_render_the_flat_image():
    sc, mats, cam, env = _scene()
    idx = np.asarray(sc["indices"], np.int64)
    xyz = np.ascontiguousarray(np.asarray(sc["xyz"], np.float32)[idx.reshape(-1)])  # unshared vertices
    iu = np.arange(len(xyz), dtype=np.uint32).reshape(-1, 3)
    e1 = xyz[1::3].astype(np.float64) - xyz[0::3]
    e2 = xyz[2::3].astype(np.float64) - xyz[0::3]
    fn = np.cross(e1, e2)
    fn /= np.linalg.norm(fn, axis=1, keepdims=True)
    nrm = np.repeat(fn, 3, axis=0).astype(np.float32)
    bvh = oracle.CpuBVH(xyz, iu, 4)
    crop = (120, 60, 48, 48)
    flat, _, r0 = oracle.pt_render(True, xyz, iu, sc["tri_material"], mats, bvh, env, cam, 8, crop=crop)
    smooth, _, r1 = oracle.pt_render(True, xyz, iu, sc["tri_material"], mats, bvh, env, cam, 8, crop=crop,
                                     normals=nrm)
    assert r0 == r1
    assert np.max(np.abs(smooth - flat) / np.maximum(np.abs(flat), 1e-3)) < 1e-5


def test_sphere_normals_change_the_image():
    sc, mats, cam, env = _scene()
    bvh = oracle.CpuBVH(sc["xyz"], sc["indices"], 4)
    crop = (120, 60, 48, 48)
    flat, _, _ = oracle.pt_render(True, sc["xyz"], sc["indices"], sc["tri_material"], mats, bvh, env, cam, 8,
                                  crop=crop)
    smooth, _, _ = oracle.pt_render(True, sc["xyz"], sc["indices"], sc["tri_material"], mats, bvh, env, cam, 8,
                                    crop=crop, normals=cornell_vertex_normals(sc))
    assert np.abs(smooth - flat).mean() > 1e-3 * np.abs(flat).mean()
