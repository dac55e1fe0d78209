"""The FP64 oracle's variance split (orc_pt_variance_split, oracle/nrc_bound.py): the first trace of
every sample is the plain estimator's path, a fork that no path reaches leaves no tail variance, and a
fork's tail variance never exceeds the plain variance beyond noise."""
import math

import numpy as np

import oracle
from oracle.nrc_bound import SUN_DIR

CROP = (944, 872, 12, 12)


def _scene():
    sc = oracle.cornell_scene(0x5EED, 2, 64, 16)
    mats = oracle.cornell_materials(0x5EED, 2, 64)
    th = float(np.float32(math.tan(math.radians(45.0) / 2.0)))
    cam = oracle.camera((0, 0, 3.4), (0, 0, 0), (0, 1, 0), th, 1920, 1080)
    env = oracle.env_procedural(256, 128, SUN_DIR)
    bvh = oracle.CpuBVH(sc["xyz"], sc["indices"], 2)
    return sc, mats, cam, env, bvh


def test_split_first_trace_is_the_plain_path_and_unreached_fork_is_empty():
    sc, mats, cam, env, bvh = _scene()
    out, rays = oracle.pt_variance_split(sc["xyz"], sc["indices"], sc["tri_material"], mats, bvh, env, cam, 8, 99,
                                         crop=CROP)
    img, sq, prays = oracle.pt_render(True, sc["xyz"], sc["indices"], sc["tri_material"], mats, bvh, env, cam, 8,
                                      crop=CROP)
    lum = 0.2126 * img[..., 0] + 0.7152 * img[..., 1] + 0.0722 * img[..., 2]
    assert np.allclose(out[..., 0], lum, rtol=1e-12, atol=1e-12)
    assert rays == prays
    assert np.all(out[..., 2] == 0) and np.all(out[..., 3] == 0)
    var = (sq - lum * lum) * 8 / 7
    assert np.allclose(out[..., 1], var, rtol=1e-9, atol=1e-9)


def test_split_tail_variance_is_part_of_the_plain_variance():
    sc, mats, cam, env, bvh = _scene()
    for fork in (0, 1, 2):
        out, _ = oracle.pt_variance_split(sc["xyz"], sc["indices"], sc["tri_material"], mats, bvh, env, cam, 96, fork,
                                          crop=CROP)
        vp, vt, reach = out[..., 1].sum(), out[..., 2].sum(), out[..., 3].mean()
        assert 0 < reach <= 1
        assert 0 <= vt <= 1.15 * vp, (fork, vt, vp)
    # later forks leave less of the variance in the tail
    t = [oracle.pt_variance_split(sc["xyz"], sc["indices"], sc["tri_material"], mats, bvh, env, cam, 96, f,
                                  crop=CROP)[0][..., 2].sum() for f in (0, 3)]
    assert t[1] < t[0]
