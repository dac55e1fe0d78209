"""Alpha-masked and blended materials in the radiance oracle (CPU only). The reference tests coverage
in its any-hit stages (raypipeline.slang:686-720, visibility_test.slang:45-87 and :131-152):

* masks whose coverage is 1 everywhere render bit for bit like the opaque scene (FP32 twin);
* spheres masked at alpha 0 render bit for bit like the scene without them (FP32 twin);
* a blended emitter of alpha a in front of another is seen by a fraction a of the paths, and a blended
  occluder lets 1 - a of a light through (FP64, one segment deep)."""
import math

import numpy as np
import pytest

import oracle
from alpha_scenes import (CROP, EYE, FOVY, HEIGHT, TARGET, UP, WIDTH, blend_quads, blend_shadow, blend_stack,
                          env_rgb, sun)
from vierkant_gb300._lib import BLEND_MASK

SUN_DIR = np.array([0.25, 0.6, 0.76])


def _cornell():
    sc = oracle.cornell_scene(0x5EED, 2, 8, 8)
    mats = oracle.cornell_materials(0x5EED, 2, 8)
    th = float(np.float32(math.tan(math.radians(45.0) / 2.0)))
    cam = oracle.camera((0, 0, 3.4), (0, 0, 0), (0, 1, 0), th, 320, 180)
    env = oracle.env_procedural(256, 128, SUN_DIR / np.linalg.norm(SUN_DIR), 50.0, 0.02)
    return sc, mats, cam, env


def _alias(weight):
    """an alias table over the environment's texel weights (Vose's method): the FP32 twin samples
    the environment through one"""
    n = len(weight)
    p = np.asarray(weight, np.float64) / np.sum(weight) * n
    prob, alias = np.ones(n, np.float32), np.arange(n, dtype=np.uint32)
    small, large = [i for i in range(n) if p[i] < 1.0], [i for i in range(n) if p[i] >= 1.0]
    while small and large:
        s, l_ = small.pop(), large.pop()
        prob[s], alias[s] = p[s], l_
        p[l_] += p[s] - 1.0
        (small if p[l_] < 1.0 else large).append(l_)
    return prob, alias


def _twin(sc, mats, cam, env, idx=None, tm=None):
    idx = sc["indices"] if idx is None else idx
    tm = sc["tri_material"] if tm is None else tm
    bvh = oracle.CpuBVH(sc["xyz"], idx, 4)
    w, _ = oracle.env_tables_fp64(env)
    prob, alias = _alias(w)
    img, _, rays = oracle.pt_render(False, sc["xyz"], idx, tm, mats, bvh, env, cam, 4, seed=21, crop=(100, 40, 96, 96),
                                    alias_prob=prob, alias=alias, weight=w)
    return img, rays


def test_full_coverage_masks_render_like_opaque():
    sc, mats, cam, env = _cornell()
    plain, r0 = _twin(sc, mats, cam, env)
    m = mats.copy()
    m["blend_mode"] = BLEND_MASK
    m["alpha"] = 1.0
    m["alpha_cutoff"] = 0.5
    masked, r1 = _twin(sc, m, cam, env)
    assert np.array_equal(plain, masked)
    assert r0 == r1


def test_zero_coverage_masks_render_like_removed_geometry():
    sc, mats, cam, env = _cornell()
    m = mats.copy()
    m["alpha"] = 1.0
    m["alpha_cutoff"] = 0.5
    gone = np.arange(7, 11)  # the last four spheres: their triangles end the index list
    m["blend_mode"][gone] = BLEND_MASK
    m["alpha"][gone] = 0.25
    masked, _ = _twin(sc, m, cam, env)
    keep = int(np.argmax(np.isin(sc["tri_material"], gone)))
    assert np.all(np.isin(sc["tri_material"][keep:], gone))
    removed, _ = _twin(sc, mats, cam, env, sc["indices"][:keep], sc["tri_material"][:keep])
    assert np.array_equal(masked, removed)
    full, _ = _twin(sc, mats, cam, env)
    assert not np.array_equal(full, removed)


def _camera():
    th = float(np.float32(math.tan(math.radians(FOVY) / 2.0)))
    return oracle.camera(EYE, TARGET, UP, th, WIDTH, HEIGHT)


@pytest.mark.parametrize("alpha", [0.3, 0.75])
def test_blended_emitter_is_seen_by_alpha_of_the_paths(alpha):
    xyz, idx, tm, m = blend_quads(alpha)
    bvh = oracle.CpuBVH(xyz, idx, 4)
    img, _, _ = oracle.pt_render(True, xyz, idx, tm, m, bvh, env_rgb(), _camera(), 256, seed=5, max_depth=1,
                                 crop=CROP)
    mean = img.mean(axis=(0, 1))
    n = CROP[2] * CROP[3] * 256
    tol = 5.0 * math.sqrt(alpha * (1 - alpha) / n) + 1e-3
    assert abs(mean[0] - alpha) < tol, mean
    assert abs(mean[2] - (1 - alpha)) < tol, mean


def test_blended_occluder_passes_one_minus_alpha_of_the_light():
    alpha = 0.35
    cam = _camera()
    out = []
    for occ in (False, True):
        xyz, idx, tm, m = blend_shadow(alpha, occ)
        bvh = oracle.CpuBVH(xyz, idx, 4)
        img, _, _ = oracle.pt_render(True, xyz, idx, tm, m, bvh, env_rgb(), cam, 128, seed=9, max_depth=1, crop=CROP,
                                     lights=sun().astype(oracle.LIGHT_DTYPE))
        out.append(img.mean())
    open_, shaded = out
    assert open_ > 0.05
    n = CROP[2] * CROP[3] * 128
    assert abs(shaded / open_ - (1 - alpha)) < 5.0 * math.sqrt(alpha * (1 - alpha) / n) + 2e-3, (open_, shaded)


def test_blended_candidates_of_a_ray_share_one_uniform():
    alpha = 0.4
    xyz, idx, tm, m = blend_stack(alpha)
    bvh = oracle.CpuBVH(xyz, idx, 4)
    img, _, _ = oracle.pt_render(True, xyz, idx, tm, m, bvh, env_rgb(), _camera(), 256, seed=3, max_depth=1,
                                 crop=CROP)
    mean = img.mean(axis=(0, 1))
    n = CROP[2] * CROP[3] * 256
    tol = 5.0 * math.sqrt(alpha * (1 - alpha) / n) + 1e-3
    assert abs(mean[0] - alpha) < tol and abs(mean[2] - (1 - alpha)) < tol, mean
    assert mean[1] < 1e-3, mean  # independent uniforms would show green at a (1 - a) = 0.24
