"""Small scenes with a known answer for alpha-blended materials, shared by the oracle and GPU tests.

* blend_quads(a): a blended emitter (red, alpha a) in front of an opaque one (blue), both facing the
  camera; traced one segment deep a path sees red with probability a: radiance (a, 0, 1 - a).
* blend_shadow(a): a white floor lit by a directional light whose shadow rays cross a blended quad
  (alpha a) off screen; one segment deep the floor gets 1 - a of its unshadowed light.
Both sit in a near-black constant environment (1e-4), so environment light adds no more than 1e-4.
"""
import math

import numpy as np

from vierkant_gb300 import geometry
from vierkant_gb300._lib import BLEND_BLEND
from vierkant_gb300.pathtracer import LIGHT_DIRECTIONAL, LIGHT_DTYPE

EYE, TARGET, UP, FOVY = (0.0, 0.0, 3.4), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 45.0
WIDTH, HEIGHT = 256, 256
CROP = (112, 112, 32, 32)


def _quad(x0, x1, y0, y1, z):
    """a quad in the plane z facing +z (the winding makes e1 x e2 point along +z)"""
    return np.array([[x0, y0, z], [x1, y0, z], [x1, y1, z], [x0, y1, z]], np.float32)


def env_rgb():
    return np.full((32, 64, 3), 1e-4, np.float32)


def blend_quads(alpha: float):
    xyz = np.concatenate([_quad(-1, 1, -1, 1, 0.5), _quad(-2, 2, -2, 2, -0.5)])
    idx = np.array([[0, 1, 2], [0, 2, 3], [4, 5, 6], [4, 6, 7]], np.uint32)
    tm = np.array([0, 0, 1, 1], np.uint32)
    m = geometry.default_materials(2)
    m["base_color"] = 0.0
    m["twosided"] = 1
    m["emission"][0] = (1.0, 0.0, 0.0)
    m["emission"][1] = (0.0, 0.0, 1.0)
    m["blend_mode"][0] = BLEND_BLEND
    m["alpha"][0] = alpha
    return xyz, idx, tm, m


def blend_stack(alpha: float):
    """two blended emitters of the same alpha (red in front, green behind it) before an opaque blue one:
    the reference's any_hit compares every candidate of a ray with the same uniform, so a ray that
    passes the red one passes the green one too: radiance (a, 0, 1 - a), where independent uniforms per
    candidate would give (a, a (1 - a), (1 - a)^2)"""
    xyz = np.concatenate([_quad(-1, 1, -1, 1, 0.5), _quad(-1.5, 1.5, -1.5, 1.5, 0.0), _quad(-2, 2, -2, 2, -0.5)])
    idx = np.array([[0, 1, 2], [0, 2, 3], [4, 5, 6], [4, 6, 7], [8, 9, 10], [8, 10, 11]], np.uint32)
    tm = np.array([0, 0, 1, 1, 2, 2], np.uint32)
    m = geometry.default_materials(3)
    m["base_color"] = 0.0
    m["twosided"] = 1
    m["emission"][0] = (1.0, 0.0, 0.0)
    m["emission"][1] = (0.0, 1.0, 0.0)
    m["emission"][2] = (0.0, 0.0, 1.0)
    m["blend_mode"][:2] = BLEND_BLEND
    m["alpha"][:2] = alpha
    return xyz, idx, tm, m


def blend_shadow(alpha: float, with_occluder: bool = True):
    floor = _quad(-1, 1, -1, 1, -0.5)
    # the occluder: the plane x = 1.5, y in [-2, 2], z in [-1.5, 3]
    occ = np.array([[1.5, -2, -1.5], [1.5, -2, 3.0], [1.5, 2, 3.0], [1.5, 2, -1.5]], np.float32)
    xyz = np.concatenate([floor, occ]) if with_occluder else floor
    idx = np.array([[0, 1, 2], [0, 2, 3], [4, 5, 6], [4, 6, 7]], np.uint32)[: 4 if with_occluder else 2]
    tm = np.array([0, 0, 1, 1], np.uint32)[: len(idx)]
    m = geometry.default_materials(2)
    m["base_color"][0] = (0.8, 0.8, 0.8)
    m["base_color"][1] = (0.5, 0.5, 0.5)
    m["twosided"] = 1
    m["blend_mode"][1] = BLEND_BLEND
    m["alpha"][1] = alpha
    return xyz, idx, tm, m


def sun():
    """a directional light from +x +z (propagating along (-1, 0, -1) / sqrt 2)"""
    L = np.zeros(1, LIGHT_DTYPE)
    L[0]["type"] = LIGHT_DIRECTIONAL
    L[0]["color"] = (1.0, 1.0, 1.0)
    L[0]["intensity"] = 2.0
    L[0]["direction"] = np.array([-1.0, 0.0, -1.0]) / math.sqrt(2.0)
    L[0]["range"] = np.inf
    L[0]["spot_angle_scale"] = 1.0
    return L
