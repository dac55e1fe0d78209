"""Scenes fed by RayBuilder's wire records render like scenes built directly: the Cornell scene (one
mesh per wall and sphere, the showcase material set) is laid out as material_struct_t and entry_t byte
images (RayBuilder.hpp:24-116), read by vkg_materials_from_wire / vkg_instances_from_wire into an
instanced scene, and rendered; the image equals the directly built instanced scene's bit for bit."""
import math

import numpy as np
import pytest
import torch

from scene_helpers import split_cornell
from test_wire import ENTRY_T, MATERIAL_STRUCT_T
from vierkant_gb300 import geometry
from vierkant_gb300.pathtracer import InstancedScene, PBRPathTracer, cornell_lights, procedural_sky, sun_direction
from vierkant_gb300.wire import instances_from_wire, materials_from_wire

pytestmark = pytest.mark.gpu


def wire_materials(mats):
    w = np.zeros(len(mats), MATERIAL_STRUCT_T)
    w["color"][:, :3] = mats["base_color"]
    w["color"][:, 3] = mats["alpha"]
    w["blend_mode"] = mats["blend_mode"]
    w["alpha_cutoff"] = mats["alpha_cutoff"]
    w["emission"][:, :3] = mats["emission"]
    w["emission"][:, 3] = 1.0
    for theirs, ours in (("metalness", "metalness"), ("roughness", "roughness"), ("transmission", "transmission"),
                         ("null_surface", "null_surface"), ("attenuation_color", "attenuation_color"),
                         ("attenuation_distance", "attenuation_distance"), ("ior", "ior"),
                         ("clearcoat_factor", "clearcoat"), ("clearcoat_roughness_factor", "clearcoat_roughness"),
                         ("sheen_roughness", "sheen_roughness"), ("iridescence_strength", "iridescence"),
                         ("iridescence_ior", "iridescence_ior"), ("two_sided", "twosided"),
                         ("phase_asymmetry_g", "phase_g"), ("scatter_factor", "scatter_factor"),
                         ("scatter_color", "scatter_color"), ("diffuse_transmission", "diffuse_transmission"),
                         ("diffuse_transmission_color", "diffuse_transmission_color")):
        w[theirs] = mats[ours]
    w["sheen_color"][:, :3] = mats["sheen_color"]
    w["iridescence_thickness_range"][:, 0] = 100.0
    w["iridescence_thickness_range"][:, 1] = mats["iridescence_thickness"]
    return w


def quat_matrix(q):
    """the rotation matrix of a unit quaternion (x, y, z, w), evaluated in double and rounded to float"""
    x, y, z, w = (float(v) for v in np.float32(q))
    R = [[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
         [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
         [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]]
    return np.float32(R)


def test_wire_scene_renders_like_the_direct_scene(ctx):
    sc = geometry.cornell_scene(0x5EED, 2, 16, 16)
    mats = geometry.showcase_materials(sc["materials"])
    meshes, inst = split_cornell(sc)
    # entry_t records: walls at identity, spheres turned about their own axis through the origin by
    # multiples of 30 degrees about z, translated by exact offsets
    e = np.zeros(len(inst), ENTRY_T)
    for k in range(len(inst)):
        ang = math.radians(30 * (k % 5)) if k >= 5 else 0.0
        q = np.float32([0.0, 0.0, math.sin(ang / 2), math.cos(ang / 2)])
        t = np.float32([0.0, 0.0, -0.125 * (k % 3)]) if k >= 5 else np.zeros(3, np.float32)
        e["transform"]["translation"][k] = t
        e["transform"]["rotation"][k] = q
        e["transform"]["scale"][k] = 1.0
        e["material_index"][k] = inst[k]["material"]
        e["buffer_index"][k] = inst[k]["blas"]
        R = quat_matrix(q)
        inst[k]["transform"] = np.concatenate([R, t[:, None]], axis=1).reshape(-1)
    wm, dropped = materials_from_wire(wire_materials(mats).tobytes())
    wi, info = instances_from_wire(e.tobytes())
    assert dropped == 0
    fields = [f for f in mats.dtype.names if f != "pad"]
    for f in fields:
        assert np.array_equal(wm[f], mats[f]), f
    assert wi.tobytes() == inst.tobytes()

    env = procedural_sky(ctx, 512, 256, sun_direction(), 50.0, 0.02)
    tw = [(x, i, int(mats[inst[k]["material"]]["twosided"])) for k, (x, i, _) in enumerate(meshes)]
    wire = InstancedScene(ctx, tw, wi, wm, env)
    direct = InstancedScene(ctx, tw, inst, mats, env)
    for s_ in (wire, direct):
        s_.set_lights(cornell_lights())
    cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, 1280, 720)
    s = PBRPathTracer.default_settings()
    s.num_samples, s.max_trace_depth, s.rr_start_depth = 4, 8, 3
    for k, c in enumerate((400, 220, 480, 280)):
        s.crop[k] = c
    a = PBRPathTracer(ctx, seed=11, settings=s)
    b = PBRPathTracer(ctx, seed=11, settings=s)
    ia = a.render_scene(wire, cam).clone()
    ib = b.render_scene(direct, cam).clone()
    assert torch.equal(ia, ib), (ia - ib).abs().max().item()
    assert ia.sum() > 0 and a.statistics().extension_rays == b.statistics().extension_rays
    a.close()
    b.close()
    wire.close()
    direct.close()
