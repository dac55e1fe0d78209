"""glTF ingestion on the GPU: the Cornell scene written as a glTF asset (one node per wall quad and
sphere, the materials as pbrMetallicRoughness factors, a KHR_lights_punctual spot) loads into an
instanced scene that renders bit for bit like the same scene built directly; packed_vertex_t
positions (24-byte records) build the same scene as packed xyz."""
import numpy as np
import pytest
import torch

from gltf_writer import write
from scene_helpers import split_cornell
from vierkant_gb300 import geometry
from vierkant_gb300.gltf import load_gltf, scene_from_gltf
from vierkant_gb300.pathtracer import (LIGHT_SPOT, PACKED_VERTEX_DTYPE, InstancedScene, PBRPathTracer,
                                       procedural_sky, sun_direction)

pytestmark = pytest.mark.gpu


def settings(spp, crop):
    s = PBRPathTracer.default_settings()
    s.num_samples, s.max_trace_depth, s.rr_start_depth = spp, 6, 3
    for k in range(4):
        s.crop[k] = crop[k]
    return s


def test_gltf_cornell_renders_like_the_direct_scene(ctx, tmp_path):
    sc = geometry.cornell_scene(0x5EED, 2, 16, 16)
    mats = sc["materials"]
    meshes, inst = split_cornell(sc)
    gm = [[(x, i, int(inst[k]["material"]), None)] for k, (x, i, _) in enumerate(meshes)]
    gmats = [{"pbrMetallicRoughness": {"baseColorFactor": [float(c) for c in m["base_color"]] + [1.0],
                                       "metallicFactor": float(m["metalness"]),
                                       "roughnessFactor": float(m["roughness"])},
              "doubleSided": bool(m["twosided"])} for m in mats]
    spot = {"type": "spot", "color": [1.0, 0.9, 0.8], "intensity": 4.0,
            "spot": {"innerConeAngle": 0.3, "outerConeAngle": 0.6}}
    q = [float(np.sin(-np.pi / 4)), 0.0, 0.0, float(np.cos(-np.pi / 4))]  # pointing down
    nodes = [dict(mesh=k) for k in range(len(meshes))] + [dict(light=0, rotation=q, translation=[0.0, 0.9, 0.0])]
    path = tmp_path / "cornell.glb"
    write(path, gm, nodes, list(range(len(nodes))), materials=gmats, lights=[spot], mode="glb")
    a = load_gltf(str(path))
    assert len(a["meshes"]) == len(meshes) and len(a["instances"]) == len(meshes) and len(a["lights"]) == 1
    for m_ref, m_g in zip(mats, a["materials"]):
        for f in ("base_color", "roughness", "metalness", "twosided"):
            assert np.array_equal(m_ref[f], m_g[f]), f
    env = procedural_sky(ctx, 512, 256, sun_direction(), 50.0, 0.02)
    loaded = scene_from_gltf(ctx, str(path), env)
    direct = InstancedScene(ctx, [(x, i, int(mats[inst[k]["material"]]["twosided"])) for k, (x, i, _) in
                                  enumerate(meshes)], inst, mats, env)
    direct.set_lights(a["lights"])
    assert a["lights"][0]["type"] == LIGHT_SPOT and np.allclose(a["lights"][0]["direction"], (0, -1, 0), atol=1e-6)
    cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, 1280, 720)
    for crop in ((560, 300, 64, 64), (0, 0, 48, 32)):
        p = PBRPathTracer(ctx, seed=4, settings=settings(4, crop))
        q_ = PBRPathTracer(ctx, seed=4, settings=settings(4, crop))
        ia = p.render_scene(loaded, cam).clone()
        ib = q_.render_scene(direct, cam).clone()
        assert torch.equal(ia, ib), (ia - ib).abs().max().item()
        assert ia.sum() > 0
        p.close()
        q_.close()
    loaded.close()
    direct.close()


def test_packed_vertex_records(ctx):
    sc = geometry.cornell_scene(0x5EED, 2, 8, 8)
    meshes, inst = split_cornell(sc, tess=8)
    packed = []
    for x, i, t in meshes:
        rec = np.zeros(len(x), PACKED_VERTEX_DTYPE)
        rec["position"] = x
        rec["normal"] = 0x7FFF7FFF
        rec["texcoord"] = 0.5
        packed.append((rec, i, t))
    env = procedural_sky(ctx, 256, 128, sun_direction(), 50.0, 0.02)
    a = InstancedScene(ctx, meshes, inst, sc["materials"], env)
    b = InstancedScene(ctx, packed, inst, sc["materials"], env)
    cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, 1280, 720)
    p = PBRPathTracer(ctx, seed=2, settings=settings(2, (600, 300, 64, 64)))
    q_ = PBRPathTracer(ctx, seed=2, settings=settings(2, (600, 300, 64, 64)))
    assert torch.equal(p.render_scene(a, cam), q_.render_scene(b, cam))
    assert a.bounds() == b.bounds()
    p.close()
    q_.close()
    a.close()
    b.close()
