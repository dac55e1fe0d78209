"""RayBuilder wire records (host only, no GPU): byte images of RayBuilder::material_struct_t and
RayBuilder::entry_t (RayBuilder.hpp:24-116), laid out here from the reference's struct definitions
with glm's default packing and cross-checked against the shader twins' std430 layout
(ray/types.slang:17-32, :64-110), read by vkg_materials_from_wire / vkg_instances_from_wire."""
import math

import numpy as np
import pytest

from vierkant_gb300.wire import WIRE_ENTRY_BYTES, WIRE_MATERIAL_BYTES, instances_from_wire, materials_from_wire

# RayBuilder::material_struct_t, field by field in declaration order (vec4 16 B, vec3 12 B, vec2 8 B)
MATERIAL_STRUCT_T = np.dtype([
    ("color", "<f4", 4), ("emission", "<f4", 4), ("metalness", "<f4"), ("roughness", "<f4"),
    ("transmission", "<f4"), ("null_surface", "<u4"), ("attenuation_color", "<f4", 3),
    ("attenuation_distance", "<f4"), ("ior", "<f4"), ("clearcoat_factor", "<f4"),
    ("clearcoat_roughness_factor", "<f4"), ("sheen_roughness", "<f4"), ("sheen_color", "<f4", 4),
    ("iridescence_strength", "<f4"), ("iridescence_ior", "<f4"), ("iridescence_thickness_range", "<f4", 2),
    ("albedo_index", "<u4"), ("normalmap_index", "<u4"), ("emission_index", "<u4"),
    ("ao_rough_metal_index", "<u4"), ("transmission_index", "<u4"), ("texture_type_flags", "<u4"),
    ("blend_mode", "<u4"), ("alpha_cutoff", "<f4"), ("two_sided", "<u4"), ("phase_asymmetry_g", "<f4"),
    ("scatter_factor", "<f4"), ("dispersion", "<f4"), ("scatter_color", "<f4", 3),
    ("diffuse_transmission", "<f4"), ("diffuse_transmission_color", "<f4", 3),
    ("diffuse_transmission_index", "<u4"), ("diffuse_transmission_color_index", "<u4"), ("pad", "<u4", 3)])

# RayBuilder::entry_t: mat4, two transform_t (translation vec3, rotation quat x y z w, scale vec3), AABB
TRANSFORM_T = np.dtype([("translation", "<f4", 3), ("rotation", "<f4", 4), ("scale", "<f4", 3)])
ENTRY_T = np.dtype([("texture_matrix", "<f4", 16), ("transform", TRANSFORM_T), ("inv_transform", TRANSFORM_T),
                    ("aabb_min", "<f4", 3), ("aabb_max", "<f4", 3), ("material_index", "<u4"),
                    ("vertex_offset", "<i4"), ("base_index", "<u4"), ("buffer_index", "<u4"), ("pad", "<u4", 2)])


def test_layouts_match_std430():
    """sizes and the offsets where std430 would align a vec3 / vec4 / vec2 member (16 / 16 / 8 bytes):
    the C++ packing puts every such member on its std430 boundary, so one byte image serves both"""
    assert MATERIAL_STRUCT_T.itemsize == WIRE_MATERIAL_BYTES == 208
    assert ENTRY_T.itemsize == WIRE_ENTRY_BYTES == 192
    f = MATERIAL_STRUCT_T.fields
    for name in ("color", "emission", "attenuation_color", "sheen_color", "scatter_color",
                 "diffuse_transmission_color"):
        assert f[name][1] % 16 == 0, name
    assert f["iridescence_thickness_range"][1] % 8 == 0
    assert ENTRY_T.fields["transform"][1] == 64 and ENTRY_T.fields["material_index"][1] == 168


def test_materials_from_wire():
    rng = np.random.default_rng(3)
    w = np.zeros(5, MATERIAL_STRUCT_T)
    for name in MATERIAL_STRUCT_T.names:
        if name == "pad":
            continue
        shape = w[name].shape
        w[name] = rng.random(shape).astype(np.float32) if w[name].dtype.kind == "f" else 0
    w["dispersion"] = 0.0
    w["null_surface"][1] = 1
    w["two_sided"][2] = 1
    w["texture_type_flags"][3] = 0x1 | 0x2 | 0x4 | 0x8 | 0x40 | 0x8000 | 0x10000
    w["albedo_index"][3], w["normalmap_index"][3], w["emission_index"][3] = 7, 8, 9
    w["ao_rough_metal_index"][3], w["transmission_index"][3] = 10, 11
    w["diffuse_transmission_index"][3], w["diffuse_transmission_color_index"][3] = 12, 13
    w["albedo_index"][2] = 5  # an index without its flag: no texture
    w["texture_type_flags"][1] = 0x80  # a clearcoat texture: not sampled, counted as dropped
    w["dispersion"][4] = 0.2
    w["blend_mode"] = (0, 2, 1, 0, 7)  # opaque, mask, blend; 7 is no BlendMode: opaque, counted as dropped
    m, dropped = materials_from_wire(w.tobytes())
    assert dropped == 2  # the clearcoat texture and the unknown blend mode; the rest is read
    assert list(m["blend_mode"]) == [0, 2, 1, 0, 0]
    assert np.array_equal(m["alpha"], w["color"][:, 3]) and np.array_equal(m["alpha_cutoff"], w["alpha_cutoff"])
    NO = 0xFFFFFFFF
    assert [int(m[f][3]) for f in ("tex_color", "tex_normal", "tex_emission", "tex_ao_rough_metal",
                                   "tex_transmission", "tex_diffuse_transmission",
                                   "tex_diffuse_transmission_color")] == [7, 8, 9, 10, 11, 12, 13]
    assert int(m["tex_color"][2]) == NO and int(m["tex_normal"][1]) == NO and int(m["tex_color"][0]) == NO
    assert np.array_equal(m["dispersion"], w["dispersion"])
    assert np.array_equal(m["base_color"], w["color"][:, :3])
    assert np.allclose(m["emission"], w["emission"][:, :3] * w["emission"][:, 3:4], rtol=1e-7, atol=0)
    for ours, theirs in (("metalness", "metalness"), ("roughness", "roughness"), ("transmission", "transmission"),
                         ("attenuation_distance", "attenuation_distance"), ("ior", "ior"),
                         ("clearcoat", "clearcoat_factor"), ("clearcoat_roughness", "clearcoat_roughness_factor"),
                         ("sheen_roughness", "sheen_roughness"), ("iridescence", "iridescence_strength"),
                         ("iridescence_ior", "iridescence_ior"), ("phase_g", "phase_asymmetry_g"),
                         ("scatter_factor", "scatter_factor"), ("diffuse_transmission", "diffuse_transmission")):
        assert np.array_equal(m[ours], w[theirs]), ours
    for ours, theirs in (("attenuation_color", "attenuation_color"), ("scatter_color", "scatter_color"),
                         ("diffuse_transmission_color", "diffuse_transmission_color")):
        assert np.array_equal(m[ours], w[theirs]), ours
    assert np.array_equal(m["sheen_color"], w["sheen_color"][:, :3])
    assert np.array_equal(m["iridescence_thickness"], w["iridescence_thickness_range"][:, 1])
    assert list(m["null_surface"]) == [0, 1, 0, 0, 0] and list(m["twosided"]) == [0, 0, 1, 0, 0]


def _quat(axis, angle):
    a = np.asarray(axis, np.float64) / np.linalg.norm(axis)
    return np.array([*(a * math.sin(angle / 2)), math.cos(angle / 2)])


def _apply_transform(t, v):
    """the shader's apply_transform (utils/transform.slang:17-24): rotate_quat(q, v * s) + t"""
    q = t["rotation"].astype(np.float64)
    v = v * t["scale"].astype(np.float64)
    qv = q[:3]
    return v + 2.0 * np.cross(qv, np.cross(qv, v) + q[3] * v) + t["translation"]


def test_instances_from_wire():
    rng = np.random.default_rng(9)
    e = np.zeros(6, ENTRY_T)
    for k in range(6):
        e["transform"]["translation"][k] = rng.uniform(-5, 5, 3)
        e["transform"]["rotation"][k] = _quat(rng.normal(size=3), rng.uniform(0, 2 * math.pi))
        e["transform"]["scale"][k] = rng.uniform(0.5, 2, 3)
        e["aabb_min"][k], e["aabb_max"][k] = -rng.random(3), rng.random(3)
    e["material_index"] = np.arange(6) * 3
    e["vertex_offset"] = [0, -4, 7, 100, 0, 3]
    e["base_index"] = np.arange(6) * 12
    e["buffer_index"] = [0, 1, 1, 2, 0, 5]
    e["texture_matrix"] = np.eye(4, dtype=np.float32).reshape(-1)
    # entry 2: a glm::mat4 (column-major) scaling u by 2, v by 3 and offsetting by (0.5, -1)
    tm = np.eye(4, dtype=np.float32)
    tm[0, 0], tm[1, 1], tm[0, 3], tm[1, 3] = 2.0, 3.0, 0.5, -1.0
    e["texture_matrix"][2] = tm.T.reshape(-1)  # column-major storage
    inst, info = instances_from_wire(e)
    assert list(info["has_uv_transform"]) == [0, 0, 1, 0, 0, 0]
    assert np.array_equal(info["uv_transform"][2], [2.0, 0.0, 0.5, 0.0, 3.0, -1.0])
    assert np.array_equal(info["uv_transform"][0], [1, 0, 0, 0, 1, 0])
    assert list(inst["blas"]) == list(e["buffer_index"]) and list(inst["material"]) == list(e["material_index"])
    assert list(info["vertex_offset"]) == list(e["vertex_offset"]) and list(info["base_index"]) == list(e["base_index"])
    assert np.array_equal(info["aabb_min"], e["aabb_min"]) and np.array_equal(info["aabb_max"], e["aabb_max"])
    pts = rng.normal(size=(50, 3))
    for k in range(6):
        M = inst["transform"][k].reshape(3, 4).astype(np.float64)
        got = pts @ M[:, :3].T + M[:, 3]
        want = np.array([_apply_transform(e["transform"][k], p) for p in pts])
        assert np.allclose(got, want, rtol=0, atol=2e-5), k


def test_bad_arguments():
    with pytest.raises(ValueError):
        materials_from_wire(bytes(100))
    with pytest.raises(ValueError):
        instances_from_wire(bytes(191))
    m, d = materials_from_wire(b"")
    assert len(m) == 0 and d == 0
