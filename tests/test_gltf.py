"""glTF 2.0 ingestion (vkg_gltf_*; host only, no GPU): the loader against assets written by
tests/gltf_writer.py — the three container forms, node hierarchies with matrix and TRS transforms
(checked against numpy compositions), uint16 / uint32 / absent indices, skipped non-triangle
primitives, materials with the KHR extensions, KHR_lights_punctual placement (convert_light), and
malformed inputs that must fail with a message."""
import json
import math

import numpy as np
import pytest

from gltf_writer import write
from vierkant_gb300.gltf import load_gltf
from vierkant_gb300.pathtracer import LIGHT_DIRECTIONAL, LIGHT_OMNI, LIGHT_SPOT

TRI = (np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32), np.array([[0, 1, 2]]))
QUAD = (np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], np.float32), np.array([[0, 1, 2], [0, 2, 3]]))


def quat(axis, angle):
    a = np.asarray(axis, np.float64) / np.linalg.norm(axis)
    s = math.sin(angle / 2)
    return [a[0] * s, a[1] * s, a[2] * s, math.cos(angle / 2)]


def trs_matrix(t=(0, 0, 0), q=(0, 0, 0, 1), s=(1, 1, 1)):
    x, y, z, w = q
    R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                  [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                  [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
    M = np.eye(4)
    M[:3, :3] = R * np.asarray(s)[None, :]
    M[:3, 3] = t
    return M


@pytest.mark.parametrize("mode", ["embedded", "external", "glb"])
def test_containers_and_hierarchy(tmp_path, mode):
    child_m = trs_matrix((0.5, -1, 2), quat((0, 1, 0), 0.3), (2, 2, 2))
    nodes = [dict(mesh=0, translation=[1, 2, 3], rotation=quat((1, 1, 0), 0.7), scale=[0.5, 0.5, 0.5],
                  children=[1, 2]),
             dict(mesh=1, matrix=list(child_m.T.reshape(-1))),   # column-major
             dict(children=[3], translation=[0, 0, -4]),
             dict(mesh=0)]
    path = tmp_path / ("a.glb" if mode == "glb" else "a.gltf")
    write(path, [[(*TRI, None, None)], [(*QUAD, None, None), (*TRI, None, None)]], nodes, [0], mode=mode)
    a = load_gltf(str(path))
    assert len(a["meshes"]) == 3  # mesh 0: one primitive, mesh 1: two
    assert np.array_equal(a["meshes"][0][0], TRI[0]) and np.array_equal(a["meshes"][1][1], QUAD[1])
    W0 = trs_matrix((1, 2, 3), quat((1, 1, 0), 0.7), (0.5, 0.5, 0.5))
    # breadth first: node 0, node 1 (two primitives), node 2 (no mesh), node 3
    expect = [(W0, 0), (W0 @ child_m, 1), (W0 @ child_m, 2), (W0 @ trs_matrix((0, 0, -4)), 0)]
    inst = a["instances"]
    assert len(inst) == len(expect)
    for k, (M, mesh) in enumerate(expect):
        assert inst[k]["blas"] == mesh and inst[k]["material"] == 0
        assert np.allclose(inst[k]["transform"].reshape(3, 4), M[:3, :], atol=1e-6)
    assert len(a["materials"]) == 1 and a["materials"][0]["ior"] == np.float32(1.5)  # the default material


@pytest.mark.parametrize("itype", [np.uint32, np.uint16, np.uint8])
def test_index_types_and_skipped_primitives(tmp_path, itype):
    path = tmp_path / "b.gltf"
    write(path, [[(*QUAD, None, None), (*QUAD, None, 1), (*TRI, 5, None), (TRI[0], None, None, None)]],
          [dict(mesh=0)], [0], index_type=itype)
    a = load_gltf(str(path))
    assert a["skipped_primitives"] == 1  # mode 1 (LINES) is left out
    assert len(a["meshes"]) == 3
    assert np.array_equal(a["meshes"][0][1], QUAD[1])
    assert np.array_equal(a["meshes"][1][1], TRI[1])
    assert np.array_equal(a["meshes"][2][1], [[0, 1, 2]])  # no indices: sequential
    assert list(a["instances"]["material"]) == [0, 0, 0]  # material 5 does not exist -> 0


def test_materials(tmp_path):
    mats = [
        {"pbrMetallicRoughness": {"baseColorFactor": [0.2, 0.4, 0.6, 1], "metallicFactor": 0.25,
                                  "roughnessFactor": 0.75},
         "emissiveFactor": [1, 0.5, 0.25], "doubleSided": True,
         "extensions": {"KHR_materials_emissive_strength": {"emissiveStrength": 4.0}}},
        {"extensions": {"KHR_materials_transmission": {"transmissionFactor": 0.9},
                        "KHR_materials_ior": {"ior": 1.33},
                        "KHR_materials_clearcoat": {"clearcoatFactor": 0.5, "clearcoatRoughnessFactor": 0.1},
                        "KHR_materials_sheen": {"sheenColorFactor": [0.1, 0.2, 0.3], "sheenRoughnessFactor": 0.4},
                        "KHR_materials_diffuse_transmission": {"diffuseTransmissionFactor": 0.3,
                                                               "diffuseTransmissionColorFactor": [1, 0.5, 0]},
                        "KHR_materials_iridescence": {"iridescenceFactor": 0.8, "iridescenceIOR": 1.4,
                                                      "iridescenceThicknessMinimum": 150,
                                                      "iridescenceThicknessMaximum": 520}}},
        {"pbrMetallicRoughness": {"baseColorFactor": [1, 1, 1, 0.3]}, "alphaMode": "MASK", "alphaCutoff": 0.25},
        {"alphaMode": "BLEND"},
        {},
    ]
    path = tmp_path / "m.gltf"
    write(path, [[(*TRI, 0, None), (*TRI, 1, None), (*TRI, None, None)]], [dict(mesh=0)], [0], materials=mats)
    a = load_gltf(str(path))
    m = a["materials"]
    assert np.allclose(m[0]["base_color"], (0.2, 0.4, 0.6)) and m[0]["metalness"] == np.float32(0.25)
    assert m[0]["roughness"] == np.float32(0.75) and m[0]["twosided"] == 1
    assert np.allclose(m[0]["emission"], (4.0, 2.0, 1.0))
    assert m[1]["transmission"] == np.float32(0.9) and m[1]["ior"] == np.float32(1.33)
    assert m[1]["clearcoat"] == np.float32(0.5) and m[1]["clearcoat_roughness"] == np.float32(0.1)
    assert np.allclose(m[1]["sheen_color"], (0.1, 0.2, 0.3)) and m[1]["sheen_roughness"] == np.float32(0.4)
    assert m[1]["diffuse_transmission"] == np.float32(0.3)
    assert np.allclose(m[1]["diffuse_transmission_color"], (1, 0.5, 0))
    assert m[1]["iridescence"] == np.float32(0.8) and m[1]["iridescence_ior"] == np.float32(1.4)
    assert m[1]["iridescence_thickness"] == 520  # the range's maximum, as the shader reads it
    assert m[0]["iridescence"] == 0 and m[0]["iridescence_ior"] == np.float32(1.3)
    # alphaMode / alphaCutoff / the base colour's alpha (the reference's gltf.cpp:323-326)
    assert (m[2]["blend_mode"], m[2]["alpha"], m[2]["alpha_cutoff"]) == (2, np.float32(0.3), np.float32(0.25))
    assert (m[3]["blend_mode"], m[3]["alpha"], m[3]["alpha_cutoff"]) == (1, 1.0, 0.5)
    # glTF defaults: metallic 1, roughness 1, white, opaque
    assert m[4]["metalness"] == 1 and m[4]["roughness"] == 1 and np.all(m[4]["base_color"] == 1)
    assert (m[4]["blend_mode"], m[4]["alpha"], m[4]["alpha_cutoff"]) == (0, 1.0, 0.5)
    assert list(a["instances"]["material"]) == [0, 1, 0]  # no material -> index 0, as the reference


def test_volume_and_scatter_materials(tmp_path):
    """KHR_materials_volume gives the attenuation colour / distance (absent distance: infinite, no
    medium); KHR_materials_scatter has a scatter factor defaulting to 0, the older
    KHR_materials_volume_scatter none (implicitly 1) (gltf.cpp:476-500, :634-657)"""
    mats = [
        {"extensions": {"KHR_materials_volume": {"thicknessFactor": 0.1, "attenuationColor": [0.5, 0.6, 0.7],
                                                 "attenuationDistance": 2.5},
                        "KHR_materials_scatter": {"multiscatterColorFactor": [0.9, 0.8, 0.7],
                                                  "scatterAnisotropy": 0.3, "scatterFactor": 0.6}}},
        {"extensions": {"KHR_materials_volume": {"attenuationColor": [0.2, 0.2, 0.2]},
                        "KHR_materials_scatter": {"multiscatterColorFactor": [0.1, 0.2, 0.3]}}},
        {"extensions": {"KHR_materials_volume": {"attenuationDistance": 0.5},
                        "KHR_materials_volume_scatter": {"scatterAnisotropy": -0.5}}},
    ]
    path = tmp_path / "v.gltf"
    write(path, [[(*TRI, 0, None), (*TRI, 1, None), (*TRI, 2, None)]], [dict(mesh=0)], [0], materials=mats)
    m = load_gltf(str(path))["materials"]
    assert np.allclose(m[0]["attenuation_color"], (0.5, 0.6, 0.7)) and m[0]["attenuation_distance"] == 2.5
    assert np.allclose(m[0]["scatter_color"], (0.9, 0.8, 0.7)) and np.isclose(m[0]["phase_g"], 0.3)
    assert np.isclose(m[0]["scatter_factor"], 0.6)
    assert np.isinf(m[1]["attenuation_distance"]) and m[1]["scatter_factor"] == 0  # unified: default 0
    assert np.allclose(m[1]["scatter_color"], (0.1, 0.2, 0.3))
    assert np.all(m[2]["attenuation_color"] == 1) and m[2]["attenuation_distance"] == 0.5
    assert m[2]["scatter_factor"] == 1 and np.isclose(m[2]["phase_g"], -0.5)  # legacy: implicit 1
    assert np.all(m[2]["scatter_color"] == 1)


def test_lights(tmp_path):
    lights = [{"type": "point", "color": [1, 0.5, 0.25], "intensity": 3.0, "range": 10.0},
              {"type": "spot", "intensity": 2.0, "spot": {"innerConeAngle": 0.2, "outerConeAngle": 0.5}},
              {"type": "directional"}]
    q = quat((1, 0, 0), -math.pi / 2)  # -z -> -y: a light pointing down
    nodes = [dict(light=0, translation=[1, 2, 3]), dict(light=1, rotation=q, translation=[0, 5, 0]),
             dict(light=2, rotation=quat((0, 1, 0), 0.4))]
    path = tmp_path / "l.gltf"
    write(path, [[(*TRI, None, None)]], nodes, [0, 1, 2], lights=lights)
    L = load_gltf(str(path))["lights"]
    assert len(L) == 3
    assert L[0]["type"] == LIGHT_OMNI and np.allclose(L[0]["position"], (1, 2, 3)) and L[0]["range"] == 10
    assert np.allclose(L[0]["color"], (1, 0.5, 0.25)) and L[0]["intensity"] == 3
    assert L[1]["type"] == LIGHT_SPOT and np.allclose(L[1]["direction"], (0, -1, 0), atol=1e-6)
    sc = 1.0 / max(0.001, math.cos(0.2) - math.cos(0.5))
    assert np.isclose(L[1]["spot_angle_scale"], sc, rtol=1e-5)
    assert np.isclose(L[1]["spot_angle_offset"], -math.cos(0.5) * sc, rtol=1e-5)
    assert L[2]["type"] == LIGHT_DIRECTIONAL and np.isinf(L[2]["range"])
    assert np.allclose(L[2]["direction"], (-math.sin(0.4), 0, -math.cos(0.4)), atol=1e-6)


@pytest.mark.parametrize("kind", ["missing", "notjson", "version", "oob_index", "short_buffer", "no_position",
                                  "bad_glb", "deep"])
def test_malformed_inputs_fail(tmp_path, kind):
    path = tmp_path / "x.gltf"
    if kind == "missing":
        path = tmp_path / "nope.gltf"
    elif kind == "notjson":
        path.write_text("{\"asset\": {\"version\": \"2.0\"},")
    elif kind == "version":
        path.write_text(json.dumps({"asset": {"version": "1.0"}}))
    elif kind == "oob_index":
        write(path, [[(TRI[0], np.array([[0, 1, 7]]), None, None)]], [dict(mesh=0)], [0])
    elif kind == "short_buffer":
        write(path, [[(*TRI, None, None)]], [dict(mesh=0)], [0])
        d = json.loads(path.read_text())
        d["buffers"][0]["byteLength"] += 100
        path.write_text(json.dumps(d))
    elif kind == "no_position":
        write(path, [[(*TRI, None, None)]], [dict(mesh=0)], [0])
        d = json.loads(path.read_text())
        d["meshes"][0]["primitives"][0]["attributes"] = {}
        path.write_text(json.dumps(d))
    elif kind == "bad_glb":
        path = tmp_path / "x.glb"
        path.write_bytes(b"glTF" + (2).to_bytes(4, "little") + (10 ** 6).to_bytes(4, "little"))
    elif kind == "deep":
        path.write_text("[" * 5000 + "]" * 5000)
    with pytest.raises(ValueError):
        load_gltf(str(path))


def test_vertex_normals(tmp_path):
    """NORMAL attributes are read per primitive (None without one); a NORMAL that is not VEC3 fails"""
    n_quad = np.array([[0, 0, 1], [0, 0.6, 0.8], [0.6, 0, 0.8], [0, 0, 1]], np.float32)
    path = tmp_path / "n.gltf"
    write(path, [[(*QUAD, None, None, n_quad), (*TRI, None, None)]], [dict(mesh=0)], [0])
    a = load_gltf(str(path))
    assert np.array_equal(a["normals"][0], n_quad)
    assert a["normals"][1] is None
    bad = tmp_path / "bad.gltf"
    write(bad, [[(*TRI, None, None, np.zeros((3, 2), np.float32))]], [dict(mesh=0)], [0])
    with pytest.raises(ValueError, match="NORMAL"):
        load_gltf(str(bad))



def _expected_rgba(img, color_type, depth, palette=None, trns=None):
    img = np.asarray(img)
    if color_type == 3:
        pal = np.asarray(palette, np.uint8).reshape(-1, 3)
        out = np.full(img.shape + (4,), 255, np.uint8)
        out[..., :3] = pal[img]
        if trns is not None:
            t = np.full(len(pal), 255, np.uint8)
            t[:len(trns)] = trns
            out[..., 3] = t[img]
        return out
    hi = (img >> 8).astype(np.uint8) if depth == 16 else img.astype(np.uint8)
    if depth < 8:
        hi = (img.astype(np.uint32) * (255 // ((1 << depth) - 1))).astype(np.uint8)
    out = np.full(img.shape[:2] + (4,), 255, np.uint8)
    if color_type in (0, 4):
        g = hi if hi.ndim == 2 else hi[..., 0]
        out[..., 0] = out[..., 1] = out[..., 2] = g
        if color_type == 4:
            out[..., 3] = hi[..., 1]
    else:
        out[..., :3] = hi[..., :3]
        if color_type == 6:
            out[..., 3] = hi[..., 3]
    return out


def test_png_images_of_every_kind(tmp_path):
    """PNG images decoded by the loader's own inflate / unfilter: the five colour types, bit depths 1,
    4, 8, 16, palettes with transparency, all five row filters, stored / fixed / dynamic DEFLATE
    blocks; a truncated PNG and a malformed JPEG are counted as skipped and leave their material slots
    empty"""
    import zlib
    from gltf_writer import png
    rng = np.random.default_rng(7)
    H, W = 13, 19
    cases = []
    for ct, ch in ((6, 4), (2, 3), (4, 2)):
        img = rng.integers(0, 256, (H, W, ch), dtype=np.uint8)
        cases.append((png(img, ct, 8), _expected_rgba(img, ct, 8)))
    gray = rng.integers(0, 256, (H, W), dtype=np.uint8)
    cases.append((png(gray, 0, 8, level=0), _expected_rgba(gray, 0, 8)))
    img16 = rng.integers(0, 65536, (H, W, 4), dtype=np.uint16)
    cases.append((png(img16, 6, 16, strategy=zlib.Z_FIXED), _expected_rgba(img16, 6, 16)))
    g4 = rng.integers(0, 16, (H, W), dtype=np.uint8)
    cases.append((png(g4, 0, 4), _expected_rgba(g4, 0, 4)))
    g1 = rng.integers(0, 2, (H, W), dtype=np.uint8)
    cases.append((png(g1, 0, 1), _expected_rgba(g1, 0, 1)))
    pal = rng.integers(0, 256, (16, 3), dtype=np.uint8)
    idx8 = rng.integers(0, 16, (H, W), dtype=np.uint8)
    trns = rng.integers(0, 256, 10, dtype=np.uint8)
    cases.append((png(idx8, 3, 8, palette=pal, trns=trns), _expected_rgba(idx8, 3, 8, pal, trns)))
    cases.append((png(idx8, 3, 4, palette=pal), _expected_rgba(idx8, 3, 4, pal)))
    bad = [png(gray, 0, 8)[:60], b"\xff\xd8\xff\xe0" + bytes(64)]
    images = [(data, 10497, 10497) for data, _ in cases] + [(b, 10497, 10497) for b in bad]
    mats = [{"pbrMetallicRoughness": {"baseColorTexture": {"index": k}}} for k in range(len(images))]
    path = tmp_path / "png.gltf"
    write(path, [[(*TRI, k, None)] for k in range(len(images))], [dict(mesh=k) for k in range(len(images))],
          list(range(len(images))), materials=mats, images=images)
    a = load_gltf(str(path))
    assert a["skipped_textures"] == 2 and len(a["textures"]) == len(images)
    for k, (_, expect) in enumerate(cases):
        got, ws, wt = a["textures"][k]
        assert np.array_equal(got, expect), k
        assert a["materials"][k]["tex_color"] == k
    for k in range(len(cases), len(images)):
        assert a["materials"][k]["tex_color"] == 0xFFFFFFFF


def test_texcoords_tangents_and_samplers(tmp_path):
    """TEXCOORD_0 as floats and as normalised bytes, TANGENT xyz, tangents computed from NORMAL and
    TEXCOORD_0 as Geometry::compute_tangents does, the samplers' wrap modes, the material texture
    slots (an emissive texture zeroes the emissive factor)"""
    from gltf_writer import png
    quad_uv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    n = np.tile([0, 0, 1], (4, 1)).astype(np.float32)
    tg = np.array([[1, 0, 0, 1]] * 4, np.float32)
    uv8 = np.array([[0, 0], [255, 0], [255, 255], [0, 255]], np.uint8)
    img = png(np.full((4, 4, 4), 200, np.uint8), 6, 8)
    meshes = [[(*QUAD, 0, None, n, {"TEXCOORD_0": quad_uv, "TANGENT": tg})],
              [(*QUAD, 0, None, n, {"TEXCOORD_0": (uv8, 5121)})],
              [(*QUAD, 0, None, None, {"TEXCOORD_0": quad_uv})]]
    mats = [{"pbrMetallicRoughness": {"baseColorTexture": {"index": 0, "extensions": {"KHR_texture_transform": {
                 "offset": [0.25, -0.5], "rotation": 0.3, "scale": [2.0, 3.0]}}}, "metallicRoughnessTexture": {"index": 1}},
             "normalTexture": {"index": 1}, "emissiveTexture": {"index": 0}, "emissiveFactor": [1, 1, 1],
             "extensions": {"KHR_materials_transmission": {"transmissionTexture": {"index": 1}}}}]
    path = tmp_path / "uv.glb"
    write(path, meshes, [dict(mesh=k) for k in range(3)], [0, 1, 2], materials=mats, mode="glb",
          images=[(img, 33071, 33648), (img, 10497, 33071)])
    a = load_gltf(str(path))
    assert np.array_equal(a["texcoords"][0], quad_uv) and np.allclose(a["tangents"][0], tg[:, :3])
    assert np.allclose(a["texcoords"][1], quad_uv)
    # computed: QUAD's u runs along +x, v along +y, normal +z -> tangent +-x, sign as compute_tangents
    xyz, ix = QUAD
    assert a["tangents"][1] is not None and np.allclose(np.abs(a["tangents"][1]), [[1, 0, 0]] * 4, atol=1e-6)
    t = np.zeros((4, 3)); b = np.zeros((4, 3))
    for tri in ix:
        v0, v1, v2 = xyz[tri]
        u0, u1, u2 = quad_uv[tri]
        x1, x2 = v1 - v0, v2 - v0
        s1, s2, t1, t2 = u1[0] - u0[0], u2[0] - u0[0], u1[1] - u0[1], u2[1] - u0[1]
        r = 1 / (s1 * t2 - s2 * t1)
        t[tri] += (t2 * x1 - t1 * x2) * r
        b[tri] += (s1 * x2 - s2 * x1) * r
    sign = np.where(np.einsum("ij,ij->i", np.cross(n, t), b) < 0, 1.0, -1.0)
    assert np.allclose(a["tangents"][1], t / np.linalg.norm(t, axis=1, keepdims=True) * sign[:, None], atol=1e-6)
    assert a["tangents"][2] is None and a["normals"][2] is None  # no normals: no tangents either
    assert [(ws, wt) for _, ws, wt in a["textures"]] == [(1, 2), (0, 1)]
    m = a["materials"][0]
    assert (m["tex_color"], m["tex_ao_rough_metal"], m["tex_normal"], m["tex_emission"], m["tex_transmission"]) == \
        (0, 1, 1, 0, 1)
    assert np.array_equal(m["emission"], [0, 0, 0])
    # the colour texture's KHR_texture_transform: T(offset) R(rotation about -z) S(scale) on (u, v, 0, 1)
    c, s_ = math.cos(0.3), math.sin(0.3)
    assert m["has_uv_transform"] == 1
    assert np.allclose(m["uv_transform"], [2 * c, 3 * s_, 0.25, -2 * s_, 3 * c, -0.5], rtol=0, atol=1e-6)


def test_jpeg_images(tmp_path):
    """JPEG images decoded by the loader's own decoder (jpeg.cpp): sequential YCbCr at 4:2:0, 4:2:2 and
    4:4:4, with and without restart intervals, and grey; progressive files of the same images
    (spectral selection, successive approximation, end-of-band runs over flat regions, restart
    intervals); RGB components under an Adobe marker; each against
    the image the encoder's quantised coefficients define (tests/jpeg_writer.py; one level of rounding
    allowed); a progressive frame header without scans is counted as skipped"""
    from jpeg_writer import jpeg
    rng = np.random.default_rng(12)
    yy, xx = np.mgrid[0:21, 0:29]
    smooth = np.stack([(120 + 80 * np.sin(xx / 4.0 + c) * np.cos(yy / 5.0)) for c in range(3)], -1)
    rgb = np.clip(smooth + rng.normal(0, 12, smooth.shape), 0, 255).astype(np.uint8)
    grey = np.clip(100 + 60 * np.sin(xx[:17, :23] / 3.0) + rng.normal(0, 20, (17, 23)), 0, 255).astype(np.uint8)
    # mostly flat with a few busy blocks: long end-of-band runs, zero runs past 16 in the refinements
    patchy = np.full((48, 56, 3), 128, np.uint8)
    patchy[8:16, 16:24] = rng.integers(0, 256, (8, 8, 3), dtype=np.uint8)
    patchy[30:38, 40:48, 0] = 255
    cases = [jpeg(rgb, (2, 2)), jpeg(rgb, (1, 1), restart=3), jpeg(rgb, (2, 1), restart=1), jpeg(grey),
             jpeg(np.full((9, 10, 3), (200, 40, 90), np.uint8), (2, 2)),
             jpeg(rgb, (2, 2), progressive=True), jpeg(rgb, (1, 1), progressive=True), jpeg(grey, progressive=True),
             jpeg(patchy, (2, 1), progressive=True), jpeg(patchy, (1, 1), progressive=True),
             jpeg(rgb, (2, 2), restart=2, progressive=True), jpeg(patchy, (2, 2), restart=5, progressive=True),
             jpeg(rgb, adobe_rgb=True), jpeg(patchy, adobe_rgb=True, progressive=True)]
    # the progressive and the sequential file of an image decode alike, restart intervals or not
    assert np.array_equal(cases[5][1], cases[0][1]) and np.array_equal(cases[7][1], cases[3][1])
    assert np.array_equal(cases[10][1], cases[0][1])
    # a progressive frame header (SOF2) after SOI
    prog = b"\xff\xd8" + bytes([0xFF, 0xC2, 0, 11, 8, 0, 8, 0, 8, 1, 1, 0x11, 0]) + b"\xff\xd9"
    images = [(data, 10497, 10497) for data, _ in cases] + [(prog, 10497, 10497)]
    mats = [{"pbrMetallicRoughness": {"baseColorTexture": {"index": k}}} for k in range(len(images))]
    path = tmp_path / "jpeg.gltf"
    write(path, [[(*TRI, k, None)] for k in range(len(images))], [dict(mesh=k) for k in range(len(images))],
          list(range(len(images))), materials=mats, images=images)
    a = load_gltf(str(path))
    assert a["skipped_textures"] == 1 and len(a["textures"]) == len(images)
    for k, (_, expect) in enumerate(cases):
        got, _, _ = a["textures"][k]
        assert got.shape == expect.shape, k
        d = np.abs(got.astype(np.int64) - expect.astype(np.int64))
        assert d.max() <= 1 and d.mean() < 0.02, (k, d.max(), d.mean())
        assert a["materials"][k]["tex_color"] == k
    assert a["materials"][len(cases)]["tex_color"] == 0xFFFFFFFF
