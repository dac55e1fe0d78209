"""Texture sampling in the radiance oracle (CPU only): the mip chain (rounded 2 x 2 means, the last row
/ column repeated for odd sizes) against a plain loop, trilinear samples against an independent numpy
transcription (texel centres, REPEAT / CLAMP_TO_EDGE / MIRRORED_REPEAT, lambda clamped to the chain),
and a textured render that differs from the untextured one."""
import math

import numpy as np
import pytest

import oracle
from vierkant_gb300 import geometry


def test_mip_chain_against_a_loop():
    rng = np.random.default_rng(4)
    img = rng.integers(0, 256, (13, 22, 4), dtype=np.uint8)
    recs, texels = oracle.texture_pool([img])
    r = recs[0]
    assert (r["width"], r["height"], r["levels"]) == (22, 13, 5)
    lvl, w, h = img.astype(np.int64), 22, 13
    for k in range(1, 5):
        pw, ph = w, h
        w, h = max(1, w // 2), max(1, h // 2)
        nxt = np.zeros((h, w, 4), np.int64)
        for y in range(h):
            for x in range(w):
                xs = (min(2 * x, pw - 1), min(2 * x + 1, pw - 1))
                ys = (min(2 * y, ph - 1), min(2 * y + 1, ph - 1))
                nxt[y, x] = (lvl[ys[0], xs[0]] + lvl[ys[0], xs[1]] + lvl[ys[1], xs[0]] + lvl[ys[1], xs[1]] + 2) // 4
        lvl = nxt
        got = texels[r["offset"][k]:r["offset"][k] + w * h]
        words = lvl[..., 0] | (lvl[..., 1] << 8) | (lvl[..., 2] << 16) | (lvl[..., 3] << 24)
        assert np.array_equal(got, words.reshape(-1).astype(np.uint32)), k


def _np_sample(levels, wrap, u, v, lam):
    def wrapi(x, n, mode):
        if mode == 1:
            return min(max(x, 0), n - 1)
        if mode == 2:
            m = x % (2 * n)
            return m if m < n else 2 * n - 1 - m
        return x % n

    def bil(img):
        h, w = img.shape[:2]
        fx, fy = u * w - 0.5, v * h - 0.5
        x0, y0 = math.floor(fx), math.floor(fy)
        ax, ay = fx - x0, fy - y0
        c = lambda x, y: img[wrapi(y, h, wrap[1]), wrapi(x, w, wrap[0])].astype(np.float64) / 255.0
        top = c(x0, y0) + (c(x0 + 1, y0) - c(x0, y0)) * ax
        bot = c(x0, y0 + 1) + (c(x0 + 1, y0 + 1) - c(x0, y0 + 1)) * ax
        return top + (bot - top) * ay

    lam = min(max(lam, 0.0), len(levels) - 1)
    l0 = int(lam)
    f = lam - l0
    a = bil(levels[l0])
    return a + (bil(levels[l0 + 1]) - a) * f if f > 0 and l0 + 1 < len(levels) else a


@pytest.mark.parametrize("wrap", [(0, 0), (1, 1), (2, 2), (0, 2)])
def test_trilinear_samples_against_numpy(wrap):
    rng = np.random.default_rng(5)
    img = rng.integers(0, 256, (16, 24, 4), dtype=np.uint8)
    recs, texels = oracle.texture_pool([(img, wrap[0], wrap[1])])
    r = recs[0]
    levels = []
    w, h = 24, 16
    for k in range(int(r["levels"])):
        words = texels[r["offset"][k]:r["offset"][k] + w * h].reshape(h, w)
        levels.append(np.stack([(words >> (8 * c)) & 0xFF for c in range(4)], axis=-1))
        w, h = max(1, w // 2), max(1, h // 2)
    for _ in range(200):
        u, v = rng.uniform(-2.5, 3.5), rng.uniform(-2.5, 3.5)
        lam = rng.uniform(-1.0, 6.0)
        got = oracle.tex_sample(recs, texels, 0, u, v, lam)
        assert np.allclose(got, _np_sample(levels, wrap, u, v, lam), atol=1e-12), (u, v, lam)


def test_textured_render_differs():
    sc = oracle.cornell_scene(0x5EED, 2, 8, 8)
    mats = oracle.cornell_materials(0x5EED, 2, 8)
    th = float(np.float32(math.tan(math.radians(45.0) / 2.0)))
    cam = oracle.camera((0, 0, 3.4), (0, 0, 0), (0, 1, 0), th, 320, 180)
    env = oracle.env_procedural(256, 128, np.array([0.2962, 0.5, 0.8138], np.float32))
    bvh = oracle.CpuBVH(sc["xyz"], sc["indices"], 4)
    uv, tg = geometry.cornell_texcoords(sc)
    nrm = geometry.cornell_vertex_normals(sc)
    tmats = geometry.textured_materials(mats)
    crop = (100, 60, 64, 64)
    a, _, _ = oracle.pt_render(True, sc["xyz"], sc["indices"], sc["tri_material"], tmats, bvh, env, cam, 8,
                               crop=crop, normals=nrm)
    b, _, _ = oracle.pt_render(True, sc["xyz"], sc["indices"], sc["tri_material"], tmats, bvh, env, cam, 8,
                               crop=crop, normals=nrm, uv=uv, tangents=tg, textures=geometry.test_textures())
    assert np.abs(a - b).mean() > 1e-2 * np.abs(a).mean()
    # without texture coordinates nothing is sampled
    c, _, _ = oracle.pt_render(True, sc["xyz"], sc["indices"], sc["tri_material"], tmats, bvh, env, cam, 8,
                               crop=crop, normals=nrm, textures=geometry.test_textures())
    assert np.array_equal(a, c)


def test_uv_transform():
    """the texture-coordinate transform of the closest-hit stage (raypipeline.slang:350): the identity
    changes nothing; scaling by 2 equals texture coordinates scaled by 2 on primary hits (where both
    read level 0: the LOD keeps the untransformed coordinates' constant); a rotation changes the image"""
    sc = oracle.cornell_scene(0x5EED, 2, 8, 8)
    mats = oracle.cornell_materials(0x5EED, 2, 8)
    th = float(np.float32(math.tan(math.radians(45.0) / 2.0)))
    cam = oracle.camera((0, 0, 3.4), (0, 0, 0), (0, 1, 0), th, 320, 180)
    env = oracle.env_procedural(256, 128, np.array([0.2962, 0.5, 0.8138], np.float32))
    bvh = oracle.CpuBVH(sc["xyz"], sc["indices"], 4)
    uv, tg = geometry.cornell_texcoords(sc)
    nrm = geometry.cornell_vertex_normals(sc)
    tmats = geometry.textured_materials(mats)
    crop = (100, 60, 64, 64)

    def render(m, tuv, depth=6):
        img, _, _ = oracle.pt_render(True, sc["xyz"], sc["indices"], sc["tri_material"], m, bvh, env, cam, 4,
                                     crop=crop, normals=nrm, uv=tuv, tangents=tg, textures=geometry.test_textures(),
                                     max_depth=depth)
        return img

    plain = render(tmats, uv)
    ident = tmats.copy()
    ident["has_uv_transform"] = 1
    ident["uv_transform"] = (1, 0, 0, 0, 1, 0)
    assert np.array_equal(plain, render(ident, uv))
    twice = tmats.copy()
    twice["has_uv_transform"] = 1
    twice["uv_transform"] = (2, 0, 0, 0, 2, 0)
    a = render(twice, uv, depth=1)
    b = render(tmats, uv * 2, depth=1)
    assert np.array_equal(a, b)
    assert not np.array_equal(a, render(tmats, uv, depth=1))
    rot = tmats.copy()
    rot["has_uv_transform"] = 1
    c, s = math.cos(0.7), math.sin(0.7)
    rot["uv_transform"] = (c, s, 0.1, -s, c, 0.2)
    assert np.abs(render(rot, uv) - plain).mean() > 1e-3 * np.abs(plain).mean()
