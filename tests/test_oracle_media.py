"""Homogeneous participating media in the FP64 oracle (no GPU): the medium of a boundary material
(raypipeline.slang:493-511), free-flight sampling with a channel pick and the segment's emission
integral (raypipeline.slang:388-474), the media stack across null surfaces (raypipeline.slang:189-194,
:516-523) and the Henyey-Greenstein phase function (phase_function.slang:10-31). Each render case
has a closed form: a null-surface box seen through its exact chord lengths (slab test in numpy,
averaged over the same jittered camera rays the tracer draws)."""
import math

import numpy as np
import pytest

import oracle
from vierkant_gb300.geometry import MATERIAL_DTYPE

H = 0.6   # half extent of the box
RES = 16


def box_mesh(h):
    """an axis-aligned box of half extent h, 12 triangles with outward (counter-clockwise) winding"""
    xyz, idx = [], []
    for a in range(3):
        b, c = (a + 1) % 3, (a + 2) % 3
        for s in (-1, 1):
            base = len(xyz)
            for u, w in ((-1, -1), (1, -1), (1, 1), (-1, 1)):
                p = [0.0, 0.0, 0.0]
                p[a], p[b], p[c] = s * h, u * h, w * h
                xyz.append(p)
            tri = [[0, 1, 2], [0, 2, 3]] if s > 0 else [[0, 2, 1], [0, 3, 2]]
            idx += [[base + i for i in t] for t in tri]
    xyz, idx = np.asarray(xyz, np.float32), np.asarray(idx, np.uint32)
    v0, v1, v2 = (xyz[idx[:, k]] for k in range(3))
    n = np.cross(v1 - v0, v2 - v0)
    assert np.all(np.einsum("ij,ij->i", n, (v0 + v1 + v2) / 3) > 0)  # outward
    return xyz, idx


def null_box_material(**kw):
    m = np.zeros(1, MATERIAL_DTYPE)
    m["null_surface"] = 1
    m["ior"] = 1.0
    m["attenuation_color"] = 1.0
    m["attenuation_distance"] = np.inf
    for k, v in kw.items():
        m[k][0] = v
    return m


def cam():
    return oracle.camera((0.3, 0.2, 4.0), (0, 0, 0), (0, 1, 0), 0.2679, RES, RES)


def chords(spp=1024):
    """per pixel: the chord length through the box of spp jittered camera rays [RES, RES, spp]"""
    r = oracle.camera_rays(cam(), 7, 3, spp)
    o, d = r["o"].astype(np.float64), r["d"].astype(np.float64)
    d = d / np.linalg.norm(d, axis=1, keepdims=True)
    with np.errstate(divide="ignore", invalid="ignore"):
        t0, t1 = (-H - o) / d, (H - o) / d
    tn = np.nanmax(np.minimum(t0, t1), axis=1)
    tf = np.nanmin(np.maximum(t0, t1), axis=1)
    L = np.where(tf > np.maximum(tn, 0), tf - np.maximum(tn, 0), 0.0)
    return L.reshape(spp, RES, RES).transpose(1, 2, 0)


def render(mat, env_value, spp, mis_mode=0, max_depth=8):
    xyz, idx = box_mesh(H)
    env = np.full((32, 64, 3), env_value, np.float32)
    img, _, _ = oracle.pt_render(True, xyz, idx, np.zeros(len(idx), np.uint32), mat, oracle.CpuBVH(xyz, idx, 4),
                                 env, cam(), spp, max_depth=max_depth, rr_depth=64, mis_mode=mis_mode)
    return img


def medium_of(mat):
    """sigma_s, sigma_a of the box's medium in float64 from the material record"""
    m = mat[0]
    st = -np.log(m["attenuation_color"].astype(np.float64)) / float(m["attenuation_distance"])
    ms = float(m["scatter_factor"]) * m["scatter_color"].astype(np.float64)
    kc = 4.09712 + 4.20863 * ms - np.sqrt(9.59217 + 41.6808 * ms + 17.7126 * ms * ms)
    ss = 1.0 - kc * kc
    return ss * st, (1.0 - ss) * st


def test_beer_lambert_absorbing_box():
    """an absorbing box (no scattering: scatter_factor 0) in a white environment: per channel the
    transmittance exp(-sigma_t chord); free-flight sampling with the channel pick weighs an escaping
    path by tr / mean(tr), so each channel's expectation is its own transmittance"""
    mat = null_box_material(attenuation_color=(0.5, 0.25, 0.8), attenuation_distance=1.0)
    ss, sa = medium_of(mat)
    assert np.all(ss < 1e-5 * (ss + sa))
    Lc = chords()
    expect = np.exp(-(ss + sa)[None, None, None, :] * Lc[..., None]).mean(axis=2)
    img = render(mat, 1.0, 256)
    inside = (Lc > 0).all(axis=2)
    assert inside.sum() > 40 and (~(Lc > 0).any(axis=2)).sum() > 20
    assert np.array_equal(img[~(Lc > 0).any(axis=2)], np.ones_like(img[~(Lc > 0).any(axis=2)]))  # misses: the sky
    for c in range(3):
        rel = img[..., c][inside].mean() / expect[..., c][inside].mean() - 1
        assert abs(rel) < 0.02, (c, rel)
    # a darker channel is darker everywhere on average: the channel pick keeps colour
    assert img[..., 1][inside].mean() < img[..., 0][inside].mean() < img[..., 2][inside].mean()


def test_emissive_box_matches_emission_integral():
    """an emissive absorbing box in a black environment: the segment through it adds
    sigma_a Le (1 - exp(-sigma_t chord)) / sigma_t (raypipeline.slang:397-403) whatever the free
    flight samples, so the estimate is exact per camera ray"""
    le = np.array([2.0, 1.0, 0.5])
    mat = null_box_material(attenuation_color=(0.3, 0.3, 0.3), attenuation_distance=1.0, emission=le)
    ss, sa = medium_of(mat)
    st = ss + sa
    Lc = chords()
    expect = (sa * le / st)[None, None, None, :] * (1 - np.exp(-st[None, None, None, :] * Lc[..., None]))
    expect = expect.mean(axis=2)
    img = render(mat, 0.0, 64)
    inside = (Lc > 0).all(axis=2)
    # pixels whose footprint sees one front and one back face: the chord varies smoothly over it, so
    # 64 jittered samples average it to well under a percent
    smooth = inside & (Lc.std(axis=2) < 0.01 * Lc.mean(axis=2))
    assert smooth.sum() > 30
    assert np.allclose(img[smooth], expect[smooth], rtol=3e-3, atol=0), np.abs(img[smooth] / expect[smooth] - 1).max()
    assert abs(img.sum() / expect.sum() - 1) < 0.02
    assert np.all(img[~(Lc > 0).any(axis=2)] == 0)


@pytest.mark.parametrize("g,mis", [(0.0, 2), (0.6, 2), (-0.4, 2), (0.3, 0), (0.3, 1)])
def test_white_scattering_furnace(g, mis):
    """a non-absorbing scatterer (scatter colour 1 at scatter factor 1: single-scattering albedo 1 by the
    Kulla-Conty inversion) in a constant unit environment: every path escapes eventually, so radiance 1
    comes back at every pixel. Scattering events take no environment NEE sample, so MIS and NEE-only
    collect the environment from the phase-sampled paths like BSDF-only does."""
    mat = null_box_material(attenuation_color=(0.3, 0.3, 0.3), attenuation_distance=1.0, scatter_factor=1.0,
                            scatter_color=(1, 1, 1), phase_g=g)
    ss, sa = medium_of(mat)
    assert np.all(sa < 1e-6 * ss)
    img = render(mat, 1.0, 128, mis_mode=mis, max_depth=64)
    assert abs(img.mean() - 1) < 0.01, img.mean()
    inside = (chords(64) > 0).all(axis=2)
    assert abs(img[inside].mean() - 1) < 0.015


def test_scattering_darkens_with_albedo():
    """a grey scatterer of multi-scatter albedo 0.5 returns less than a white one and more than a pure
    absorber of the same extinction"""
    kw = dict(attenuation_color=(0.3, 0.3, 0.3), attenuation_distance=1.0, phase_g=0.2)
    white = render(null_box_material(scatter_factor=1.0, scatter_color=(1, 1, 1), **kw), 1.0, 64, 2, 64).mean()
    half = render(null_box_material(scatter_factor=0.5, scatter_color=(1, 1, 1), **kw), 1.0, 64, 2, 64).mean()
    black = render(null_box_material(**kw), 1.0, 64, 2, 64).mean()
    assert black + 0.02 < half < white - 0.02


@pytest.mark.parametrize("g", [0.0, 0.5, -0.7, 0.9])
def test_phase_hg_normalised_and_sampled(g):
    """phase_hg integrates to 1 over the sphere, the sampler's pdf is phase_hg of its own cosine, and
    the sampled mean cosine is g"""
    mu = np.linspace(-1, 1, 20001)
    p = np.array([oracle.phase_hg(m, g) for m in mu])
    assert abs(2 * math.pi * np.trapezoid(p, mu) - 1) < 2e-3
    rng = np.random.default_rng(5)
    cos = []
    for x, y in rng.random((4000, 2)):
        d, pdf = oracle.phase_hg_sample(x, y, g)
        assert abs(np.linalg.norm(d) - 1) < 1e-9
        assert math.isclose(pdf, oracle.phase_hg(d[2], g), rel_tol=1e-9)
        cos.append(d[2])
    assert abs(np.mean(cos) - g) < 0.03


def test_null_surface_without_medium_is_invisible():
    """a null surface that bounds no medium (infinite attenuation distance) neither shades nor
    attenuates: the environment comes through unchanged"""
    img = render(null_box_material(), 0.75, 4)
    assert np.allclose(img, 0.75, rtol=0, atol=1e-12)


def test_camera_inside_medium():
    """a camera inside an absorbing box (raypipeline.slang:128-135): paths start with the camera's medium
    on their stack, so a ray that leaves through the box wall at distance t carries exp(-sigma_t t);
    the medium given as parameters and as the box material's render identically; without a camera
    medium the exit wall pops nothing and the environment comes through unattenuated"""
    big = 5.0
    xyz, idx = box_mesh(big)
    mat = null_box_material(attenuation_color=(0.5, 0.7, 0.9), attenuation_distance=6.0)
    env = np.ones((32, 64, 3), np.float32)
    args = (True, xyz, idx, np.zeros(len(idx), np.uint32), mat, oracle.CpuBVH(xyz, idx, 4), env, cam(), 16)
    kw = dict(max_depth=4, rr_depth=64, mis_mode=0)
    given, _, _ = oracle.pt_render(*args, camera_medium=oracle.medium_params(attenuation_color=(0.5, 0.7, 0.9),
                                                                             attenuation_distance=6.0), **kw)
    by_mat, _, _ = oracle.pt_render(*args, camera_material=0, **kw)
    vacuum, _, _ = oracle.pt_render(*args, **kw)
    assert np.array_equal(given, by_mat)
    assert np.all(vacuum == 1.0)
    r = oracle.camera_rays(cam(), 7, 3, 256)
    o, d = r["o"].astype(np.float64), r["d"].astype(np.float64)
    d = d / np.linalg.norm(d, axis=1, keepdims=True)
    with np.errstate(divide="ignore", invalid="ignore"):
        tf = np.nanmin(np.maximum((-big - o) / d, (big - o) / d), axis=1)
    st = -np.log(np.array([0.5, 0.7, 0.9])) / 6.0
    expect = np.exp(-st[None, :] * tf[:, None]).reshape(256, RES, RES, 3).mean(axis=0)
    # free-flight escapes weigh tr / mean(tr): per channel unbiased, 16 spp x 256 pixels
    for c in range(3):
        assert abs(given[..., c].mean() / expect[..., c].mean() - 1) < 0.03, c
