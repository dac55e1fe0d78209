"""The reference's random streams on the GPU (settings.rng_mode = VKG_RNG_REFERENCE): every random
number the tracer's kernels draw, recorded through vkg_diag_tracer_uniforms, equals the reference
shaders' streams restated by the oracle (oracle/rng.c: xxhash32 of hash.slang, the rnd() LCG of
random.slang) bit for bit: the batch seed from std::minstd_rand0(seed), the per-pixel chain
xxhash32(batch seed, width * y + x), the sub-pixel offset, the lens sample, the jitter
frac(Hammersley(s, N) + offset) and, per segment i, the chain hashed with i feeding the LCG."""
import ctypes as C
import math

import numpy as np
import pytest
import torch

import oracle
from vierkant_gb300 import _lib, geometry
from vierkant_gb300.pathtracer import PBRPathTracer, Scene, procedural_sky, sun_direction

pytestmark = pytest.mark.gpu

W, H, CROP, SPP, DEPTH = 64, 36, (8, 4, 16, 12), 4, 6
STRIDE = 2 + 16 * DEPTH


def minstd_rand0(seed, k):
    """the k-th output (k = 0, 1, ...) of std::minstd_rand0 seeded with `seed`"""
    m = 2147483647
    x = seed % m or 1
    for _ in range(k + 1):
        x = x * 16807 % m
    return x


class RefStream:
    def __init__(self, L):
        self.L = L

    def xxhash(self, a, b):
        return int(self.L.orc_xxhash32(a & 0xFFFFFFFF, b & 0xFFFFFFFF))

    def rnd(self, state):
        s = C.c_uint32(state)
        v = self.L.orc_rnd(C.byref(s))
        return np.float32(v), s.value


def expected_check(rec, bseed, x, y, rs):
    """walks one pixel's records (SPP samples) through the reference's streams; returns the number of
    segments checked"""
    f = np.float32
    chain = rs.xxhash(bseed, W * y + x)
    r, chain = rs.rnd(chain)
    off = f(f(2.0) * r) - f(1.0)
    checked = 0
    for s in range(SPP):
        d = rec[s]
        _, chain = rs.rnd(chain)
        _, chain = rs.rnd(chain)
        hx = f(s) / f(SPP)
        hy = f(int("{:032b}".format(s)[::-1], 2)) * f(2.3283064365386963e-10)
        ax, ay = f(hx + off), f(hy + off)
        jx, jy = f(ax - f(math.floor(ax))), f(ay - f(math.floor(ay)))
        assert d[0].tobytes() == jx.tobytes() and d[1].tobytes() == jy.tobytes(), (x, y, s)
        for i in range(DEPTH):
            seg = d[2 + 16 * i: 2 + 16 * i + 8]
            if np.isnan(seg[0]):
                assert np.all(np.isnan(d[2 + 16 * i:])), (x, y, s, i)
                break
            chain = rs.xxhash(chain, i)
            l = chain
            want = []
            for _ in range(8):
                v, l = rs.rnd(l)
                want.append(v)
            assert seg.tobytes() == np.array(want, np.float32).tobytes(), (x, y, s, i)
            checked += 1
    return checked


def test_reference_streams_equal_the_oracle(ctx):
    sc = geometry.cornell_scene(0x5EED, 2, 16, 8)
    env = procedural_sky(ctx, 256, 128, sun_direction(), 50.0, 0.02)
    scene = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], sc["materials"], env)
    cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, W, H)
    s = PBRPathTracer.default_settings()
    s.resolution[0], s.resolution[1] = W, H
    s.num_samples, s.max_trace_depth, s.rr_start_depth = SPP, DEPTH, 3
    for k in range(4):
        s.crop[k] = CROP[k]
    s.rng_mode = _lib.RNG_REFERENCE
    seed = 1234
    pt = PBRPathTracer(ctx, seed=seed, settings=s)
    npix = CROP[2] * CROP[3]
    buf = torch.empty(SPP * npix * STRIDE, dtype=torch.float32, device="cuda")
    _lib.check(_lib.lib().vkg_diag_tracer_uniforms(pt.handle, C.c_void_p(buf.data_ptr()), DEPTH))
    rs = RefStream(oracle.orc())
    total = 0
    for batch in range(2):
        buf.fill_(float("nan"))
        img = pt.render_scene(scene, cam)
        torch.cuda.synchronize()
        assert torch.isfinite(img).all() and img.sum() > 0
        rec = buf.cpu().numpy().reshape(SPP, npix, STRIDE)
        bseed = minstd_rand0(seed, batch)
        for p in range(npix):
            x, y = CROP[0] + p % CROP[2], CROP[1] + p // CROP[2]
            total += expected_check(rec[:, p], bseed, x, y, rs)
    assert total > 2 * npix * SPP  # most paths run several segments
    _lib.check(_lib.lib().vkg_diag_tracer_uniforms(pt.handle, None, 0))
    # PCG32 and reference streams give different (both finite) images of the same scene
    ref_img = img.clone()
    s.rng_mode = _lib.RNG_PCG32
    pt2 = PBRPathTracer(ctx, seed=seed, settings=s)
    pcg_img = pt2.render_scene(scene, cam)
    assert not torch.equal(pcg_img, ref_img)
    pt.close()
    pt2.close()
    scene.close()


def test_reference_streams_refused_with_a_cache(ctx):
    from vierkant_gb300.nrc import NeuralRadianceCache
    sc = geometry.cornell_scene(0x5EED, 2, 4, 4)
    env = procedural_sky(ctx, 64, 32, sun_direction(), 50.0, 0.02)
    scene = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], sc["materials"], env)
    cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, 32, 32)
    s = PBRPathTracer.default_settings()
    s.resolution[0], s.resolution[1] = 32, 32
    s.rng_mode = _lib.RNG_REFERENCE
    pt = PBRPathTracer(ctx, seed=1, settings=s)
    cache = NeuralRadianceCache(ctx, NeuralRadianceCache.default_config())
    pt.attach_cache(cache)
    with pytest.raises(_lib.VkgError):
        pt.render_scene(scene, cam)
    pt.close()
    cache.close()
    scene.close()
