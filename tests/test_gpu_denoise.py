"""Pixel records and the a-trous denoiser on the GPU.

* pixel records: coverage, object id, albedo and normal of the tracer's records equal the FP32 twin's
  (the same paths, the same last sample), depth to float rounding, radiance equals the render output;
* denoise: vkg_denoise equals the C restatement of denoise.slang on the same records (one fused
  exponential per tap on the GPU vs three in the restatement: rounding only), for a frame, a crop and
  degenerate sizes; the tracer's `denoising` setting outputs exactly vkg_denoise of its records;
* the denoised 4-spp crop is closer to the FP64 oracle than the raw one.
"""
import math

import numpy as np
import pytest
import torch

import oracle
from vierkant_gb300 import geometry
from vierkant_gb300.pathtracer import PIXEL_DTYPE, PBRPathTracer, Scene, denoise, procedural_sky, sun_direction
from test_gpu_pathtracer import d2h

pytestmark = pytest.mark.gpu

W, H = 256, 144


def settings(spp, res=(W, H), crop=(0, 0, 0, 0), denoising=False):
    s = PBRPathTracer.default_settings()
    s.resolution[0], s.resolution[1] = res
    s.num_samples, s.max_trace_depth, s.rr_start_depth = spp, 6, 3
    for k in range(4):
        s.crop[k] = crop[k]
    s.denoising = int(denoising)
    return s


@pytest.fixture(scope="module")
def box(ctx):
    sc = geometry.cornell_scene(0x5EED, 2, 64, 16)
    env = procedural_sky(ctx, 2048, 1024, sun_direction(), 5e4, 3.8e-5)
    scene = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], sc["materials"], env)
    yield {"sc": sc, "env": env, "scene": scene}
    scene.close()


def records(pt):
    return pt.pixel_data().cpu().numpy().view(PIXEL_DTYPE)[..., 0]


def test_pixel_records_match_twin(ctx, box):
    cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, W, H)
    pt = PBRPathTracer(ctx, seed=0x5EED, settings=settings(4))
    img = pt.render_scene(box["scene"], cam).cpu().numpy()
    rec = records(pt)
    pt.close()
    wptr, aptr, EW, EH = box["scene"].env_tables()
    n = EW * EH
    w = d2h(wptr, 4 * n, np.float32)
    tab = d2h(aptr, 8 * n, np.uint32).reshape(n, 2)
    sc = box["sc"]
    th = float(np.float32(math.tan(math.radians(45.0) / 2.0)))
    ocam = oracle.camera((0, 0, 3.4), (0, 0, 0), (0, 1, 0), th, W, H)
    twin = np.zeros((H, W), oracle.PIXEL_DTYPE)
    oracle.pt_render(False, sc["xyz"], sc["indices"], sc["tri_material"], sc["materials"],
                     oracle.CpuBVH(sc["xyz"], sc["indices"], 4), box["env"].cpu().numpy(), ocam, 4, seed=0x5EED,
                     rr_depth=3, alias_prob=np.ascontiguousarray(tab[:, 0].view(np.float32)),
                     alias=np.ascontiguousarray(tab[:, 1]), weight=w, pixels=twin)
    assert np.array_equal(rec["radiance"], img)
    assert np.array_equal(rec["alpha"], twin["alpha"])
    assert np.array_equal(rec["object_id"], twin["object_id"])
    assert np.array_equal(rec["albedo"], twin["albedo"])
    assert np.mean(rec["normal"] == twin["normal"]) > 0.999
    assert np.allclose(rec["depth"], twin["depth"], rtol=1e-5, atol=0)
    hit = twin["object_id"] != 0xFFFF
    assert 0.2 < hit.mean() < 1.0 and np.all(rec["depth"][~hit] == 0) and np.all(rec["depth"][hit] > 0)


@pytest.mark.parametrize("crop", [(0, 0, 0, 0), (40, 30, 97, 61), (100, 70, 1, 1), (10, 10, 3, 4)])
def test_denoise_matches_restatement(ctx, box, crop):
    cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, W, H)
    pt = PBRPathTracer(ctx, seed=3, settings=settings(2, crop=crop))
    pt.render_scene(box["scene"], cam)
    px = pt.pixel_data()
    cw, ch = (crop[2], crop[3]) if crop[2] else (W, H)
    out, dep = denoise(ctx, px, cw, ch, with_depth=True)
    out, dep = out.cpu().numpy(), dep.cpu().numpy()
    rec = px.cpu().numpy().view(PIXEL_DTYPE)[..., 0]
    pt.close()
    ref = oracle.denoise(rec)
    assert np.array_equal(dep, rec["depth"])
    assert np.all(out[..., 3] == 0)
    err = np.abs(out - ref) / np.maximum(np.abs(ref), 1e-3)
    print("max rel err", err.max())
    assert err.max() < 2e-4


def test_denoising_setting_outputs_the_denoised_records(ctx, box):
    cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, W, H)
    a = PBRPathTracer(ctx, seed=5, settings=settings(2, denoising=True))
    da = a.render_scene(box["scene"], cam)
    dn = denoise(ctx, a.pixel_data(), W, H)
    assert torch.equal(da, dn[..., :3])
    b = PBRPathTracer(ctx, seed=5, settings=settings(2))
    raw = b.render_scene(box["scene"], cam)
    assert torch.equal(raw.cpu(), torch.from_numpy(records(a)["radiance"].copy()))
    a.close()
    b.close()


def test_denoised_crop_is_closer_to_the_oracle(ctx, box, golden):
    g = golden("pt_oracle_crop")
    crop = tuple(int(v) for v in g["crop"])
    cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, 1280, 720)
    pt = PBRPathTracer(ctx, seed=11, settings=settings(4, res=(1280, 720), crop=crop, denoising=True))
    den = pt.render_scene(box["scene"], cam).cpu().numpy().astype(np.float64)
    raw = records(pt)["radiance"].astype(np.float64)
    pt.close()
    ref = g["mean"].astype(np.float64)
    lum = lambda a: 0.2126 * a[..., 0] + 0.7152 * a[..., 1] + 0.0722 * a[..., 2]
    e_raw = math.sqrt(np.mean((lum(raw) - lum(ref)) ** 2))
    e_den = math.sqrt(np.mean((lum(den) - lum(ref)) ** 2))
    print(f"4 spp crop RMSE: raw {e_raw:.4f}, denoised {e_den:.4f}")
    assert e_den < 0.8 * e_raw


def test_denoise_empty_image(ctx):
    px = torch.zeros((0, 0, 32), dtype=torch.uint8, device="cuda")
    out = denoise(ctx, px, 0, 0)
    assert out.numel() == 0
