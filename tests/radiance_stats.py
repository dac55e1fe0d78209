"""Statistical comparison of a GPU radiance estimate with an FP64 oracle fixture.

The GPU image is the mean of B independent batches (tracers with different seeds), so its per-pixel
variance is measured from the batches themselves; the fixture holds the oracle's mean and the per-pixel
variance of one path's luminance, so the oracle mean's variance is lum_var / spp. Pixels are independent
in both estimators (each pixel's paths draw their own random streams). On luminance:

  bias     = (sum L_gpu - sum L_ref) / sum L_ref
  se       = sqrt(sum var_gpu + sum var_ref)          standard error of the difference of the sums
  z        = (sum L_gpu - sum L_ref) / se            |z| < 3 for an unbiased estimator
  rmse     = sqrt(mean (L_gpu - L_ref)^2)
  expected = sqrt(mean (var_gpu + var_ref))          the RMSE an unbiased estimator shows
  ratio    = rmse / expected                         about 1; <= 1.2 passes
  bound    = 3 se / sum L_ref                        the smallest relative bias the comparison resolves
"""
from __future__ import annotations

import math

import numpy as np


def lum(a):
    return 0.2126 * a[..., 0] + 0.7152 * a[..., 1] + 0.0722 * a[..., 2]


def render_batches(make_tracer, scene, cam, batches: int, seed0: int = 0x5EED):
    """Per-batch images (B, H, W, 3) float64: batch k is one render of a fresh tracer seeded seed0 + k."""
    out = []
    for k in range(batches):
        pt = make_tracer(seed0 + k)
        out.append(pt.render_scene(scene, cam).cpu().numpy().astype(np.float64))
        pt.close()
    return np.stack(out)


def compare(batch_imgs, ref_mean, ref_lum_var, ref_spp, crop=None):
    """Statistics of the batch mean against the oracle (see the module docstring). crop: (x0, y0, w, h)
    cut from the GPU images when the fixture covers a window of them."""
    imgs = np.asarray(batch_imgs, np.float64)
    if crop is not None:
        x0, y0, w, h = crop
        imgs = imgs[:, y0:y0 + h, x0:x0 + w]
    B = imgs.shape[0]
    Lb = lum(imgs)
    Lg = Lb.mean(axis=0)
    var_gpu = Lb.var(axis=0, ddof=1) / B
    Lr = lum(np.asarray(ref_mean, np.float64))
    var_ref = np.asarray(ref_lum_var, np.float64) / float(ref_spp)
    Sg, Sr = Lg.sum(), Lr.sum()
    se = math.sqrt(var_gpu.sum() + var_ref.sum())
    rmse = math.sqrt(float(np.mean((Lg - Lr) ** 2)))
    expected = math.sqrt(float(np.mean(var_gpu + var_ref)))
    mean = imgs.mean(axis=0)
    return {"bias": (Sg - Sr) / Sr, "z": (Sg - Sr) / se, "se_rel": se / Sr, "bound": 3 * se / Sr,
            "rmse": rmse, "expected": expected, "ratio": rmse / expected, "batches": B,
            "rgb_bias": float((mean.sum() - np.asarray(ref_mean, np.float64).sum()) /
                              np.asarray(ref_mean, np.float64).sum())}


def report(name, s):
    print(f"{name}: bias {s['bias']:+.5f} z {s['z']:+.2f} (3 se = {s['bound']:.5f}), rmse {s['rmse']:.4f} vs "
          f"expected {s['expected']:.4f} (ratio {s['ratio']:.3f}), {s['batches']} batches")


def check(s, max_ratio=1.2, max_bound=0.005):
    assert abs(s["z"]) < 3.0, s
    assert s["ratio"] <= max_ratio, s
    assert s["bound"] < max_bound, s
