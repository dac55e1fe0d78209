"""Generate the FP64 radiance-oracle fixture for the plain path tracer (CPU only, no reference needed).

    python tests/golden/make_pt_oracle.py [spp] [width height]

Scene: Cornell box + 64 cube-spheres (PCG32 seed 0x5EED, stream 2), procedural 2048x1024 equirect
environment (environment_white gradient + sun lobe 5e4 * exp((cos g - 1) / 3.8e-5) toward elevation
30 deg, azimuth 20 deg from +z), camera (0,0,3.4) -> origin, fovy 45 deg, 1280x720 (or 1920x1080,
the radiance-cache workload), max 6 segments, Russian roulette from the 3rd interaction, MIS. The
oracle (oracle/pathtrace.c, FP64, independent CDF environment sampler) renders a 128x128 crop
((576, 528) at 1280x720, (896, 824) at 1920x1080: both centred on the same image point) with `spp` paths per
pixel (default 4096) and stores the mean radiance plus the per-pixel variance of the luminance of
one path. Output: pt_oracle_crop.npz (1280x720) or pt_oracle_crop_1080.npz.
"""
from __future__ import annotations

import math
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
import oracle  # noqa: E402

CROPS = {(1280, 720): (576, 528, 128, 128), (1920, 1080): (896, 824, 128, 128)}
NAMES = {(1280, 720): "pt_oracle_crop.npz", (1920, 1080): "pt_oracle_crop_1080.npz"}
SUN_DIR = np.array([math.sin(math.radians(20)) * math.cos(math.radians(30)), math.sin(math.radians(30)),
                    math.cos(math.radians(20)) * math.cos(math.radians(30))], np.float32)


def scene(width=1280, height=720):
    sc = oracle.cornell_scene(0x5EED, 2, 64, 16)
    mats = oracle.cornell_materials(0x5EED, 2, 64)
    th = float(np.float32(math.tan(math.radians(45.0) / 2.0)))
    cam = oracle.camera((0, 0, 3.4), (0, 0, 0), (0, 1, 0), th, width, height)
    env = oracle.env_procedural(2048, 1024, SUN_DIR)
    return sc, mats, cam, env


def main():
    spp = int(sys.argv[1]) if len(sys.argv) > 1 else 4096
    res = (int(sys.argv[2]), int(sys.argv[3])) if len(sys.argv) > 3 else (1280, 720)
    CROP = CROPS[res]
    sc, mats, cam, env = scene(*res)
    bvh = oracle.CpuBVH(sc["xyz"], sc["indices"], 4)
    t0 = time.time()
    img, sq, stats = oracle.pt_render(True, sc["xyz"], sc["indices"], sc["tri_material"], mats, bvh, env, cam, spp,
                                      seed=0x0DDBA11, batch=0, max_depth=6, rr_depth=3, mis_mode=0, crop=CROP)
    dt = time.time() - t0
    lum = 0.2126 * img[..., 0] + 0.7152 * img[..., 1] + 0.0722 * img[..., 2]
    var = np.maximum(sq - lum * lum, 0.0)  # variance of one path's luminance
    out = ROOT / "tests" / "golden" / NAMES[res]
    np.savez_compressed(out, mean=img.astype(np.float32), lum_var=var.astype(np.float32), spp=np.int32(spp),
                        crop=np.int32(CROP), sun_dir=SUN_DIR, seconds=np.float32(dt),
                        rays=np.int64(stats))
    print(f"{spp} spp in {dt:.1f} s, mean {img.mean(axis=(0, 1))}, rays {stats}, written {out}")


if __name__ == "__main__":
    main()
