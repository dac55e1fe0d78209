"""Generate the FP64 radiance-oracle fixture for the plain path tracer (CPU only, no reference needed).

    python tests/golden/make_pt_oracle.py [spp]

Scene: Cornell box + 64 cube-spheres (PCG32 seed 0x5EED, stream 2), procedural 2048x1024 equirect
environment (environment_white gradient + sun lobe 5e4 * exp((cos g - 1) / 3.8e-5) toward elevation
30 deg, azimuth 20 deg from +z), camera (0,0,3.4) -> origin, fovy 45 deg, 1280x720, max 6 segments,
Russian roulette from the 3rd interaction, MIS. The oracle (oracle/pathtrace.c, FP64, independent
CDF environment sampler) renders the 128x128 crop at (576, 528) with `spp` paths per pixel (default
4096) and stores the mean radiance plus the per-pixel variance of the luminance of one path.
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

CROP = (576, 528, 128, 128)
SUN_DIR = np.array([math.sin(math.radians(20)) * math.cos(math.radians(30)), math.sin(math.radians(30)),
                    math.cos(math.radians(20)) * math.cos(math.radians(30))], np.float32)


def scene():
    sc = oracle.cornell_scene(0x5EED, 2, 64, 16)
    mats = oracle.cornell_materials(0x5EED, 2, 64)
    th = float(np.float32(math.tan(math.radians(45.0) / 2.0)))
    cam = oracle.camera((0, 0, 3.4), (0, 0, 0), (0, 1, 0), th, 1280, 720)
    env = oracle.env_procedural(2048, 1024, SUN_DIR)
    return sc, mats, cam, env


def main():
    spp = int(sys.argv[1]) if len(sys.argv) > 1 else 4096
    sc, mats, cam, env = scene()
    bvh = oracle.CpuBVH(sc["xyz"], sc["indices"], 4)
    t0 = time.time()
    img, sq, stats = oracle.pt_render(True, sc["xyz"], sc["indices"], sc["tri_material"], mats, bvh, env, cam, spp,
                                      seed=0x0DDBA11, batch=0, max_depth=6, rr_depth=3, mis_mode=0, crop=CROP)
    dt = time.time() - t0
    lum = 0.2126 * img[..., 0] + 0.7152 * img[..., 1] + 0.0722 * img[..., 2]
    var = np.maximum(sq - lum * lum, 0.0)  # variance of one path's luminance
    out = ROOT / "tests" / "golden" / "pt_oracle_crop.npz"
    np.savez_compressed(out, mean=img.astype(np.float32), lum_var=var.astype(np.float32), spp=np.int32(spp),
                        crop=np.int32(CROP), sun_dir=SUN_DIR, seconds=np.float32(dt),
                        rays=np.int64(stats))
    print(f"{spp} spp in {dt:.1f} s, mean {img.mean(axis=(0, 1))}, rays {stats}, written {out}")


if __name__ == "__main__":
    main()
