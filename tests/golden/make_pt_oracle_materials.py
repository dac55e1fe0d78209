"""Generate the FP64 radiance-oracle fixture for the Disney material set (CPU only, no reference needed).

    python tests/golden/make_pt_oracle_materials.py [spp]

Scene: the Cornell box + 64 cube-spheres of the plain fixture (PCG32 seed 0x5EED, stream 2) with the
spheres cycled through metal-rough, smooth glass (ior 1.5), rough glass (ior 1.33, roughness 0.35),
clearcoat, sheen and diffuse transmission (vierkant_gb300.geometry.showcase_materials). Environment:
the procedural 2048x1024 equirect sky with a broad sun lobe, 50 * exp((cos g - 1) / 0.02) toward
elevation 30 deg, azimuth 20 deg from +z, so that caustics through the glass stay finite-variance.
Camera (0,0,3.4) -> origin, fovy 45 deg, full frame at 256x144; max 8 segments, Russian roulette from
the 3rd interaction, MIS. Stores the mean radiance and the per-pixel variance of one path's luminance.
Output: pt_oracle_materials.npz.
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
from vierkant_gb300.geometry import showcase_materials  # noqa: E402

WIDTH, HEIGHT = 256, 144
SUN_PEAK, SUN_WIDTH = 50.0, 0.02
MAX_DEPTH = 8
SUN_DIR = np.array([math.sin(math.radians(20)) * math.cos(math.radians(30)), math.sin(math.radians(30)),
                    math.cos(math.radians(20)) * math.cos(math.radians(30))], np.float32)


def scene():
    sc = oracle.cornell_scene(0x5EED, 2, 64, 16)
    mats = showcase_materials(oracle.cornell_materials(0x5EED, 2, 64))
    th = float(np.float32(math.tan(math.radians(45.0) / 2.0)))
    cam = oracle.camera((0, 0, 3.4), (0, 0, 0), (0, 1, 0), th, WIDTH, HEIGHT)
    env = oracle.env_procedural(2048, 1024, SUN_DIR, SUN_PEAK, SUN_WIDTH)
    return sc, mats, cam, env


def main():
    spp = int(sys.argv[1]) if len(sys.argv) > 1 else 2048
    sc, mats, cam, env = scene()
    bvh = oracle.CpuBVH(sc["xyz"], sc["indices"], 4)
    t0 = time.time()
    img, sq, stats = oracle.pt_render(True, sc["xyz"], sc["indices"], sc["tri_material"], mats, bvh, env, cam, spp,
                                      seed=0x0DDBA11, batch=0, max_depth=MAX_DEPTH, rr_depth=3, mis_mode=0)
    dt = time.time() - t0
    lum = 0.2126 * img[..., 0] + 0.7152 * img[..., 1] + 0.0722 * img[..., 2]
    var = np.maximum(sq - lum * lum, 0.0)  # variance of one path's luminance
    out = ROOT / "tests" / "golden" / "pt_oracle_materials.npz"
    np.savez_compressed(out, mean=img.astype(np.float32), lum_var=var.astype(np.float32), spp=np.int32(spp),
                        size=np.int32((WIDTH, HEIGHT)), sun_dir=SUN_DIR, sun=np.float32((SUN_PEAK, SUN_WIDTH)),
                        max_depth=np.int32(MAX_DEPTH), seconds=np.float32(dt), rays=np.int64(stats))
    print(f"{spp} spp in {dt:.1f} s, mean {img.mean(axis=(0, 1))}, rays {stats}, written {out}")


if __name__ == "__main__":
    main()
