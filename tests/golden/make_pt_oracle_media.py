"""Generate the FP64 radiance-oracle fixture for homogeneous media (CPU only, no reference needed).

    python tests/golden/make_pt_oracle_media.py [spp]

Scene: the Cornell box + 16 cube-spheres (PCG32 seed 0x5EED, stream 2) with the spheres cycled
through metal-rough, fog (null surface, forward-scattering medium), absorbing glass, emissive gas
(null surface, absorbing and emitting medium) and scattering glass
(vierkant_gb300.geometry.media_materials); the spheres overlap, so media nest on the per-path stack.
Lit by one light of each analytic type (vierkant_gb300.pathtracer.cornell_lights) in a constant 0.2
environment: volume NEE toward the lights and the environment with the phase function, light shadow
rays through null surfaces and glass with Beer-Lambert attenuation. Camera (0,0,3.4) -> origin, fovy
45 deg, full frame at 256x144; max 10 segments, Russian roulette from the 3rd interaction, MIS.
Stores the mean radiance and the per-pixel variance of one path's luminance.
Output: pt_oracle_media.npz.
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
from vierkant_gb300.geometry import media_materials  # noqa: E402
from vierkant_gb300.pathtracer import cornell_lights  # noqa: E402

WIDTH, HEIGHT = 256, 144
MAX_DEPTH = 10
ENV = 0.2
NUM_SPHERES = 16


def lights():
    return cornell_lights().astype(oracle.LIGHT_DTYPE)


def scene():
    sc = oracle.cornell_scene(0x5EED, 2, NUM_SPHERES, 16)
    mats = media_materials(oracle.cornell_materials(0x5EED, 2, NUM_SPHERES))
    th = float(np.float32(math.tan(math.radians(45.0) / 2.0)))
    cam = oracle.camera((0, 0, 3.4), (0, 0, 0), (0, 1, 0), th, WIDTH, HEIGHT)
    env = np.full((64, 128, 3), ENV, np.float32)
    return sc, mats, cam, env


def main():
    spp = int(sys.argv[1]) if len(sys.argv) > 1 else 2048
    sc, mats, cam, env = scene()
    bvh = oracle.CpuBVH(sc["xyz"], sc["indices"], 4)
    t0 = time.time()
    img, sq, stats = oracle.pt_render(True, sc["xyz"], sc["indices"], sc["tri_material"], mats, bvh, env, cam, spp,
                                      seed=0x0DDBA11, batch=0, max_depth=MAX_DEPTH, rr_depth=3, mis_mode=0,
                                      lights=lights())
    dt = time.time() - t0
    lum = 0.2126 * img[..., 0] + 0.7152 * img[..., 1] + 0.0722 * img[..., 2]
    var = np.maximum(sq - lum * lum, 0.0)  # variance of one path's luminance
    out = ROOT / "tests" / "golden" / "pt_oracle_media.npz"
    np.savez_compressed(out, mean=img.astype(np.float32), lum_var=var.astype(np.float32), spp=np.int32(spp),
                        size=np.int32((WIDTH, HEIGHT)), max_depth=np.int32(MAX_DEPTH), env=np.float32(ENV),
                        num_spheres=np.int32(NUM_SPHERES), seconds=np.float32(dt), rays=np.int64(stats))
    print(f"{spp} spp in {dt:.1f} s, mean {img.mean(axis=(0, 1))}, rays {stats}, written {out}")


if __name__ == "__main__":
    main()
