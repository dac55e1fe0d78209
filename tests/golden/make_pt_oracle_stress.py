"""Generate the FP64 radiance-oracle fixture of the stress workload (CPU only, no reference needed).

    python tests/golden/make_pt_oracle_stress.py [spp]

Scene: vierkant_gb300.geometry.stress_scene() (2048^2-vertex fBm terrain + 100,000 instances of 20
cube-spheres, PCG32 seed 0x5EED), procedural 2048x1024 environment as the Cornell workload, camera
(0, 120, 300) -> origin, fovy 40 deg, 3840x2160, 8 segments, Russian roulette from the 3rd
interaction, MIS. The FP64 oracle (oracle/pathtrace.c, instanced path: a binary BVH over the exact
instance boxes, object-space double-precision traversal of each mesh's BVH, CDF environment
sampler) renders the 128x128 crop at (1856, 1016) with `spp` paths per pixel (default 1024) and
stores the mean radiance and the per-pixel variance of one path's luminance.
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
from vierkant_gb300 import geometry  # noqa: E402

CROP = (1856, 1016, 128, 128)
SUN_DIR = np.array([math.sin(math.radians(20)) * math.cos(math.radians(30)), math.sin(math.radians(30)),
                    math.cos(math.radians(20)) * math.cos(math.radians(30))], np.float32)


def main():
    spp = int(sys.argv[1]) if len(sys.argv) > 1 else 1024
    st = geometry.stress_scene()
    th = float(np.float32(math.tan(math.radians(40.0) / 2.0)))
    cam = oracle.camera((0, 120, 300), (0, 0, 0), (0, 1, 0), th, 3840, 2160)
    env = oracle.env_procedural(2048, 1024, SUN_DIR)
    inst = st["instances"]
    t0 = time.time()
    img, sq, rays = oracle.pt_render_instanced(st["meshes"], inst["transform"], inst["blas"], inst["material"],
                                               st["materials"], env, cam, spp, seed=0x0DDBA11, max_depth=8,
                                               rr_depth=3, crop=CROP)
    dt = time.time() - t0
    lum = 0.2126 * img[..., 0] + 0.7152 * img[..., 1] + 0.0722 * img[..., 2]
    var = np.maximum(sq - lum * lum, 0.0)
    out = ROOT / "tests" / "golden" / "pt_oracle_stress_crop.npz"
    np.savez_compressed(out, mean=img.astype(np.float32), lum_var=var.astype(np.float32), spp=np.int32(spp),
                        crop=np.int32(CROP), seconds=np.float32(dt), rays=np.int64(rays))
    print(f"{spp} spp in {dt:.1f} s, mean {img.mean(axis=(0, 1))}, rays {rays}, written {out}")


if __name__ == "__main__":
    main()
