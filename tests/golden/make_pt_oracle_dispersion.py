"""Generate the FP64 radiance-oracle fixture for chromatic dispersion (CPU only, no reference needed).

    python tests/golden/make_pt_oracle_dispersion.py [spp]

The scene of pt_oracle_materials.npz (Cornell box + 64 showcase spheres, broad-sun sky, 256x144,
8 segments, Russian roulette from the 3rd interaction, MIS) with every transmissive sphere dispersive
(dispersion 3.0: vierkant_gb300.geometry.dispersive_materials). Stores the mean radiance and the
per-pixel variance of one path's luminance. Output: pt_oracle_dispersion.npz.
"""
from __future__ import annotations

import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests" / "golden"))
import oracle  # noqa: E402
from make_pt_oracle_materials import MAX_DEPTH, SUN_DIR, SUN_PEAK, SUN_WIDTH, WIDTH, HEIGHT, scene  # noqa: E402
from vierkant_gb300.geometry import dispersive_materials  # noqa: E402

DISPERSION = 3.0


def main():
    spp = int(sys.argv[1]) if len(sys.argv) > 1 else 4096
    sc, mats, cam, env = scene()
    mats = dispersive_materials(mats, DISPERSION)
    bvh = oracle.CpuBVH(sc["xyz"], sc["indices"], 4)
    t0 = time.time()
    img, sq, stats = oracle.pt_render(True, sc["xyz"], sc["indices"], sc["tri_material"], mats, bvh, env, cam, spp,
                                      seed=0x0DDBA11, batch=0, max_depth=MAX_DEPTH, rr_depth=3, mis_mode=0)
    dt = time.time() - t0
    lum = 0.2126 * img[..., 0] + 0.7152 * img[..., 1] + 0.0722 * img[..., 2]
    var = np.maximum(sq - lum * lum, 0.0)
    out = ROOT / "tests" / "golden" / "pt_oracle_dispersion.npz"
    np.savez_compressed(out, mean=img.astype(np.float32), lum_var=var.astype(np.float32), spp=np.int32(spp),
                        size=np.int32((WIDTH, HEIGHT)), sun_dir=SUN_DIR, sun=np.float32((SUN_PEAK, SUN_WIDTH)),
                        max_depth=np.int32(MAX_DEPTH), dispersion=np.float32(DISPERSION), seconds=np.float32(dt),
                        rays=np.int64(stats))
    print(f"{spp} spp in {dt:.1f} s, mean {img.mean(axis=(0, 1))}, rays {stats}, written {out}")


if __name__ == "__main__":
    main()
