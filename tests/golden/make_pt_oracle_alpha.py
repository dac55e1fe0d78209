"""Generate the FP64 radiance-oracle fixture for alpha-masked / blended materials (CPU only, no
reference needed).

    python tests/golden/make_pt_oracle_alpha.py [spp]

The scene, camera, environment and crop of pt_oracle_crop.npz (make_pt_oracle.py) with smooth vertex
normals (geometry.cornell_vertex_normals), texture coordinates and tangents
(geometry.cornell_texcoords), the textures of geometry.alpha_textures() and the materials of
geometry.alpha_materials(): the left wall masked by a cut-out texture, the spheres in turn masked by
the cut-out, blended by a ramp texture, blended at alpha 0.4, or opaque. Stores the mean radiance and
the per-pixel variance of one path's luminance. Output: pt_oracle_alpha.npz.
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
from make_pt_oracle import CROPS, SUN_DIR, scene  # noqa: E402
from vierkant_gb300.geometry import (alpha_materials, alpha_textures, cornell_texcoords,  # noqa: E402
                                     cornell_vertex_normals)


def main():
    spp = int(sys.argv[1]) if len(sys.argv) > 1 else 4096
    crop = CROPS[(1280, 720)]
    sc, mats, cam, env = scene(1280, 720)
    uv, tg = cornell_texcoords(sc)
    bvh = oracle.CpuBVH(sc["xyz"], sc["indices"], 4)
    t0 = time.time()
    img, sq, stats = oracle.pt_render(True, sc["xyz"], sc["indices"], sc["tri_material"], alpha_materials(mats),
                                      bvh, env, cam, spp, seed=0x0DDBA11, batch=0, max_depth=6, rr_depth=3,
                                      mis_mode=0, crop=crop, normals=cornell_vertex_normals(sc), uv=uv, tangents=tg,
                                      textures=alpha_textures())
    dt = time.time() - t0
    lum = 0.2126 * img[..., 0] + 0.7152 * img[..., 1] + 0.0722 * img[..., 2]
    var = np.maximum(sq - lum * lum, 0.0)
    out = ROOT / "tests" / "golden" / "pt_oracle_alpha.npz"
    np.savez_compressed(out, mean=img.astype(np.float32), lum_var=var.astype(np.float32), spp=np.int32(spp),
                        crop=np.int32(crop), sun_dir=SUN_DIR, seconds=np.float32(dt), rays=np.int64(stats))
    print(f"{spp} spp in {dt:.1f} s, mean {img.mean(axis=(0, 1))}, rays {stats}, written {out}")


if __name__ == "__main__":
    main()
