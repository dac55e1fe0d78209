"""The best equal-RMSE time a radiance cache could reach on the 1920x1080 Cornell workload, from the
FP64 oracle's variance split (TEST INFRASTRUCTURE: an analysis of the oracle, not product code).

    python -m oracle.nrc_bound [spp] [fork_segment]

The cache tracer ends every rendering path at the surface its segment `fork_segment` reaches (the
tracer's terminate_depth, 2: the third surface of a path) and adds the cache's estimate there. Even an
exact cache only removes the variance of the path's tail beyond that surface: with L = prefix + tail,
Var(L) = Var(prefix + E[tail | prefix]) + E[Var(tail | prefix)], and orc_pt_variance_split measures the
second term by tracing every sample's tail twice from a shared prefix. Over the 128x128 crop the RMSE
criterion weighs pixels by their variance, so an exact, free cache needs

    r = sum(var_plain - var_tail) / sum(var_plain)

times the plain tracer's samples for the same RMSE, and its time ratio is at least r times the cost of
a cache sample over a plain one. Prints r, the fraction of samples reaching the cut, and the extension
segments per sample of the cut and the full paths (the cost of an exact cache's sample in rays).
"""
from __future__ import annotations

import json
import math
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))
import oracle  # noqa: E402

CROP_1080 = (896, 824, 128, 128)
SUN_DIR = np.array([math.sin(math.radians(20)) * math.cos(math.radians(30)), math.sin(math.radians(30)),
                    math.cos(math.radians(20)) * math.cos(math.radians(30))], np.float32)


def split(spp=256, fork_segment=2, crop=CROP_1080, size=(1920, 1080), max_depth=6):
    sc = oracle.cornell_scene(0x5EED, 2, 64, 16)
    mats = oracle.cornell_materials(0x5EED, 2, 64)
    th = float(np.float32(math.tan(math.radians(45.0) / 2.0)))
    cam = oracle.camera((0, 0, 3.4), (0, 0, 0), (0, 1, 0), th, size[0], size[1])
    env = oracle.env_procedural(2048, 1024, SUN_DIR)
    bvh = oracle.CpuBVH(sc["xyz"], sc["indices"], 2)
    t0 = time.time()
    out, rays = oracle.pt_variance_split(sc["xyz"], sc["indices"], sc["tri_material"], mats, bvh, env, cam, spp,
                                         fork_segment, seed=0x0DDBA11, max_depth=max_depth, rr_depth=3, crop=crop)
    dt = time.time() - t0
    var_plain, var_tail, reach = out[..., 1], out[..., 2], out[..., 3]
    _, cut_rays = oracle.pt_variance_split(sc["xyz"], sc["indices"], sc["tri_material"], mats, bvh, env, cam, spp,
                                           fork_segment, seed=0x0DDBA11, max_depth=fork_segment + 1, rr_depth=3,
                                           crop=crop)
    n = crop[2] * crop[3] * spp
    return {"spp": spp, "fork_segment": fork_segment, "crop": list(crop), "seconds": round(dt, 1),
            "var_plain_mean": float(var_plain.mean()), "var_tail_mean": float(var_tail.mean()),
            "r_exact_cache": float((var_plain.sum() - var_tail.sum()) / var_plain.sum()),
            "reach_fraction": float(reach.mean()),
            "ext_rays_per_sample_plain": rays[0] / n, "ext_rays_per_sample_cut": cut_rays[0] / n,
            "shadow_rays_per_sample_plain": rays[1] / n, "shadow_rays_per_sample_cut": cut_rays[1] / n}


def main():
    spp = int(sys.argv[1]) if len(sys.argv) > 1 else 256
    fork = int(sys.argv[2]) if len(sys.argv) > 2 else 2
    print(json.dumps(split(spp, fork), indent=1))


if __name__ == "__main__":
    main()
