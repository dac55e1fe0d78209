"""Host side of the batched uneven workload: the Python PCG32 behind its parameters reproduces the
golden PCG32 stream, and the 32 scenes' parameters stay within the workload's ranges."""
import numpy as np

from vierkant_gb300 import geometry


def test_host_pcg32_matches_golden(golden):
    g = golden("rng")
    r = geometry._Pcg32(0x5EED, 1)
    out = np.array([r.next() for _ in range(4096)], np.uint32)
    assert np.array_equal(out, g["pcg32_5eed_1"])


def test_batch_scene_params():
    ps = [geometry.batch_scene_params(i) for i in range(32)]
    assert ps == [geometry.batch_scene_params(i) for i in range(32)]  # deterministic
    for p in ps:
        assert p["resolution"] in (256, 512, 768, 1024) and p["spp"] in (4, 16, 64)
        assert 3_082 <= p["triangles"] <= 2_000_000 + 3_072
        assert p["triangles"] == 10 + 3072 * p["spheres"]
    # log-uniform over [5k, 2M]: both ends of the range occur among 32 draws
    tris = sorted(p["triangles"] for p in ps)
    assert tris[0] < 20_000 and tris[-1] > 500_000
    assert len({p["resolution"] for p in ps}) == 4 and len({p["spp"] for p in ps}) == 3
