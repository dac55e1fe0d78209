"""Material-class grouping of the shade queue (k_pt_bin_count / k_pt_bin_scatter) changes only which
warp shades which path: each path's result depends on its own state alone, so a render with the
grouping equals one in queue order (VKG_PT_BINNING=0) bit for bit, ray counts included."""
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
SCRIPT = r'''
import sys, numpy as np, torch
sys.path.insert(0, sys.argv[1])
from vierkant_gb300 import geometry
from vierkant_gb300.raytracing import Context
from vierkant_gb300.pathtracer import PBRPathTracer, Scene, cornell_lights
ctx = Context(0)
sc = geometry.cornell_scene(0x5EED, 2, 16, 16)
mats = geometry.showcase_materials(sc["materials"]) if sys.argv[3] == "showcase" else geometry.media_materials(sc["materials"])
env = torch.full((32, 64, 3), 0.3, dtype=torch.float32, device="cuda")
scene = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], mats, env)
scene.set_lights(cornell_lights())
cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, 96, 54)
s = PBRPathTracer.default_settings()
s.resolution[0], s.resolution[1] = 96, 54
s.num_samples, s.max_trace_depth, s.rr_start_depth = 8, 8, 3
pt = PBRPathTracer(ctx, seed=3, settings=s)
img = pt.render_scene(scene, cam).cpu().numpy()
st = pt.statistics()
np.savez(sys.argv[2], img=img, rays=np.array([st.extension_rays, st.shadow_rays], np.int64))
'''


def _render(tmp_path, binning, kind):
    out = tmp_path / f"{kind}_{binning}.npz"
    env = dict(os.environ, VKG_PT_BINNING=binning)
    subprocess.run([sys.executable, "-c", SCRIPT, str(ROOT), str(out), kind], env=env, check=True, timeout=600)
    return np.load(out)


@pytest.mark.parametrize("kind", ["showcase", "media"])
def test_grouping_is_bit_exact(tmp_path, kind):
    a = _render(tmp_path, "1", kind)
    b = _render(tmp_path, "0", kind)
    assert np.array_equal(a["rays"], b["rays"])
    assert a["img"].tobytes() == b["img"].tobytes()
