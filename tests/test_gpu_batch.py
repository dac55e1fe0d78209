"""Batched uneven rendering (vkg_batch_*): every job's image equals the single-scene tracer's render of
the same scene, camera, settings and seed, bit for bit, whatever the tuning (queue kernels, grid,
wave size, CUDA graph or not) and across accumulated batches; the autotuner keeps one of its
candidates and leaves the images unchanged."""
import numpy as np
import pytest
import torch

from vierkant_gb300 import geometry
from vierkant_gb300.batch import BatchJob, BatchRenderer
from vierkant_gb300.pathtracer import PBRPathTracer, Scene, procedural_sky, sun_direction

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def jobs(ctx):
    env = procedural_sky(ctx, 512, 256, sun_direction(), 5e4, 3.8e-5)
    out = []
    specs = [  # (spheres, tess, width, height, crop, spp, depth, rr, mis, seed)
        (3, 8, 64, 48, None, 3, 6, 3, 0, 11),
        (1, 4, 96, 64, None, 5, 4, 0, 1, 12),
        (6, 8, 1280, 720, (600, 500, 40, 24), 1, 6, 3, 0, 13),
        (12, 16, 128, 128, None, 8, 8, 2, 2, 14),
    ]
    scenes = []
    for k, (ns, tess, w, h, crop, spp, depth, rr, mis, seed) in enumerate(specs):
        sc = geometry.cornell_scene(0x5EED, 3 + k, ns, tess)
        scene = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], sc["materials"], env)
        scenes.append(scene)
        cam = geometry.camera_lookat((0, 0, 3.4), (0.1 * k, 0, 0), (0, 1, 0), 45.0 + 5 * k, w, h)
        s = PBRPathTracer.default_settings()
        s.resolution[0], s.resolution[1] = w, h
        s.num_samples, s.max_trace_depth, s.rr_start_depth, s.mis_mode = spp, depth, rr, mis
        if crop:
            for i in range(4):
                s.crop[i] = crop[i]
        out.append(BatchJob(scene, cam, s, seed))
    yield out
    for s in scenes:
        s.close()


def single(ctx, job, renders):
    pt = PBRPathTracer(ctx, seed=job.seed, settings=job.settings)
    for _ in range(renders):
        img = pt.render_scene(job.scene, job.camera).clone()
    pt.close()
    return img


@pytest.mark.parametrize("extend,cps,wave,graph,bs,stack", [(1, 16, 8 << 20, 1, 128, 128), (2, 8, 20_000, 1, 64, 64),
                                                             (1, 4, 5_000, 0, 64, 128), (2, 16, 1024, 0, 128, 64)])
def test_batch_equals_single_scene_tracer(ctx, jobs, extend, cps, wave, graph, bs, stack):
    t = BatchRenderer.default_tuning()
    t.extend_kernel, t.ctas_per_sm, t.wave_paths, t.use_graph = extend, cps, wave, graph
    t.block_size, t.stack_depth = bs, stack
    br = BatchRenderer(ctx, jobs, t)
    for r in (1, 2):
        imgs = [i.clone() for i in br.render()]
        torch.cuda.synchronize()
        for k, job in enumerate(jobs):
            ref = single(ctx, job, r)
            assert torch.equal(imgs[k], ref), (k, r, (imgs[k] - ref).abs().max().item())
    st = br.statistics()
    assert st.batch == 2 and st.render_ms > 0 and st.extension_rays > 0
    assert st.paths == sum(j.settings.num_samples * imgs[k].shape[0] * imgs[k].shape[1] for k, j in enumerate(jobs))
    if wave <= 20_000:
        assert st.waves > len(jobs)  # jobs were split across waves
    br.close()


def test_autotune_keeps_images(ctx, jobs):
    br = BatchRenderer(ctx, jobs)
    t = br.autotune()
    assert t.extend_kernel in (1, 2) and t.ctas_per_sm in (8, 16) and t.wave_paths in (8 << 20, 16 << 20)
    assert t.block_size in (64, 128) and t.stack_depth in (64, 128)
    assert br.statistics().batch == 0
    imgs = [i.clone() for i in br.render()]
    for k, job in enumerate(jobs):
        assert torch.equal(imgs[k], single(ctx, job, 1))
    br.reset_accumulator()
    again = [i.clone() for i in br.render()]
    assert all(torch.equal(a, b) for a, b in zip(imgs, again))
    br.close()


@pytest.mark.parametrize("extend,lit", [(1, False), (2, False), (1, True)])
def test_batch_textures_and_alpha_equal_single_scene_tracer(ctx, extend, lit):
    """jobs with textures (the textured Cornell scene) and with alpha-tested materials (the alpha
    scene) render in a batch bit for bit like the tracer renders them; an untextured job of the same
    batch shades with the textured variant and equals its tracer render up to that variant's rounding.
    lit: the alpha scene also has the analytic lights (light shadow rays through the coverage test);
    the other jobs then shade with the batch's full variant, equal up to its rounding"""
    from vierkant_gb300.pathtracer import cornell_lights
    env = procedural_sky(ctx, 256, 128, sun_direction(), 50.0, 0.02)
    scenes, jobs = [], []
    for k, (mats_of, tex) in enumerate(((geometry.alpha_materials, geometry.alpha_textures()),
                                        (geometry.textured_materials, geometry.test_textures()),
                                        (None, None))):
        sc = geometry.cornell_scene(0x5EED, 2, 8, 8)
        mats = mats_of(sc["materials"]) if mats_of else sc["materials"]
        scene = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], mats, env)
        if tex is not None:
            uv, tg = geometry.cornell_texcoords(sc)
            scene.set_normals(geometry.cornell_vertex_normals(sc))
            scene.set_texcoords(uv)
            scene.set_tangents(tg)
            scene.set_textures(tex)
        if lit and k == 0:
            scene.set_lights(cornell_lights())
        scenes.append(scene)
        w, h = (160, 96) if k < 2 else (64, 48)
        cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, w, h)
        s = PBRPathTracer.default_settings()
        s.resolution[0], s.resolution[1] = w, h
        s.num_samples, s.max_trace_depth, s.rr_start_depth = 4, 6, 3
        jobs.append(BatchJob(scene, cam, s, 21 + k))
    t = BatchRenderer.default_tuning()
    t.extend_kernel = extend
    br = BatchRenderer(ctx, jobs, t)
    imgs = [i.clone() for i in br.render()]
    torch.cuda.synchronize()
    for k, job in enumerate(jobs):
        ref = single(ctx, job, 1)
        if k == 0 or (k == 1 and not lit):
            assert torch.equal(imgs[k], ref), (k, (imgs[k] - ref).abs().max().item())
        else:
            a, b = imgs[k].cpu().numpy().astype(np.float64), ref.cpu().numpy().astype(np.float64)
            close = np.mean(np.all(np.abs(a - b) <= 1e-3 * np.maximum(np.abs(b), 1e-2), axis=-1))
            assert close > 0.97, close
    br.close()
    for s in scenes:
        s.close()
