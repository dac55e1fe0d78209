"""Benchmark: closest-hit ray casting over the 196,618-triangle Cornell + 64-sphere scene.

Workload (one step = one vkg_closest_hit launch over one resident batch):
  scene   : 5-quad Cornell box + 64 cube-spheres of 3,072 triangles (PCG32 seed 0x5EED, stream 2),
            fp32 xyz / uint32 indices, 8-wide BVH built on the GPU
  batch   : 1280x720 pixels x 4 spp camera rays (fovy 45 deg, eye (0,0,3.4) -> origin, PCG32 jitter,
            stream 2 + rank) plus one bounce ray per primary hit, leaving the hit point in a uniformly
            random direction (seeded torch RNG): coherent and incoherent rays in one batch
  metric  : Mrays/s closest-hit (hit ids bit-exact to brute force over the reference's ray-triangle
            test; the GPU tests check this on the same scene)
Inputs exceed L2 (rays + hits ~ 290 MB per step), so no explicit flush is needed between steps.

--impl reference: the reference's CPU ray cast (brute-force closest hit over all triangles with
vierkant's ray-triangle test, all host threads) on a bounded sample of the same batch.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WIDTH, HEIGHT, SPP = 1280, 720, 4
SEED = 0x5EED
NODE_BYTES, TRI_BYTES, RAY_BYTES, HIT_BYTES = 96, 48, 32, 16
METRIC = "Mrays/s closest-hit"
WORKLOAD = ("closest-hit, Cornell box + 64 cube-spheres (196,618 triangles), 1280x720x4 spp camera rays "
            "+ one uniform bounce ray per primary hit")


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x: float, device) -> float:
    """The largest of every rank's x: the slowest replica sets the whole job's time (a no-op without
    an initialised process group of more than one rank)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    t = torch.tensor([x], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank: int, world_size: int, ms: float) -> float:
    """Whole-job throughput of weak-scaled replicas in millions of units per second: every rank
    processed units_per_rank units in at most ms milliseconds."""
    return units_per_rank * world_size / (ms * 1e-3) / 1e6


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic_per_ray():
    """DRAM bytes per ray of the traversal kernel from the committed ncu capture summary, if any."""
    p = ROOT / "profiles" / "traversal_dram_bytes.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["dram_bytes_per_ray"])
        except (KeyError, ValueError):
            return None
    return None


def make_batch(ctx, bvh, rank):
    """camera rays + bounce rays from their hit points (built on the GPU, untimed)."""
    import torch
    from vierkant_gb300 import geometry
    cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, WIDTH, HEIGHT)
    prim = ctx.camera_rays(cam, SEED, 2 + rank, SPP)
    hits = bvh.closest_hit(prim)
    hit = hits[:, 0] != -1
    t = hits[:, 1].view(torch.float32)
    pos = prim[:, 0:3] + prim[:, 4:7] * t[:, None]
    g = torch.Generator(device=prim.device)
    g.manual_seed(SEED + rank)
    d = torch.randn((prim.shape[0], 3), device=prim.device, generator=g)
    d = d / d.norm(dim=1, keepdim=True)
    n2 = int(hit.sum())
    sec = torch.empty((n2, 8), device=prim.device, dtype=torch.float32)
    sec[:, 0:3] = pos[hit]
    sec[:, 3] = 1e-4
    sec[:, 4:7] = d[hit]
    sec[:, 7] = 1e4
    batch = torch.cat([prim, sec]).contiguous()
    del hits, pos, d, sec
    return batch


def run_ours(args):
    import numpy as np
    import torch
    import torch.distributed as dist
    from vierkant_gb300 import geometry
    from vierkant_gb300._lib import RAY_COUNT_STATS
    from vierkant_gb300.raytracing import BVH, Context

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        dist.init_process_group("nccl", device_id=torch.device(f"cuda:{local}"))
    ctx = Context(local)
    sc = geometry.cornell_scene(SEED, 2, 64, 16)
    bvh = BVH(ctx, torch.from_numpy(sc["xyz"]).cuda(), torch.from_numpy(sc["indices"].astype(np.int32)).cuda())
    info = bvh.info()
    batch = make_batch(ctx, bvh, rank)
    n = batch.shape[0]
    hits = torch.empty((n, 4), dtype=torch.int32, device=batch.device)

    # algorithmic work per ray, counted by the traversal itself (untimed; the GPU tests check these
    # counters against the CPU traversal of the same BVH)
    ctx.stats(reset=True)
    bvh.closest_hit(batch, hits, flags=RAY_COUNT_STATS)
    visits, tests = ctx.stats(reset=True)
    bytes_per_launch = n * (RAY_BYTES + HIT_BYTES) + visits * NODE_BYTES + tests * TRI_BYTES

    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        bvh.closest_hit(batch, hits)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        bvh.closest_hit(batch, hits)
    e1.record(stream)
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    ms_total = e0.elapsed_time(e1)
    clk = clocks.stop()
    ms_step = max_over_ranks(ms_total / args.steps, batch.device)
    value = replica_throughput(n, ws, ms_step)

    # end to end through the host-buffer entry point: H2D rays, trace, D2H hits, synchronise
    rays_host = batch.cpu().pin_memory()
    hits_host = torch.empty((n, 4), dtype=torch.int32).pin_memory()
    for _ in range(max(1, args.warmup // 2)):
        bvh.closest_hit_host(rays_host, hits_host)
    if ws > 1:
        dist.barrier()
    e2e_steps = max(3, args.steps // 2)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        bvh.closest_hit_host(rays_host, hits_host)
    e2e_ms = max_over_ranks((time.perf_counter() - t0) * 1e3 / e2e_steps, batch.device)
    e2e_value = replica_throughput(n, ws, e2e_ms)
    # the host-buffer results must equal the device results
    dev_hits = hits.cpu()
    e2e_ok = bool(torch.equal(dev_hits, hits_host))

    peak, peak_kind = measured_peaks()
    achieved = bytes_per_launch / (ms_step * 1e-3) / 1e9
    tpr = profiled_traffic_per_ray()
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": (round(tpr * n) if tpr is not None else None),
                "peak_source": peak_kind,
                "algorithmic_bytes_per_ray": round(bytes_per_launch / n, 1),
                "node_visits_per_ray": round(visits / n, 3), "tri_tests_per_ray": round(tests / n, 3),
                "note": "node (96 B) + triangle (48 B) reads per ray are served mostly from L2/L1; "
                        "HBM sees the 48 B/ray ray+hit stream"}

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        cpu = cpu_baseline(sc, batch, budget_s=args.cpu_seconds)
    pt_block = batch_block = stress = features = None
    if rank == 0 and not args.no_pt:
        pt_block = path_tracer_block(ctx, frames=args.nrc_frames)
        batch_block = batched_block(ctx)
        stress = stress_block(ctx)
        features = features_block(ctx)

    if rank == 0:
        line = {"metric": METRIC, "value": round(value, 1), "unit": "Mrays/s", "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(ms_step, 4), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": WORKLOAD, "triangles": int(info.num_tris), "rays_per_step": n,
                           "bvh_nodes": int(info.num_nodes), "bvh_depth": int(info.depth),
                           "bvh_build_ms": round(float(info.build_ms), 3), "leaf_max": int(info.leaf_max),
                           "l2": "inputs larger than L2 (%.0f MB rays+hits per step)" % (n * 48 / 1e6),
                           "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"},
                "e2e": {"value": round(e2e_value, 1), "unit": "Mrays/s", "h2d_bytes_per_step": n * RAY_BYTES,
                        "d2h_bytes_per_step": n * HIT_BYTES, "matches_device": e2e_ok},
                "gpu_launches": args.steps, "roofline": roofline, "clocks": clk}
        if cpu is not None:
            line["cpu_baseline"] = cpu
        if pt_block is not None:
            line["path_tracer"] = pt_block
        if batch_block is not None:
            line["batched"] = batch_block
        if stress is not None:
            line["stress"] = stress
        if features is not None:
            line["materials_lights"] = features
        print(json.dumps(line), flush=True)
    bvh.close()
    ctx.close()
    if ws > 1:
        dist.destroy_process_group()


def _lum(a):
    return 0.2126 * a[..., 0] + 0.7152 * a[..., 1] + 0.0722 * a[..., 2]


def _crop_error(img, golden):
    """(RMSE of the luminance, relative bias) of an image crop against the FP64 oracle fixture"""
    import numpy as np
    ref = golden["mean"].astype(np.float64)
    x0, y0, w, h = (int(v) for v in golden["crop"])
    c = img[y0:y0 + h, x0:x0 + w].astype(np.float64)
    return math.sqrt(float(np.mean((_lum(c) - _lum(ref)) ** 2))), float((c.sum() - ref.sum()) / ref.sum())


def denoise_timing(ctx, pixels, w, h, reps=20):
    """The a-trous denoise pass (5 passes) over a frame of pixel records: CUDA-event time per call on
    the context's stream, and its bytes against the measured HBM copy bandwidth. Bytes per pixel: the
    32-byte record read once, per pass the demodulated colour written and read (2 x 16 B), the
    geometry and albedo float4s (32 B) and the output (16 B) — the 25 taps per pass are L1/L2 hits."""
    import torch
    from vierkant_gb300.pathtracer import denoise
    for _ in range(3):
        denoise(ctx, pixels, w, h)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(torch.cuda.current_stream())
    for _ in range(reps):
        denoise(ctx, pixels, w, h)
    e1.record(torch.cuda.current_stream())
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    byts = w * h * (32 + 5 * (2 * 16 + 32 + 16) + 16)
    peak, src = measured_peaks()
    return {"ms": round(ms, 4), "mpix_per_s": round(w * h / ms / 1e3, 1), "bytes_per_pixel": byts // (w * h),
            "gbs": round(byts / ms / 1e6, 1), "frac_of_hbm": round(byts / ms / 1e6 / peak, 3), "peak": src}


def post_fx_timing(ctx, rgb, w, h, reps=20):
    """Bloom + tonemap (threshold to half resolution, 3 x 2 blur passes, composition) of one frame:
    CUDA-event time per call. Bytes per full-resolution pixel: the HDR image read twice (16 B each:
    threshold, composition) and the output (16 B); per half-resolution pixel the threshold write and
    2 x 3 blur passes reading and writing RGBA16F (8 B each) and the composition's read."""
    import torch
    from vierkant_gb300.pathtracer import post_fx
    hdr = torch.cat([rgb, torch.ones_like(rgb[..., :1])], dim=-1).contiguous()
    for _ in range(3):
        post_fx(ctx, hdr)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(torch.cuda.current_stream())
    for _ in range(reps):
        post_fx(ctx, hdr)
    e1.record(torch.cuda.current_stream())
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    byts = w * h * 48 + (w // 2) * (h // 2) * (8 + 6 * 16 + 8)
    peak, src = measured_peaks()
    return {"ms": round(ms, 4), "mpix_per_s": round(w * h / ms / 1e3, 1), "gbs": round(byts / ms / 1e6, 1),
            "frac_of_hbm": round(byts / ms / 1e6 / peak, 3), "peak": src}


def path_tracer_block(ctx, frames=256):
    """The radiance estimator on the same scene: the plain tracer at 1280x720 x 64 spp (samples/s,
    Mrays/s, RMSE / bias against the FP64 oracle crop), and the equal-RMSE comparison at 1920x1080:
    GPU time for the plain tracer's 64-spp image vs the radiance-cache tracer (1 spp per frame, trained
    online) to reach the same crop RMSE. Times are CUDA-event totals of the renders (training included)."""
    import numpy as np
    from vierkant_gb300 import geometry
    from vierkant_gb300.nrc import cache_for_scene
    from vierkant_gb300.pathtracer import PBRPathTracer, Scene, procedural_sky, sun_direction

    g720 = np.load(ROOT / "tests" / "golden" / "pt_oracle_crop.npz")
    g1080 = np.load(ROOT / "tests" / "golden" / "pt_oracle_crop_1080.npz")
    sc = geometry.cornell_scene(SEED, 2, 64, 16)
    env = procedural_sky(ctx, 2048, 1024, sun_direction(), 5e4, 3.8e-5)
    scene = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], sc["materials"], env)

    def settings(spp, w, h):
        s = PBRPathTracer.default_settings()
        s.num_samples, s.max_trace_depth, s.rr_start_depth = spp, 6, 3
        s.resolution[0], s.resolution[1] = w, h
        return s

    out = {}
    cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, 1280, 720)
    pt = PBRPathTracer(ctx, seed=SEED, settings=settings(64, 1280, 720))
    pt.render_scene(scene, cam)
    pt.reset_accumulator()
    img = pt.render_scene(scene, cam).cpu().numpy()
    st = pt.statistics()
    rmse, bias = _crop_error(img, g720)
    rays = st.extension_rays + st.shadow_rays
    out["plain_720p_64spp"] = {"ms": round(st.total_ms, 2), "samples_per_s": round(st.paths / st.total_ms * 1e3),
                               "mrays_per_s": round(rays / st.total_ms / 1e3, 1), "rays": int(rays),
                               "rmse": round(rmse, 4), "bias": round(bias, 5),
                               "oracle": "FP64 4096 spp, 128x128 crop at (576, 528)"}
    out["denoise_720p"] = denoise_timing(ctx, pt.pixel_data(), 1280, 720)
    out["post_fx_720p"] = post_fx_timing(ctx, pt.render_scene(scene, cam), 1280, 720)
    pt.close()

    cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, 1920, 1080)
    pt = PBRPathTracer(ctx, seed=SEED, settings=settings(64, 1920, 1080))
    pt.render_scene(scene, cam)
    pt.reset_accumulator()
    img = pt.render_scene(scene, cam).cpu().numpy()
    st = pt.statistics()
    target, pbias = _crop_error(img, g1080)
    plain_ms = st.total_ms
    pt.close()

    pt = PBRPathTracer(ctx, seed=SEED + 1, settings=settings(1, 1920, 1080))
    cache = cache_for_scene(ctx, scene)
    pt.attach_cache(cache)
    tot = render = train = 0.0
    reached = None
    rmse = bias = None
    for f in range(frames):
        img = pt.render_scene(scene, cam)
        st = pt.statistics()
        tot += st.total_ms
        render += st.raytrace_ms
        train += st.train_ms
        rmse, bias = _crop_error(img.cpu().numpy(), g1080)
        if reached is None and rmse <= target:
            reached = {"frames": f + 1, "ms": round(tot, 2)}
    pt.close()
    cache.close()
    scene.close()
    out["equal_rmse_1080p"] = {
        "rmse_target": round(target, 4), "plain_64spp_ms": round(plain_ms, 2), "plain_bias": round(pbias, 5),
        "nrc_reached": reached, "nrc_vs_plain_time": round(reached["ms"] / plain_ms, 3) if reached else None,
        "nrc_frames": frames, "nrc_ms_total": round(tot, 2), "nrc_ms_per_frame": round(tot / frames, 3),
        "nrc_render_ms_per_frame": round(render / frames, 3), "nrc_train_ms_per_frame": round(train / frames, 3),
        "nrc_rmse_final": round(rmse, 4), "nrc_bias_final": round(bias, 5),
        "oracle": "FP64 4096 spp, 128x128 crop at (896, 824)",
        "protocol": "1 spp per frame, 65,536 training paths per frame, terminate after 2 bounces"}
    return out


def features_block(ctx):
    """The full material and light set: the Cornell box with the showcase materials (glass, rough
    glass, clearcoat, sheen, diffuse transmission, iridescence, metal-rough), one light of every
    analytic type and a sun disc, and the same box with its spheres cycled through homogeneous media
    (fog, absorbing glass, emissive gas, scattering glass) and the same lights, against the box with
    metal-rough materials and no lights, all at 1280x720 x 64 spp, 8 segments (samples/s, Mrays/s).
    Parity: the 16-sphere lit scene and the 16-sphere media scene at 256x144 x 1024 spp against their
    FP64 oracles (4096 spp full frame)."""
    import math
    import numpy as np
    import torch
    from vierkant_gb300 import geometry
    from vierkant_gb300.pathtracer import PBRPathTracer, Scene, cornell_lights

    sun = dict(color=(1.0, 0.95, 0.9), intensity=3.0, coords=(math.radians(30), math.radians(200)), angular=0.05)

    def settings(spp, w, h, lit):
        s = PBRPathTracer.default_settings()
        s.num_samples, s.max_trace_depth, s.rr_start_depth = spp, 8, 3
        s.resolution[0], s.resolution[1] = w, h
        if lit:
            for c in range(3):
                s.sun_color[c] = sun["color"][c]
            s.sun_intensity = sun["intensity"]
            s.sun_spherical_coords[0], s.sun_spherical_coords[1] = sun["coords"]
            s.sun_angular_size = sun["angular"]
        return s

    env = torch.full((64, 128, 3), 0.1, dtype=torch.float32, device="cuda")
    out = {}
    sc = geometry.cornell_scene(SEED, 2, 64, 16)
    cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, 1280, 720)
    for name, mats, lit in (("plain_720p_64spp_8seg", sc["materials"], False),
                            ("materials_lights_720p_64spp_8seg", geometry.showcase_materials(sc["materials"]), True),
                            ("media_lights_720p_64spp_8seg", geometry.media_materials(sc["materials"]), True)):
        scene = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], mats, env)
        if lit:
            scene.set_lights(cornell_lights())
        pt = PBRPathTracer(ctx, seed=SEED, settings=settings(64, 1280, 720, lit))
        pt.render_scene(scene, cam)
        pt.reset_accumulator()
        pt.render_scene(scene, cam)
        st = pt.statistics()
        rays = st.extension_rays + st.shadow_rays
        out[name] = {"ms": round(st.total_ms, 2), "samples_per_s": round(st.paths / st.total_ms * 1e3),
                     "mrays_per_s": round(rays / st.total_ms / 1e3, 1), "rays": int(rays)}
        pt.close()
        scene.close()
    out["materials_lights_time_vs_plain"] = round(out["materials_lights_720p_64spp_8seg"]["ms"] /
                                                  out["plain_720p_64spp_8seg"]["ms"], 3)
    out["media_lights_time_vs_plain"] = round(out["media_lights_720p_64spp_8seg"]["ms"] /
                                              out["plain_720p_64spp_8seg"]["ms"], 3)
    g = np.load(ROOT / "tests" / "golden" / "pt_oracle_lights.npz")
    sc = geometry.cornell_scene(SEED, 2, int(g["num_spheres"]), 16)
    scene = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], geometry.showcase_materials(sc["materials"]),
                  env)
    scene.set_lights(cornell_lights())
    cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, 256, 144)
    pt = PBRPathTracer(ctx, seed=SEED, settings=settings(1024, 256, 144, True))
    img = pt.render_scene(scene, cam).cpu().numpy().astype(np.float64)
    pt.close()
    scene.close()
    ref = g["mean"].astype(np.float64)
    rmse = math.sqrt(np.mean((_lum(img) - _lum(ref)) ** 2))
    out["lights_parity_256x144_1024spp"] = {
        "rmse": round(rmse, 4), "bias": round(float((img.sum() - ref.sum()) / ref.sum()), 5),
        "expected_noise": round(math.sqrt(np.mean(g["lum_var"]) / 1024 + np.mean(g["lum_var"]) / int(g["spp"])), 4),
        "oracle": "FP64 %d spp, full frame" % int(g["spp"])}
    # media: fog, absorbing glass, emissive gas and scattering glass spheres, the analytic lights, a
    # constant 0.2 environment, 10 segments, against its FP64 oracle
    g = np.load(ROOT / "tests" / "golden" / "pt_oracle_media.npz")
    sc = geometry.cornell_scene(SEED, 2, int(g["num_spheres"]), 16)
    env_m = torch.full((64, 128, 3), float(g["env"]), dtype=torch.float32, device="cuda")
    scene = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], geometry.media_materials(sc["materials"]), env_m)
    scene.set_lights(cornell_lights())
    s = settings(1024, 256, 144, False)
    s.max_trace_depth = int(g["max_depth"])
    pt = PBRPathTracer(ctx, seed=SEED, settings=s)
    img = pt.render_scene(scene, cam).cpu().numpy().astype(np.float64)
    pt.close()
    scene.close()
    ref = g["mean"].astype(np.float64)
    rmse = math.sqrt(np.mean((_lum(img) - _lum(ref)) ** 2))
    out["media_parity_256x144_1024spp"] = {
        "rmse": round(rmse, 4), "bias": round(float((img.sum() - ref.sum()) / ref.sum()), 5),
        "expected_noise": round(math.sqrt(np.mean(g["lum_var"]) / 1024 + np.mean(g["lum_var"]) / int(g["spp"])), 4),
        "oracle": "FP64 %d spp, full frame" % int(g["spp"])}
    return out


def batched_block(ctx):
    """The batched uneven workload: 32 Cornell + cube-sphere scenes, triangle counts log-uniform in
    [5k, 2M], square resolutions from {256, 512, 768, 1024}, spp from {4, 16, 64} (PCG32 seed 0x5EED,
    stream 3 + scene), all rendered by one CUDA-graph launch per render after the autotuner picked the
    queue kernels, grid and wave size; beside it the same jobs one scene at a time through the
    single-scene tracer. Times are CUDA-event totals of whole renders."""
    import torch
    from vierkant_gb300 import geometry
    from vierkant_gb300.batch import BatchJob, BatchRenderer
    from vierkant_gb300.pathtracer import PBRPathTracer, Scene, procedural_sky, sun_direction

    env = procedural_sky(ctx, 2048, 1024, sun_direction(), 5e4, 3.8e-5)
    jobs, scenes, params = [], [], []
    for i in range(32):
        p = geometry.batch_scene_params(i)
        sc = geometry.cornell_scene(SEED, p["stream"], p["spheres"], 16)
        scene = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], sc["materials"], env)
        scenes.append(scene)
        params.append(p)
        r = p["resolution"]
        cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, r, r)
        s = PBRPathTracer.default_settings()
        s.resolution[0] = s.resolution[1] = r
        s.num_samples, s.max_trace_depth, s.rr_start_depth = p["spp"], 6, 3
        jobs.append(BatchJob(scene, cam, s, SEED + i))
    br = BatchRenderer(ctx, jobs)
    t0 = time.perf_counter()
    tun = br.autotune()
    tune_s = time.perf_counter() - t0
    br.render()
    ms = []
    for _ in range(2):
        br.render()
        st = br.statistics()
        ms.append(st.render_ms)
    rays = st.extension_rays + st.shadow_rays
    best = min(ms)
    seq_ms = 0.0
    for jb in jobs:
        pt = PBRPathTracer(ctx, seed=jb.seed, settings=jb.settings)
        pt.render_scene(jb.scene, jb.camera)
        seq_ms += pt.statistics().total_ms
        pt.close()
    br.close()
    for sc in scenes:
        sc.close()
    torch.cuda.synchronize()
    return {"scenes": 32, "triangles": sum(p["triangles"] for p in params), "paths": int(st.paths),
            "rays": int(rays), "render_ms": round(best, 2), "mrays_per_s": round(rays / best / 1e3, 1),
            "samples_per_s": round(st.paths / best * 1e3), "waves": int(st.waves),
            "tuning": {"extend_kernel": "persistent" if tun.extend_kernel == 2 else "grid-stride",
                       "ctas_per_sm": int(tun.ctas_per_sm), "wave_paths": int(tun.wave_paths),
                       "block_size": int(tun.block_size), "stack_depth": int(tun.stack_depth),
                       "autotune_s": round(tune_s, 2), "graph": True},
            "one_scene_at_a_time_ms": round(seq_ms, 2), "speedup_vs_one_at_a_time": round(seq_ms / best, 3)}


def stress_block(ctx):
    """The stress workload: an 8,380,418-triangle fBm terrain (2048^2 vertices) plus 100,000 instances of
    20 cube-spheres (5,292 to 50,700 triangles) under a two-level BVH, rendered at 3840x2160 x 16 spp,
    8 segments, Russian roulette from the 3rd interaction, environment as the Cornell workload."""
    import torch
    from vierkant_gb300 import geometry
    from vierkant_gb300.pathtracer import InstancedScene, PBRPathTracer, procedural_sky, sun_direction

    t0 = time.perf_counter()
    st = geometry.stress_scene()
    gen_s = time.perf_counter() - t0
    env = procedural_sky(ctx, 2048, 1024, sun_direction(), 5e4, 3.8e-5)
    t0 = time.perf_counter()
    scene = InstancedScene(ctx, st["meshes"], st["instances"], st["materials"], env)
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    W, H = 3840, 2160
    cam = geometry.camera_lookat((0, 120, 300), (0, 0, 0), (0, 1, 0), 40.0, W, H)
    s = PBRPathTracer.default_settings()
    s.resolution[0], s.resolution[1] = W, H
    s.num_samples, s.max_trace_depth, s.rr_start_depth = 16, 8, 3
    pt = PBRPathTracer(ctx, seed=SEED, settings=s)
    pt.render_scene(scene, cam)
    best = None
    for _ in range(2):
        pt.reset_accumulator()
        img = pt.render_scene(scene, cam)
        stt = pt.statistics()
        if best is None or stt.total_ms < best.total_ms:
            best = stt
    pt.close()
    tris = sum(len(m[1]) for m in st["meshes"])
    inst_tris = sum(len(st["meshes"][int(b)][1]) for b in st["instances"]["blas"])
    rays = best.extension_rays + best.shadow_rays
    out = {"terrain_triangles": len(st["meshes"][0][1]), "instances": len(st["instances"]) - 1,
           "mesh_triangles": tris, "instanced_triangles": int(inst_tris), "resolution": [W, H], "spp": 16,
           "segments": 8, "render_ms": round(best.total_ms, 1), "samples_per_s": round(best.paths / best.total_ms * 1e3),
           "mrays_per_s": round(rays / best.total_ms / 1e3, 1), "rays": int(rays),
           "generate_s": round(gen_s, 2), "scene_build_s": round(build_s, 2)}
    fixture = ROOT / "tests" / "golden" / "pt_oracle_stress_crop.npz"
    if fixture.exists():
        # the plain tracer's 16-spp image and the radiance-cache tracer (1 spp per frame) against the FP64
        # oracle crop: GPU time for the cache tracer to reach the plain tracer's RMSE
        import numpy as np
        g = np.load(fixture)
        target, pbias = _crop_error(img.cpu().numpy(), g)
        from vierkant_gb300.nrc import cache_for_scene
        s1 = PBRPathTracer.default_settings()
        s1.resolution[0], s1.resolution[1] = W, H
        s1.num_samples, s1.max_trace_depth, s1.rr_start_depth = 1, 8, 3
        ptc = PBRPathTracer(ctx, seed=SEED + 1, settings=s1)
        cache = cache_for_scene(ctx, scene)
        ptc.attach_cache(cache)
        tot, reached, rmse, bias = 0.0, None, None, None
        frames = 48
        for f in range(frames):
            im = ptc.render_scene(scene, cam)
            tot += ptc.statistics().total_ms
            rmse, bias = _crop_error(im.cpu().numpy(), g)
            if reached is None and rmse <= target:
                reached = {"frames": f + 1, "ms": round(tot, 1)}
                break
        ptc.close()
        cache.close()
        out["equal_rmse"] = {"oracle": "FP64 %d spp, 128x128 crop at (1856, 1016)" % int(g["spp"]),
                             "plain_16spp_rmse": round(target, 4), "plain_bias": round(pbias, 5),
                             "plain_16spp_ms": round(best.total_ms, 1), "nrc_reached": reached,
                             "nrc_vs_plain_time": round(reached["ms"] / best.total_ms, 3) if reached else None,
                             "nrc_frames_run": f + 1, "nrc_ms_total": round(tot, 1),
                             "nrc_rmse_last": round(rmse, 4), "nrc_bias_last": round(bias, 5)}
    scene.close()
    return out


def profile_case(name: str):
    """Small workloads for profiler captures (ncu): one case per call, no JSON line.
    pt-frame   plain path tracer, Cornell scene, 1280x720 x 4 spp
    nrc        radiance-cache kernels: 4 training steps of 65,536 records, inference of 262,144 queries
               with the mma.sync, tcgen05 and fused tcgen05 kernels
    batch      batched renderer, 4 scenes of the batched workload at 1 spp
    stress     instanced scene: 512^2 terrain + 10,000 instances, 960x540 x 2 spp, 8 segments
    features   Cornell scene with the showcase materials, the six analytic lights and a sun disc,
               1280x720 x 4 spp, 8 segments"""
    import numpy as np
    import torch
    from vierkant_gb300 import geometry
    from vierkant_gb300.raytracing import Context
    from vierkant_gb300.pathtracer import InstancedScene, PBRPathTracer, Scene, procedural_sky, sun_direction
    ctx = Context(0)
    env = procedural_sky(ctx, 2048, 1024, sun_direction(), 5e4, 3.8e-5)
    if name == "pt-frame":
        sc = geometry.cornell_scene(SEED, 2, 64, 16)
        scene = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], sc["materials"], env)
        cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, 1280, 720)
        s = PBRPathTracer.default_settings()
        s.num_samples, s.max_trace_depth, s.rr_start_depth = 4, 6, 3
        pt = PBRPathTracer(ctx, seed=SEED, settings=s)
        pt.render_scene(scene, cam)
    elif name == "nrc":
        from vierkant_gb300.nrc import NeuralRadianceCache
        g = torch.Generator(device="cuda").manual_seed(1)

        def feats(n):
            p = torch.rand((n, 3), device="cuda", generator=g) * 2 - 1
            d = torch.nn.functional.normalize(torch.randn((n, 3), device="cuda", generator=g), dim=1)
            nn_ = torch.nn.functional.normalize(torch.randn((n, 3), device="cuda", generator=g), dim=1)
            return torch.cat([p, d, nn_, torch.rand((n, 4), device="cuda", generator=g)], dim=1).contiguous()
        caches = []
        for kind in (1, 2, 3):
            cfg = NeuralRadianceCache.default_config()
            cfg.infer_kernel = kind
            caches.append(NeuralRadianceCache(ctx, cfg))
        x, t = feats(65536), torch.rand((65536, 3), device="cuda", generator=g)
        for _ in range(4):
            caches[0].train_step(x, t)
        q = feats(262144)
        for c in caches:
            c.infer(q)
    elif name == "batch":
        from vierkant_gb300.batch import BatchJob, BatchRenderer
        jobs = []
        for i in range(4):
            p = geometry.batch_scene_params(i)
            sc = geometry.cornell_scene(SEED, p["stream"], p["spheres"], 16)
            scene = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], sc["materials"], env)
            r = p["resolution"]
            cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, r, r)
            s = PBRPathTracer.default_settings()
            s.resolution[0] = s.resolution[1] = r
            s.num_samples, s.max_trace_depth, s.rr_start_depth = 1, 6, 3
            jobs.append(BatchJob(scene, cam, s, SEED + i))
        BatchRenderer(ctx, jobs).render()
    elif name == "stress":
        st = geometry.stress_scene(terrain_n=512, num_instances=10_000)
        scene = InstancedScene(ctx, st["meshes"], st["instances"], st["materials"], env)
        cam = geometry.camera_lookat((0, 120, 300), (0, 0, 0), (0, 1, 0), 40.0, 960, 540)
        s = PBRPathTracer.default_settings()
        s.resolution[0], s.resolution[1] = 960, 540
        s.num_samples, s.max_trace_depth, s.rr_start_depth = 2, 8, 3
        PBRPathTracer(ctx, seed=SEED, settings=s).render_scene(scene, cam)
    elif name == "features":
        import math
        from vierkant_gb300.pathtracer import cornell_lights
        sc = geometry.cornell_scene(SEED, 2, 64, 16)
        envc = torch.full((64, 128, 3), 0.1, dtype=torch.float32, device="cuda")
        scene = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], geometry.showcase_materials(sc["materials"]),
                      envc)
        scene.set_lights(cornell_lights())
        cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, 1280, 720)
        s = PBRPathTracer.default_settings()
        s.num_samples, s.max_trace_depth, s.rr_start_depth = 4, 8, 3
        s.sun_color[0] = s.sun_color[1] = s.sun_color[2] = 1.0
        s.sun_intensity, s.sun_angular_size = 3.0, 0.05
        s.sun_spherical_coords[0], s.sun_spherical_coords[1] = math.radians(30), math.radians(200)
        PBRPathTracer(ctx, seed=SEED, settings=s).render_scene(scene, cam)
    elif name == "media":
        from vierkant_gb300.pathtracer import cornell_lights
        sc = geometry.cornell_scene(SEED, 2, 64, 16)
        envc = torch.full((64, 128, 3), 0.1, dtype=torch.float32, device="cuda")
        scene = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], geometry.media_materials(sc["materials"]),
                      envc)
        scene.set_lights(cornell_lights())
        cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, 1280, 720)
        s = PBRPathTracer.default_settings()
        s.num_samples, s.max_trace_depth, s.rr_start_depth = 4, 8, 3
        PBRPathTracer(ctx, seed=SEED, settings=s).render_scene(scene, cam)
    else:
        raise SystemExit(f"unknown profile case {name}")
    torch.cuda.synchronize()
    print(f"profile case {name} done")


def cpu_reference_lib():
    """The reference's own ray-triangle code when it was compiled here (oracle/_ref), else the
    oracle's C port of it (bit-identical; checked by the tests)."""
    import oracle
    R = oracle.ref()
    if R is not None:
        return "reference", (lambda *a: R.vkref_closest_hit_bruteforce(*a))
    L = oracle.orc()
    return "port", (lambda *a: L.orc_closest_hit_bruteforce(*a))


def cpu_baseline(sc, batch_gpu, budget_s=12.0, sample_rays=None):
    """Time the reference's brute-force CPU ray cast over all host threads on a bounded, evenly
    strided sample of the batch (keeps the primary/bounce mix)."""
    import numpy as np
    import oracle
    kind, fn = cpu_reference_lib()
    rays = batch_gpu.cpu().numpy() if hasattr(batch_gpu, "cpu") else batch_gpu
    n = rays.shape[0]
    xyz = np.ascontiguousarray(sc["xyz"])
    idx = np.ascontiguousarray(sc["indices"])
    cores = os.cpu_count() or 1
    # calibrate on a small sample, then size the timed sample to the budget
    probe = np.ascontiguousarray(rays[:: max(1, n // 256)][:256])
    hits = np.zeros((len(probe), 4), np.uint32)
    t0 = time.perf_counter()
    fn(oracle.ptr(xyz), oracle.ptr(idx), idx.shape[0], oracle.ptr(probe), len(probe), oracle.ptr(hits), 0, 0)
    dt = max(time.perf_counter() - t0, 1e-6)
    m = sample_rays or int(max(256, min(n, len(probe) * budget_s / dt)))
    sample = np.ascontiguousarray(rays[:: max(1, n // m)][:m])
    hits = np.zeros((len(sample), 4), np.uint32)
    t0 = time.perf_counter()
    used = fn(oracle.ptr(xyz), oracle.ptr(idx), idx.shape[0], oracle.ptr(sample), len(sample), oracle.ptr(hits), 0,
              0)
    dt = time.perf_counter() - t0
    return {"value": round(len(sample) / dt / 1e6, 5), "unit": "Mrays/s", "cores": int(used or cores),
            "kind": kind,
            "sample": f"{len(sample)} rays (every {max(1, n // m)}th of the batch) x {idx.shape[0]} triangles, "
                      f"brute force, {dt:.1f} s"}


def run_reference(args):
    """Reference arm: the reference's CPU ray cast on the host cores (rank 0 only)."""
    ws, rank, local = dist_env()
    if rank != 0:
        return
    import numpy as np
    import torch
    from vierkant_gb300 import geometry
    sc = geometry.cornell_scene(SEED, 2, 64, 16)
    if torch.cuda.is_available():
        from vierkant_gb300.raytracing import BVH, Context
        ctx = Context(local)
        bvh = BVH(ctx, torch.from_numpy(sc["xyz"]).cuda(), torch.from_numpy(sc["indices"].astype(np.int32)).cuda())
        batch = make_batch(ctx, bvh, 0).cpu().numpy()
        bvh.close()
        ctx.close()
    else:
        raise SystemExit("the benchmark batch is generated on the GPU")
    per_step_budget = max(1.0, min(20.0, args.cpu_seconds / max(1, args.steps)))
    for _ in range(args.warmup):
        cpu_baseline(sc, batch, budget_s=0.2)
    results = [cpu_baseline(sc, batch, budget_s=per_step_budget) for _ in range(args.steps)]
    value = statistics.median(r["value"] for r in results)
    cb = dict(results[-1])
    cb["value"] = value
    line = {"metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD, "triangles": int(sc["indices"].shape[0])},
            "cpu_baseline": cb,
            "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-pt", action="store_true", help="skip the path-tracer / radiance-cache block")
    ap.add_argument("--nrc-frames", type=int, default=256)
    ap.add_argument("--profile-case", choices=["pt-frame", "nrc", "batch", "stress", "features", "media"], default=None,
                    help="run one small workload for a profiler capture and exit (no JSON line)")
    args = ap.parse_args()
    if args.profile_case:
        profile_case(args.profile_case)
        return
    if args.warmup < 3 and args.impl == "ours":
        print("note: timing rules want >= 3 warm-up steps", file=sys.stderr)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
