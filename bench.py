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
BIN_MIN_RAYS = 1 << 19  # vkg_closest_hit traces batches this large in bins
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


def traversal_sources_digest():
    """sha256 prefix of the closest-hit kernel's sources (traverse.cu, traverse.cuh, vkg_common.cuh):
    the committed capture summary records the digest of the sources it was taken on, so a bench line
    says whether its traffic figure still describes the kernel it timed"""
    import hashlib
    h = hashlib.sha256()
    for f in ("traverse.cu", "traverse.cuh", "vkg_common.cuh"):
        h.update((ROOT / "vierkant_gb300" / "csrc" / f).read_bytes())
    return h.hexdigest()[:16]


def profiled_counters():
    """Per-ray DRAM bytes and issue statistics of the traversal kernel from the committed ncu capture
    summary (one launch on this batch), or None. These are profile figures: the bench cannot read
    hardware counters while it times."""
    p = ROOT / "profiles" / "k_trace_cornell_mixed_batch.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except ValueError:
            return None
    return None


# ---- the benchmark batch, built identically by both arms -------------------------------------------
PCG_MULT = 6364136223846793005
_M64 = (1 << 64) - 1


def _pcg_output(old):
    import numpy as np
    xs = (((old >> np.uint64(18)) ^ old) >> np.uint64(27)).astype(np.uint32)
    rot = (old >> np.uint64(59)).astype(np.uint32)
    return (xs >> rot) | (xs << ((np.uint32(32) - rot) & np.uint32(31)))


def pcg32_fill(seed: int, stream: int, count: int, lanes: int = 4096):
    """The first `count` outputs of PCG32 (O'Neill's pcg32_random_r, seeded with pcg32_srandom_r(seed,
    stream)) as uint32, computed by `lanes` interleaved generators that each start at their offset
    with the LCG jump-ahead."""
    import numpy as np
    inc = ((stream << 1) | 1) & _M64
    state = inc
    state = (state + seed) & _M64
    state = (state * PCG_MULT + inc) & _M64
    per = -(-count // lanes) if count else 0
    delta = np.arange(lanes, dtype=np.uint64) * np.uint64(per)
    acc_mult = np.ones(lanes, np.uint64)
    acc_plus = np.zeros(lanes, np.uint64)
    cur_mult, cur_plus = PCG_MULT, inc
    d = delta.copy()
    while d.any():
        sel = (d & np.uint64(1)).astype(bool)
        acc_plus = np.where(sel, acc_plus * np.uint64(cur_mult) + np.uint64(cur_plus), acc_plus)
        acc_mult = np.where(sel, acc_mult * np.uint64(cur_mult), acc_mult)
        cur_plus = ((cur_mult + 1) * cur_plus) & _M64
        cur_mult = (cur_mult * cur_mult) & _M64
        d >>= np.uint64(1)
    st = acc_mult * np.uint64(state) + acc_plus
    out = np.empty((lanes, per), np.uint32)
    m, c = np.uint64(PCG_MULT), np.uint64(inc)
    for k in range(per):
        out[:, k] = _pcg_output(st)
        st = st * m + c
    return out.reshape(-1)[:count]


def bounce_batch(prim, hits, stream: int):
    """The benchmark batch from the camera rays `prim` ((n, 8) float32 ray records) and their closest
    hits `hits` ((n, 4) uint32 hit records): the camera rays, then for every primary hit, in ray order,
    a ray from the hit point o + d*t (float32) in a uniformly random direction. Primary ray r draws
    PCG32(0x5EED, stream) outputs 2r and 2r+1: z = 1 - 2 u1, phi = 2 pi u2 (u = (x >> 8) 2^-24)."""
    import numpy as np
    n = prim.shape[0]
    hit = hits[:, 0] != 0xFFFFFFFF
    t = hits[:, 1].view(np.float32)
    x = pcg32_fill(SEED, stream, 2 * n)
    u1 = (x[0::2] >> 8).astype(np.float64) * 2.0 ** -24
    u2 = (x[1::2] >> 8).astype(np.float64) * 2.0 ** -24
    z = 1.0 - 2.0 * u1
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    phi = 2.0 * math.pi * u2
    d = np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1).astype(np.float32)
    pos = prim[:, 0:3] + prim[:, 4:7] * t[:, None]
    nh = int(hit.sum())
    sec = np.empty((nh, 8), np.float32)
    sec[:, 0:3] = pos[hit]
    sec[:, 3] = np.float32(1e-4)
    sec[:, 4:7] = d[hit]
    sec[:, 7] = np.float32(1e4)
    return np.ascontiguousarray(np.concatenate([prim, sec]))


def batch_digest(batch) -> str:
    import hashlib
    return hashlib.sha256(batch.tobytes()).hexdigest()[:16]


def bench_config(num_tris: int, batch) -> dict:
    """The workload description both arms print: identical for the same scene and batch."""
    n = batch.shape[0]
    return {"workload": WORKLOAD, "triangles": int(num_tris), "rays_per_step": int(n),
            "batch_sha256_16": batch_digest(batch),
            "l2": "inputs larger than L2 (%.0f MB rays+hits per step)" % (n * 48 / 1e6)}


def make_batch(ctx, bvh, rank):
    """camera rays and their hits on the GPU (untimed), the bounce rays on the host, uploaded"""
    import numpy as np
    import torch
    from vierkant_gb300 import geometry
    cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, WIDTH, HEIGHT)
    prim = ctx.camera_rays(cam, SEED, 2 + rank, SPP)
    hits = bvh.closest_hit(prim)
    batch = bounce_batch(prim.cpu().numpy(), hits.cpu().numpy().view(np.uint32), 4 + rank)
    del prim, hits
    return torch.from_numpy(batch).cuda(), batch


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
    batch, batch_np = make_batch(ctx, bvh, rank)
    config = bench_config(sc["indices"].shape[0], batch_np)
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
    # per-call wall times (each call synchronises); the median call, so that one slow host-side call
    # does not set the figure; the mean is reported beside it
    e2e_steps = max(10, args.steps)
    e2e_times = []
    for _ in range(e2e_steps):
        t0 = time.perf_counter()
        bvh.closest_hit_host(rays_host, hits_host)
        e2e_times.append((time.perf_counter() - t0) * 1e3)
    e2e_ms = max_over_ranks(statistics.median(e2e_times), batch.device)
    e2e_mean_ms = max_over_ranks(statistics.mean(e2e_times), batch.device)
    e2e_value = replica_throughput(n, ws, e2e_ms)
    # the host-buffer results must equal the device results
    dev_hits = hits.cpu()
    e2e_ok = bool(torch.equal(dev_hits, hits_host))
    hits_digest = batch_digest(dev_hits.numpy())

    # per call: five ray-binning kernels (batches of 2^19 rays or more) and the traversal kernel
    launches_per_call = 6 if n >= BIN_MIN_RAYS else 1
    peak, peak_kind = measured_peaks()
    achieved = bytes_per_launch / (ms_step * 1e-3) / 1e9
    prof = profiled_counters()
    roofline = {"bound": "issue", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": None, "peak_source": peak_kind,
                "algorithmic_bytes_per_ray": round(bytes_per_launch / n, 1),
                "node_visits_per_ray": round(visits / n, 3), "tri_tests_per_ray": round(tests / n, 3),
                "note": "achieved/frac: algorithmic bytes (48 B ray+hit, 96 B per node visit, 48 B per "
                        "triangle test) per second against the measured HBM copy bandwidth, over the whole "
                        "call (the ray-binning kernels included); the node and triangle reads are L1/L2 "
                        "hits, so the traversal's limiter is instruction issue, not DRAM (dram_frac)"}
    if prof is not None:
        dram = prof["dram_bytes_per_ray"] * n
        roofline.update({
            "traffic": round(dram), "traffic_source": "profile: " + prof["source"],
            # the capture was taken on the sources the bench runs (else the figure is stale)
            "traffic_current": prof.get("sources_sha256_16") == traversal_sources_digest(),
            "dram_frac": round(dram / (ms_step * 1e-3) / 1e9 / peak, 4),
            "threads_per_instruction": prof.get("threads_per_instruction"),
            "warp_instructions_per_ray": prof.get("warp_instructions_per_ray"),
            "alu_pipe_pct": prof.get("alu_pipe_pct")})

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        cpu = cpu_baseline(sc, batch_np, budget_s=args.cpu_seconds)
    c1 = None
    if rank == 0 and not args.no_pt:
        c1 = config1_block(ctx, args, run_cpu=(ws == 1 and not args.no_cpu))
    pt_block = batch_block = stress = features = None
    if rank == 0 and not args.no_pt:
        pt_block = path_tracer_block(ctx, frames=args.nrc_frames, bytes_per_ray=bytes_per_launch / n,
                                     cpu=(ws == 1 and not args.no_cpu))
        batch_block = batched_block(ctx)
        stress = stress_block(ctx, cpu=(ws == 1 and not args.no_cpu))
        twin = pt_block.get("plain_720p_64spp", {}).get("cpu_baseline")
        if twin:
            # the batched jobs on the host cores, extrapolated from the FP32 twin's per-sample rate on
            # the Cornell crop (the same scene family, 6 segments)
            cpu_s = batch_block["paths"] / twin["value"]
            batch_block["cpu_baseline"] = {
                "value": round(batch_block["rays"] / cpu_s / 1e6, 4), "unit": "Mrays/s", "cores": twin["cores"],
                "kind": "port", "sample": "extrapolated: %d paths at the FP32 twin's %.0f samples/s on the Cornell "
                                          "crop = %.0f s" % (batch_block["paths"], twin["value"], cpu_s)}
        batch_block["traversal_roofline"] = {
            "achieved": round(batch_block["rays"] * bytes_per_launch / n / (batch_block["render_ms"] * 1e-3) / 1e9, 1),
            "unit": "GB/s", "peak": measured_peaks()[0], "peak_source": measured_peaks()[1],
            "bytes_per_ray": round(bytes_per_launch / n, 1),
            "note": "rays x the closest-hit batch's algorithmic bytes per ray over the whole render time"}
        batch_block["traversal_roofline"]["frac"] = round(batch_block["traversal_roofline"]["achieved"] /
                                                          batch_block["traversal_roofline"]["peak"], 4)
        features = features_block(ctx)

    if rank == 0:
        line = {"metric": METRIC, "value": round(value, 1), "unit": "Mrays/s", "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(ms_step, 4), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": config,
                "gpu_config": {"bvh_nodes": int(info.num_nodes), "bvh_depth": int(info.depth),
                               "bvh_build_ms": round(float(info.build_ms), 3), "leaf_max": int(info.leaf_max),
                               "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"},
                "hits_sha256_16": hits_digest,
                "e2e": {"value": round(e2e_value, 1), "unit": "Mrays/s", "h2d_bytes_per_step": n * RAY_BYTES,
                        "d2h_bytes_per_step": n * HIT_BYTES, "matches_device": e2e_ok,
                        "timing": f"median of {e2e_steps} host-buffer calls (wall clock, each synchronised)",
                        "mean_value": round(replica_throughput(n, ws, e2e_mean_ms), 1)},
                "gpu_launches": args.steps * launches_per_call, "roofline": roofline, "clocks": clk}
        if cpu is not None:
            line["cpu_baseline"] = cpu
        if c1 is not None:
            line["config1"] = c1
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


def _parity(img, g, spp):
    """one render of `spp` samples per pixel against an FP64 full-frame fixture, on luminance: relative
    bias, its z-score and RMSE against the noise both estimates carry, the GPU's per-sample variance
    taken as the fixture's (the statistical tests in tests/ measure it from independent batches)"""
    import numpy as np
    ref = g["mean"].astype(np.float64)
    lv = g["lum_var"].astype(np.float64)
    lg, lr = _lum(img.astype(np.float64)), _lum(ref)
    var = lv / spp + lv / int(g["spp"])
    return {"rmse": round(math.sqrt(float(np.mean((lg - lr) ** 2))), 4),
            "expected_noise": round(math.sqrt(float(np.mean(var))), 4),
            "bias": round(float((lg.sum() - lr.sum()) / lr.sum()), 5),
            "z": round(float((lg.sum() - lr.sum()) / math.sqrt(var.sum())), 2),
            "oracle": "FP64 %d spp, full frame" % int(g["spp"])}


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


def pt_cpu_baseline(sc, scene, env, pt_settings_crop, spp=4, budget_s=12.0):
    """The estimator on the host cores: the oracle's FP32 twin of the tracer (the same arithmetic,
    BVH hits, alias-table environment sampling and PCG32 streams, oracle/pathtrace.c) over all threads
    on the 128x128 crop of the 1280x720 frame, 6 segments, roulette from the 3rd interaction; samples
    (paths) per second, repeated until about budget_s."""
    import numpy as np
    import oracle
    from vierkant_gb300.raytracing import _cudart
    import ctypes as C

    def d2h(ptr_, nbytes, dtype):
        a = np.empty(nbytes // np.dtype(dtype).itemsize, dtype)
        _cudart().cudaMemcpy(a.ctypes.data_as(C.c_void_p), C.c_void_p(ptr_), C.c_size_t(nbytes), 2)
        return a

    wptr, aptr, W, H = scene.env_tables()
    n = W * H
    w = d2h(wptr, 4 * n, np.float32)
    tab = d2h(aptr, 8 * n, np.uint32).reshape(n, 2)
    prob = np.ascontiguousarray(tab[:, 0].view(np.float32))
    alias = np.ascontiguousarray(tab[:, 1])
    env = env.cpu().numpy()
    bvh = oracle.CpuBVH(sc["xyz"], sc["indices"], 2)
    th = float(np.float32(math.tan(math.radians(45.0) / 2.0)))
    cam = oracle.camera((0, 0, 3.4), (0, 0, 0), (0, 1, 0), th, 1280, 720)
    total, paths, batches = 0.0, 0, 0
    while total < budget_s or batches < 2:
        t0 = time.perf_counter()
        oracle.pt_render(False, sc["xyz"], sc["indices"], sc["tri_material"], sc["materials"], bvh, env, cam, spp,
                         seed=SEED, batch=batches, rr_depth=3, crop=pt_settings_crop, alias_prob=prob, alias=alias,
                         weight=w)
        total += time.perf_counter() - t0
        paths += pt_settings_crop[2] * pt_settings_crop[3] * spp
        batches += 1
    return {"value": round(paths / total, 1), "unit": "samples/s", "cores": os.cpu_count() or 1, "kind": "port",
            "sample": f"{batches} x {spp} spp on the 128x128 crop at ({pt_settings_crop[0]}, {pt_settings_crop[1]}), "
                      f"{total:.1f} s",
            "method": "the oracle's FP32 twin of the tracer (oracle/pathtrace.c) on all host threads; the reference "
                      "has no CPU path tracer (its estimator runs in Vulkan ray-tracing shaders)"}


def path_tracer_block(ctx, frames=256, bytes_per_ray=None, cpu=True):
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
    if bytes_per_ray:
        peak, src = measured_peaks()
        gbs = rays * bytes_per_ray / (st.total_ms * 1e-3) / 1e9
        out["plain_720p_64spp"]["traversal_roofline"] = {
            "achieved": round(gbs, 1), "peak": peak, "unit": "GB/s", "frac": round(gbs / peak, 4), "peak_source": src,
            "bytes_per_ray": round(bytes_per_ray, 1),
            "note": "extension + shadow rays x the algorithmic bytes per ray of the closest-hit batch (camera and "
                    "bounce rays of this scene) over the whole frame time, shading included: a lower bound for "
                    "the traversal kernels alone (their share of a frame: "
                    "profiles/path_tracer_cornell_720p_4spp_launches.md)"}
    if cpu:
        out["plain_720p_64spp"]["cpu_baseline"] = pt_cpu_baseline(sc, scene, env, pt_settings_crop=(576, 528, 128, 128))
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


def nrc_cut_sweep(frames=256):
    """The radiance cache's cut point on the 1920x1080 Cornell workload: for terminate_depth 0, 1 and 2
    (the surface interaction at which rendering paths end in the cache; 2 is the workload's), the GPU
    time the cache tracer (1 spp per frame, 65,536 training paths per frame) needs to reach the plain
    tracer's 64-spp crop RMSE against the FP64 oracle, over the plain tracer's time. Prints one JSON
    line; not part of the default run."""
    import numpy as np
    from vierkant_gb300 import geometry
    from vierkant_gb300.nrc import NeuralRadianceCache, cache_for_scene
    from vierkant_gb300.pathtracer import PBRPathTracer, Scene, procedural_sky, sun_direction
    from vierkant_gb300.raytracing import Context
    ctx = Context(0)
    g1080 = np.load(ROOT / "tests" / "golden" / "pt_oracle_crop_1080.npz")
    sc = geometry.cornell_scene(SEED, 2, 64, 16)
    env = procedural_sky(ctx, 2048, 1024, sun_direction(), 5e4, 3.8e-5)
    scene = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], sc["materials"], env)

    def settings(spp):
        s = PBRPathTracer.default_settings()
        s.num_samples, s.max_trace_depth, s.rr_start_depth = spp, 6, 3
        s.resolution[0], s.resolution[1] = 1920, 1080
        return s

    cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, 1920, 1080)
    pt = PBRPathTracer(ctx, seed=SEED, settings=settings(64))
    pt.render_scene(scene, cam)
    pt.reset_accumulator()
    target, _ = _crop_error(pt.render_scene(scene, cam).cpu().numpy(), g1080)
    plain_ms = pt.statistics().total_ms
    pt.close()
    out = {"plain_64spp_ms": round(plain_ms, 2), "rmse_target": round(target, 4), "frames": frames, "cuts": []}
    for term in (0, 1, 2):
        cfg = NeuralRadianceCache.default_config()
        cfg.terminate_depth = term
        pt = PBRPathTracer(ctx, seed=SEED + 1, settings=settings(1))
        cache = cache_for_scene(ctx, scene, cfg)
        pt.attach_cache(cache)
        tot, reached, rmse, bias = 0.0, None, None, None
        for f in range(frames):
            im = pt.render_scene(scene, cam)
            tot += pt.statistics().total_ms
            rmse, bias = _crop_error(im.cpu().numpy(), g1080)
            if reached is None and rmse <= target:
                reached = {"frames": f + 1, "ms": round(tot, 1)}
        out["cuts"].append({"terminate_depth": term, "reached": reached,
                            "time_vs_plain": round(reached["ms"] / plain_ms, 3) if reached else None,
                            "ms_per_frame": round(tot / frames, 3), "rmse_last": round(rmse, 4),
                            "bias_last": round(bias, 4), "kernel_error": int(cache.info().kernel_error)})
        pt.close()
        cache.close()
    scene.close()
    print(json.dumps(out), flush=True)


def features_block(ctx):
    """The full material and light set: the Cornell box with the showcase materials (glass, rough
    glass, clearcoat, sheen, diffuse transmission, iridescence, metal-rough), one light of every
    analytic type and a sun disc, and the same box with its spheres cycled through homogeneous media
    (fog, absorbing glass, emissive gas, scattering glass) and the same lights, against the box with
    metal-rough materials and no lights, all at 1280x720 x 64 spp, 8 segments (samples/s, Mrays/s);
    also the textured box (smooth normals; checker, ao-rough-metal, normal and emission maps) and the
    alpha box (a cut-out wall, masked and blended spheres), unlit. Parity: the 16-sphere lit scene and the 16-sphere media scene at 256x144 x 1024 spp against their
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
    nrm = geometry.cornell_vertex_normals(sc)
    uv, tg = geometry.cornell_texcoords(sc)
    for name, mats, lit, tex in (("plain_720p_64spp_8seg", sc["materials"], False, None),
                                 ("materials_lights_720p_64spp_8seg", geometry.showcase_materials(sc["materials"]),
                                  True, None),
                                 ("media_lights_720p_64spp_8seg", geometry.media_materials(sc["materials"]), True,
                                  None),
                                 ("textured_720p_64spp_8seg", geometry.textured_materials(sc["materials"]), False,
                                  geometry.test_textures()),
                                 ("alpha_720p_64spp_8seg", geometry.alpha_materials(sc["materials"]), False,
                                  geometry.alpha_textures())):
        scene = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], mats, env)
        if lit:
            scene.set_lights(cornell_lights())
        if tex is not None:
            # smooth normals, texture coordinates, tangents and the textures (the textured and the
            # alpha-masked / blended Cornell scenes of the parity tests)
            scene.set_normals(nrm)
            scene.set_texcoords(uv)
            scene.set_tangents(tg)
            scene.set_textures(tex)
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
    out["textured_time_vs_plain"] = round(out["textured_720p_64spp_8seg"]["ms"] / out["plain_720p_64spp_8seg"]["ms"],
                                          3)
    out["alpha_time_vs_textured"] = round(out["alpha_720p_64spp_8seg"]["ms"] / out["textured_720p_64spp_8seg"]["ms"],
                                          3)
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
    out["lights_parity_256x144_1024spp"] = _parity(img, g, 1024)
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
    out["media_parity_256x144_1024spp"] = _parity(img, g, 1024)
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


def stress_cpu_baseline(st, env_rgb, budget_s=15.0):
    """The stress scene on the host cores: the oracle's FP64 instanced estimator (a BVH per mesh, an
    instance BVH, double arithmetic) on a 32x32 crop of the 3840x2160 frame at 1 spp per pass, 8
    segments, all threads; samples/s (the FP32 twin has no instanced mode)."""
    import numpy as np
    import oracle
    W, H, crop = 3840, 2160, (1856, 1016, 32, 32)
    th = float(np.float32(math.tan(math.radians(40.0) / 2.0)))
    cam = oracle.camera((0, 120, 300), (0, 0, 0), (0, 1, 0), th, W, H)
    inst = st["instances"]
    t0 = time.perf_counter()
    bvhs = [oracle.CpuBVH(m[0], m[1], 2) for m in st["meshes"]]
    build_s = time.perf_counter() - t0
    total, paths, passes, rays = 0.0, 0, 0, 0
    while total < budget_s or passes < 2:
        t0 = time.perf_counter()
        _, _, r = oracle.pt_render_instanced(st["meshes"], inst["transform"], inst["blas"], inst["material"],
                                             st["materials"], env_rgb, cam, 1, seed=SEED, batch=passes, max_depth=8,
                                             rr_depth=3, crop=crop, mesh_bvhs=bvhs)
        total += time.perf_counter() - t0
        paths += crop[2] * crop[3]
        rays += r[0] + r[1]
        passes += 1
    return {"value": round(paths / total, 1), "unit": "samples/s", "cores": os.cpu_count() or 1, "kind": "port",
            "mrays_per_s": round(rays / total / 1e6, 4),
            "sample": f"{passes} passes x 1 spp on the 32x32 crop at (1856, 1016), {total:.1f} s "
                      f"(+ {build_s:.1f} s building the mesh BVHs, untimed)",
            "method": "the oracle's FP64 instanced estimator (oracle/pathtrace.c) on all host threads; the "
                      "reference has no CPU path tracer"}


def stress_block(ctx, cpu=False):
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
    if cpu:
        out["cpu_baseline"] = stress_cpu_baseline(st, env.cpu().numpy())
    scene.close()
    return out


def profile_case(name: str):
    """Small workloads for profiler captures (ncu): one case per call, no JSON line.
    pt-frame   plain path tracer, Cornell scene, 1280x720 x 4 spp
    nrc        radiance-cache kernels: 2 training steps of 65,536 records with each training forward
               (mma.sync, tcgen05), inference of 262,144 queries with the mma.sync, tcgen05 and fused
               tcgen05 kernels
    batch      batched renderer, 4 scenes of the batched workload at 1 spp
    stress     instanced scene: 512^2 terrain + 10,000 instances, 960x540 x 2 spp, 8 segments
    features   Cornell scene with the showcase materials, the six analytic lights and a sun disc,
               1280x720 x 4 spp, 8 segments
    alpha      Cornell scene with the alpha materials and textures (a cut-out wall, masked and blended
               spheres), 1280x720 x 4 spp, 8 segments"""
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
            cfg.train_kernel = 3 if kind == 2 else 2
            caches.append(NeuralRadianceCache(ctx, cfg))
        x, t = feats(65536), torch.rand((65536, 3), device="cuda", generator=g)
        for _ in range(2):
            caches[0].train_step(x, t)  # mma.sync forward, tcgen05 weight gradients
            caches[1].train_step(x, t)  # tcgen05 forward and weight gradients
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
    elif name == "alpha":
        sc = geometry.cornell_scene(SEED, 2, 64, 16)
        envc = torch.full((64, 128, 3), 0.1, dtype=torch.float32, device="cuda")
        scene = Scene(ctx, sc["xyz"], sc["indices"], sc["tri_material"], geometry.alpha_materials(sc["materials"]),
                      envc)
        uv, tg = geometry.cornell_texcoords(sc)
        scene.set_normals(geometry.cornell_vertex_normals(sc))
        scene.set_texcoords(uv)
        scene.set_tangents(tg)
        scene.set_textures(geometry.alpha_textures())
        cam = geometry.camera_lookat((0, 0, 3.4), (0, 0, 0), (0, 1, 0), 45.0, 1280, 720)
        s = PBRPathTracer.default_settings()
        s.num_samples, s.max_trace_depth, s.rr_start_depth = 4, 8, 3
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


def cpu_bvh_tracer(xyz, idx):
    """The CPU closest-hit ray cast timed as the baseline: the oracle's 8-wide BVH of the same scene
    (leaf size 2, the same build as the GPU's) traversed over all host threads, with every triangle
    test done by the reference's own vierkant::intersect(const Triangle&, const Ray&)
    (src/intersection.cpp:114-129, compiled unmodified into oracle/_ref) — kind "reference" — or, where
    that library was not built, by the oracle's bit-identical C port of it — kind "port".
    Returns (kind, trace) with trace(rays) -> (hits, threads used)."""
    import oracle
    bvh = oracle.CpuBVH(xyz, idx, leaf_max=2)
    if oracle.ref() is not None:
        mesh = oracle.RefMesh(xyz, idx)
        return "reference", (lambda rays: bvh.closest_hit_ref(mesh, rays))
    return "port", (lambda rays: (bvh.closest_hit(rays), os.cpu_count() or 1))


def _strided(rays, m):
    import numpy as np
    n = len(rays)
    stride = max(1, n // max(1, m))
    return np.ascontiguousarray(rays[::stride][:m]), stride


def time_cpu_bvh(trace, rays, budget_s):
    """Mrays/s of trace() on an evenly strided sample of `rays`: the whole batch when one pass takes
    less than budget_s / 3, then as many passes as fit the budget (at least 3; the median pass is
    reported), else one pass over a sample sized to the budget."""
    n = len(rays)
    probe, _ = _strided(rays, min(n, 65536))
    t0 = time.perf_counter()
    trace(probe)
    dt = max(time.perf_counter() - t0, 1e-6)
    m = int(max(1024, min(n, len(probe) * budget_s / dt)))
    sample, stride = _strided(rays, m)
    rates, total, used = [], 0.0, 1
    while len(rates) < 3 or total < budget_s:
        t0 = time.perf_counter()
        _, used = trace(sample)
        dt = time.perf_counter() - t0
        rates.append(len(sample) / dt / 1e6)
        total += dt
        if total >= budget_s and len(rates) >= 1 and m < n:
            break
    return statistics.median(rates), int(used), len(sample), stride, total


def bruteforce_rate(xyz, idx, rays, budget_s):
    """The reference's brute-force ray cast (every ray against every triangle with vierkant::intersect,
    all host threads) on a strided sample: Mrays/s, a second figure beside the BVH baseline."""
    import numpy as np
    import oracle
    R = oracle.ref()
    if R is not None:
        kind, fn = "reference", R.vkref_closest_hit_bruteforce
    else:
        kind, fn = "port", oracle.orc().orc_closest_hit_bruteforce
    xyz, idx = np.ascontiguousarray(xyz), np.ascontiguousarray(idx)
    n = len(rays)
    probe, _ = _strided(rays, min(n, 256))
    hits = np.zeros((len(probe), 4), np.uint32)
    t0 = time.perf_counter()
    fn(oracle.ptr(xyz), oracle.ptr(idx), idx.shape[0], oracle.ptr(probe), len(probe), oracle.ptr(hits), 0, 0)
    dt = max(time.perf_counter() - t0, 1e-6)
    sample, stride = _strided(rays, int(max(256, min(n, len(probe) * budget_s / dt))))
    hits = np.zeros((len(sample), 4), np.uint32)
    t0 = time.perf_counter()
    used = fn(oracle.ptr(xyz), oracle.ptr(idx), idx.shape[0], oracle.ptr(sample), len(sample), oracle.ptr(hits), 0,
              0)
    dt = time.perf_counter() - t0
    return {"value": round(len(sample) / dt / 1e6, 5), "unit": "Mrays/s", "cores": int(used), "kind": kind,
            "sample": f"{len(sample)} rays (every {stride}th) x {idx.shape[0]} triangles, brute force, {dt:.1f} s"}


def cpu_baseline(sc, batch_np, budget_s=12.0):
    """The CPU BVH ray cast with the reference's triangle test on a bounded sample of the batch (see
    cpu_bvh_tracer), plus the brute-force figure."""
    kind, trace = cpu_bvh_tracer(sc["xyz"], sc["indices"])
    rate, used, m, stride, dt = time_cpu_bvh(trace, batch_np, budget_s)
    return {"value": round(rate, 4), "unit": "Mrays/s", "cores": used, "kind": kind,
            "sample": f"{m} rays (every {stride}th of the batch) per pass, CPU BVH traversal, median of the passes "
                      f"in {dt:.1f} s",
            "method": "the oracle's 8-wide BVH (leaf size 2) traversed on all host threads; every triangle "
                      "test is vierkant::intersect(Triangle, Ray), src/intersection.cpp:114-129",
            "bruteforce": bruteforce_rate(sc["xyz"], sc["indices"], batch_np, min(6.0, budget_s / 2))}


def config1_block(ctx, args, run_cpu=True):
    """The closest-hit workload on the 20,480-triangle icosphere (IcoSphere(1, 5)): a 1024x1024 pinhole
    camera at (0,0,3) looking at the origin, fovy 60 deg, one ray per pixel jittered by PCG32(0x5EED,
    stream 1). 48 MB of rays + hits fit in L2, so a 512 MB buffer is written between timed launches and
    each launch is timed alone with CUDA events on the launching stream. e2e: the host-buffer entry
    point (pinned rays in, hits out, synchronised) per call."""
    import numpy as np
    import torch
    from vierkant_gb300 import geometry
    from vierkant_gb300._lib import RAY_COUNT_STATS
    from vierkant_gb300.raytracing import BVH
    xyz, idx = geometry.icosphere(1.0, 5)
    bvh = BVH(ctx, torch.from_numpy(xyz).cuda(), torch.from_numpy(idx.astype(np.int32)).cuda())
    cam = geometry.camera_lookat((0, 0, 3), (0, 0, 0), (0, 1, 0), 60.0, 1024, 1024)
    rays = ctx.camera_rays(cam, SEED, 1, 1)
    n = rays.shape[0]
    hits = torch.empty((n, 4), dtype=torch.int32, device=rays.device)
    ctx.stats(reset=True)
    bvh.closest_hit(rays, hits, flags=RAY_COUNT_STATS)
    visits, tests = ctx.stats(reset=True)
    byts = n * (RAY_BYTES + HIT_BYTES) + visits * NODE_BYTES + tests * TRI_BYTES
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=rays.device)
    stream = torch.cuda.current_stream()
    for _ in range(max(3, args.warmup)):
        bvh.closest_hit(rays, hits)
    steps = max(10, args.steps)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    torch.cuda.synchronize()
    for e0, e1 in ev:
        flush.fill_(1)
        e0.record(stream)
        bvh.closest_hit(rays, hits)
        e1.record(stream)
    torch.cuda.synchronize()
    ms = statistics.mean(e0.elapsed_time(e1) for e0, e1 in ev)
    rays_h = rays.cpu().pin_memory()
    hits_h = torch.empty((n, 4), dtype=torch.int32).pin_memory()
    for _ in range(3):
        bvh.closest_hit_host(rays_h, hits_h)
    t0 = time.perf_counter()
    for _ in range(steps):
        bvh.closest_hit_host(rays_h, hits_h)
    e2e_ms = (time.perf_counter() - t0) * 1e3 / steps
    ok = bool(torch.equal(hits.cpu(), hits_h))
    peak, src = measured_peaks()
    out = {"workload": "closest-hit, IcoSphere(1, 5) (20,480 triangles), 1024x1024 camera rays",
           "rays": n, "ms": round(ms, 4), "mrays_per_s": round(n / ms / 1e3, 1),
           "e2e_mrays_per_s": round(n / e2e_ms / 1e3, 1), "e2e_matches_device": ok,
           "l2": "512 MB written between timed launches", "hits_sha256_16": batch_digest(hits.cpu().numpy()),
           "roofline": {"achieved": round(byts / ms / 1e6, 1), "peak": peak, "unit": "GB/s",
                        "frac": round(byts / ms / 1e6 / peak, 4), "peak_source": src,
                        "algorithmic_bytes_per_ray": round(byts / n, 1),
                        "node_visits_per_ray": round(visits / n, 3), "tri_tests_per_ray": round(tests / n, 3)}}
    if run_cpu:
        kind, trace = cpu_bvh_tracer(xyz, idx)
        rate, used, m, stride, dt = time_cpu_bvh(trace, rays.cpu().numpy(), 6.0)
        out["cpu_baseline"] = {"value": round(rate, 4), "unit": "Mrays/s", "cores": used, "kind": kind,
                               "sample": f"{m} rays (every {stride}th), CPU BVH traversal, {dt:.1f} s"}
    bvh.close()
    del flush
    return out


def run_reference(args):
    """Reference arm: the CPU closest-hit ray cast of cpu_bvh_tracer on the host cores (rank 0 only),
    over the same batch as the GPU arm, built here on the CPU without the GPU library: the oracle's
    camera rays and CPU BVH hits (both bit-identical to the GPU's), then bounce_batch."""
    ws, rank, local = dist_env()
    if rank != 0:
        return
    import numpy as np
    import oracle
    sc = oracle.cornell_scene(SEED, 2, 64, 16)
    th = float(np.float32(math.tan(math.radians(45.0) / 2.0)))
    cam = oracle.camera((0, 0, 3.4), (0, 0, 0), (0, 1, 0), th, WIDTH, HEIGHT)
    prim = oracle.camera_rays(cam, SEED, 2, SPP).view(np.float32).reshape(-1, 8)
    kind, trace = cpu_bvh_tracer(sc["xyz"], sc["indices"])
    hits, _ = trace(prim)
    batch = bounce_batch(prim, hits.view(np.uint32).reshape(-1, 4), 4)
    config = bench_config(sc["indices"].shape[0], batch)
    n = batch.shape[0]
    t0 = time.perf_counter()
    all_hits, used = trace(batch)
    full_s = time.perf_counter() - t0
    digest = batch_digest(all_hits.view(np.uint32).reshape(-1, 4))
    per_step_budget = max(0.5, min(20.0, args.cpu_seconds / max(1, args.steps)))
    m = int(max(1024, min(n, n * per_step_budget / max(full_s, 1e-6))))
    sample, stride = _strided(batch, m)
    for _ in range(args.warmup):
        trace(sample[: max(1024, m // 8)])
    rates = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        _, used = trace(sample)
        rates.append(len(sample) / (time.perf_counter() - t0) / 1e6)
    value = round(statistics.median(rates), 4)
    cb = {"value": value, "unit": "Mrays/s", "cores": int(used), "kind": kind,
          "sample": f"{len(sample)} rays per step (every {stride}th of the {n}-ray batch), CPU BVH traversal",
          "method": "the oracle's 8-wide BVH (leaf size 2) traversed on all host threads; every triangle test is "
                    "vierkant::intersect(Triangle, Ray), src/intersection.cpp:114-129",
          "bruteforce": bruteforce_rate(sc["xyz"], sc["indices"], batch, min(4.0, args.cpu_seconds / 3))}
    line = {"metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(len(sample) / value / 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
            "config": config, "hits_sha256_16": digest,
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
    ap.add_argument("--profile-case", choices=["pt-frame", "nrc", "batch", "stress", "features", "media", "alpha"], default=None,
                    help="run one small workload for a profiler capture and exit (no JSON line)")
    ap.add_argument("--nrc-cut-sweep", action="store_true",
                    help="measure the radiance cache's equal-RMSE time for terminate_depth 0, 1, 2 and exit")
    args = ap.parse_args()
    if args.nrc_cut_sweep:
        nrc_cut_sweep(args.nrc_frames)
        return
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
