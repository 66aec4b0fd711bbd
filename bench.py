#!/usr/bin/env python3
"""Benchmark of the ray-traced visibility + deferred-lighting frame.

Workload: the large two-level scene at 1920x1080 — 64 icospheres (subdivision 6,
81,920 triangles each, radially displaced by 8 seeded spherical sinusoids), 1024
instances in a 200^3 box (83.9 M instanced triangles), 1 directional + 32 point + 8
spot lights, 1 shadow ray per light and 16 cosine-weighted AO rays (radius 2.0) per
lit pixel, FP32. Synthetic, seeded scene (seed 1002).

A step is one frame: TLAS rebuild from the host instance array, primary-ray
G-buffer, shadow + AO visibility, deferred light pass. Rays per frame = primary
rays (one per pixel) + lit pixels x (41 shadow + 16 AO). The BLAS are built once
before timing, as the reference builds them at import.

value: Grays/s with every input resident in device memory (CUDA events around each
frame on the launching stream; a 256 MB buffer is written between frames to flush
L2). e2e: the same frame through the C ABI from pinned host buffers — scene,
light and model blocks and the instance array copied host->device, the RGBA32F
light image read back — timed on the host around the synchronised call.

--impl reference runs the reference path's CPU restatement (the oracle, tracing
every ray light.frag traces) on all host cores over the same frame (each step one
whole frame; --cpu-rows bounds it to a band of rows).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ms/frame @1080p: denoised 1spp vs plain at equal AO RMSE vs 1024spp; Grays/s"
UNIT = "Grays/s"
CONFIG = {"workload": "two-level scene 1920x1080: 64 displaced icospheres (81,920 tris) x 1024 instances, "
                      "41 lights (1 dir + 32 point + 8 spot), 1 shadow ray/light + 16 AO rays/px, FP32",
          "width": 1920, "height": 1080, "instances": 1024, "blas": 64, "triangles_per_blas": 81920,
          "shadow_rays_per_px": 41, "ao_rays_per_px": 16, "seed": 1002, "l2": "flushed between frames (256 MB write)"}
FALLBACK_HBM_GBS = 6800.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-rows", type=int, default=1080,
                    help="rows of the CPU baseline sample (default: the whole 1080-row frame)")
    ap.add_argument("--width", type=int, default=1920, help="smaller sizes only for profiling captures")
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-denoise", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--batch-scenes", type=int, default=64, help="scenes of the batched workload (64 as configured)")
    ap.add_argument("--batch-no-tune", action="store_true",
                    help="keep the default traversal launch shape in the batched workload (profiling captures)")
    ap.add_argument("--no-stress", action="store_true", help="skip the 4K 4096-instance stress scene")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x: float, device=None) -> float:
    """The largest x over the ranks of the default process group (x itself when there
    is none): every rank's step time is bounded by the slowest replica's."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world: int, units_per_rank: float, ms: float) -> float:
    """Units per second of all ranks together (each rank processes units_per_rank per
    step; ms is the max-over-ranks step time), in G units/s."""
    return world * units_per_rank / (ms * 1e-3) / 1e9


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", FALLBACK_HBM_GBS), "measured"
    return FALLBACK_HBM_GBS, "fallback"


class Clocks:
    """nvidia-smi samples during the timed region (200 ms period)."""

    def __init__(self, index: int):
        self.index = index
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.proc = None

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.flush()
        self.file.seek(0)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.file.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.file.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------- CPU baseline
def cpu_baseline(scene, rows: int, repeats: int = 1):
    """Oracle frame (by default all of it; else a band of rows at the image centre) on
    all host cores, `repeats` times; the BLAS build is not timed."""
    import numpy as np

    import luz_gb300 as L
    import oracle as O

    meshes = scene.meshes()
    ob = [O.OracleBlas(v, i) for v, i in meshes]          # BLAS: built once, not timed
    im = scene.instance_mesh()
    tr = scene.transforms()
    b, lights, models = scene.block(), scene.lights(), scene.models()
    W, H = scene.width, scene.height
    y0 = max(0, H // 2 - rows // 2)
    y1 = min(H, y0 + rows)
    bn = L.blue_noise()
    nthreads = O.threads()
    S = sum(lights[i].num_shadow_samples for i in range(scene.light_count)) + b.ao_num_samples
    times, rays_list = [], []
    for _ in range(repeats):
        t0 = time.perf_counter()
        tl = O.OracleTlas([ob[m] for m in im], tr)
        f = O.OracleFrame(tl, b, lights, scene.light_count, models, scene.instance_count, W, H)
        f.gbuffer(nthreads, y0, y1)
        f.visibility(0, bn, y0, y1, nthreads=nthreads, cull=False)   # every ray light.frag traces
        f.light_pass(nthreads=nthreads, y0=y0, y1=y1)
        dt = time.perf_counter() - t0
        lit = int((np.linalg.norm(f.normal[y0 * W:y1 * W, :3], axis=1) > 0).sum())
        rays_list.append((y1 - y0) * W + lit * S)
        times.append(dt)
    value = sum(rays_list) / sum(times) / 1e9
    # G-buffer + visibility + light pass on one core over the two centre rows (the
    # TLAS built before the clock starts)
    tl = O.OracleTlas([ob[m] for m in im], tr)
    f = O.OracleFrame(tl, b, lights, scene.light_count, models, scene.instance_count, W, H)
    yc = max(0, H // 2 - 1)
    t0 = time.perf_counter()
    f.gbuffer(1, yc, yc + 2)
    f.visibility(0, bn, yc, yc + 2, nthreads=1, cull=False)
    f.light_pass(nthreads=1, y0=yc, y1=yc + 2)
    dt1 = time.perf_counter() - t0
    lit1 = int((np.linalg.norm(f.normal[yc * W:(yc + 2) * W, :3], axis=1) > 0).sum())
    single = (2 * W + lit1 * S) / dt1 / 1e9
    return {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port", "single_thread_value": single,
            "sample": f"rows {y0}-{y1} of 1920x1080 ({(y1 - y0) * W} px, {rays_list[0]} rays per sample, "
                      f"{len(times)} samples): "
                      f"TLAS build + G-buffer + shadow/AO any-hit + light pass; BLAS build untimed; "
                      f"single_thread_value: rows {yc}-{yc + 2} on one core, TLAS build untimed"}, times


def run_reference(args, rank):
    if rank != 0:
        return
    import luz_gb300 as L
    scene = L.HostScene(2, width=args.width, height=args.height)
    K = args.steps
    res, times = cpu_baseline(scene, args.cpu_rows, repeats=max(1, args.warmup) + K)
    times = times[max(1, args.warmup):]
    value = res["value"]
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": K, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generator)", "config": CONFIG,
            "cpu_baseline": res, "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                                         "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------- denoised vs plain
def denoised_vs_plain(g, ctx, stream, flush, K, W, restore_ao=16, curve_spp=(1, 2, 4, 8, 16, 32, 64),
                      target_spp=1024):
    """The headline comparison. The denoised frame traces 1 AO ray and 1 shadow ray per
    light per lit pixel and filters the shadow ratio and AO with the network; the plain
    frame traces N AO rays and N shadow rays per light (the reference's one sample-count
    knob, lightSamples, sets every light's numShadowSamples: GPUScene.cpp:248). RMSE
    over the lit pixels against the target_spp-sample frame, for the AO value and for
    the radiance (RGB light-pass output); the equal-quality N is the smallest plain
    sample count whose AO RMSE and radiance RMSE are both at or below the denoised
    frame's; ms/frame of both frames (TLAS build, G-buffer, visibility, denoiser / light
    pass), CUDA events, L2 flushed between frames."""
    import numpy as np
    import torch

    import luz_gb300 as L
    from luz_gb300 import denoiser as D

    if not D.DEFAULT_WEIGHTS.exists():
        return None
    den = D.Denoiser(ctx)
    den.load(D.DEFAULT_WEIGHTS)
    fr, tl, sc = g.frame, g.tlas, g.scene
    t0 = time.perf_counter()
    tl.build(g.instances, g.n_instances)
    fr.gbuffer(tl)
    lit = np.linalg.norm(fr.read(L.PLANE_NORMAL)[..., :3], axis=-1) > 0
    t_rad, t_sig = D.reference(fr, tl, sc, target_spp, per_trace=16)   # torch and the context share `stream`
    t_ao = t_sig[..., 3]
    t_target = time.perf_counter() - t0

    def rmse_pair(ao_plane):
        return (D.lit_rmse(fr.read(ao_plane), t_ao, lit), D.lit_rmse(fr.read(L.PLANE_LIGHT)[..., :3], t_rad, lit))

    def plain(n):
        D.set_samples(fr, sc, n, n)
        fr.trace(tl, 7)
        fr.light_pass(L.LIGHT_PASS_PLAIN)
        fr.ao_resolve()
        return rmse_pair(L.PLANE_AO)

    curve = {n: plain(n) for n in curve_spp}
    D.set_samples(fr, sc, 1, 1)
    fr.trace(tl, 7)
    den.denoise(fr)
    fr.light_pass(L.LIGHT_PASS_DENOISED)
    r_den = rmse_pair(L.PLANE_AO_DENOISED)

    def passes(n):
        r = curve[n] if n in curve else curve.setdefault(n, plain(n))
        return r[0] <= r_den[0] and r[1] <= r_den[1]

    # smallest N that matches the denoised frame on both: first passing point of the
    # measured curve, then a bisection over the integers below it
    ns = sorted(curve)
    hi = next((n for n in ns if passes(n)), None)
    matched = hi is not None
    if matched:
        lo = max([n for n in ns if n < hi] or [0])
        while hi - lo > 1:
            mid = (lo + hi) // 2
            if passes(mid):
                hi = mid
            else:
                lo = mid
        n_star = hi
    else:
        n_star = ns[-1]          # the denoised frame beats every measured N: a lower bound
    ao_curve = {n: v[0] for n, v in curve.items()}
    rad_curve = {n: v[1] for n, v in curve.items()}

    def timed(fn, profile=False):
        for w in range(W):
            fn(w)
        torch.cuda.synchronize()
        if profile:
            ctx.profile(True)
        ts = []
        for k in range(K):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn(100 + k)
            e1.record(stream)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return statistics.mean(ts)

    def frame_denoised(fi):
        tl.build(g.instances, g.n_instances)
        fr.gbuffer(tl)
        fr.trace(tl, fi)
        den.denoise(fr)
        fr.light_pass(L.LIGHT_PASS_DENOISED)

    def frame_plain(fi):
        tl.build(g.instances, g.n_instances)
        fr.gbuffer(tl)
        fr.trace(tl, fi)
        fr.light_pass(L.LIGHT_PASS_PLAIN)

    D.set_samples(fr, sc, 1, 1)
    ms_den = timed(frame_denoised, profile=True)
    stages = {}
    for name in ("tlas_build", "gbuffer", "raygen", "traversal", "features", "light_pass", "denoise"):
        tot, n = ctx.profile_read(name)
        stages[name] = tot / K
    ctx.profile(False)
    D.set_samples(fr, sc, n_star, n_star)
    ms_plain = timed(frame_plain)
    # back to the benchmark's sampling
    sc.set_sampling(restore_ao, light_samples=1, sampler=L.SAMPLER_PARITY)
    fr.upload(sc.block(), sc.lights(), sc.light_count, sc.models(), sc.instance_count)
    nlit = int(lit.sum())
    flops = 2.0 * (72 * 64 + 64 * 64 + 64 * 64 + 64 * 49) * nlit
    return {"target_spp": target_spp, "target": f"{target_spp // 16} traces of 16 AO + 16 shadow samples per light",
            "target_s": t_target,
            "rmse_vs_target": {"denoised_1spp": {"ao": r_den[0], "radiance": r_den[1]},
                               "plain": {str(k): {"ao": v[0], "radiance": v[1]} for k, v in sorted(curve.items())}},
            "equal_rmse_spp": n_star, "equal_rmse_matched": matched,
            "equal_rmse_spp_interpolated": {"ao": D.equal_rmse_spp(ao_curve, r_den[0]),
                                            "radiance": D.equal_rmse_spp(rad_curve, r_den[1])},
            "ms_per_frame_denoised": ms_den, "ms_per_frame_plain_equal_rmse": ms_plain,
            "frame_speedup": ms_plain / ms_den,
            "denoised_frame_kernel_ms": stages,
            "denoiser_tflops_bf16": flops / (stages["denoise"] * 1e-3) / 1e12 if stages["denoise"] else None,
            "denoised_pixels": nlit, "plain_rays_per_px": "N AO + N shadow per light",
            "sampler": "stratified (8x8-block R2)", "weights": D.DEFAULT_WEIGHTS.name}


# ---------------------------------------------------------------------------- denoiser training
def denoiser_training(ctx, stream, steps=20, scenes=32):
    """Training throughput of the denoiser: Adam steps on batches of 16 config-3 pairs at
    256x256 (1-sample input, 64-sample target: the target count does not change the
    step's work). Per step the tcgen05 forward + backward + weight-gradient kernel, the
    partial sum, Adam and the BF16 repack; the kernel's own time from the event pairs
    around its launches."""
    import torch

    from luz_gb300 import denoiser as D

    pairs = D.render_pairs(ctx, scenes, size=256, target_spp=64, per_trace=32)
    ctx.set_stream(stream.cuda_stream)      # render_pairs ran on a stream of its own
    torch.cuda.set_stream(stream)
    den = D.Denoiser(ctx, seed=2)
    batch = 16
    for w in range(3):
        den.train_step(pairs.batch((w * batch) % (scenes - batch + 1), batch), 1e-3)
    torch.cuda.synchronize()
    ctx.profile(True)
    t0 = time.perf_counter()
    for k in range(steps):
        den.train_step(pairs.batch((k * batch) % (scenes - batch + 1), batch), 1e-3)
    torch.cuda.synchronize()
    wall = (time.perf_counter() - t0) / steps
    kern, n = ctx.profile_read("denoise_train")
    ctx.profile(False)
    px = batch * 256 * 256
    flop = 3.0 * 2.0 * (72 * 64 + 64 * 64 + 64 * 64 + 64 * 49) * px    # forward + backward (dX and dW)
    kms = kern / max(n, 1)
    den.close()
    return {"pixels_per_step": px, "ms_per_step": wall * 1e3, "kernel_ms_per_step": kms,
            "kernel_tflops_bf16": flop / (kms * 1e-3) / 1e12, "step_tflops_bf16": flop / wall / 1e12,
            "kernel": "denoise_train_tc_kernel (tcgen05, TMEM accumulators)",
            "note": "FLOP = 3 x forward (forward, dX, dW); the step also runs the partial sum, Adam, the repack "
                    "and a 4-byte loss read-back"}


# ---------------------------------------------------------------------------- post passes
def post_passes(g, stream, flush, K, W):
    """TAA (taa.comp), compose / ACES (present.frag) and the luminance histogram on the
    1080p frame: ms per pass and the HBM byte rate of its algorithmic traffic (TAA 52
    B/px: light 16 + history 16 + depth 4 + output 16; compose 20 B/px; histogram 16 B/px)."""
    import torch

    fr = g.frame
    px = fr.width * fr.height
    peak, _ = measured_peaks()
    passes = {"taa": (lambda: fr.taa(True), 52), "compose": (lambda: fr.compose(True, 0), 20),
              "histogram": (lambda: fr.luminance_histogram(True), 16)}
    out = {}
    for name, (fn, bpp) in passes.items():
        for _ in range(W):
            fn()
        ts = []
        for _ in range(K):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        ms = statistics.mean(ts)
        gbs = bpp * px / (ms * 1e-3) / 1e9
        out[name] = {"ms": ms, "bytes_per_px": bpp, "achieved_gbs": gbs, "frac_of_measured_hbm": gbs / peak}
    out["note"] = "histogram includes its 1 KB read-back (a host sync); TAA/compose are device-only"
    return out


# ---------------------------------------------------------------------------- stress scene
def stress_config5(ctx, stream, flush, K, W):
    """The stress scene: 4096 instances of the 64 displaced icospheres (335.5 M
    instanced triangles) at 3840x2160, 145 lights (128 point + 16 spot + 1
    directional, above the reference's 64-light block), 1 shadow ray per light and 64
    AO rays per pixel on the plain path. Reports the BVH device bytes, the plain
    frame (ms, Grays/s) and the denoised 1-spp frame against the plain frame at equal
    AO RMSE."""
    import torch

    import luz_gb300 as L

    scene = L.HostScene(5)
    g = L.GPUScene(ctx, scene)
    g.update_resources_gpu()
    fr, tl = g.frame, g.tlas
    mem = {"blas": {}, "tlas": tl.memory()}
    for b in g.blas:
        for k, v in b.memory().items():
            mem["blas"][k] = mem["blas"].get(k, 0) + v
    mem["total"] = mem["blas"]["total"] + mem["tlas"]["total"]

    def frame(fi):
        tl.build(g.instances, g.n_instances)
        fr.gbuffer(tl)
        fr.trace(tl, fi)
        fr.light_pass(False)

    for w in range(W):
        frame(w)
    torch.cuda.synchronize()
    lit = fr.lit_count()
    S = sum(g.lights[i].num_shadow_samples for i in range(scene.light_count)) + g.block.ao_num_samples
    rays = scene.width * scene.height + lit * S
    traversed = scene.width * scene.height + fr.trace_stats(tl, 0)["rays"]
    ts = []
    for k in range(K):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        frame(W + k)
        e1.record(stream)
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    if ctx.device_status() != 0:
        raise RuntimeError("device status word raised in the stress scene")
    ms = statistics.mean(ts)
    out = {"workload": "4096 instances x 64 displaced icospheres (335.5 M instanced tris), 3840x2160, "
                       "145 lights, 1 shadow ray/light + 64 AO rays/px",
           "lights": scene.light_count, "lit_pixels": lit, "rays_per_frame": rays,
           "rays_traversed_per_frame": traversed, "ms_per_frame": ms,
           "grays_per_s": rays / (ms * 1e-3) / 1e9, "bvh_device_bytes": mem,
           "blas_build_ms": g.blas_build_ms}
    out["denoised_vs_plain"] = denoised_vs_plain(g, ctx, stream, flush, K, W, restore_ao=64,
                                                 curve_spp=(1, 2, 4, 8, 16, 32, 64))
    for b in g.blas:
        b.close()
    tl.close()
    fr.close()
    return out


# ---------------------------------------------------------------------------- batched workload
def batched_uneven(ctx, stream, flush, K, W, count=64, seed=4004, tune=True):
    """count scenes, triangles log-uniform in [1e3, 2e6] from the cube/quad and
    displaced-icosphere generators, resolutions from {256^2, 512^2, 1280x720,
    1920x1080}, 4 AO rays per pixel; one batched BLAS build at creation, then every
    frame ONE persistent launch (the frame kernel: all TLAS builds, G-buffers, the
    traversal of every scene's rays and the light passes) replayed as a CUDA graph, its
    traversal launch shape picked by the autotuner. The staged form (separate launches
    per scene around one batched traversal launch) is timed beside it."""
    import numpy as np
    import torch

    import luz_gb300 as L

    rng = np.random.default_rng(seed)
    sizes = [(256, 256), (512, 512), (1280, 720), (1920, 1080)]
    scenes = []
    t0 = time.perf_counter()
    for i in range(count):
        tris = int(round(10 ** rng.uniform(3.0, np.log10(2e6))))
        w, h = sizes[int(rng.integers(4))]
        scenes.append(L.HostScene(6, seed=4000 + i, width=w, height=h, triangles=tris, ao_samples=4))
    t_gen = time.perf_counter() - t0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b = L.Batch(ctx, scenes)
    ctx.synchronize()
    t_build = time.perf_counter() - t0
    pixels = sum(sc.width * sc.height for sc in scenes)

    def replay_ms():
        b.capture(0)
        for _ in range(W):
            b.replay()
        torch.cuda.synchronize()
        ts = []
        for _ in range(K):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            b.replay()
            e1.record(stream)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        if ctx.device_status() != 0:
            raise RuntimeError("device status word raised in the batched workload")
        return statistics.mean(ts)

    out = {"scenes": count, "pixels": pixels, "instanced_triangles": b.triangles, "blas_meshes": len(b.blas),
           "host_generation_s": t_gen, "blas_build_and_setup_s": t_build}
    staged = None
    if b.fused:
        b.set_fused(False)
        staged = replay_ms()
        b.set_fused(True)
    tun, tune_ms = b.autotune(3) if tune else (ctx.vis_tuning(), None)
    b.render(0)
    st = b.stats(0)
    # light.frag's rays (the unit of grays_per_s, as for the single frame) and the
    # rays actually traversed
    rays = pixels + sum(f.lit_count() * (sum(sc.lights()[i].num_shadow_samples for i in range(sc.light_count)) +
                                         sc.block().ao_num_samples)
                        for f, sc in zip(b.frames, scenes))
    traversed = st["rays"] + pixels
    ms = replay_ms()
    # graph launches counted by the library: one frame kernel per replay when fused
    out.update({"rays_per_replay": rays, "rays_traversed_per_replay": traversed, "ms_per_replay": ms,
                "grays_per_s": rays / (ms * 1e-3) / 1e9,
                "graph": ("one CUDA graph per batch frame: a memset of the work counters and ONE persistent "
                          "frame-kernel launch" if b.fused else "one CUDA graph of staged launches"),
                "fused": b.fused, "staged_ms_per_replay": staged,
                "autotuned_shape": tun, "autotune_best_frame_ms": tune_ms})
    b.close()
    return out


# ---------------------------------------------------------------------------- GPU arm
def run_ours(args, rank, world, local):
    import numpy as np
    import torch

    import luz_gb300 as L
    from luz_gb300 import _abi

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    scene = L.HostScene(2, width=args.width, height=args.height)
    ctx = L.Context(local)
    # One explicit stream for the library's kernels, the L2 flush and the events.
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    g = L.GPUScene(ctx, scene)
    g.update_resources_gpu()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    fr, tl = g.frame, g.tlas

    def frame(fi: int, ev=None):
        if ev:
            ev[0].record(stream)
        tl.build(g.instances, g.n_instances)
        if ev:
            ev[1].record(stream)
        fr.gbuffer(tl)
        if ev:
            ev[2].record(stream)
        fr.trace(tl, fi)
        if ev:
            ev[3].record(stream)
        fr.light_pass(False)
        if ev:
            ev[4].record(stream)

    for w in range(args.warmup):
        frame(w)
    torch.cuda.synchronize()
    lit = fr.lit_count()
    S = fr_shadow = sum(g.lights[i].num_shadow_samples for i in range(scene.light_count))
    S = fr_shadow + g.block.ao_num_samples
    rays_per_frame = scene.width * scene.height + lit * S
    stats = fr.trace_stats(tl, 0)
    torch.cuda.synchronize()
    assert 0 < stats["rays"] <= lit * S, (stats, lit, S)
    if ctx.device_status() != 0:
        raise RuntimeError("device status word raised during warm-up")

    K = args.steps
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(5)] for _ in range(K)]
    clocks = Clocks(local)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    launches0 = ctx.launch_count()
    ctx.profile(True)          # an event pair around each launch of the instrumented kernels
    for k in range(K):
        flush.zero_()
        frame(args.warmup + k, evs[k])
    torch.cuda.synchronize()
    launches = ctx.launch_count() - launches0
    kernel_ms = {}
    for name in ("tlas_build", "gbuffer", "raygen", "traversal", "light_pass"):
        tot, n = ctx.profile_read(name)
        kernel_ms[name] = {"ms_per_launch": tot / max(n, 1), "launches": n}
    ctx.profile(False)
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    frame_ms = [e[0].elapsed_time(e[4]) for e in evs]
    stage_ms = {name: statistics.mean(e[i].elapsed_time(e[i + 1]) for e in evs)
                for i, name in enumerate(["tlas_build", "gbuffer", "visibility", "light_pass"])}
    ms = max_over_ranks(statistics.mean(frame_ms), dev)
    value = whole_job_rate(world, rays_per_frame, ms)
    if ctx.device_status() != 0:
        raise RuntimeError("device status word raised during timing")

    # Roofline of the dominant kernel, the traversal (visibility_kernel): algorithmic
    # bytes per launch = ray records read (32 B per item, written by ray generation) +
    # hit bits (1/8 B per traversed ray) + 4-wide node visits x 112 B (7 of the 8
    # float4) + triangle tests x 48 B + instance entries x 80 B, with the visits counted
    # by the counting build of the same kernel over the same frame. The node and triangle
    # loads are served by L1 and L2 (the BVH is read from HBM about once per frame), so
    # the bound is the L2 read bandwidth, measured in this run by L2-only 16-B loads
    # over a 48 MiB buffer on every SM.
    trav_bytes = (lit * S * 32 + stats["rays"] * 0.125 + (stats["tlas_nodes"] + stats["blas_nodes"]) * 112 +
                  stats["tris"] * 48 + stats["instances"] * 80)
    trav_ms = kernel_ms["traversal"]["ms_per_launch"]
    l2_gbs = ctx.probe_l2_read_gbs(48 << 20, 50)
    peak, peak_kind = measured_peaks()
    achieved = trav_bytes / (trav_ms * 1e-3) / 1e9
    roofline = {"bound": "l2", "kernel": "visibility_kernel", "achieved": achieved, "peak": l2_gbs,
                "peak_source": "measured in this run (L2-only loads, 48 MiB, every SM)", "unit": "GB/s",
                "frac": achieved / l2_gbs, "traffic": None, "algorithmic_bytes": trav_bytes,
                "ms_per_launch": trav_ms,
                "note": "traffic (DRAM bytes per launch) comes from an ncu capture, not from this run; "
                        "the kernel is issue-bound (about 69 % of issue slots and 13 of 32 lanes per instruction in an ncu capture)",
                "per_ray": {k: stats[k] / max(stats["rays"], 1) for k in
                            ("tlas_nodes", "blas_nodes", "tris", "instances")}}
    # the light pass against HBM: per lit pixel the 32-B surface record, the 16-B record of
    # its albedo / material / emission words, its shadow and AO bits and the 16-B
    # RGBA32F result
    lp_bytes = lit * (32 + 16 + 16 + S / 8.0)
    lp_ms = kernel_ms["light_pass"]["ms_per_launch"]
    light_pass = {"bound": "hbm", "achieved": lp_bytes / (lp_ms * 1e-3) / 1e9, "peak": peak,
                  "peak_source": peak_kind, "unit": "GB/s", "algorithmic_bytes": lp_bytes, "ms_per_launch": lp_ms}
    light_pass["frac"] = light_pass["achieved"] / peak

    # e2e through the C ABI from pinned host buffers
    e2e = None
    if not args.no_e2e:
        nbytes = fr.plane_bytes(L.PLANE_LIGHT)
        out = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
        models_p = torch.empty(C.sizeof(g.models), dtype=torch.uint8, pin_memory=True)
        lights_p = torch.empty(C.sizeof(g.lights), dtype=torch.uint8, pin_memory=True)
        scene_p = torch.empty(C.sizeof(g.block), dtype=torch.uint8, pin_memory=True)
        inst_p = torch.empty(C.sizeof(g.instances), dtype=torch.uint8, pin_memory=True)
        C.memmove(models_p.data_ptr(), g.models, C.sizeof(g.models))
        C.memmove(lights_p.data_ptr(), g.lights, C.sizeof(g.lights))
        C.memmove(scene_p.data_ptr(), C.byref(g.block), C.sizeof(g.block))
        C.memmove(inst_p.data_ptr(), g.instances, C.sizeof(g.instances))
        lib = L.lib
        sp = C.cast(C.c_void_p(scene_p.data_ptr()), C.POINTER(_abi.Scene))
        lp = C.cast(C.c_void_p(lights_p.data_ptr()), C.POINTER(_abi.Light))
        mp = C.cast(C.c_void_p(models_p.data_ptr()), C.POINTER(_abi.Model))
        ip = C.cast(C.c_void_p(inst_p.data_ptr()), C.POINTER(_abi.Instance))

        def e2e_step(fi):
            st = lib.luz_frame_upload(ctx.handle, fr.handle, sp, lp, scene.light_count, mp, scene.instance_count)
            st |= lib.luz_render_frame(ctx.handle, fr.handle, tl.handle, ip, g.n_instances, fi)
            st |= lib.luz_frame_read(ctx.handle, fr.handle, L.PLANE_LIGHT, C.c_void_p(out.data_ptr()), nbytes)
            if st != 0:
                raise RuntimeError(lib.luz_last_error(ctx.handle).decode())

        for w in range(args.warmup):
            e2e_step(w)
        torch.cuda.synchronize()
        ts = []
        for k in range(K):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            e2e_step(k)
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        e2e_s = max_over_ranks(statistics.mean(ts), dev)
        h2d = C.sizeof(g.block) + C.sizeof(_abi.Light) * scene.light_count + \
            C.sizeof(_abi.Model) * scene.instance_count + C.sizeof(_abi.Instance) * g.n_instances
        e2e = {"value": whole_job_rate(world, rays_per_frame, e2e_s * 1e3), "unit": UNIT, "ms_per_step": e2e_s * 1e3,
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(nbytes)}

    denoised = None
    if not args.no_denoise:
        denoised = denoised_vs_plain(g, ctx, stream, flush, K, args.warmup)
        if ctx.device_status() != 0:
            raise RuntimeError("device status word raised during the denoised comparison")

    training = None
    if not args.no_denoise:
        training = denoiser_training(ctx, stream)
        if ctx.device_status() != 0:
            raise RuntimeError("device status word raised during denoiser training")

    batched = None
    if not args.no_batch:
        saved = ctx.vis_tuning()
        batched = batched_uneven(ctx, stream, flush, K, args.warmup, count=args.batch_scenes,
                                 tune=not args.batch_no_tune)
        ctx.set_vis_tuning(**saved)

    post = post_passes(g, stream, flush, K, args.warmup)

    stress = None
    if not args.no_stress:
        stress = stress_config5(ctx, stream, flush, min(K, 5), args.warmup)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu, _ = cpu_baseline(scene, args.cpu_rows, repeats=3)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator)",
                "config": dict(CONFIG, width=args.width, height=args.height,
                               parallelism=f"replicas{world}" if world > 1 else "single"),
                "rays_per_frame": rays_per_frame, "rays_traversed_per_frame": scene.width * scene.height + stats["rays"],
                "rays_note": "rays_per_frame (the unit of value) counts the rays light.frag traces: primary "
                             "+ lit pixels x (41 shadow + 16 AO). A shadow ray whose light's term in "
                             "the light pass cannot depend on it (weight max(dot(N, L), 0) = 0 or zero "
                             "unshadowed radiance) is resolved at generation without traversal, the "
                             "image is unchanged; rays_traversed_per_frame are the rays actually traced.",
                "traversed_grays_per_s": whole_job_rate(world, scene.width * scene.height + stats["rays"], ms),
                "lit_pixels": lit, "stage_ms": stage_ms, "kernel_ms": kernel_ms,
                "kernel_ms_note": "gbuffer includes its two tile-list kernels, raygen the near-list check of "
                                  "the AO rays and the beam-list kernel of the shadow rays",
                "blas_build": {"ms": g.blas_build_ms, "device_ms": g.blas_build_device_ms,
                               "triangles": g.blas_prims, "meshes": len(g.blas),
                               "algorithmic_bytes_per_triangle": 248,
                               "device_gbs": 248.0 * g.blas_prims / (g.blas_build_device_ms * 1e-3) / 1e9,
                               "hbm_frac": 248.0 * g.blas_prims / (g.blas_build_device_ms * 1e-3) / 1e9 / peak,
                               "note": "one batched build; ms includes the host->device vertex/index copies, "
                                       "device_ms is the device pipeline after them (CUDA events)"},
                "gpu_launches": launches, "roofline": roofline, "light_pass_roofline": light_pass,
                "cpu_baseline": cpu, "e2e": e2e,
                "clocks": clk, "denoised_vs_plain": denoised, "denoiser_training": training,
                "batched_uneven_64": batched,
                "stress_4k_4096_instances": stress, "post_passes_1080p": post}
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank)
        return
    run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
