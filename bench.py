"""Benchmark of the GB300 rendering path on the BVH-stress workload.

Workload (one step): 16 samples per pixel of the 1024x1024 path-traced image
of a level-8 displaced icosphere (1,310,720 triangles, one material per
face) on a ground quad under a uniform infinite light, max depth 8 -- one
pass of the hot path over 16,777,216 pixel samples.  Metric: Msamples/s.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

N > 1 runs under torchrun as N independent replicas (one per GPU, weak
scaling, no data-path collective); rank 0 prints one JSON line.
`--impl reference` times the reference algorithm on the host cores (the
float64 restatement in oracle/, 64x64 tiles on all host threads, scene build
excluded) on a bounded sample of the same workload.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "go-progressive-raytracer_gb300")
for _p in (PKG, ROOT):
    if _p not in sys.path:
        sys.path.insert(0, _p)

WIDTH = 1024
SPP = 16
DEPTH = 8
LEVEL = 8
METRIC = "Msamples/s at fixed image RMSE, batched-serving vs plain; p50/p99 first-pass ms"
WORKLOAD = "icosphere-L8 displaced (1,310,720 tris, per-face Lambertian/metal), ground quad, uniform sky; " \
           "1024x1024, 16 spp per step, max depth 8, path tracing"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gprt", choices=["gprt", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def build_libs():
    import importlib.util
    for path, name in ((os.path.join(PKG, "build.py"), "gprt_build"), (os.path.join(ROOT, "oracle", "build.py"), "ob")):
        spec = importlib.util.spec_from_file_location(name, path)
        m = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(m)
        m.build()


def make_scene():
    from gprt import scenes
    return scenes.icosphere_scene(level=LEVEL, width=WIDTH, max_depth=DEPTH)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    Q = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown," \
        "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown," \
        "clocks_event_reasons.sw_power_cap"

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def committed_traffic():
    """DRAM bytes per extend launch from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "extend_traffic.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("dram_bytes_per_launch"), d
    return None, None


def cpu_baseline(flat, seconds=15.0, threads=None, seed=101):
    """The oracle (float64 restatement of the reference's CPU path) on a
    bounded sample of the workload: whole 64x64 tiles at 16 spp."""
    from oracle import client
    threads = threads or os.cpu_count()
    t0 = time.time()
    sc = client.OracleScene(flat)
    build_s = time.time() - t0
    r = client.OracleRenderer(sc, 0, max_spp=SPP, max_passes=1, seed=seed, threads=threads)
    probe = max(1, threads)
    secs, st = r.render_pass(1, only_tiles=probe)
    rate = st[1] / max(secs, 1e-9)  # samples/s (tiles beyond `probe` hold 0 samples)
    tiles = int(min(256, max(probe, probe * seconds / max(secs, 1e-3))))
    r2 = client.OracleRenderer(sc, 0, max_spp=SPP, max_passes=1, seed=seed + 1, threads=threads)
    secs2, st2 = r2.render_pass(1, only_tiles=tiles)
    r.close()
    r2.close()
    sc.close()
    return {"value": st2[1] / secs2 / 1e6, "unit": "Msamples/s", "cores": threads, "kind": "port",
            "sample": "%d of 256 64x64 tiles of the 1024x1024 image at 16 spp (%d samples, %.1f s); scene build "
                      "%.1f s excluded" % (tiles, st2[1], secs2, build_s)}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    build_libs()
    from oracle import client
    flat = make_scene().to_desc()
    sc = client.OracleScene(flat)
    threads = os.cpu_count()
    tiles = max(threads, 16)
    times, samples = [], []
    for i in range(args.warmup + args.steps):
        r = client.OracleRenderer(sc, 0, max_spp=SPP, max_passes=1, seed=1000 + i, threads=threads)
        secs, st = r.render_pass(1, only_tiles=tiles)
        r.close()
        if i >= args.warmup:
            times.append(secs)
            samples.append(st[1])
    v = sum(samples) / sum(times) / 1e6
    line = {"metric": METRIC, "value": v, "unit": "Msamples/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD, "parallelism": "host threads", "sample": "%d tiles per step" % tiles},
            "cpu_baseline": {"value": v, "unit": "Msamples/s", "cores": threads, "kind": "port",
                             "sample": "%d of 256 64x64 tiles at 16 spp per step" % tiles},
            "e2e": {"value": v, "unit": "Msamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_gprt(args):
    rank, world, local = dist_env()
    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    build_libs()
    import gprt
    from gprt import capi

    scene = make_scene()
    flat = scene.to_desc()
    ctx = gprt.Context(local)
    g = gprt.GpuScene(ctx, flat)
    npix = g.width * g.height
    samples_per_step = npix * SPP

    # work per extend launch, counted once on the same inputs (not timed)
    cj = gprt.ProgressiveRaytracer(g, gprt.ProgressiveConfig(max_samples_per_pixel=SPP, max_passes=1, seed=1,
                                                             flags=capi.JOB_COUNT_TRAVERSAL | capi.JOB_TIME_KERNELS))
    cj.add_samples(SPP)
    cnt = cj.counters()
    cj.close()

    # autotuned wavefront size / traversal variants / block size (not timed)
    tuned, tune = gprt.renderer.autotune(g, spp=SPP, config=gprt.ProgressiveConfig(max_samples_per_pixel=SPP))
    job = gprt.ProgressiveRaytracer(g, gprt.ProgressiveConfig(max_samples_per_pixel=1 << 30, max_passes=1, seed=1,
                                                              flags=capi.JOB_TIME_KERNELS | tuned.flags,
                                                              block_size=tuned.block_size,
                                                              chunk_paths=tuned.chunk_paths))
    stream = torch.cuda.ExternalStream(job.stream())
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    for _ in range(args.warmup):
        with torch.cuda.stream(stream):
            flush.zero_()
        job.add_samples(SPP)
    job.sync()
    job.counters(reset=True)
    launches0 = job.launches()
    clocks = ClockSampler(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()  # L2 flush: 512 MB write before every step
        job.add_samples(SPP)
    ev1.record(stream)
    job.sync()
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    clk = clocks.stop()
    timed_launches = job.launches() - launches0 + args.steps  # + the flush kernels
    kc = job.counters()
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        dist.barrier()
    value = world * samples_per_step * args.steps / (ms / 1e3) / 1e6

    # roofline of the dominant kernel: closest-hit traversal ("extend")
    peak, peak_kind = measured_peaks()
    ray_b = 32 + 16
    alg_bytes = cnt["extend_rays"] * ray_b + 24 * cnt["extend_boxes"] + 36 * cnt["extend_prims"]
    per_launch = alg_bytes / max(1, cnt["extend_launches"])
    avg_ms = kc["extend_ms"] / max(1, kc["extend_launches"])
    achieved = per_launch / (avg_ms / 1e3) / 1e9
    traffic, _ = committed_traffic()
    roof = {"bound": "hbm", "kernel": "k_pt_extend (closest-hit BVH4 traversal)", "achieved": achieved,
            "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
            "traffic": traffic, "alg_bytes_per_launch": per_launch, "avg_launch_ms": avg_ms,
            "rays_per_launch": cnt["extend_rays"] / max(1, cnt["extend_launches"]),
            "box_tests_per_ray": cnt["extend_boxes"] / max(1, cnt["extend_rays"]),
            "tri_tests_per_ray": cnt["extend_prims"] / max(1, cnt["extend_rays"])}
    kernel_share = {k: kc[k + "_ms"] for k in ("extend", "shade", "shadow", "other")}
    rays_total = (cnt["extend_rays"] + cnt["shadow_rays"]) * args.steps  # per-step rays x steps (same workload)

    # end to end through the C ABI with host buffers
    e2e = None
    if args.e2e_steps > 0:
        rgba = np.zeros((g.height, g.width, 4), dtype=np.uint8)
        h2d = 0
        t_total = 0.0
        parts = {"scene_create_ms": 0.0, "render_ms": 0.0, "readback_ms": 0.0}
        for i in range(args.e2e_steps + 1):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s2 = gprt.GpuScene(ctx, flat)
            t1 = time.perf_counter()
            j2 = gprt.ProgressiveRaytracer(s2, gprt.ProgressiveConfig(max_samples_per_pixel=SPP, max_passes=1, seed=7 + i))
            j2.add_samples(SPP)
            j2.sync()
            t2 = time.perf_counter()
            ctx.check(ctx.lib.gprt_job_read_rgba8(j2.h, rgba.ctypes.data_as(capi.U8P)))
            t3 = time.perf_counter()
            h2d = s2.info.device_bytes
            j2.close()
            s2.close()
            if i == 0:
                continue  # first call warms allocations
            t_total += t3 - t0
            parts["scene_create_ms"] += 1e3 * (t1 - t0) / args.e2e_steps
            parts["render_ms"] += 1e3 * (t2 - t1) / args.e2e_steps
            parts["readback_ms"] += 1e3 * (t3 - t2) / args.e2e_steps
        e2e = {"value": samples_per_step * args.e2e_steps / t_total / 1e6, "unit": "Msamples/s",
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(rgba.nbytes),
               "includes": "scene upload + host BVH build, job create, 16 spp, RGBA8 read-back", **parts}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            cpu = cpu_baseline(flat)
        except Exception as e:  # the baseline never blocks the GPU line
            cpu = {"value": None, "error": str(e)}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "Msamples/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded icosphere, no dataset)",
                "config": {"workload": WORKLOAD, "samples_per_step": samples_per_step, "triangles": 1310720,
                           "l2": "flushed (512 MB write before every timed step)",
                           "parallelism": "replicas" if world > 1 else "single GPU",
                           "autotuned": {"chunk_paths": tuned.chunk_paths, "block_size": tuned.block_size,
                                         "simple_extend": bool(tuned.flags & capi.JOB_SIMPLE_EXTEND),
                                         "simple_shadow": bool(tuned.flags & capi.JOB_SIMPLE_SHADOW),
                                         "candidates": tune["candidates"], "tuning_pass_ms": tune["best_ms"],
                                         "default_pass_ms": tune["default_ms"]}},
                "mrays_per_s": rays_total * world / (ms / 1e3) / 1e6,
                "roofline": roof, "kernel_ms": kernel_share, "cpu_baseline": cpu, "e2e": e2e,
                "gpu_launches": int(timed_launches), "clocks": clk,
                "scene": {"nodes": int(g.info.n_nodes), "device_mb": g.info.device_bytes / 2 ** 20,
                          "host_bvh_build_ms": g.info.build_ms}}
        print(json.dumps(line))
    job.close()
    g.close()
    ctx.close()
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_gprt(args)


if __name__ == "__main__":
    sys.exit(main())
