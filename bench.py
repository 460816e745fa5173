"""Benchmark of the GB300 rendering path: batched serving vs the plain path.

Headline workload (one step): the heterogeneous batch -- 256 seeded
default-style sphere scenes (ground sphere, 3 feature spheres, 10-500 small
spheres of 60/25/15 % Lambertian / metal / glass, gradient sky) at
resolutions drawn from {128^2, 256^2, 512^2, 1024x768}, spp ~ U[1,64], max
depth 8, about 2.14 G pixel samples -- rendered to completion by the batched
render server (many jobs per wavefront, bounce sequences replayed from CUDA
graphs, autotuned step size / block size / traversal variant).  Metric:
aggregate Msamples/s.  Beside it, on the same GPU:
  plain      the same 256 jobs one at a time through the per-job path;
  serving    Poisson request streams mixing the Cornell (400^2), icosphere
             (1024^2, 1.3 M triangles), Cornell-boxes (512^2) and
             default-style scenes, target spp 16-256 in passes of 4 spp:
             p50/p99 time-to-first-pass and per-pass latency, aggregate
             Msamples/s, batched server vs plain one-job-at-a-time;
  per_config every configuration of the reference's path through the
             autotuned per-job path: Cornell 400^2 64 spp, the reference
             Cornell spheres 400^2 64 spp, the icosphere 1024^2 16 spp (with
             its traversal roofline), Cornell boxes 512^2 64 spp under BDPT,
             and the raw 2^24-ray intersection batch (closest and any hit).
Every job's film is the same alone and in the batch (bit for bit), so the
comparison is at equal image RMSE.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

N > 1 runs under torchrun as N independent replicas (one per GPU, weak
scaling, no data-path collective); rank 0 prints one JSON line.
`--impl reference` times the reference algorithm on the host cores (the
float64 restatement in oracle/, 64x64 tiles on all host threads) on a bounded
sample of the same batch.
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

NJOBS = 256
JOB_SEED = 17
DEPTH = 8
METRIC = "Msamples/s at fixed image RMSE, batched-serving vs plain; p50/p99 first-pass ms"
WORKLOAD = "256 heterogeneous default-style sphere scenes (seed 17; 10-500 spheres each; 128^2/256^2/512^2/1024x768; " \
           "spp U[1,64]; max depth 8), path tracing, batched render server"
ICO_WIDTH, ICO_SPP, ICO_LEVEL = 1024, 16, 8


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gprt", choices=["gprt", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--stream-requests", type=int, default=48)
    ap.add_argument("--rates", default="20,50,100,200")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-per-config", action="store_true")
    ap.add_argument("--no-stream", action="store_true")
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


def l2_absorption(traffic, alg_bytes, avg_ms, peak):
    """How much of a traversal launch's algorithmic bytes reach DRAM (the
    ncu traffic per launch scaled to the timed launch) and the DRAM-side
    fraction of the HBM peak.  The upper BVH levels and, for scenes of a
    few hundred spheres, whole trees stay in the 129 MB L2, so the
    algorithmic fraction can exceed 1 while DRAM is far from busy: the
    kernel is then bound by L2 and memory latency, not HBM bandwidth."""
    if not traffic or not alg_bytes or not avg_ms:
        return {}
    dram_gbs = traffic / (avg_ms / 1e3) / 1e9
    return {"dram_share_of_alg_bytes": traffic / alg_bytes, "dram_gbs": dram_gbs, "dram_frac": dram_gbs / peak}


_L2_PEAK = {}


def l2_copy_gbs(torch):
    """L2-resident copy bandwidth of this GPU, measured like the HBM peak (a
    torch copy, read + write bytes) but over a 2 x 40 MB working set that the
    129 MB L2 holds: 64 copies captured in one CUDA graph (no launch gaps),
    best of 5 replays after a warm-up.  The denominator for traversal
    kernels whose upper tree levels stay in L2."""
    if "gbs" in _L2_PEAK:
        return _L2_PEAK["gbs"]
    n = 20 * 1024 * 1024  # bf16 elements: 40 MB per buffer
    a = torch.ones(n, dtype=torch.bfloat16, device="cuda")
    b = torch.empty_like(a)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        for _ in range(3):
            b.copy_(a)
    torch.cuda.current_stream().wait_stream(s)
    g = torch.cuda.CUDAGraph()
    reps = 64
    with torch.cuda.graph(g):
        for _ in range(reps):
            b.copy_(a)
    best = None
    for k in range(6):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        g.replay()
        e1.record()
        e1.synchronize()
        if k:
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
    gbs = 2 * a.numel() * a.element_size() * reps / (best / 1e3) / 1e9
    del g, a, b
    _L2_PEAK["gbs"] = gbs
    return gbs


def l2_fraction(achieved, torch):
    """The traversal kernel's algorithmic bandwidth against the L2 copy
    bandwidth (the node and primitive fetches that L2 and L1 serve)."""
    try:
        gbs = l2_copy_gbs(torch)
    except Exception as e:  # reported, not fatal: the HBM roofline stands
        return {"l2_peak_error": str(e)}
    return {"l2_copy_gbs": gbs, "frac_of_l2": (achieved / gbs) if achieved else None,
            "l2_peak_how": "torch bf16 copy over 2 x 40 MB (L2-resident), 64 copies per CUDA graph, best of 5"}


# Path-state bytes of one shading step (the SoA queues of the wavefront):
# a shaded path reads ray origin, direction, hit, weight, roulette
# throughput, radiance and ids (7 x 16 B), except at bounce 0 (one shaded
# path per sample), where weight, throughput and radiance are implied
# (4 x 16 B); a
# continuing path writes all but the hit to the next queue (6 x 16 B); a
# finished path writes its radiance (16 B); a shadow ray writes origin,
# direction, contribution (3 x 16 B) and its BVH root (4 B).
SHADE_READ_B, SHADE_BOUNCE0_B, SHADE_CONT_B, SHADE_DONE_B, SHADE_SHADOW_B = 112, 64, 96, 16, 52


def shade_roofline(cnt, kc, kc_batches, samples, peak, peak_kind, timing_source):
    """Roofline of the multi-job shading kernel.  Paths shaded = extend rays
    (every queued path is traced, then shaded); each sample's path finishes
    exactly once, so continuing paths = shaded - samples.  Material, light
    and item tables (a few KB per job, L1-resident) are not counted."""
    shaded, shadow = cnt["extend_rays"], cnt["shadow_rays"]
    alg = (SHADE_READ_B * (shaded - samples) + SHADE_BOUNCE0_B * samples + SHADE_CONT_B * (shaded - samples) +
           SHADE_DONE_B * samples + SHADE_SHADOW_B * shadow)
    # per launch of the timed configuration: the counting run may split the
    # batch into steps of another size
    launches = max(1.0, kc["shade_launches"] / kc_batches)
    per_launch = alg / launches
    avg_ms = kc["shade_ms"] / max(1, kc["shade_launches"])
    achieved = per_launch / (avg_ms / 1e3) / 1e9 if kc["shade_launches"] else None
    traffic, _ = committed_traffic("shade_batch_traffic.json", shaded / launches, key="dram_bytes_per_path")
    r = {"bound": "hbm", "kernel": "k_srv_shade (one bounce of every path of a step, all jobs)",
         "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": (achieved / peak) if achieved else None,
         "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)", "traffic": traffic,
         "alg_bytes_per_launch": per_launch, "avg_launch_ms": avg_ms, "launch_timing": timing_source,
         "paths_per_launch": shaded / launches, "shadow_rays_per_path": shadow / max(1, shaded),
         "alg_bytes_per_path": alg / max(1, shaded)}
    if traffic and avg_ms:
        r["dram_gbs"] = traffic / (avg_ms / 1e3) / 1e9
        r["dram_frac"] = r["dram_gbs"] / peak
    return r


def committed_traffic(name, rays_per_launch, key="dram_bytes_per_ray"):
    """DRAM bytes per launch of the extend kernel: the committed ncu capture's
    DRAM bytes per ray (a smaller case of the same kernel) x rays per launch."""
    p = os.path.join(ROOT, "profiles", name)
    if os.path.exists(p):
        d = json.load(open(p))
        return d[key] * rays_per_launch, d
    return None, None


def aggregate_over_ranks(ms, samples_per_rank, steps, dist=None, device="cpu"):
    """Max timed-region duration over the replicas and the whole-job rate
    (weak scaling: every rank renders its own copy of the workload, no
    data-path collective).  Returns (ms, Msamples/s)."""
    world = 1
    if dist is not None and dist.is_initialized():
        import torch
        t = torch.tensor([ms], device=device, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        world = dist.get_world_size()
    return ms, world * samples_per_rank * steps / (ms / 1e3) / 1e6


def batch_jobs():
    from gprt import scenes
    return [(s.to_desc(), spp) for s, spp in scenes.batched_jobs(NJOBS, JOB_SEED, DEPTH)]


def job_config(spp, seed=1):
    import gprt
    return gprt.ProgressiveConfig(initial_samples=spp, max_samples_per_pixel=spp, max_passes=1, seed=seed)


# ----------------------------------------------------------------- CPU side
def oracle_sample(jobs, seconds, threads, seed):
    """Renders whole 64x64 tiles of the batch's jobs (in order, at each job's
    spp) with the oracle until about `seconds` of work; returns
    (samples, seconds, description)."""
    from oracle import client
    done_s, done_n, parts = 0.0, 0, []
    for k, (flat, spp) in enumerate(jobs):
        if done_s >= seconds:
            break
        sc = client.OracleScene(flat)
        ntiles = ((sc.width + 63) // 64) * ((sc.height + 63) // 64)
        r = client.OracleRenderer(sc, 0, max_spp=spp, max_passes=1, seed=seed + k, threads=threads)
        probe = min(ntiles, threads)
        secs, st = r.render_pass(1, only_tiles=probe)
        r.close()
        per_tile = secs / probe
        want = int(min(ntiles, max(probe, (seconds - done_s) / max(per_tile, 1e-6))))
        used = probe
        if want > probe:
            r = client.OracleRenderer(sc, 0, max_spp=spp, max_passes=1, seed=seed + k, threads=threads)
            secs, st = r.render_pass(1, only_tiles=want)
            r.close()
            used = want
        sc.close()
        done_s += secs
        done_n += st[1]
        parts.append("job %d: %d tiles at %d spp" % (k, used, spp))
    return done_n, done_s, "; ".join(parts)


def cpu_baseline(jobs, seconds=15.0):
    threads = os.cpu_count()
    n, s, desc = oracle_sample(jobs, seconds, threads, 101)
    return {"value": n / s / 1e6, "unit": "Msamples/s", "cores": threads, "kind": "port",
            "sample": "oracle (float64 restatement of the reference CPU path), %d host threads, %d samples in %.1f s "
                      "of whole 64x64 tiles of the batch's first jobs (%s); scene builds excluded"
                      % (threads, n, s, desc)}


def cpu_per_config(seconds=5.0):
    """The oracle on each of the other workloads, about `seconds` of whole
    64x64 tiles each (scene builds excluded): the CPU figure beside each
    per-config GPU number."""
    from oracle import client
    threads = os.cpu_count()
    out = {}
    for name, spp, bdpt in PER_CONFIG:
        integ = 1 if bdpt else 0
        sc = client.OracleScene(config_scene(name).to_desc())
        r = client.OracleRenderer(sc, integ, max_spp=spp, max_passes=1, seed=11, threads=threads)
        secs, st = r.render_pass(1, only_tiles=threads)
        r.close()
        ntiles = ((sc.width + 63) // 64) * ((sc.height + 63) // 64)
        want = int(min(ntiles, max(threads, threads * seconds / max(secs, 1e-3))))
        r = client.OracleRenderer(sc, integ, max_spp=spp, max_passes=1, seed=12, threads=threads)
        secs, st = r.render_pass(1, only_tiles=want)
        r.close()
        sc.close()
        out[name] = {"msamples_per_s": st[1] / secs / 1e6, "tiles": want, "seconds": secs}
    return {"cores": threads, "kind": "port", "configs": out}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    build_libs()
    jobs = batch_jobs()
    threads = os.cpu_count()
    per_step = 4.0  # seconds of host work per step
    times, samples = [], []
    for i in range(args.warmup + args.steps):
        n, s, desc = oracle_sample(jobs[i % 8:], per_step, threads, 1000 + 17 * i)
        if i >= args.warmup:
            times.append(s)
            samples.append(n)
    v = sum(samples) / sum(times) / 1e6
    line = {"metric": METRIC, "value": v, "unit": "Msamples/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD, "parallelism": "%d host threads" % threads,
                       "sample": "about %.0f s of whole 64x64 tiles of the batch's jobs per step" % per_step},
            "cpu_baseline": {"value": v, "unit": "Msamples/s", "cores": threads, "kind": "port",
                             "sample": "about %.0f s of whole 64x64 tiles of the batch's jobs per step" % per_step},
            "e2e": {"value": v, "unit": "Msamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ----------------------------------------------------------------- GPU side
def run_batch(sv, gscenes, spps, seed=1):
    """Submits every job, steps the server until all are done and releases
    them; returns the jobs' sample total."""
    tickets = [sv.submit(g, job_config(s, seed)) for g, s in zip(gscenes, spps)]
    sv.run_until_idle()
    for t in tickets:
        sv.release(t)
    return sum(g.width * g.height * s for g, s in zip(gscenes, spps))


def run_plain_batch(gscenes, spps, seed=1):
    """The same jobs one at a time through the per-job path."""
    import gprt
    n = 0
    for g, s in zip(gscenes, spps):
        r = gprt.ProgressiveRaytracer(g, gprt.ProgressiveConfig(max_samples_per_pixel=s, max_passes=1, seed=seed))
        r.add_samples(s)
        r.sync()
        r.close()
        n += g.width * g.height * s
    return n


# request kinds of the serving stream rendered with BDPT (the Cornell-boxes
# scene, kind 2 of scenes.serving_requests)
BDPT_KINDS = (2,)


# Path capacity of a serving step at most: the offline batch may tune larger
# steps (fewer, longer launches), but a step is what a new request waits for
# before its first pass, so serving keeps them at 2^23 paths (about 5-10 ms).
SERVING_STEP_PATHS = 1 << 23


def stream_batched(ctx, server_kw, tune, reqs, arrivals, gs):
    """Serves a request stream with the batched server's loop thread."""
    import gprt
    sv = gprt.RenderServer(ctx, **server_kw)
    sv.configure(min(tune["chunk_paths"], SERVING_STEP_PATHS), tune["block_size"], tune["flags"])
    sv.start()
    t0 = time.perf_counter()
    tickets = []
    for (kind, spp), at in zip(reqs, arrivals):
        while time.perf_counter() - t0 < at:
            time.sleep(0.0002)
        cfg = gprt.ProgressiveConfig(initial_samples=4, max_samples_per_pixel=spp, max_passes=spp // 4, seed=5)
        tickets.append(sv.submit(gs[kind], cfg, integrator=gprt.BDPTIntegrator() if kind in BDPT_KINDS else None))
    ev = []
    deadline = time.perf_counter() + 600
    while len({e.ticket for e in ev if e.kind == "done"}) < len(tickets) and time.perf_counter() < deadline:
        ev += sv.poll(1024, timeout_ms=20)
    sv.stop()
    st = sv.stats()
    for t in tickets:
        sv.release(t)
    sv.close()
    first_submit = min((e.submit_ms for e in ev), default=0.0)
    last_done = max((e.t_ms for e in ev if e.kind == "done"), default=first_submit)
    return ev, tickets, (last_done - first_submit) / 1e3, st


def stream_plain(reqs, arrivals, gs):
    """The same stream served one job at a time, in arrival order, by the
    per-job path (passes of 4 spp)."""
    import gprt
    ev = []
    t0 = time.perf_counter()
    for k, ((kind, spp), at) in enumerate(zip(reqs, arrivals)):
        now = time.perf_counter() - t0
        if now < at:
            time.sleep(at - now)
        r = gprt.ProgressiveRaytracer(gs[kind], gprt.ProgressiveConfig(max_samples_per_pixel=spp, max_passes=spp // 4,
                                                                       seed=5),
                                      integrator=gprt.BDPTIntegrator() if kind in BDPT_KINDS else None)
        for p in range(spp // 4):
            r.add_samples(4)
            r.sync()
            ev.append(gprt.ServerEvent(k, "pass", p + 1, 4 * (p + 1), 0, 1e3 * (time.perf_counter() - t0), 1e3 * at))
        r.close()
        ev.append(gprt.ServerEvent(k, "done", spp // 4, spp, 0, 1e3 * (time.perf_counter() - t0), 1e3 * at))
    last = max(e.t_ms for e in ev) / 1e3
    return ev, last - arrivals[0]


def serving_section(ctx, args, server_kw, tune, flats):
    """Request streams at each rate, batched and (at the middle rate) plain."""
    import gprt
    from gprt import scenes
    gs = [gprt.GpuScene(ctx, f) for f in flats]
    sizes = [g.width * g.height for g in gs]
    reqs = scenes.serving_requests(args.stream_requests)
    samples = sum(sizes[k] * spp for k, spp in reqs)
    out = {"requests": len(reqs), "mix": "Cornell 400^2 PT / icosphere 1024^2 PT / Cornell boxes 512^2 BDPT / "
                                         "default-style 512^2 scene PT, target spp U{16..256} in passes of 4 spp",
           "bdpt_requests": sum(1 for k, _ in reqs if k in BDPT_KINDS),
           "requests_512sq_pt": sum(1 for k, _ in reqs if sizes[k] == 512 * 512 and k not in BDPT_KINDS),
           "samples_per_stream": samples, "rates": {}}
    rates = [float(x) for x in args.rates.split(",") if x]
    for rate in rates:
        arr = scenes.poisson_arrivals(len(reqs), rate)
        ev, tickets, span, st = stream_batched(ctx, server_kw, tune, reqs, arr, gs)
        t512 = [t for t, (k, _) in zip(tickets, reqs) if gs[k].width == 512 and gs[k].height == 512]
        pt512 = [t for t, (k, _) in zip(tickets, reqs) if t in t512 and k not in BDPT_KINDS]
        bd512 = [t for t, (k, _) in zip(tickets, reqs) if t in t512 and k in BDPT_KINDS]
        out["rates"][str(int(rate))] = {
            "batched": {"msamples_per_s": samples / span / 1e6, "makespan_s": span,
                        **gprt.latency_summary(ev),
                        "ttfp_p99_ms_512sq": gprt.latency_summary(ev, t512)["ttfp_p99_ms"],
                        "ttfp_p99_ms_512sq_pt": gprt.latency_summary(ev, pt512)["ttfp_p99_ms"] if pt512 else None,
                        "ttfp_p99_ms_512sq_bdpt": gprt.latency_summary(ev, bd512)["ttfp_p99_ms"] if bd512 else None,
                        "ttfp_p50_ms_512sq_bdpt": gprt.latency_summary(ev, bd512)["ttfp_p50_ms"] if bd512 else None,
                        "steps": st["steps"], "graph_launches": st["graph_launches"]}}
    mid = rates[len(rates) // 2] if rates else None
    if mid is not None:
        arr = scenes.poisson_arrivals(len(reqs), mid)
        ev, span = stream_plain(reqs, arr, gs)
        idx512 = [k for k, (kind, _) in enumerate(reqs) if gs[kind].width == 512 and gs[kind].height == 512]
        out["rates"][str(int(mid))]["plain"] = {"msamples_per_s": samples / span / 1e6, "makespan_s": span,
                                                **gprt.latency_summary(ev),
                                                "ttfp_p99_ms_512sq": gprt.latency_summary(ev, idx512)["ttfp_p99_ms"]}
    for g in gs:
        g.close()
    return out


def _event_frames(torch, stream, flush, frames, render):
    """Mean device time of `frames` calls of render() on `stream`: CUDA
    events around each call, an L2 flush (512 MB write) before each, outside
    the events."""
    evs = []
    for _ in range(frames):
        with torch.cuda.stream(stream):
            flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        render()
        e1.record(stream)
        evs.append((e0, e1))
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in evs) / frames


def _tuned_job(g, integ, spp, extra_flags=0):
    import gprt
    tuned, _ = gprt.renderer.autotune(g, integ, spp=spp, config=gprt.ProgressiveConfig(max_samples_per_pixel=spp))
    conf = gprt.ProgressiveConfig(max_samples_per_pixel=1 << 30, max_passes=1, seed=1, flags=tuned.flags | extra_flags,
                                  block_size=tuned.block_size, chunk_paths=tuned.chunk_paths)
    job = gprt.ProgressiveRaytracer(g, conf, integ) if integ else gprt.ProgressiveRaytracer(g, conf)
    return job, tuned


def render_config(ctx, torch, flush, flat, spp, bdpt=False, frames=8):
    """One benchmark configuration through the autotuned per-job path: mean
    device time per frame (`spp` samples per pixel, CUDA events on the job
    stream, L2 flushed before every frame), the kernel split of a frame, and
    the first progressive pass (1 spp) of a fresh job on the host clock."""
    import gprt
    from gprt import capi
    g = gprt.GpuScene(ctx, flat)
    integ = gprt.BDPTIntegrator() if bdpt else None
    job, tuned = _tuned_job(g, integ, spp, capi.JOB_TIME_KERNELS)
    stream = torch.cuda.ExternalStream(job.stream())
    for _ in range(2):
        job.add_samples(spp)
    job.sync()
    job.counters(reset=True)
    ms = _event_frames(torch, stream, flush, frames, lambda: job.add_samples(spp))
    kc = job.counters()
    job.close()
    conf = gprt.ProgressiveConfig(initial_samples=1, max_samples_per_pixel=spp, max_passes=max(2, spp // 4), seed=2)
    first = gprt.ProgressiveRaytracer(g, conf, integ) if integ else gprt.ProgressiveRaytracer(g, conf)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    first.render_pass(1)
    ttfp = (time.perf_counter() - t0) * 1e3
    first.close()
    n = g.width * g.height * spp
    out = {"width": g.width, "height": g.height, "spp": spp, "integrator": "bdpt" if bdpt else "path tracing",
           "ms_per_frame": ms, "msamples_per_s": n / ms / 1e3, "first_pass_ms": ttfp,
           "kernel_ms_per_frame": {k: kc[k + "_ms"] / frames for k in ("extend", "shade", "shadow", "other")},
           "autotuned": {"chunk_paths": tuned.chunk_paths, "block_size": tuned.block_size, "flags": tuned.flags}}
    return out, g, tuned


def icosphere_extras(ctx, torch, flush, g, flat, tuned, frame_ms):
    """The icosphere's closest-hit roofline (algorithmic bytes per ray = 32 B
    ray in + 16 B hit out + 24 B per child-box test + 36 B per triangle test,
    counted on the same frame by the counting kernels) and the same scene
    built on the GPU (GPRT_BUILD_DEVICE)."""
    import gprt
    from gprt import capi
    cj = gprt.ProgressiveRaytracer(g, gprt.ProgressiveConfig(max_samples_per_pixel=ICO_SPP, max_passes=1, seed=1,
                                                             flags=capi.JOB_COUNT_TRAVERSAL))
    cj.add_samples(ICO_SPP)
    cnt = cj.counters()
    cj.close()
    job = gprt.ProgressiveRaytracer(g, gprt.ProgressiveConfig(max_samples_per_pixel=1 << 30, max_passes=1, seed=1,
                                                              flags=capi.JOB_TIME_KERNELS | tuned.flags,
                                                              block_size=tuned.block_size,
                                                              chunk_paths=tuned.chunk_paths))
    stream = torch.cuda.ExternalStream(job.stream())
    job.add_samples(ICO_SPP)
    job.sync()
    job.counters(reset=True)
    steps = 6
    _event_frames(torch, stream, flush, steps, lambda: job.add_samples(ICO_SPP))
    kc = job.counters()
    job.close()
    peak, peak_kind = measured_peaks()
    alg = cnt["extend_rays"] * 48 + 24 * cnt["extend_boxes"] + 36 * cnt["extend_prims"]
    launches = max(1.0, kc["extend_launches"] / steps)
    per_launch = alg / launches
    avg_ms = kc["extend_ms"] / max(1, kc["extend_launches"])
    achieved = per_launch / (avg_ms / 1e3) / 1e9
    traffic, _ = committed_traffic("extend_traffic.json", cnt["extend_rays"] / launches)
    out = {"mrays_per_s": (cnt["extend_rays"] + cnt["shadow_rays"]) / (frame_ms / 1e3) / 1e6,
           "extend_roofline": {"kernel": "k_pt_extend", "achieved": achieved, "peak": peak, "unit": "GB/s",
                               "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
                               "alg_bytes_per_launch": per_launch, "avg_launch_ms": avg_ms,
                               **l2_absorption(traffic, per_launch, avg_ms, peak), **l2_fraction(achieved, torch)}}
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    gd = gprt.GpuScene(ctx, flat, device_bvh=True)
    create_dev = (time.perf_counter() - t0) * 1e3
    jd = gprt.ProgressiveRaytracer(gd, gprt.ProgressiveConfig(max_samples_per_pixel=1 << 30, max_passes=1, seed=1,
                                                              flags=tuned.flags, block_size=tuned.block_size,
                                                              chunk_paths=tuned.chunk_paths))
    sd = torch.cuda.ExternalStream(jd.stream())
    jd.add_samples(ICO_SPP)
    jd.sync()
    out["scene_build"] = {"host_sah_ms": g.info.build_ms, "host_sah_flatten_ms": g.info.flatten_ms,
                          "device_lbvh_create_ms": create_dev, "device_lbvh_build_ms": gd.info.build_ms,
                          "device_lbvh_nodes": int(gd.info.n_nodes), "host_sah_nodes": int(g.info.n_nodes),
                          "device_lbvh_ms_per_frame": _event_frames(torch, sd, flush, 3,
                                                                    lambda: jd.add_samples(ICO_SPP))}
    jd.close()
    gd.close()
    return out


def raw_batch(ctx, torch, flush, flat, mesh, frames=6):
    """The raw intersection batch: 2^24 rays on the level-8 icosphere (half
    camera rays at 1024^2, half surface-point rays in uniform directions,
    seed 13), closest and any hit, through gprt_intersect on device
    buffers.  Roofline bytes per ray as for the render's extend kernel,
    counted on a 1/64 sample of the batch."""
    import gprt
    from gprt import capi, scenes
    n = 1 << 24
    rays = scenes.ray_batch(mesh.vertices, mesh.faces, n, seed=13, width=ICO_WIDTH)
    g = gprt.GpuScene(ctx, flat)
    d_rays = torch.from_numpy(rays).cuda()
    d_hits = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    st = torch.cuda.Stream()  # a real stream handle (NULL would mean the library's own stream)
    st.wait_stream(torch.cuda.current_stream())
    peak, _ = measured_peaks()
    sample = rays[::64]
    out = {"rays": n}
    for name, flag in (("closest", capi.CLOSEST), ("any", capi.ANY)):
        call = lambda: ctx.check(ctx.lib.gprt_intersect(g.h, d_rays.data_ptr(), n, flag, d_hits.data_ptr(),
                                                        st.cuda_stream))
        for _ in range(2):
            call()
        ms = _event_frames(torch, st, flush, frames, call)
        nodes, boxes, prims = g.traversal_counts(sample, any_hit=(flag == capi.ANY))
        scale = n / len(sample)
        alg = n * 48 + scale * (24 * boxes + 36 * prims)
        achieved = alg / (ms / 1e3) / 1e9
        out[name] = {"ms_per_batch": ms, "mrays_per_s": n / ms / 1e3,
                     "roofline": {"achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                                  "box_tests_per_ray": boxes / len(sample), "tri_tests_per_ray": prims / len(sample),
                                  **l2_fraction(achieved, torch)}}
    out["hit_fraction"] = float((d_hits[:, 0] >= 0).float().mean().item())
    g.close()
    return out


PER_CONFIG = (("c0a_cornell_400_64spp_pt", 64, False), ("c0b_cornell_spheres_400_64spp_pt", 64, False),
              ("c1_icosphere_1024_16spp_pt", ICO_SPP, False), ("c2_cornell_boxes_512_64spp_bdpt", 64, True))


def config_scene(name):
    from gprt import scenes
    from gprt.scene import CameraConfig
    if name.startswith("c0a"):
        return scenes.cornell_baseline(400)
    if name.startswith("c0b"):  # the reference Cornell scene, every pixel taking every sample
        s = scenes.cornell_scene(scenes.CORNELL_SPHERES, camera=CameraConfig(width=400))
        s.sampling.adaptive_min_samples, s.sampling.adaptive_threshold = 1.0, 0.0
        return s
    if name.startswith("c1"):
        return scenes.icosphere_scene(level=ICO_LEVEL, width=ICO_WIDTH)
    return scenes.cornell_boxes_bdpt(512)


def per_config_section(ctx, torch):
    """Every benchmark configuration of the reference's path on the GPU:
    Cornell 400^2 64 spp, reference Cornell spheres 400^2 64 spp, the
    icosphere 1024^2 16 spp (with its extend roofline and the device-built
    BVH), Cornell boxes 512^2 64 spp under BDPT, and the raw 2^24-ray batch.
    The ALU-side figures of the L1-resident scenes come from committed ncu
    summaries (profiles/*_alu.json) when present."""
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    out = {}
    ico = None
    for name, spp, bdpt in PER_CONFIG:
        scene = config_scene(name)
        flat = scene.to_desc()
        r, g, tuned = render_config(ctx, torch, flush, flat, spp, bdpt)
        if name.startswith("c1"):
            r.update(icosphere_extras(ctx, torch, flush, g, flat, tuned, r["ms_per_frame"]))
            ico = (flat, scene.shapes[0].mesh)
        g.close()
        alu = os.path.join(ROOT, "profiles", name.split("_")[0] + "_alu.json")
        if os.path.exists(alu):
            r["alu"] = json.load(open(alu))
        out[name] = r
    out["raw_batch_2_24"] = raw_batch(ctx, torch, flush, *ico)
    del flush
    return out


def plain_section(ctx, torch, gscenes, spps, film0, batched_value, tune, world):
    """The plain per-job path on the same batch, analysed: the host-clock
    rate of one job at a time (job creation included, as a caller sees
    it), the device time of each job's pass (CUDA events on the job's
    stream) and the share of the wall clock the GPU sits idle between jobs,
    the same jobs with the launch configuration autotuned once per
    resolution class, and per resolution class the batched server on that
    class alone against the plain path on it."""
    import gprt
    run_plain_batch(gscenes[:16], spps[:16])  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    dev_ms, per_job = 0.0, []
    evs = []
    for g, s in zip(gscenes, spps):
        r = gprt.ProgressiveRaytracer(g, gprt.ProgressiveConfig(max_samples_per_pixel=s, max_passes=1, seed=1))
        st = torch.cuda.ExternalStream(r.stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        r.add_samples(s)
        e1.record(st)
        r.sync()
        r.close()
        evs.append((e0, e1))
    torch.cuda.synchronize()
    tp = time.perf_counter() - t0
    per_job = [a.elapsed_time(b) for a, b in evs]
    dev_ms = sum(per_job)
    n = sum(g.width * g.height * s for g, s in zip(gscenes, spps))
    r = gprt.ProgressiveRaytracer(gscenes[0], gprt.ProgressiveConfig(max_samples_per_pixel=spps[0], max_passes=1,
                                                                     seed=1))
    r.add_samples(spps[0])
    same = all(np.array_equal(a, b) for a, b in zip(r.film(), film0))
    r.close()
    classes = {}
    for k, g in enumerate(gscenes):
        classes.setdefault("%dx%d" % (g.width, g.height), []).append(k)
    # plain, launch configuration autotuned on the first job of each class
    tuned_ms = 0.0
    by_class = {}
    for cls, idx in classes.items():
        g0 = gscenes[idx[0]]
        tuned, _ = gprt.renderer.autotune(g0, spp=spps[idx[0]],
                                          config=gprt.ProgressiveConfig(max_samples_per_pixel=spps[idx[0]]))
        cms, tevs = 0.0, []
        for k in idx:
            job = gprt.ProgressiveRaytracer(gscenes[k], gprt.ProgressiveConfig(
                max_samples_per_pixel=spps[k], max_passes=1, seed=1, flags=tuned.flags, block_size=tuned.block_size,
                chunk_paths=tuned.chunk_paths))
            st = torch.cuda.ExternalStream(job.stream())
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            job.add_samples(spps[k])
            e1.record(st)
            job.sync()
            job.close()
            tevs.append((e0, e1))
        torch.cuda.synchronize()
        cms = sum(a.elapsed_time(b) for a, b in tevs)
        tuned_ms += cms
        samples = sum(gscenes[k].width * gscenes[k].height * spps[k] for k in idx)
        # the batched server on this class alone (one warm-up batch, one timed)
        sv = gprt.RenderServer(ctx, step_paths=tune["chunk_paths"], block_size=tune["block_size"],
                               flags=tune["flags"])
        sv.configure(tune["chunk_paths"], tune["block_size"], tune["flags"])
        sub_g, sub_s = [gscenes[k] for k in idx], [spps[k] for k in idx]
        run_batch(sv, sub_g, sub_s)
        stream = torch.cuda.ExternalStream(sv.stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        run_batch(sv, sub_g, sub_s)
        e1.record(stream)
        torch.cuda.synchronize()
        bms = e0.elapsed_time(e1)
        sv.close()
        plain_dev = sum(per_job[k] for k in idx)
        by_class[cls] = {"jobs": len(idx), "msamples": samples / 1e6,
                         "plain_device_msamples_per_s": samples / plain_dev / 1e3,
                         "plain_tuned_device_msamples_per_s": samples / cms / 1e3,
                         "batched_class_alone_msamples_per_s": samples / bms / 1e3,
                         "batched_over_plain_device": plain_dev / bms, "batched_over_plain_tuned": cms / bms,
                         "plain_mean_job_ms": plain_dev / len(idx)}
    return {"msamples_per_s": n / tp / 1e6, "s_per_batch": tp, "timing": "host clock, device-synchronised, "
            "job creation included",
            "batched_over_plain": batched_value / world / (n / tp / 1e6),
            "device_msamples_per_s": n / dev_ms / 1e3, "device_ms_per_batch": dev_ms,
            "gpu_idle_fraction": max(0.0, 1.0 - dev_ms / (tp * 1e3)),
            "batched_over_plain_device": batched_value / world / (n / dev_ms / 1e3),
            "tuned_per_class_msamples_per_s": n / tuned_ms / 1e3,
            "batched_over_plain_tuned": batched_value / world / (n / tuned_ms / 1e3),
            "by_resolution": by_class, "film_of_job0_identical": bool(same)}


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

    jobs = batch_jobs()
    ctx = gprt.Context(local)
    gscenes = [gprt.GpuScene(ctx, f) for f, _ in jobs]
    spps = [s for _, s in jobs]
    samples_per_step = sum(g.width * g.height * s for g, s in zip(gscenes, spps))
    cap = 1 << 25

    # work per extend launch, counted once on the same batch (not timed)
    sv = gprt.RenderServer(ctx, step_paths=cap,
                           flags=capi.JOB_COUNT_TRAVERSAL | capi.JOB_TIME_KERNELS | capi.SERVER_NO_GRAPHS)
    run_batch(sv, gscenes, spps)
    cnt = sv.counters()
    sv.close()

    # the batched server, autotuned on the admitted batch (tuning steps change no film)
    sv = gprt.RenderServer(ctx, step_paths=cap)
    tickets = [sv.submit(g, job_config(s)) for g, s in zip(gscenes, spps)]
    tune = sv.autotune()
    sv.run_until_idle()
    film0 = sv.film(tickets[0])
    for t in tickets:
        sv.release(t)
    sv.configure(tune["chunk_paths"], tune["block_size"], tune["flags"] | capi.JOB_TIME_KERNELS)
    stream = torch.cuda.ExternalStream(sv.stream())
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    for _ in range(args.warmup):
        with torch.cuda.stream(stream):
            flush.zero_()
        run_batch(sv, gscenes, spps)
    sv.counters(reset=True)
    st0 = sv.stats()
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
        run_batch(sv, gscenes, spps)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    clk = clocks.stop()
    st1 = sv.stats()
    kc = sv.counters()
    kc_batches = args.steps  # the launch counts cover the timed batches
    timed_kernels = st1["kernels"] - st0["kernels"] + args.steps  # + the flush kernels
    ms, value = aggregate_over_ranks(ms, samples_per_step, args.steps, dist, "cuda")
    if dist:
        dist.barrier()
    server_kw = {"step_paths": cap, "block_size": tune["block_size"], "flags": tune["flags"]}
    timing_source = "CUDA events captured in the step graphs of the timed region"
    if kc["extend_launches"] == 0:
        # no event-record nodes fired: time one more batch with direct launches
        sv.configure(tune["chunk_paths"], tune["block_size"],
                     tune["flags"] | capi.JOB_TIME_KERNELS | capi.SERVER_NO_GRAPHS)
        with torch.cuda.stream(stream):
            flush.zero_()
        sv.counters(reset=True)
        run_batch(sv, gscenes, spps)
        kc = sv.counters()
        kc = {k: (v * args.steps if k.endswith("_ms") else v) for k, v in kc.items()}
        kc_batches = 1  # launch counts of the one extra batch
        timing_source = "CUDA events around direct launches, one batch after the timed region"
    sv.close()
    del flush

    # rooflines of the two largest kernels; `roofline` is the one with the
    # larger measured time.  Closest-hit traversal ("extend") over the pooled
    # sphere BVHs: algorithmic bytes per ray = ray in (32 B) + hit out (16 B)
    # + 24 B per child-box test + 16 B (center, radius) per sphere test.
    peak, peak_kind = measured_peaks()
    alg = cnt["extend_rays"] * 48 + 24 * cnt["extend_boxes"] + 16 * cnt["extend_prims"]
    # launches of the timed configuration per batch (the counting run above may
    # use another step size; the per-batch counts do not depend on it)
    launches_timed = max(1.0, kc["extend_launches"] / kc_batches)
    per_launch = alg / launches_timed
    avg_ms = kc["extend_ms"] / max(1, kc["extend_launches"])
    achieved = per_launch / (avg_ms / 1e3) / 1e9 if kc["extend_launches"] else None
    traffic, _ = committed_traffic("extend_batch_traffic.json", cnt["extend_rays"] / launches_timed)
    roof = {"bound": "hbm", "kernel": "k_pt_extend (closest-hit BVH4 traversal, all jobs of a step)",
            "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": (achieved / peak) if achieved else None,
            "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)", "traffic": traffic,
            "alg_bytes_per_launch": per_launch, "avg_launch_ms": avg_ms, "launch_timing": timing_source,
            "rays_per_launch": cnt["extend_rays"] / launches_timed,
            "box_tests_per_ray": cnt["extend_boxes"] / max(1, cnt["extend_rays"]),
            "sphere_tests_per_ray": cnt["extend_prims"] / max(1, cnt["extend_rays"])}
    roof.update(l2_absorption(traffic, per_launch, avg_ms, peak))
    roof.update(l2_fraction(achieved, torch))
    roof_shade = shade_roofline(cnt, kc, kc_batches, samples_per_step, peak, peak_kind, timing_source)
    kernel_ms = {k: kc[k + "_ms"] / args.steps for k in ("extend", "shade", "shadow", "other")}
    rooflines = {"extend": roof, "shade": roof_shade}
    if kc["shade_ms"] > kc["extend_ms"]:
        roof = roof_shade

    # the plain per-job path on the same batch
    plain = plain_section(ctx, torch, gscenes, spps, film0, value, tune, world) if rank == 0 else None

    # end to end through the public API with host buffers: scene descriptions
    # in (host BVH build + upload), every job's RGBA8 image out.  As a serving
    # front door runs it: the server's loop thread renders the jobs already
    # submitted while the host builds the next scenes, and each job's image
    # is read (on the server's read-back stream) and the job released as its
    # `done` event arrives, while the others render.
    e2e = None
    if args.e2e_steps > 0 and rank == 0:
        sv = gprt.RenderServer(ctx, **server_kw)
        sv.configure(tune["chunk_paths"], tune["block_size"], tune["flags"])
        total_t, h2d, d2h = 0.0, 0, 0
        phases = [0.0, 0.0, 0.0]  # build + submit, until every image is read, releases after (s, timed steps)
        bvh_ms = 0.0  # host BVH builds inside gprt_scene_create (ms, timed steps)
        for i in range(args.e2e_steps + 1):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            sv.start()
            gs2, tickets = [], []
            for (f, _), s in zip(jobs, spps):
                gs2.append(gprt.GpuScene(ctx, f))
                tickets.append(sv.submit(gs2[-1], job_config(s, 7 + i)))
            ta = time.perf_counter()
            imgs, deadline = {}, time.perf_counter() + 600
            while len(imgs) < len(tickets):
                if time.perf_counter() > deadline:
                    raise RuntimeError("e2e: jobs did not finish within 600 s")
                for e in sv.poll(1024, timeout_ms=5):
                    if e.kind in ("failed", "refused", "cancelled"):
                        raise RuntimeError("e2e: job %d %s (status %d)" % (e.ticket, e.kind, e.status))
                    if e.kind == "done":
                        imgs[e.ticket] = sv.rgba8(e.ticket)
                        sv.release(e.ticket)
            tb = time.perf_counter()
            sv.stop()
            t1 = time.perf_counter()
            imgs = [imgs[t] for t in tickets]
            if i > 0:
                bvh_ms += sum(g.info.build_ms for g in gs2)
                phases[0] += ta - t0
                phases[1] += tb - ta
                phases[2] += t1 - tb
            h2d = sum(g.info.device_bytes for g in gs2)
            d2h = sum(im.nbytes for im in imgs)
            for g in gs2:
                g.close()
            if i > 0:
                total_t += t1 - t0
        sv.close()
        e2e = {"value": samples_per_step * args.e2e_steps / total_t / 1e6, "unit": "Msamples/s",
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
               "phases_ms_per_step": {"build_and_submit": phases[0] * 1e3 / args.e2e_steps,
                                      "until_all_read": phases[1] * 1e3 / args.e2e_steps,
                                      "stop": phases[2] * 1e3 / args.e2e_steps,
                                      "host_bvh_builds": bvh_ms / args.e2e_steps},
               "includes": "256 scene builds (host BVH) + uploads, each job submitted as its scene is built to the "
                           "server's loop thread (rendering overlaps the remaining builds), 256 RGBA8 read-backs, each "
                           "as its job's done event arrives (overlapping the other jobs' rendering)"}

    ico_flat = None
    serving = None
    if rank == 0 and not args.no_stream:
        from gprt import scenes
        ico_flat = scenes.icosphere_scene(level=ICO_LEVEL, width=ICO_WIDTH).to_desc()
        # C3's kind: the batch's first 512^2 job, so that 512^2 requests of both integrators arrive
        c3 = next(f for (f, _), g in zip(jobs, gscenes) if g.width == 512 and g.height == 512)
        flats = [scenes.cornell_baseline(400).to_desc(), ico_flat, scenes.cornell_boxes_bdpt(512).to_desc(), c3]
        serving = serving_section(ctx, args, server_kw, tune, flats)

    per_config = None
    if rank == 0 and not args.no_per_config:
        per_config = per_config_section(ctx, torch)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            cpu = cpu_baseline(jobs)
            cpu["per_config"] = cpu_per_config()
            if per_config:
                for k, v in cpu["per_config"]["configs"].items():
                    if k in per_config:
                        per_config[k]["cpu_msamples_per_s"] = v["msamples_per_s"]
                        per_config[k]["gpu_over_cpu"] = per_config[k]["msamples_per_s"] / v["msamples_per_s"]
        except Exception as e:  # the baseline never blocks the GPU line
            cpu = {"value": None, "error": str(e)}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "Msamples/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scenes, no dataset)",
                "config": {"workload": WORKLOAD, "jobs": NJOBS, "samples_per_step": samples_per_step,
                           "l2": "flushed (512 MB write before every timed step); path state 4.6 GB > L2",
                           "parallelism": "replicas" if world > 1 else "single GPU",
                           "autotuned": {"step_paths": tune["chunk_paths"], "block_size": tune["block_size"],
                                         "simple_extend": bool(tune["flags"] & capi.JOB_SIMPLE_EXTEND),
                                         "simple_shadow": bool(tune["flags"] & capi.JOB_SIMPLE_SHADOW),
                                         "candidates": tune["candidates"]},
                           "server_steps_per_batch": (st1["steps"] - st0["steps"]) / args.steps},
                "plain": plain, "serving": serving, "per_config": per_config,
                "roofline": roof, "rooflines": rooflines, "kernel_ms_per_step": kernel_ms, "cpu_baseline": cpu, "e2e": e2e,
                "gpu_launches": int(timed_kernels), "clocks": clk}
        print(json.dumps(line))
    for g in gscenes:
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
