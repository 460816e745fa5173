"""Throughput of the per-job GPU path on each reference workload.

    python -m gprt.configs_report [--steps 5]

Prints one JSON object per workload: the Cornell box of the path-tracing
workload (400^2, 64 spp), the reference Cornell scene with spheres (400^2,
64 spp), the displaced icosphere (1024^2, 16 spp), the Cornell-boxes scene
under BDPT (512^2, 64 spp) and the raw 2^24-ray intersection batch on the
icosphere.  Each render is autotuned first (untimed), then `--steps` frames
are timed with CUDA events on the job's stream; the first progressive pass
(1 spp) of a fresh job is timed on the host (time to first pass).  Run from
the package directory.
"""
import argparse
import json
import os
import sys
import time


def _setup():
    here = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    if here not in sys.path:
        sys.path.insert(0, here)


def _render(ctx, torch, name, scene, spp, integrator, steps):
    import gprt
    from gprt import capi
    g = gprt.GpuScene(ctx, scene.to_desc())
    integ = integrator()
    cfg, tune = gprt.renderer.autotune(g, integ, spp=spp, config=gprt.ProgressiveConfig(max_samples_per_pixel=spp))
    job = gprt.ProgressiveRaytracer(g, gprt.ProgressiveConfig(max_samples_per_pixel=1 << 30, max_passes=1, seed=1,
                                                              flags=cfg.flags | capi.JOB_TIME_KERNELS,
                                                              block_size=cfg.block_size, chunk_paths=cfg.chunk_paths),
                                    integ)
    st = torch.cuda.ExternalStream(job.stream())
    for _ in range(2):
        job.add_samples(spp)
    job.sync()
    job.counters(reset=True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(steps):
        job.add_samples(spp)
    e1.record(st)
    job.sync()
    ms = e0.elapsed_time(e1) / steps
    kc = job.counters()
    job.close()
    # time to first pass: a fresh job's pass 1 (1 spp) on the host clock
    first = gprt.ProgressiveRaytracer(g, gprt.ProgressiveConfig(initial_samples=1, max_samples_per_pixel=spp,
                                                                max_passes=max(2, spp // 4), seed=2), integ)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    first.render_pass(1)
    ttfp = (time.perf_counter() - t0) * 1e3
    first.close()
    n = g.width * g.height * spp
    out = {"workload": name, "width": g.width, "height": g.height, "spp": spp, "ms_per_frame": ms,
           "msamples_per_s": n / ms / 1e3, "first_pass_ms": ttfp,
           "kernel_ms_per_frame": {k: kc[k + "_ms"] / steps for k in ("extend", "shade", "shadow", "other")},
           "autotuned": {"chunk_paths": cfg.chunk_paths, "block_size": cfg.block_size, "flags": cfg.flags}}
    g.close()
    return out


def _raw_batch(ctx, torch, steps):
    import numpy as np
    import gprt
    from gprt import capi, scenes
    scene = scenes.icosphere_scene(level=8, width=1024)
    mesh = scene.shapes[0].mesh
    n = 1 << 24
    rays = scenes.ray_batch(mesh.vertices, mesh.faces, n, seed=13, width=1024)
    g = gprt.GpuScene(ctx, scene.to_desc())
    d_rays = torch.from_numpy(rays).cuda()
    d_hits = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    st = torch.cuda.Stream()  # a real stream handle (0 would mean the library's own stream)
    st.wait_stream(torch.cuda.current_stream())
    out = {}
    for name, flag in (("closest", capi.CLOSEST), ("any", capi.ANY)):
        for _ in range(2):
            ctx.check(ctx.lib.gprt_intersect(g.h, d_rays.data_ptr(), n, flag, d_hits.data_ptr(), st.cuda_stream))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(steps):
            ctx.check(ctx.lib.gprt_intersect(g.h, d_rays.data_ptr(), n, flag, d_hits.data_ptr(), st.cuda_stream))
        e1.record(st)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        out[name] = {"ms_per_batch": ms, "mrays_per_s": n / ms / 1e3}
    hits = d_hits.cpu().numpy()
    g.close()
    return {"workload": "raw batch: 2^24 rays on the level-8 icosphere (half camera rays at 1024^2, half "
                        "surface-point rays in uniform directions), seed 13", **out,
            "hit_fraction": float((hits[:, 0] >= 0).mean())}


def main(argv=None):
    _setup()
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--only", default="", help="comma list of: cornell, spheres, icosphere, bdpt, raw")
    a = ap.parse_args(argv)
    only = set(x for x in a.only.split(",") if x)
    import torch
    import gprt
    from gprt import scenes
    ctx = gprt.Context(0)
    PT, BD = gprt.PathTracingIntegrator, gprt.BDPTIntegrator
    cases = [("cornell", "cornell (path-tracing workload), PT", lambda: scenes.cornell_baseline(400), 64, PT),
             ("spheres", "reference cornell with spheres, PT", lambda: scenes.cornell_scene(), 64, PT),
             ("icosphere", "icosphere L8 (1,310,720 tris), PT", lambda: scenes.icosphere_scene(level=8, width=1024), 16,
              PT),
             ("bdpt", "cornell-boxes, BDPT", lambda: scenes.cornell_boxes_bdpt(512), 64, BD)]
    for key, name, make, spp, integ in cases:
        if not only or key in only:
            print(json.dumps(_render(ctx, torch, name, make(), spp, integ, a.steps)), flush=True)
    if not only or "raw" in only:
        print(json.dumps(_raw_batch(ctx, torch, a.steps)), flush=True)
    ctx.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
