"""Small, self-contained render cases for kernel profiling (ncu).

    python profile_cases.py batch [--jobs 24] [--spp N] [--step-paths P] [--count]
    python profile_cases.py icosphere [--width 512] [--spp 4] [--count]
    python profile_cases.py bdpt [--width 512] [--spp 4]
    python profile_cases.py cornell [--width 400] [--spp 64]

`batch` renders the first jobs of the heterogeneous default-style batch
(seed 17; each job at its own spp, or at --spp N) through the batched render
server; `icosphere` renders the displaced level-8 icosphere (1,310,720
triangles) through the per-job path; `bdpt` renders the Cornell-boxes scene
under BDPT through the per-job path.  All keep a few GB on the device at
most and run each kernel a bounded number of times, so a capture of a few
launches of one kernel ends by itself.  With --count the same case runs with
the traversal counters on (and direct launches) and prints the rays, node
visits, box tests and primitive tests of the extend and shadow kernels, the
units that scale a capture's DRAM bytes to other launch sizes.  A
measurement helper beside bench.py (the profiles/ summaries cite its
command lines); run it from the repository root.
"""
import argparse
import json
import os
import sys


def _setup():
    pkg = os.path.join(os.path.dirname(os.path.abspath(__file__)), "go-progressive-raytracer_gb300")
    if pkg not in sys.path:
        sys.path.insert(0, pkg)


def batch(jobs, step_paths, spp=None, count=False, seed=17):
    import gprt
    from gprt import capi, scenes
    ctx = gprt.Context(0)
    gs, spps = [], []
    for s, n in scenes.batched_jobs(jobs, seed):
        gs.append(gprt.GpuScene(ctx, s.to_desc()))
        spps.append(spp or n)
    flags = (capi.JOB_COUNT_TRAVERSAL | capi.JOB_TIME_KERNELS | capi.SERVER_NO_GRAPHS) if count else 0
    sv = gprt.RenderServer(ctx, step_paths=step_paths, flags=flags)
    ts = [sv.submit(g, gprt.ProgressiveConfig(initial_samples=s, max_samples_per_pixel=s, max_passes=1, seed=1))
          for g, s in zip(gs, spps)]
    sv.run_until_idle()
    st = sv.stats()
    c = sv.counters() if count else None
    for t in ts:
        sv.release(t)
    sv.close()
    for g in gs:
        g.close()
    ctx.close()
    print(json.dumps({"case": "batch", "jobs": jobs, "samples": st["samples"], "steps": st["steps"],
                      "kernels": st["kernels"], "counters": c}))


def icosphere(width, spp, count=False):
    import gprt
    from gprt import capi, scenes
    ctx = gprt.Context(0)
    g = gprt.GpuScene(ctx, scenes.icosphere_scene(level=8, width=width).to_desc())
    flags = (capi.JOB_COUNT_TRAVERSAL | capi.JOB_TIME_KERNELS) if count else 0
    r = gprt.ProgressiveRaytracer(g, gprt.ProgressiveConfig(max_samples_per_pixel=spp, max_passes=1, seed=1,
                                                            flags=flags))
    r.add_samples(spp)
    r.sync()
    c = r.counters() if count else None
    r.close()
    g.close()
    ctx.close()
    print(json.dumps({"case": "icosphere", "width": width, "spp": spp, "counters": c}))


def cornell(width, spp):
    """The Cornell box of the path-tracing workload (cornell_baseline) through
    the per-job path: one frame of `spp` samples per pixel."""
    import gprt
    from gprt import scenes
    ctx = gprt.Context(0)
    g = gprt.GpuScene(ctx, scenes.cornell_baseline(width).to_desc())
    r = gprt.ProgressiveRaytracer(g, gprt.ProgressiveConfig(max_samples_per_pixel=spp, max_passes=1, seed=1))
    r.add_samples(spp)
    r.sync()
    r.close()
    g.close()
    ctx.close()
    print(json.dumps({"case": "cornell", "width": width, "spp": spp}))


def bdpt(width, spp):
    import gprt
    from gprt import scenes
    ctx = gprt.Context(0)
    g = gprt.GpuScene(ctx, scenes.cornell_boxes_bdpt(width).to_desc())
    r = gprt.ProgressiveRaytracer(g, gprt.ProgressiveConfig(max_samples_per_pixel=spp, max_passes=1, seed=1),
                                  gprt.BDPTIntegrator())
    r.add_samples(spp)
    r.sync()
    r.close()
    g.close()
    ctx.close()
    print(json.dumps({"case": "bdpt", "width": width, "spp": spp}))


def main(argv=None):
    _setup()
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["batch", "icosphere", "bdpt", "cornell"])
    ap.add_argument("--jobs", type=int, default=24)
    ap.add_argument("--step-paths", type=int, default=1 << 22)
    ap.add_argument("--width", type=int, default=512)
    ap.add_argument("--spp", type=int, default=0)
    ap.add_argument("--count", action="store_true")
    a = ap.parse_args(argv)
    if a.case == "batch":
        batch(a.jobs, a.step_paths, a.spp or None, a.count)
    elif a.case == "bdpt":
        bdpt(a.width, a.spp or 4)
    elif a.case == "cornell":
        cornell(a.width, a.spp or 64)
    else:
        icosphere(a.width, a.spp or 4, a.count)
    return 0


if __name__ == "__main__":
    sys.exit(main())
