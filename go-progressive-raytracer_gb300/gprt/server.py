"""Device-resident render server with continuous batching (gprt_server_*).

The reference serves concurrent progressive renders from its web server, one
``ProgressiveRaytracer`` with its own worker pool per request
(web/server/render.go:45-82,183-227).  ``RenderServer`` is the GPU form: many
requests share every wavefront, scenes and films stay on the device, and
admission is bounded by an HBM budget.  Requests carry the progressive pass
schedule of ``ProgressiveConfig`` (getSamplesForPass, progressive.go:98-123).
"""
import ctypes as C
from dataclasses import dataclass
from typing import Dict, List, Optional

import numpy as np

from . import _capi as capi
from .renderer import Context, GpuScene, ProgressiveConfig


@dataclass
class ServerEvent:
    ticket: int
    kind: str  # admitted | pass | done | refused | cancelled | failed
    pass_number: int
    samples_per_pixel: int
    status: int
    t_ms: float
    submit_ms: float


class RenderServer:
    def __init__(self, ctx: Context, hbm_budget_bytes=0, max_jobs=0, step_paths=0, block_size=0, flags=0):
        self.ctx = ctx
        d = capi.ServerDesc()
        d.hbm_budget_bytes = hbm_budget_bytes
        d.max_jobs = max_jobs
        d.step_paths = step_paths
        d.block_size = block_size
        d.flags = flags
        h = C.c_void_p()
        ctx.check(ctx.lib.gprt_server_create(ctx.h, C.byref(d), C.byref(h)))
        self.h = h
        self.sizes: Dict[int, tuple] = {}

    def submit(self, gscene: GpuScene, config: ProgressiveConfig, integrator=None) -> int:
        """Queues a render of `gscene` (path tracing unless `integrator` is a
        BDPTIntegrator; BDPT requests render pass by pass between the batched
        path-tracing steps, on the server's own copy of the scene)."""
        d = capi.JobDesc()
        d.integrator = integrator.kind if integrator is not None else capi.INTEGRATOR_PATH_TRACING
        d.initial_samples = config.initial_samples
        d.max_samples_per_pixel = config.max_samples_per_pixel
        d.max_passes = config.max_passes
        d.seed = config.seed
        t = C.c_uint64()
        self.ctx.check(self.ctx.lib.gprt_server_submit(self.h, gscene.h, C.byref(d), C.byref(t)))
        self.sizes[t.value] = (gscene.height, gscene.width)
        return t.value

    def cancel(self, ticket: int):
        self.ctx.check(self.ctx.lib.gprt_server_cancel(self.h, ticket))

    def release(self, ticket: int):
        self.ctx.check(self.ctx.lib.gprt_server_release(self.h, ticket))

    def step(self) -> int:
        """One batched step on this thread; returns the jobs still busy."""
        busy = C.c_uint32()
        self.ctx.check(self.ctx.lib.gprt_server_step(self.h, C.byref(busy)))
        return busy.value

    def start(self):
        self.ctx.check(self.ctx.lib.gprt_server_start(self.h))

    def stop(self):
        self.ctx.check(self.ctx.lib.gprt_server_stop(self.h))

    def poll(self, max_events=256, timeout_ms=0) -> List[ServerEvent]:
        buf = (capi.Event * max_events)()
        n = C.c_uint32()
        self.ctx.check(self.ctx.lib.gprt_server_poll(self.h, buf, max_events, timeout_ms, C.byref(n)))
        return [ServerEvent(e.ticket, capi.EVENT_NAMES.get(e.kind, str(e.kind)), e.pass_number, e.samples_per_pixel,
                            e.status, e.t_ms, e.submit_ms) for e in buf[:n.value]]

    def run_until_idle(self, max_steps=1_000_000) -> List[ServerEvent]:
        """Steps on this thread until no job is busy; returns every event."""
        events = []
        for _ in range(max_steps):
            busy = self.step()
            events += self.poll()
            if busy == 0:
                break
        return events + self.poll()

    def film(self, ticket: int):
        h, w = self.sizes[ticket]
        n = h * w
        rgb = np.zeros((n, 3), dtype=np.float32)
        lum = np.zeros(n, dtype=np.float32)
        lum2 = np.zeros(n, dtype=np.float32)
        cnt = np.zeros(n, dtype=np.uint32)
        self.ctx.check(self.ctx.lib.gprt_server_read_film(self.h, ticket, rgb.ctypes.data_as(capi.F32P),
                                                          lum.ctypes.data_as(capi.F32P),
                                                          lum2.ctypes.data_as(capi.F32P),
                                                          cnt.ctypes.data_as(capi.U32P)))
        return rgb, lum, lum2, cnt

    def image(self, ticket: int):
        h, w = self.sizes[ticket]
        out = np.zeros((h, w, 3), dtype=np.float32)
        self.ctx.check(self.ctx.lib.gprt_server_read_image(self.h, ticket, out.ctypes.data_as(capi.F32P)))
        return out

    def rgba8(self, ticket: int):
        h, w = self.sizes[ticket]
        out = np.zeros((h, w, 4), dtype=np.uint8)
        self.ctx.check(self.ctx.lib.gprt_server_read_rgba8(self.h, ticket, out.ctypes.data_as(capi.U8P)))
        return out

    def tile(self, ticket: int, x0: int, y0: int, x1: int, y1: int):
        """RGBA8 of tile [x0, x1) x [y0, y1) (only its bytes leave the device)."""
        out = np.zeros((y1 - y0, x1 - x0, 4), dtype=np.uint8)
        self.ctx.check(self.ctx.lib.gprt_server_read_tile(self.h, ticket, x0, y0, x1, y1,
                                                          out.ctypes.data_as(capi.U8P)))
        return out

    def tiles(self, ticket: int, pass_number: int, total_passes: int, tile_size: int = 64):
        """The TileCompletionResult events of a finished pass (progressive.go:
        266-276), in the reference's row-major tile order: every tile of a
        pass is complete when the job's `pass` event arrives."""
        from .renderer import TileCompletionResult
        h, w = self.sizes[ticket]
        rects = [(x0, y0) for y0 in range(0, h, tile_size) for x0 in range(0, w, tile_size)]
        for k, (x0, y0) in enumerate(rects):
            img = self.tile(ticket, x0, y0, min(x0 + tile_size, w), min(y0 + tile_size, h))
            yield TileCompletionResult(x0 // tile_size, y0 // tile_size, img, pass_number, k + 1, len(rects),
                                       total_passes)

    def stats(self) -> dict:
        s = capi.ServerStats()
        self.ctx.check(self.ctx.lib.gprt_server_get_stats(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in capi.ServerStats._fields_}

    def counters(self, reset=False) -> dict:
        c = capi.JobCounters()
        self.ctx.check(self.ctx.lib.gprt_server_get_counters(self.h, C.byref(c), 1 if reset else 0))
        return {k: getattr(c, k) for k, _ in capi.JobCounters._fields_}

    def stream(self) -> int:
        """The cudaStream_t (as an int) the server runs on."""
        s = C.c_void_p()
        self.ctx.check(self.ctx.lib.gprt_server_stream(self.h, C.byref(s)))
        return s.value or 0

    def configure(self, step_paths: int, block_size: int, flags: int):
        self.ctx.check(self.ctx.lib.gprt_server_configure(self.h, step_paths, block_size, flags))

    def autotune(self, max_step_ms: float = 0.0) -> dict:
        r = capi.TuneResult()
        self.ctx.check(self.ctx.lib.gprt_server_autotune(self.h, max_step_ms, C.byref(r)))
        return {k: getattr(r, k) for k, _ in capi.TuneResult._fields_}

    def close(self):
        if self.h and self.ctx.h:
            self.ctx.lib.gprt_server_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def latency_summary(events: List[ServerEvent], tickets: Optional[List[int]] = None) -> dict:
    """p50 / p99 time-to-first-pass and per-pass latency (ms) from events."""
    first: Dict[int, float] = {}
    last: Dict[int, float] = {}
    per_pass = []
    for e in sorted(events, key=lambda e: e.t_ms):
        if tickets is not None and e.ticket not in tickets:
            continue
        if e.kind != "pass":
            continue
        if e.ticket not in first:
            first[e.ticket] = e.t_ms - e.submit_ms
        else:
            per_pass.append(e.t_ms - last[e.ticket])
        last[e.ticket] = e.t_ms
    ttfp = np.array(list(first.values())) if first else np.zeros(0)
    pp = np.array(per_pass) if per_pass else np.zeros(0)

    def pct(a, q):
        return float(np.percentile(a, q)) if a.size else None

    return {"ttfp_p50_ms": pct(ttfp, 50), "ttfp_p99_ms": pct(ttfp, 99), "pass_p50_ms": pct(pp, 50),
            "pass_p99_ms": pct(pp, 99), "jobs": int(ttfp.size), "passes": int(pp.size + ttfp.size)}
