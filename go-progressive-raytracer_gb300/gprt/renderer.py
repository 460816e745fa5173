"""Renderer API mirroring pkg/renderer and pkg/integrator over the C ABI.

``ProgressiveRaytracer`` follows renderer.ProgressiveRaytracer
(pkg/renderer/progressive.go:48-368): ``render_pass`` is RenderPass and
``render_progressive`` yields the PassResult / TileCompletionResult events of
RenderProgressive.  ``PathTracingIntegrator`` / ``BDPTIntegrator`` select the
integrator (pkg/integrator/path_tracing.go:40, bdpt.go:64).
"""
import ctypes as C
from dataclasses import dataclass
from typing import Callable, Iterator, Optional

import numpy as np

from . import _capi as capi


class Context:
    """A device context (one per GPU)."""

    def __init__(self, device=0):
        self.lib = capi.load()
        h = C.c_void_p()
        rc = self.lib.gprt_ctx_create(device, C.byref(h))
        if rc != capi.GPRT_OK:
            raise capi.GprtError(rc, "cannot create a context on CUDA device %d" % device)
        self.h = h

    def check(self, rc):
        capi.check(rc, self.h)

    def close(self):
        if self.h:
            self.lib.gprt_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GpuScene:
    """scene.Scene after Preprocess, resident on the device."""

    def __init__(self, ctx: Context, scene, device_bvh: bool = False, test_stack_cap: bool = False):
        """device_bvh: build the BVH on the GPU (GPRT_BUILD_DEVICE) instead of
        the host SAH builder.  test_stack_cap (tests only): a 1-entry
        traversal stack, so that rays overflow it and the scene's renders
        fail with GPRT_E_BOUND."""
        self.ctx = ctx
        self.flat = scene.to_desc() if hasattr(scene, "to_desc") else scene
        self.flat.desc.build_flags = ((capi.BUILD_DEVICE if device_bvh else 0) |
                                      (capi.BUILD_TEST_STACK_CAP if test_stack_cap else 0))
        h = C.c_void_p()
        ctx.check(ctx.lib.gprt_scene_create(ctx.h, self.flat.ptr(), C.byref(h)))
        self.h = h
        info = capi.SceneInfo()
        ctx.check(ctx.lib.gprt_scene_get_info(h, C.byref(info)))
        self.info = info
        self.width, self.height = info.image_width, info.image_height

    def primitive_map(self):
        n = self.info.n_primitives
        shape = np.zeros(n, dtype=np.uint32)
        sub = np.zeros(n, dtype=np.uint32)
        self.ctx.check(self.ctx.lib.gprt_scene_primitive_map(self.h, shape.ctypes.data_as(capi.U32P),
                                                             sub.ctypes.data_as(capi.U32P)))
        return shape, sub

    def intersect(self, rays: np.ndarray, any_hit=False):
        """BVH.Hit over a host batch of rays ((n, 8) float32, gprt_ray layout).
        Returns a structured array of (t, prim, u, v)."""
        rays = np.ascontiguousarray(rays, dtype=np.float32)
        n = rays.shape[0]
        hits = np.zeros(n, dtype=[("t", "<f4"), ("prim", "<u4"), ("u", "<f4"), ("v", "<f4")])
        self.ctx.check(self.ctx.lib.gprt_intersect_host(self.h, rays.ctypes.data, n, capi.ANY if any_hit else capi.CLOSEST,
                                                        hits.ctypes.data))
        return hits

    def traversal_counts(self, rays: np.ndarray, any_hit=False):
        rays = np.ascontiguousarray(rays, dtype=np.float32)
        a, b, c = C.c_uint64(), C.c_uint64(), C.c_uint64()
        self.ctx.check(self.ctx.lib.gprt_traversal_counts(self.h, rays.ctypes.data, rays.shape[0],
                                                          capi.ANY if any_hit else capi.CLOSEST, C.byref(a), C.byref(b),
                                                          C.byref(c)))
        return a.value, b.value, c.value

    def close(self):
        # a destroyed context has already released its scenes
        if self.h and self.ctx.h:
            self.ctx.lib.gprt_scene_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune(gscene: "GpuScene", integrator=None, spp=1, config: Optional["ProgressiveConfig"] = None):
    """gprt_autotune: the fastest wavefront size / traversal variant / block
    size for this scene.  Returns (config with the choice applied, details)."""
    cfg = config or ProgressiveConfig()
    d = capi.JobDesc()
    d.integrator = (integrator or PathTracingIntegrator()).kind
    d.max_samples_per_pixel = max(cfg.max_samples_per_pixel, 2 * spp)
    d.max_passes = 1
    d.seed = cfg.seed
    r = capi.TuneResult()
    gscene.ctx.check(gscene.ctx.lib.gprt_autotune(gscene.h, C.byref(d), spp, C.byref(r)))
    out = ProgressiveConfig(**cfg.__dict__)
    out.flags = (cfg.flags & ~(capi.JOB_SIMPLE_EXTEND | capi.JOB_SIMPLE_SHADOW | capi.JOB_SHADE_OCCUPANCY)) | r.flags
    out.block_size = r.block_size
    out.chunk_paths = r.chunk_paths
    return out, {k: getattr(r, k) for k, _ in capi.TuneResult._fields_}


@dataclass
class PathTracingIntegrator:  # integrator.NewPathTracingIntegrator
    kind: int = capi.INTEGRATOR_PATH_TRACING


@dataclass
class BDPTIntegrator:  # integrator.NewBDPTIntegrator
    kind: int = capi.INTEGRATOR_BDPT


@dataclass
class ProgressiveConfig:  # renderer.ProgressiveConfig (progressive.go:29-46)
    tile_size: int = 64
    initial_samples: int = 1
    max_samples_per_pixel: int = 50
    max_passes: int = 7
    chunk_paths: int = 0
    block_size: int = 0
    seed: int = 1
    flags: int = 0  # capi.JOB_TIME_KERNELS | capi.JOB_COUNT_TRAVERSAL


@dataclass
class RenderStats:  # renderer.RenderStats (stats.go:10-17)
    total_pixels: int
    total_samples: int
    average_samples: float
    max_samples: int
    min_samples: int
    max_samples_used: int
    pass_ms: float


@dataclass
class PassResult:  # progressive.go:258-263
    pass_number: int
    image: np.ndarray  # (h, w, 4) uint8
    stats: RenderStats
    is_last: bool


@dataclass
class TileCompletionResult:  # progressive.go:266-276
    tile_x: int
    tile_y: int
    tile_image: np.ndarray
    pass_number: int
    tile_number: int
    total_tiles: int
    total_passes: int


class ProgressiveRaytracer:
    """renderer.NewProgressiveRaytracer (progressive.go:62-95)."""

    def __init__(self, gscene: GpuScene, config: ProgressiveConfig, integrator=None):
        self.scene = gscene
        self.ctx = gscene.ctx
        self.config = config
        integ = integrator or PathTracingIntegrator()
        d = capi.JobDesc()
        d.integrator = integ.kind
        d.tile_size = config.tile_size
        d.initial_samples = config.initial_samples
        d.max_samples_per_pixel = config.max_samples_per_pixel
        d.max_passes = config.max_passes
        d.chunk_paths = config.chunk_paths
        d.block_size = config.block_size
        d.flags = config.flags
        d.seed = config.seed
        h = C.c_void_p()
        self.ctx.check(self.ctx.lib.gprt_job_create(gscene.h, C.byref(d), C.byref(h)))
        self.h = h
        self.width, self.height = gscene.width, gscene.height

    # ------------------------------------------------------------ passes
    def render_pass(self, pass_number: int, tile_callback: Optional[Callable] = None):
        """RenderPass (progressive.go:126-223): returns (RGBA image, stats)."""
        st = capi.RenderStats()
        self.ctx.check(self.ctx.lib.gprt_job_render_pass(self.h, pass_number, C.byref(st)))
        img = self.rgba8()
        stats = RenderStats(st.total_pixels, st.total_samples, st.average_samples, st.max_samples, st.min_samples,
                            st.max_samples_used, st.pass_ms)
        if tile_callback is not None:
            ts = self.config.tile_size
            tiles = [(x0, y0) for y0 in range(0, self.height, ts) for x0 in range(0, self.width, ts)]
            for i, (x0, y0) in enumerate(tiles):
                tile_callback(TileCompletionResult(x0 // ts, y0 // ts, img[y0:y0 + ts, x0:x0 + ts].copy(),
                                                   pass_number, i + 1, len(tiles), self.config.max_passes))
        return img, stats

    def render_progressive(self, tile_updates=False, cancelled: Optional[Callable[[], bool]] = None) -> Iterator:
        """RenderProgressive (progressive.go:286-368) as a generator of
        PassResult (and TileCompletionResult when tile_updates)."""
        for p in range(1, self.config.max_passes + 1):
            if cancelled is not None and cancelled():
                raise capi.GprtError(capi.GPRT_E_CANCELLED, "rendering cancelled before pass %d" % p)
            events = []
            img, stats = self.render_pass(p, events.append if tile_updates else None)
            yield from events
            actual = int(stats.average_samples)
            last = p == self.config.max_passes or actual >= self.config.max_samples_per_pixel
            yield PassResult(p, img, stats, last)
            if actual >= self.config.max_samples_per_pixel:
                break

    def add_samples(self, spp: int):
        self.ctx.check(self.ctx.lib.gprt_job_add_samples(self.h, spp))

    def sync(self):
        self.ctx.check(self.ctx.lib.gprt_job_sync(self.h))

    # ------------------------------------------------------------ read-back
    def rgba8(self):
        out = np.zeros((self.height, self.width, 4), dtype=np.uint8)
        self.ctx.check(self.ctx.lib.gprt_job_read_rgba8(self.h, out.ctypes.data_as(capi.U8P)))
        return out

    def image(self):
        """Per-pixel mean linear radiance, (h, w, 3) float32."""
        out = np.zeros((self.height, self.width, 3), dtype=np.float32)
        self.ctx.check(self.ctx.lib.gprt_job_read_image(self.h, out.ctypes.data_as(capi.F32P)))
        return out

    def film(self):
        n = self.width * self.height
        rgb = np.zeros((n, 3), dtype=np.float32)
        lum = np.zeros(n, dtype=np.float32)
        lum2 = np.zeros(n, dtype=np.float32)
        cnt = np.zeros(n, dtype=np.uint32)
        self.ctx.check(self.ctx.lib.gprt_job_read_film(self.h, rgb.ctypes.data_as(capi.F32P), lum.ctypes.data_as(capi.F32P),
                                                       lum2.ctypes.data_as(capi.F32P), cnt.ctypes.data_as(capi.U32P)))
        return rgb, lum, lum2, cnt

    def tile(self, x0, y0, x1, y1):
        out = np.zeros((y1 - y0, x1 - x0, 4), dtype=np.uint8)
        self.ctx.check(self.ctx.lib.gprt_job_read_tile(self.h, x0, y0, x1, y1, out.ctypes.data_as(capi.U8P)))
        return out

    def launches(self):
        v = C.c_uint64()
        self.ctx.check(self.ctx.lib.gprt_job_launch_count(self.h, C.byref(v)))
        return v.value

    def counters(self, reset=False):
        """Instrumentation summed since the last reset (synchronises the job)."""
        c = capi.JobCounters()
        self.ctx.check(self.ctx.lib.gprt_job_get_counters(self.h, C.byref(c)))
        if reset:
            self.ctx.check(self.ctx.lib.gprt_job_reset_counters(self.h))
        return {k: getattr(c, k) for k, _ in capi.JobCounters._fields_}

    def stream(self):
        """The cudaStream_t (as an int) the job's kernels run on."""
        s = C.c_void_p()
        self.ctx.check(self.ctx.lib.gprt_job_stream(self.h, C.byref(s)))
        return s.value or 0

    def close(self):
        # a destroyed scene or context has already released its jobs
        if self.h and self.scene.h and self.ctx.h:
            self.ctx.lib.gprt_job_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
