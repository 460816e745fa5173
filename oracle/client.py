"""ctypes client of the oracle library.  TEST INFRASTRUCTURE ONLY.

Used by tests/, __graft_entry__.smoke() and bench.py's CPU baseline to run
the float64 restatement of the reference (oracle.hpp) on the same scene
descriptions the GPU library consumes.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
KAT = os.path.join(HERE, "_build", "kat")

_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            from . import build as _b  # noqa: F401  (package import when available)
        _lib = C.CDLL(LIB)
        P = C.c_void_p
        _lib.oracle_last_error.restype = C.c_char_p
        _lib.oracle_scene_create.restype = P
        _lib.oracle_scene_create.argtypes = [P]
        _lib.oracle_scene_destroy.argtypes = [P]
        _lib.oracle_scene_info.argtypes = [P, P, P, P, P]
        _lib.oracle_intersect.argtypes = [P, P, C.c_uint32, P, P, P, P, P, C.c_int]
        _lib.oracle_renderer_create.restype = P
        _lib.oracle_renderer_create.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint64, C.c_int,
                                                C.c_int]
        _lib.oracle_renderer_destroy.argtypes = [P]
        _lib.oracle_render_pass.argtypes = [P, C.c_int, C.c_int, P, P]
        _lib.oracle_render_tiles.argtypes = [P, C.c_int, P, C.c_int, P, P]
        _lib.oracle_renderer_read.argtypes = [P, P, P, P, P, P]
        _lib.oracle_renderer_rgba8.argtypes = [P, P]
        _lib.oracle_samples_for_pass.argtypes = [P, C.c_int]
        _lib.oracle_camera_rays.argtypes = [P, C.c_uint32, P, P, P]
        _lib.oracle_pt_ray_color.argtypes = [P, P, P, C.c_int, P, C.c_int, P, C.c_int, P]
    return _lib


def ensure_built():
    import importlib.util
    spec = importlib.util.spec_from_file_location("oracle_build", os.path.join(HERE, "build.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m.build()


class OracleScene:
    def __init__(self, flat):
        """`flat`: a FlatScene (gprt.scene) whose desc both libraries read."""
        self.flat = flat
        lib = load()
        self.h = lib.oracle_scene_create(C.addressof(flat.desc))
        if not self.h:
            raise RuntimeError("oracle scene: " + lib.oracle_last_error().decode())
        c = (C.c_double * 3)()
        r = C.c_double()
        w, h = C.c_int(), C.c_int()
        lib.oracle_scene_info(self.h, C.addressof(c), C.addressof(r), C.addressof(w), C.addressof(h))
        self.world_center = tuple(c)
        self.world_radius = r.value
        self.width, self.height = w.value, h.value

    def intersect(self, rays, threads=8):
        rays = np.ascontiguousarray(rays, dtype=np.float32)
        n = rays.shape[0]
        t = np.zeros(n)
        shape = np.zeros(n, dtype=np.int32)
        sub = np.zeros(n, dtype=np.int32)
        uv = np.zeros((n, 2))
        nrm = np.zeros((n, 3))
        load().oracle_intersect(self.h, rays.ctypes.data, n, t.ctypes.data, shape.ctypes.data, sub.ctypes.data,
                                uv.ctypes.data, nrm.ctypes.data, threads)
        return t, shape, sub, uv, nrm

    def close(self):
        if self.h:
            load().oracle_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class OracleRenderer:
    """The progressive renderer on host threads (64x64 tiles)."""

    def __init__(self, scene: OracleScene, integrator=0, max_spp=16, max_passes=1, initial=1, seed=101, threads=8,
                 tile=64, counter_stream=False):
        self.scene = scene
        self.h = load().oracle_renderer_create(scene.h, integrator, tile, initial, max_spp, max_passes, seed, threads,
                                               1 if counter_stream else 0)

    def render_pass(self, p, only_tiles=-1):
        secs = C.c_double()
        st = (C.c_longlong * 4)()
        rc = load().oracle_render_pass(self.h, p, only_tiles, C.addressof(secs), C.addressof(st))
        if rc != 0:
            raise RuntimeError(load().oracle_last_error().decode())
        return secs.value, tuple(st)

    def render_tiles(self, p, tile_ids):
        """RenderPass `p` over the listed tile ids only (row-major 64x64 grid)."""
        ids = np.ascontiguousarray(tile_ids, dtype=np.int32)
        secs = C.c_double()
        st = (C.c_longlong * 4)()
        rc = load().oracle_render_tiles(self.h, p, ids.ctypes.data, len(ids), C.addressof(secs), C.addressof(st))
        if rc != 0:
            raise RuntimeError(load().oracle_last_error().decode())
        return secs.value, tuple(st)

    def image(self):
        n = self.scene.width * self.scene.height
        out = np.zeros((n, 3))
        load().oracle_renderer_read(self.h, out.ctypes.data, None, None, None, None)
        return out.reshape(self.scene.height, self.scene.width, 3)

    def film(self):
        n = self.scene.width * self.scene.height
        rgb, lum, lum2 = np.zeros((n, 3)), np.zeros(n), np.zeros(n)
        cnt = np.zeros(n, dtype=np.int32)
        load().oracle_renderer_read(self.h, None, rgb.ctypes.data, lum.ctypes.data, lum2.ctypes.data, cnt.ctypes.data)
        return rgb, lum, lum2, cnt

    def rgba8(self):
        out = np.zeros((self.scene.height, self.scene.width, 4), dtype=np.uint8)
        load().oracle_renderer_rgba8(self.h, out.ctypes.data)
        return out

    def close(self):
        if self.h:
            load().oracle_renderer_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def render(flat, integrator=0, spp=16, seed=101, threads=8, counter_stream=False):
    """Fixed-spp single-pass render; returns the (h, w, 3) mean image."""
    s = OracleScene(flat)
    r = OracleRenderer(s, integrator, max_spp=spp, max_passes=1, seed=seed, threads=threads,
                       counter_stream=counter_stream)
    r.render_pass(1)
    img = r.image()
    r.close()
    s.close()
    return img
