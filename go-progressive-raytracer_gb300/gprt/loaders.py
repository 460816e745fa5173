"""Scene files: PBRT-v4 subset scenes and binary PLY meshes.

``load_pbrt`` / ``parse_pbrt`` mirror loaders.LoadPBRT / ParsePBRT
(pkg/loaders/pbrt.go) followed by scene.NewPBRTScene
(pkg/scene/pbrt_scene.go); the parsing and conversion run in the library
(``gprt_pbrt_load`` / ``gprt_pbrt_parse``), which hands back a finished scene
description.  ``load_ply`` mirrors loaders.LoadPLY (pkg/loaders/ply.go).
"""
import ctypes as C
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _capi as capi
from .scene import CameraConfig, Mesh, TriangleMesh


def _camera_desc(cfg: Optional[CameraConfig]):
    if cfg is None:
        return None
    d = capi.CameraDesc()
    for k in range(3):
        d.center[k] = cfg.center[k]
        d.look_at[k] = cfg.look_at[k]
        d.up[k] = cfg.up[k]
    d.width = cfg.width
    d.aspect_ratio = cfg.aspect_ratio
    d.vfov_deg = cfg.vfov
    d.aperture = cfg.aperture
    d.focus_distance = cfg.focus_distance
    return C.byref(d)


class LoadedScene:
    """A scene description built by the library from a scene file; use it
    where a flattened Scene goes (GpuScene, the oracle)."""

    def __init__(self, handle):
        self._lib = capi.load()
        self.h = handle
        self.desc = self._lib.gprt_loaded_desc(handle).contents

    def ptr(self):
        return C.byref(self.desc)

    def to_desc(self):
        return self

    @property
    def width(self):
        return self.desc.sampling.width

    @property
    def height(self):
        return self.desc.sampling.height

    def close(self):
        if self.h:
            self._lib.gprt_loaded_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _loaded(rc, h, err):
    if rc != capi.GPRT_OK:
        raise capi.GprtError(rc, err.value.decode(errors="replace"))
    return LoadedScene(h)


def parse_pbrt(text: str, camera: Optional[CameraConfig] = None) -> LoadedScene:
    """loaders.ParsePBRT + scene.NewPBRTScene on PBRT text."""
    lib = capi.load()
    raw = text.encode()
    h, err = C.c_void_p(), C.create_string_buffer(512)
    return _loaded(lib.gprt_pbrt_parse(raw, len(raw), _camera_desc(camera), C.byref(h), err, 512), h, err)


def load_pbrt(path: str, camera: Optional[CameraConfig] = None) -> LoadedScene:
    """loaders.LoadPBRT + scene.NewPBRTScene: the path must lie under a
    scenes/ directory or the temporary directory and end in .pbrt."""
    lib = capi.load()
    h, err = C.c_void_p(), C.create_string_buffer(512)
    return _loaded(lib.gprt_pbrt_load(path.encode(), _camera_desc(camera), C.byref(h), err, 512), h, err)


@dataclass
class PlyData:  # loaders.PLYData (ply.go:45-63), the attributes the renderer uses
    vertices: np.ndarray  # (n, 3) float64
    faces: np.ndarray  # (m, 3) uint32
    normals: Optional[np.ndarray] = None
    colors: Optional[np.ndarray] = None  # [0, 1]
    texcoords: Optional[np.ndarray] = None

    def mesh(self, material) -> "Mesh":
        """A TriangleMesh shape of one material (NewTriangleMesh)."""
        return Mesh(TriangleMesh(vertices=self.vertices, faces=self.faces, material=material))


def load_ply(path: str) -> PlyData:
    """loaders.LoadPLY: binary little-endian, triangular faces."""
    lib = capi.load()
    h, err = C.c_void_p(), C.create_string_buffer(512)
    rc = lib.gprt_ply_load(path.encode(), C.byref(h), err, 512)
    if rc != capi.GPRT_OK:
        raise capi.GprtError(rc, err.value.decode(errors="replace"))
    try:
        info = capi.PlyInfo()
        v, i, n, c, t = (C.POINTER(C.c_double)(), C.POINTER(C.c_uint32)(), C.POINTER(C.c_double)(),
                         C.POINTER(C.c_double)(), C.POINTER(C.c_double)())
        capi.check(lib.gprt_ply_get(h, C.byref(info), C.byref(v), C.byref(i), C.byref(n), C.byref(c), C.byref(t)))
        nv, nt = info.n_vertices, info.n_triangles

        def arr(p, count, cols, dtype):
            if not p or count == 0:
                return np.zeros((0, cols), dtype=dtype)
            return np.ctypeslib.as_array(p, shape=(count * cols,)).astype(dtype).reshape(count, cols)

        return PlyData(vertices=arr(v, nv, 3, np.float64), faces=arr(i, nt, 3, np.uint32),
                       normals=arr(n, nv, 3, np.float64) if info.has_normals else None,
                       colors=arr(c, nv, 3, np.float64) if info.has_colors else None,
                       texcoords=arr(t, nv, 2, np.float64) if info.has_texcoords else None)
    finally:
        lib.gprt_ply_free(h)
