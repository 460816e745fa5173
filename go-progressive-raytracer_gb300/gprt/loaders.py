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


# ---------------------------------------------------------------- images
def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = np.abs(p - a), np.abs(p - b), np.abs(p - c)
    return np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))


def _unfilter(raw: bytes, height: int, stride: int, bpp: int) -> np.ndarray:
    """Reverses the PNG scanline filters (None, Sub, Up, Average, Paeth)."""
    out = np.zeros((height, stride), dtype=np.int64)
    data = np.frombuffer(raw, dtype=np.uint8)
    prev = np.zeros(stride, dtype=np.int64)
    pos = 0
    for y in range(height):
        ftype = int(data[pos])
        line = data[pos + 1:pos + 1 + stride].astype(np.int64)
        pos += 1 + stride
        if ftype == 0:
            cur = line
        elif ftype == 2:
            cur = (line + prev) & 0xFF
        else:  # Sub, Average and Paeth depend on the bytes to the left: per pixel column
            cur = np.zeros(stride, dtype=np.int64)
            for x in range(0, stride, bpp):
                left = cur[x - bpp:x] if x >= bpp else np.zeros(bpp, dtype=np.int64)
                up = prev[x:x + bpp]
                if ftype == 1:
                    cur[x:x + bpp] = (line[x:x + bpp] + left) & 0xFF
                elif ftype == 3:
                    cur[x:x + bpp] = (line[x:x + bpp] + ((left + up) >> 1)) & 0xFF
                elif ftype == 4:
                    ul = prev[x - bpp:x] if x >= bpp else np.zeros(bpp, dtype=np.int64)
                    cur[x:x + bpp] = (line[x:x + bpp] + _paeth(left, up, ul)) & 0xFF
                else:
                    raise ValueError("failed to decode image: bad PNG filter %d" % ftype)
        out[y] = cur
        prev = cur
    return out


def load_image(path: str):
    """loaders.LoadImage (pkg/loaders/image.go:21-61) for PNG files: an
    ImageTexture of colours in [0,1], row 0 at the top, each pixel the
    colour Go's image.At(x, y).RGBA() gives (alpha-premultiplied, 16-bit)
    divided by 65535.  Non-interlaced 8- and 16-bit grey, RGB, palette, grey
    + alpha and RGBA images; JPEG is not decoded here."""
    import struct
    import zlib
    from .scene import ImageTexture
    try:
        blob = open(path, "rb").read()
    except OSError as e:
        raise ValueError("failed to open image file: %s" % e)
    if blob[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("failed to decode image: only PNG images are decoded")
    pos, idat, plte, trns = 8, b"", None, None
    w = h = depth = ctype = interlace = None
    while pos + 8 <= len(blob):
        n, kind = struct.unpack(">I4s", blob[pos:pos + 8])
        body = blob[pos + 8:pos + 8 + n]
        pos += 12 + n
        if kind == b"IHDR":
            w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body)
        elif kind == b"PLTE":
            plte = np.frombuffer(body, dtype=np.uint8).reshape(-1, 3)
        elif kind == b"tRNS":
            trns = body
        elif kind == b"IDAT":
            idat += body
        elif kind == b"IEND":
            break
    if w is None or interlace != 0 or depth not in (8, 16) or ctype not in (0, 2, 3, 4, 6):
        raise ValueError("failed to decode image: unsupported PNG (8/16-bit, non-interlaced only)")
    if ctype == 3 and depth != 8:
        raise ValueError("failed to decode image: unsupported PNG palette depth")
    channels = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    bpp = channels * depth // 8
    rows = _unfilter(zlib.decompress(idat), h, w * bpp, bpp)
    if depth == 16:
        vals = (rows[:, 0::2] << 8) | rows[:, 1::2]  # big-endian samples, 0..65535
    else:
        vals = rows * 257  # 8-bit sample v as v | v << 8
    vals = vals.reshape(h, w, channels).astype(np.float64)
    if ctype == 3:
        idx = rows.reshape(h, w)
        rgb = plte[idx].astype(np.float64) * 257
        alpha = np.full((h, w), 65535.0)
        if trns is not None:
            a = np.full(len(plte), 255, dtype=np.int64)
            a[:len(trns)] = np.frombuffer(trns, dtype=np.uint8)
            alpha = a[idx].astype(np.float64) * 257
    elif ctype in (0, 4):
        rgb = np.repeat(vals[..., :1], 3, axis=-1)
        alpha = vals[..., 1] if ctype == 4 else np.full((h, w), 65535.0)
    else:
        rgb = vals[..., :3]
        alpha = vals[..., 3] if ctype == 6 else np.full((h, w), 65535.0)
    # color.NRGBA(64).RGBA(): premultiplied, truncating division
    rgb = np.floor(rgb * alpha[..., None] / 65535.0)
    return ImageTexture(rgb / 65535.0)
