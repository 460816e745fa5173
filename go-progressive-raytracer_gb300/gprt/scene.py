"""Scene description API mirroring the reference's Go scene model.

``Scene`` follows ``scene.Scene`` (pkg/scene/scene.go:11-141): an ordered list
of shapes, a list of lights, camera and sampling configuration.  Materials
follow pkg/material (NewLambertian, NewMetal, NewDielectric, NewEmissive,
NewLayered); shapes follow pkg/geometry (NewSphere, NewQuad, NewBox,
NewTriangleMesh, NewTriangle); lights follow pkg/lights and the Scene.Add*Light
helpers.  ``Scene.to_desc()`` flattens it into the C ``gprt_scene_desc``.
"""
import ctypes as C
import math
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from . import _capi as capi

Vec3 = Sequence[float]


# ---------------------------------------------------------------- textures
@dataclass(eq=False)
class ImageTexture:  # material.ImageTexture (image_texture.go:8-23)
    pixels: np.ndarray  # (height, width, 3) float64, row y = 0 first

    @property
    def width(self):
        return self.pixels.shape[1]

    @property
    def height(self):
        return self.pixels.shape[0]


def NewCheckerboardTexture(width, height, check_size, color1, color2):  # procedural_textures.go:8-30
    y, x = np.mgrid[0:height, 0:width]
    even = ((x // check_size + y // check_size) % 2) == 0
    return ImageTexture(np.where(even[..., None], np.array(color1, dtype=np.float64), np.array(color2, dtype=np.float64)))


def NewUVDebugTexture(width, height):  # procedural_textures.go:34-46: (u, v, 0) per texel
    y, x = np.mgrid[0:height, 0:width]
    return ImageTexture(np.stack([x / float(width - 1), y / float(height - 1), np.zeros((height, width))], axis=-1))


def NewGradientTexture(width, height, color1, color2):  # procedural_textures.go:49-63: color1 at row 0
    t = (np.arange(height, dtype=np.float64) / float(height - 1))[:, None, None]
    row = np.array(color1, dtype=np.float64) * (1.0 - t) + np.array(color2, dtype=np.float64) * t
    return ImageTexture(np.broadcast_to(row, (height, width, 3)).copy())


# ---------------------------------------------------------------- materials
@dataclass
class Material:
    kind: int
    albedo: Vec3 = (0.0, 0.0, 0.0)
    fuzz: float = 0.0
    ior: float = 1.0
    emission: Vec3 = (0.0, 0.0, 0.0)
    outer: Optional["Material"] = None
    inner: Optional["Material"] = None
    texture: Optional[ImageTexture] = None


def Lambertian(albedo):  # material.NewLambertian (lambertian.go:15-18)
    return Material(capi.MAT_LAMBERTIAN, albedo=tuple(albedo))


def Metal(albedo, fuzz):  # material.NewMetal (metal.go:18-30), fuzz clamped to [0,1]
    return Material(capi.MAT_METAL, albedo=tuple(albedo), fuzz=min(1.0, max(0.0, fuzz)))


def TexturedLambertian(texture):  # material.NewTexturedLambertian (lambertian.go:19-24)
    return Material(capi.MAT_LAMBERTIAN, texture=texture)


def TexturedMetal(texture, fuzz):  # material.NewTexturedMetal (metal.go:25-36)
    return Material(capi.MAT_METAL, texture=texture, fuzz=min(1.0, max(0.0, fuzz)))


def Dielectric(ior):  # material.NewDielectric (dielectric.go:15-17)
    return Material(capi.MAT_DIELECTRIC, ior=ior)


def Emissive(emission):  # material.NewEmissive (emissive.go:12-14)
    return Material(capi.MAT_EMISSIVE, emission=tuple(emission))


def Layered(outer, inner):  # material.NewLayered (layered.go:16-21)
    return Material(capi.MAT_LAYERED, outer=outer, inner=inner)


def Mix(material1, material2, ratio):  # material.NewMix (mix.go:17-27), ratio clamped to [0,1]
    return Material(capi.MAT_MIX, outer=material1, inner=material2, fuzz=min(1.0, max(0.0, ratio)))


def SpotEmissive(emission, direction):  # discSpotLightMaterial (disc_spot_light.go:13-51)
    return Material(capi.MAT_SPOT_EMISSIVE, albedo=tuple(direction), emission=tuple(emission))


# ---------------------------------------------------------------- shapes
@dataclass
class Shape:
    kind: int
    material: Optional[Material]
    p: Sequence[float] = ()
    mesh: Optional["TriangleMesh"] = None


def Sphere(center, radius, material):  # geometry.NewSphere (sphere.go:18-24)
    return Shape(capi.SHAPE_SPHERE, material, tuple(center) + (radius,))


def Quad(corner, u, v, material):  # geometry.NewQuad (quad.go:109-130)
    return Shape(capi.SHAPE_QUAD, material, tuple(corner) + tuple(u) + tuple(v))


def Box(center, size, rotation, material):  # geometry.NewBox (box.go:21-33), size = half extents
    return Shape(capi.SHAPE_BOX, material, tuple(center) + tuple(size) + tuple(rotation))


def Triangle(v0, v1, v2, material):  # geometry.NewTriangle (triangle.go:20-33)
    return Shape(capi.SHAPE_TRIANGLE, material, tuple(v0) + tuple(v1) + tuple(v2))


def Disc(center, normal, radius, material):  # geometry.NewDisc (disc.go:21-44)
    return Shape(capi.SHAPE_DISC, material, tuple(center) + tuple(normal) + (radius,))


def Cylinder(base, top, radius, capped, material):  # geometry.NewCylinder (cylinder.go:24-39)
    return Shape(capi.SHAPE_CYLINDER, material, tuple(base) + tuple(top) + (radius, 1.0 if capped else 0.0))


def Cone(base, base_radius, top, top_radius, capped, material):  # geometry.NewCone (cone.go:27-77)
    return Shape(capi.SHAPE_CONE, material,
                 tuple(base) + tuple(top) + (base_radius, top_radius, 1.0 if capped else 0.0))


# numpy layout of gprt_material_desc (include/gprt.h)
MATERIAL_DTYPE = np.dtype([("kind", "<u4"), ("outer", "<u4"), ("inner", "<u4"), ("texture", "<u4"),
                           ("albedo", "<f8", 3), ("fuzz", "<f8"), ("ior", "<f8"), ("emission", "<f8", 3)])
assert MATERIAL_DTYPE.itemsize == C.sizeof(capi.MaterialDesc)


@dataclass
class MaterialTable:
    """A block of non-layered materials given as arrays (one row per material),
    for meshes whose faces each carry their own material."""
    rows: np.ndarray  # MATERIAL_DTYPE


@dataclass
class TriangleMesh:
    """geometry.NewTriangleMesh(vertices, faces, material, &TriangleMeshOptions{...})
    (pkg/geometry/triangle_mesh.go:33-146).  TriangleMeshOptions: Materials
    (``materials`` + ``material_index``), Normals (``normals``, one per
    triangle), VertexUVs (``vertex_uvs``, one per vertex) and Rotation /
    Center (applied to the vertices here, as rotateVertex does)."""
    vertices: np.ndarray  # (n, 3) float64
    faces: np.ndarray  # (m, 3) uint32
    material: Optional[Material] = None
    materials: Optional[object] = None  # list of Material, or a MaterialTable
    material_index: Optional[np.ndarray] = None  # (m,) index into `materials`
    normals: Optional[np.ndarray] = None  # (m, 3) custom triangle normals
    vertex_uvs: Optional[np.ndarray] = None  # (n, 2) texture coordinates
    rotation: Optional[Vec3] = None  # radians about X, then Y, then Z
    center: Optional[Vec3] = None  # the point rotated about

    def placed_vertices(self) -> np.ndarray:
        """The vertices after Rotation / Center (triangle_mesh.go:53-67, 170-199)."""
        v = np.asarray(self.vertices, dtype=np.float64).reshape(-1, 3)
        if self.rotation is None:
            return v
        v = v.copy()
        if self.center is not None:
            v -= np.asarray(self.center, dtype=np.float64)
        rx, ry, rz = self.rotation
        if rx != 0:
            c, s = math.cos(rx), math.sin(rx)
            v[:, 1], v[:, 2] = v[:, 1] * c - v[:, 2] * s, v[:, 1] * s + v[:, 2] * c
        if ry != 0:
            c, s = math.cos(ry), math.sin(ry)
            v[:, 0], v[:, 2] = v[:, 0] * c + v[:, 2] * s, -v[:, 0] * s + v[:, 2] * c
        if rz != 0:
            c, s = math.cos(rz), math.sin(rz)
            v[:, 0], v[:, 1] = v[:, 0] * c - v[:, 1] * s, v[:, 0] * s + v[:, 1] * c
        if self.center is not None:
            v += np.asarray(self.center, dtype=np.float64)
        return v


def Mesh(mesh: TriangleMesh):
    return Shape(capi.SHAPE_MESH, mesh.material, (), mesh)


def NewGroundQuad(center, size, material):  # scene.NewGroundQuad (scene.go:34-42)
    corner = (center[0] - size / 2, center[1], center[2] - size / 2)
    return Quad(corner, (size, 0.0, 0.0), (0.0, 0.0, size), material)


# ---------------------------------------------------------------- lights
@dataclass
class Light:
    kind: int
    shape: Optional[Shape] = None
    color_a: Vec3 = (0.0, 0.0, 0.0)
    color_b: Vec3 = (0.0, 0.0, 0.0)
    weight: float = 1.0
    from_: Vec3 = (0.0, 0.0, 0.0)  # spot lights: position and aim point
    to: Vec3 = (0.0, 0.0, 0.0)
    cone_deg: float = 0.0
    cone_delta_deg: float = 0.0
    radius: float = 0.0  # a sphere light with no shape: its radius (centre in from_)


@dataclass
class CameraConfig:  # geometry.CameraConfig (camera.go:18-32)
    """Field defaults are Go's zero values, so that a partly filled config
    (CameraConfig(width=96)) overrides only what it names when merged, as a
    Go composite literal does; a camera used directly names every field."""
    center: Vec3 = (0.0, 0.0, 0.0)
    look_at: Vec3 = (0.0, 0.0, 0.0)
    up: Vec3 = (0.0, 0.0, 0.0)
    width: int = 0
    aspect_ratio: float = 0.0
    vfov: float = 0.0
    aperture: float = 0.0
    focus_distance: float = 0.0

    def merged(self, o: Optional["CameraConfig"]):
        """MergeCameraConfig (camera.go:320-349): non-zero fields override."""
        if o is None:
            return self
        r = CameraConfig(**self.__dict__)
        if o.width:
            r.width = o.width
        if o.aspect_ratio:
            r.aspect_ratio = o.aspect_ratio
        if any(o.center):
            r.center = o.center
        if any(o.look_at):
            r.look_at = o.look_at
        if any(o.up):
            r.up = o.up
        if o.vfov:
            r.vfov = o.vfov
        if o.aperture:
            r.aperture = o.aperture
        if o.focus_distance:
            r.focus_distance = o.focus_distance
        return r

    @property
    def height(self):
        return int(float(self.width) / self.aspect_ratio)  # camera.go:91


@dataclass
class SamplingConfig:  # scene.SamplingConfig (scene.go:22-30)
    width: int = 0
    height: int = 0
    samples_per_pixel: int = 0
    max_depth: int = 5
    russian_roulette_min_bounces: int = 0
    adaptive_min_samples: float = 0.0
    adaptive_threshold: float = 0.0


@dataclass
class Scene:
    camera: CameraConfig = field(default_factory=CameraConfig)
    sampling: SamplingConfig = field(default_factory=SamplingConfig)
    shapes: List[Shape] = field(default_factory=list)
    lights: List[Light] = field(default_factory=list)
    light_weights: Optional[List[float]] = None  # lights.NewWeightedLightSampler

    def add(self, *shapes):
        self.shapes.extend(shapes)
        return self

    # Scene.Add*Light helpers (scene.go:102-141)
    def add_quad_light(self, corner, u, v, emission):
        q = Quad(corner, u, v, Emissive(emission))
        self.lights.append(Light(capi.LIGHT_QUAD, shape=q))
        self.shapes.append(q)
        return q

    def add_sphere_light(self, center, radius, emission):
        s = Sphere(center, radius, Emissive(emission))
        self.lights.append(Light(capi.LIGHT_SPHERE, shape=s))
        self.shapes.append(s)
        return s

    def add_disc_light(self, center, normal, radius, emission):  # lights.NewDiscLight (disc_light.go:17-22)
        d = Disc(center, normal, radius, Emissive(emission))
        self.lights.append(Light(capi.LIGHT_DISC, shape=d))
        self.shapes.append(d)
        return d

    def add_spot_light(self, from_, to, emission, cone_deg, cone_delta_deg, radius):
        """scene.AddSpotLight (scene.go:117-123): a disc spot light whose disc
        (facing `to`, directional emissive material) is also a shape."""
        dv = [t - f for f, t in zip(from_, to)]
        n = math.sqrt(sum(x * x for x in dv))
        direction = tuple(x / n for x in dv)
        d = Disc(from_, direction, radius, SpotEmissive(emission, direction))
        self.lights.append(Light(capi.LIGHT_DISC_SPOT, shape=d, color_a=tuple(emission), from_=tuple(from_), to=tuple(to),
                                 cone_deg=cone_deg, cone_delta_deg=cone_delta_deg))
        self.shapes.append(d)
        return d

    def add_point_spot_light(self, from_, to, emission, cone_deg, cone_delta_deg, radius=0.0):
        """scene.AddPointSpotLight (scene.go:125-129); `radius` is unused, as there."""
        self.lights.append(Light(capi.LIGHT_POINT_SPOT, color_a=tuple(emission), from_=tuple(from_), to=tuple(to),
                                 cone_deg=cone_deg, cone_delta_deg=cone_delta_deg))

    def add_uniform_infinite_light(self, emission):
        self.lights.append(Light(capi.LIGHT_UNIFORM_INFINITE, color_a=tuple(emission)))

    def add_gradient_infinite_light(self, top, bottom):
        self.lights.append(Light(capi.LIGHT_GRADIENT_INFINITE, color_a=tuple(top), color_b=tuple(bottom)))

    def finalize_size(self):
        """Image size from the camera, as main.go:188-193 does."""
        self.sampling.width = self.camera.width
        self.sampling.height = self.camera.height
        return self

    # ------------------------------------------------------------ flattening
    def to_desc(self) -> "FlatScene":
        return FlatScene(self)


class FlatScene:
    """A ``gprt_scene_desc`` with the arrays it points to kept alive."""

    def __init__(self, scene: Scene):
        mats: List[Material] = []
        tables = []  # (first material index, MaterialTable)
        index = {}

        def n_mats():
            return len(mats) + sum(t.rows.shape[0] for _, t in tables)

        def mat_id(m):
            if m is None:
                m = Lambertian((0.0, 0.0, 0.0))
            k = id(m)
            if k not in index:
                if m.kind in (capi.MAT_LAYERED, capi.MAT_MIX):
                    mat_id(m.outer)
                    mat_id(m.inner)
                index[k] = n_mats()
                mats.append((index[k], m))
            return index[k]

        shapes = scene.shapes
        shape_index = {id(s): i for i, s in enumerate(shapes)}
        meshes = []
        self._keep = []
        sdesc = (capi.ShapeDesc * max(1, len(shapes)))()
        for i, s in enumerate(shapes):
            d = sdesc[i]
            d.kind = s.kind
            if s.kind == capi.SHAPE_MESH:
                m = s.mesh
                v = np.ascontiguousarray(m.placed_vertices(), dtype=np.float64).reshape(-1, 3)
                f = np.ascontiguousarray(m.faces, dtype=np.uint32).reshape(-1, 3)
                md = capi.MeshDesc()
                md.vertices = v.ctypes.data_as(C.POINTER(C.c_double))
                md.indices = f.ctypes.data_as(C.POINTER(C.c_uint32))
                md.n_vertices = v.shape[0]
                md.n_triangles = f.shape[0]
                self._keep += [v, f]
                if m.normals is not None:
                    nrm = np.ascontiguousarray(m.normals, dtype=np.float64).reshape(-1, 3)
                    if nrm.shape[0] != f.shape[0]:  # NewTriangleMesh panics (triangle_mesh.go:41-44)
                        raise ValueError("number of normals must match number of triangles")
                    md.tri_normals = nrm.ctypes.data_as(C.POINTER(C.c_double))
                    self._keep.append(nrm)
                if m.vertex_uvs is not None:
                    uvs = np.ascontiguousarray(m.vertex_uvs, dtype=np.float64).reshape(-1, 2)
                    if uvs.shape[0] != v.shape[0]:  # triangle_mesh.go:47-50
                        raise ValueError("number of vertex UVs must match number of vertices")
                    md.vertex_uvs = uvs.ctypes.data_as(C.POINTER(C.c_double))
                    self._keep.append(uvs)
                if isinstance(m.materials, MaterialTable):
                    first = n_mats()
                    tables.append((first, m.materials))
                    tm = np.ascontiguousarray(np.asarray(m.material_index, dtype=np.int64) + first, dtype=np.uint32)
                    md.tri_materials = tm.ctypes.data_as(C.POINTER(C.c_uint32))
                    self._keep.append(tm)
                elif m.materials is not None:
                    ids = np.array([mat_id(x) for x in m.materials], dtype=np.uint32)
                    tm = np.ascontiguousarray(ids[np.asarray(m.material_index, dtype=np.int64)], dtype=np.uint32)
                    md.tri_materials = tm.ctypes.data_as(C.POINTER(C.c_uint32))
                    self._keep.append(tm)
                d.material = mat_id(m.material) if (m.material is not None or not isinstance(m.materials, MaterialTable)) \
                    else first
                d.mesh = len(meshes)
                meshes.append(md)
            else:
                d.material = mat_id(s.material)
                for k, x in enumerate(s.p):
                    d.p[k] = float(x)
        total = n_mats()
        mdesc = np.zeros(max(1, total), dtype=MATERIAL_DTYPE)
        textures, tex_index = [], {}
        for i, m in mats:
            d = mdesc[i]
            d["kind"] = m.kind
            if m.texture is not None:
                if id(m.texture) not in tex_index:
                    tex_index[id(m.texture)] = len(textures)
                    textures.append(m.texture)
                d["texture"] = tex_index[id(m.texture)] + 1
            d["albedo"] = m.albedo
            d["emission"] = m.emission
            d["fuzz"] = m.fuzz
            d["ior"] = m.ior
            if m.kind in (capi.MAT_LAYERED, capi.MAT_MIX):
                d["outer"] = index[id(m.outer)]
                d["inner"] = index[id(m.inner)]
        for first, t in tables:
            mdesc[first:first + t.rows.shape[0]] = t.rows
        ldesc = (capi.LightDesc * max(1, len(scene.lights)))()
        for i, l in enumerate(scene.lights):
            d = ldesc[i]
            d.kind = l.kind
            if l.shape is not None:
                d.shape = shape_index[id(l.shape)]
            elif l.kind == capi.LIGHT_SPHERE:
                d.shape = capi.NO_SHAPE
            for k in range(3):
                d.color_a[k] = l.color_a[k]
                d.color_b[k] = l.color_b[k]
                d.from_[k] = l.from_[k]
                d.to[k] = l.to[k]
            d.cone_deg = l.cone_deg
            d.cone_delta_deg = l.cone_delta_deg
            d.radius = l.radius
            d.weight = scene.light_weights[i] if scene.light_weights else 1.0
        meshd = (capi.MeshDesc * max(1, len(meshes)))(*meshes) if meshes else (capi.MeshDesc * 1)()
        desc = capi.SceneDesc()
        desc.materials = mdesc.ctypes.data_as(C.POINTER(capi.MaterialDesc))
        desc.shapes = C.cast(sdesc, C.POINTER(capi.ShapeDesc))
        desc.meshes = C.cast(meshd, C.POINTER(capi.MeshDesc))
        desc.lights = C.cast(ldesc, C.POINTER(capi.LightDesc))
        desc.n_materials = total
        desc.n_shapes = len(shapes)
        desc.n_meshes = len(meshes)
        desc.n_lights = len(scene.lights)
        desc.weighted_sampler = 1 if scene.light_weights else 0
        tdesc = (capi.TextureDesc * max(1, len(textures)))()
        for k, t in enumerate(textures):
            px = np.ascontiguousarray(t.pixels, dtype=np.float64)
            self._keep.append(px)
            tdesc[k].width, tdesc[k].height = t.width, t.height
            tdesc[k].pixels = px.ctypes.data_as(C.POINTER(C.c_double))
        desc.textures = C.cast(tdesc, C.POINTER(capi.TextureDesc))
        desc.n_textures = len(textures)
        cam = scene.camera
        for k in range(3):
            desc.camera.center[k] = cam.center[k]
            desc.camera.look_at[k] = cam.look_at[k]
            desc.camera.up[k] = cam.up[k]
        desc.camera.aspect_ratio = cam.aspect_ratio
        desc.camera.vfov_deg = cam.vfov
        desc.camera.aperture = cam.aperture
        desc.camera.focus_distance = cam.focus_distance
        desc.camera.width = cam.width
        sc = scene.sampling
        desc.sampling.width = sc.width or cam.width
        desc.sampling.height = sc.height or cam.height
        desc.sampling.samples_per_pixel = sc.samples_per_pixel
        desc.sampling.max_depth = sc.max_depth
        desc.sampling.rr_min_bounces = sc.russian_roulette_min_bounces
        desc.sampling.adaptive_min_samples = sc.adaptive_min_samples
        desc.sampling.adaptive_threshold = sc.adaptive_threshold
        self._keep += [mdesc, sdesc, ldesc, meshd]
        self.desc = desc
        self.materials = mats
        self.width = desc.sampling.width
        self.height = desc.sampling.height

    def ptr(self):
        return C.byref(self.desc)
