"""Built-in scenes.

``cornell_scene`` mirrors scene.NewCornellScene (pkg/scene/cornell.go:32-257)
and ``default_scene`` mirrors scene.NewDefaultScene
(pkg/scene/default_scene.go:11-95).  The other constructors build the
synthetic workloads of this project from the same primitives:

* ``cornell_baseline``: the Cornell box with both boxes white, a (15,15,15)
  130x105 quad light, depth 8 and fixed samples per pixel.
* ``icosphere_scene``: a level-8 subdivided icosahedron (1,310,720
  triangles) displaced by 3-octave value noise, with one material per face,
  on a ground quad under a uniform infinite light.
* ``default_style_scene``: the seeded many-sphere scenes of the batched
  workload (one ground sphere of radius 1000, three feature spheres and
  10-500 small spheres) under a gradient sky.
* ``cone_test_scene`` / ``cylinder_test_scene`` / ``sphere_grid_scene``
  mirror scene.NewConeTestScene, scene.NewCylinderTestScene and
  scene.NewSphereGridScene.
* ``quadric_scene``: discs, capped and open cylinders, a pointed cone and
  frustums (the reference's Disc / Cylinder / Cone shapes) with Lambertian,
  metal and glass under a quad light and a gradient sky.
* ``ray_batch``: seeded raw ray batches (coherent primaries and incoherent
  surface-to-sphere rays) for the intersection benchmark and parity tests.
"""
import math

import numpy as np

from . import _capi as capi
from .scene import (MATERIAL_DTYPE, Box, CameraConfig, Cone, Cylinder, Dielectric, Disc, Emissive, Lambertian, Layered,
                    MaterialTable, Mesh, Metal, Mix, NewCheckerboardTexture, NewGradientTexture, NewGroundQuad,
                    NewUVDebugTexture, Quad, SamplingConfig, Scene, Sphere, TexturedLambertian, TexturedMetal, Triangle,
                    TriangleMesh)

CORNELL_SPHERES, CORNELL_BOXES, CORNELL_EMPTY = 0, 1, 2
CORNELL_QUAD_LIGHT, CORNELL_POINT_LIGHT, CORNELL_SPHERE_LIGHT = 0, 1, 2


def _cornell_camera(override=None):  # setupCornellCamera (cornell.go:59-77)
    base = CameraConfig(center=(278.0, 278.0, -800.0), look_at=(278.0, 278.0, 0.0), up=(0.0, 1.0, 0.0), width=400,
                        aspect_ratio=1.0, vfov=40.0, aperture=0.0, focus_distance=0.0)
    return base.merged(override)


def _cornell_walls(s):  # addCornellWalls (cornell.go:91-147)
    white = Lambertian((0.73, 0.73, 0.73))
    red = Lambertian((0.65, 0.05, 0.05))
    green = Lambertian((0.12, 0.45, 0.15))
    s.add(Quad((0.0, 0.0, 0.0), (556.0, 0.0, 0.0), (0.0, 0.0, 556.0), white),
          Quad((0.0, 556.0, 0.0), (556.0, 0.0, 0.0), (0.0, 0.0, 556.0), white),
          Quad((0.0, 0.0, 556.0), (556.0, 0.0, 0.0), (0.0, 556.0, 0.0), white),
          Quad((0.0, 0.0, 0.0), (0.0, 0.0, 556.0), (0.0, 556.0, 0.0), red),
          Quad((556.0, 0.0, 0.0), (0.0, 0.0, 556.0), (0.0, 556.0, 0.0), green))


def cornell_scene(geometry=CORNELL_SPHERES, light=CORNELL_QUAD_LIGHT, camera=None):
    """scene.NewCornellScene (pkg/scene/cornell.go:32-257) with its quad,
    point and sphere light variants."""
    s = Scene(camera=_cornell_camera(camera))
    # createCornellSamplingConfig (cornell.go:80-88)
    s.sampling = SamplingConfig(samples_per_pixel=150, max_depth=5, russian_roulette_min_bounces=16,
                                adaptive_min_samples=0.20, adaptive_threshold=0.005)
    _cornell_walls(s)
    emission = (18.0, 15.0, 8.0)
    if light == CORNELL_QUAD_LIGHT:  # addCornellLight (cornell.go:150-197)
        s.add_quad_light((213.0, 556.0 - 0.001, 227.0), (130.0, 0.0, 0.0), (0.0, 0.0, 105.0),
                         tuple(2.5 * e for e in emission))
    elif light == CORNELL_SPHERE_LIGHT:
        s.add_sphere_light((278.0, 556.0 - 0.001, 279.5), 52.5, tuple(2.05 * e for e in emission))
    elif light == CORNELL_POINT_LIGHT:
        # a 180-degree point spot light aimed at (0,-1,0) (cornell.go:170-182)
        s.add_point_spot_light((278.0, 556.0 - 0.001, 279.5), (0.0, -1.0, 0.0), tuple(20000.0 * e for e in emission),
                               180.0, 0.0)
    else:
        raise ValueError("unsupported Cornell light type")
    if geometry == CORNELL_SPHERES:  # addCornellSpheres (cornell.go:212-226)
        s.add(Sphere((185.0, 82.5, 169.0), 82.5, Metal((0.8, 0.8, 0.9), 0.0)),
              Sphere((370.0, 90.0, 351.0), 90.0, Dielectric(1.5)))
    elif geometry == CORNELL_BOXES:  # addCornellBoxes (cornell.go:229-257)
        white = Lambertian((0.73, 0.73, 0.73))
        mirror = Metal((0.9, 0.9, 0.9), 0.0)
        s.add(Box((370.0, 82.5, 169.0), (82.5, 82.5, 82.5), (0.0, 18 * math.pi / 180, 0.0), white),
              Box((185.0, 165.0, 351.0), (82.5, 165.0, 82.5), (0.0, -20 * math.pi / 180, 0.0), mirror))
    return s.finalize_size()


def cornell_baseline(width=400, max_depth=8):
    """The Cornell box of the path-tracing workload: five Lambertian walls,
    one 130x105 ceiling quad light of emission (15,15,15), two rotated white
    boxes (geometry of cornell.go:238-253), depth 8, fixed spp."""
    s = Scene(camera=_cornell_camera(CameraConfig(width=width)))
    s.sampling = SamplingConfig(max_depth=max_depth, russian_roulette_min_bounces=16, adaptive_min_samples=1.0,
                                adaptive_threshold=0.0)
    _cornell_walls(s)
    s.add_quad_light((213.0, 556.0 - 0.001, 227.0), (130.0, 0.0, 0.0), (0.0, 0.0, 105.0), (15.0, 15.0, 15.0))
    white = Lambertian((0.73, 0.73, 0.73))
    s.add(Box((370.0, 82.5, 169.0), (82.5, 82.5, 82.5), (0.0, 18 * math.pi / 180, 0.0), white),
          Box((185.0, 165.0, 351.0), (82.5, 165.0, 82.5), (0.0, -20 * math.pi / 180, 0.0), white))
    return s.finalize_size()


def cornell_boxes_bdpt(width=512, max_depth=8):
    """scene.NewCornellScene(CornellBoxes, CornellQuadLight, {Width: width})
    with MaxDepth = max_depth and fixed samples per pixel."""
    s = cornell_scene(CORNELL_BOXES, CORNELL_QUAD_LIGHT, CameraConfig(width=width))
    s.sampling.max_depth = max_depth
    s.sampling.adaptive_min_samples = 1.0
    s.sampling.adaptive_threshold = 0.0
    return s


def default_scene(camera=None):
    """scene.NewDefaultScene (pkg/scene/default_scene.go:11-95)."""
    base = CameraConfig(center=(0.0, 0.75, 2.0), look_at=(0.0, 0.5, -1.0), up=(0.0, 1.0, 0.0), width=400,
                        aspect_ratio=16.0 / 9.0, vfov=40.0, aperture=0.05, focus_distance=0.0)
    s = Scene(camera=base.merged(camera))
    s.sampling = SamplingConfig(samples_per_pixel=200, max_depth=50, russian_roulette_min_bounces=20,
                                adaptive_min_samples=0.15, adaptive_threshold=0.01)
    green = Lambertian((0.8 * 0.6, 0.8 * 0.6, 0.0))
    blue = Lambertian((0.1, 0.2, 0.5))
    red = Lambertian((0.65, 0.25, 0.2))
    silver = Metal((0.8, 0.8, 0.8), 0.0)
    gold = Metal((0.8, 0.6, 0.2), 0.3)
    glass = Dielectric(1.5)
    coated = Layered(glass, red)
    s.add_sphere_light((30.0, 30.5, 15.0), 10.0, (15.0, 14.0, 13.0))
    s.add(Sphere((0.0, 0.5, -1.0), 0.5, coated), Sphere((-1.0, 0.5, -1.0), 0.5, silver),
          Sphere((1.0, 0.5, -1.0), 0.5, gold), NewGroundQuad((0.0, 0.0, 0.0), 10000.0, green),
          Sphere((0.5, 0.25, -0.5), 0.25, glass), Sphere((-0.5, 0.25, -0.5), 0.25, glass),
          Sphere((-0.5, 0.25, -0.5), -0.24, glass), Sphere((-0.5, 0.25, -0.5), 0.20, blue))
    s.add_gradient_infinite_light((0.5, 0.7, 1.0), (1.0, 1.0, 1.0))
    return s.finalize_size()


def quadric_scene(width=64, max_depth=8, disc_light=False):
    """Discs, cylinders and cones (geometry.NewDisc / NewCylinder / NewCone)
    of every kind: a floor disc, capped and open cylinders, a pointed cone,
    capped and open frustums, an axis-tilted cylinder; Lambertian, metal and
    glass; a quad light (or a downward disc light, lights.NewDiscLight) and a
    gradient sky."""
    cam = CameraConfig(center=(0.0, 2.5, 7.0), look_at=(0.0, 0.8, 0.0), up=(0.0, 1.0, 0.0), width=width,
                       aspect_ratio=1.0, vfov=45.0)
    s = Scene(camera=cam)
    s.sampling = SamplingConfig(max_depth=max_depth, russian_roulette_min_bounces=16, adaptive_min_samples=1.0,
                                adaptive_threshold=0.0)
    white, red, blue = Lambertian((0.73, 0.73, 0.73)), Lambertian((0.65, 0.1, 0.1)), Lambertian((0.1, 0.2, 0.6))
    steel, glass = Metal((0.8, 0.8, 0.85), 0.1), Dielectric(1.5)
    s.add(Disc((0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 4.0, white),
          Cylinder((-2.0, 0.0, -0.5), (-2.0, 1.6, -0.5), 0.5, True, red),
          Cylinder((2.0, 0.0, -0.5), (2.0, 1.2, -0.5), 0.6, False, steel),
          Cone((0.0, 0.0, -1.2), 0.8, (0.0, 2.0, -1.2), 0.0, True, blue),
          Cone((-0.8, 0.0, 1.2), 0.5, (-0.8, 0.9, 1.2), 0.25, True, glass),
          Cone((1.0, 0.0, 1.3), 0.45, (1.0, 0.7, 1.3), 0.2, False, white),
          Cylinder((0.2, 0.4, 0.9), (1.0, 0.9, 0.3), 0.2, True, glass),
          Disc((-1.2, 2.2, -2.0), (0.3, -0.2, 1.0), 0.7, steel))
    if disc_light:
        s.add_disc_light((0.0, 4.0, 0.0), (0.0, -1.0, 0.0), 1.1, (8.0, 8.0, 8.0))
    else:
        s.add_quad_light((-1.0, 4.0, -1.0), (2.0, 0.0, 0.0), (0.0, 0.0, 2.0), (6.0, 6.0, 6.0))
    s.add_gradient_infinite_light((0.3, 0.4, 0.6), (0.7, 0.7, 0.7))
    return s.finalize_size()


def _quadric_test_base(camera):
    # the camera, sampling, ground and lighting shared by NewConeTestScene
    # (cone_scene.go:10-179) and NewCylinderTestScene (cylinder_scene.go:10-119)
    base = CameraConfig(center=(0.0, 1.5, 4.0), look_at=(0.0, 1.0, 0.0), up=(0.0, 1.0, 0.0), width=400,
                        aspect_ratio=16.0 / 9.0, vfov=50.0, aperture=0.0, focus_distance=0.0)
    s = Scene(camera=base.merged(camera))
    s.sampling = SamplingConfig(samples_per_pixel=200, max_depth=50, russian_roulette_min_bounces=20,
                                adaptive_min_samples=0.15, adaptive_threshold=0.01)
    s.add(NewGroundQuad((0.0, 0.0, 0.0), 10000.0, Lambertian((0.5, 0.5, 0.5))))
    return s


def _quadric_test_lights(s):
    s.add_sphere_light((3.0, 5.0, 3.0), 1.5, (10.0, 10.0, 10.0))
    s.add_gradient_infinite_light((0.5, 0.7, 1.0), (1.0, 1.0, 1.0))
    return s.finalize_size()


def cone_test_scene(camera=None):
    """scene.NewConeTestScene (pkg/scene/cone_scene.go:10-179)."""
    s = _quadric_test_base(camera)
    red, blue, green = Lambertian((0.8, 0.2, 0.2)), Lambertian((0.2, 0.2, 0.8)), Lambertian((0.2, 0.8, 0.2))
    gold, glass = Metal((0.8, 0.6, 0.2), 0.1), Dielectric(1.5)
    s.add(Cone((0.0, 0.0, 0.0), 0.5, (0.0, 2.0, 0.0), 0.0, True, red),
          Cone((-2.0, 0.8, -0.8), 0.5, (-2.0, 0.2, 0.5), 0.2, True, gold),
          Cone((2.0, 0.0, 0.0), 0.8, (2.0, 0.6, 0.0), 0.5, True, blue),
          Cone((2.0, 0.6, 0.0), 0.5, (2.0, 1.8, 0.0), 0.0, True, glass),
          Cone((-1.5, 0.0, -0.5), 0.4, (-1.2, 1.2, -0.3), 0.15, False, green),
          Cone((-0.8, 0.0, 1.2), 0.3, (-0.8, 0.8, 1.2), 0.0, True, glass),
          Cone((0.8, 0.2, 1.2), 0.3, (0.8, 1.0, 1.2), 0.0, True, glass))
    return _quadric_test_lights(s)


def cylinder_test_scene(camera=None):
    """scene.NewCylinderTestScene (pkg/scene/cylinder_scene.go:10-119)."""
    s = _quadric_test_base(camera)
    red, blue = Lambertian((0.8, 0.2, 0.2)), Lambertian((0.2, 0.2, 0.8))
    gold, glass = Metal((0.8, 0.6, 0.2), 0.1), Dielectric(1.5)
    s.add(Cylinder((-0.3, 1.0, -1.5), (0.0, 1.2, 2.0), 0.35, False, gold),
          Cylinder((-2.5, 0.3, 0.0), (-1.5, 0.3, 0.0), 0.3, True, blue),
          Cylinder((1.8, 0.0, 0.0), (1.8, 2.0, 0.0), 0.5, True, red),
          Cylinder((0.5, 0.0, 1.0), (0.5, 0.6, 1.0), 0.2, True, glass))
    return _quadric_test_lights(s)


def _oklch_to_rgb(l, c, h):
    """OKLCH -> linear sRGB clamped to [0,1] (the OKLab transform published by
    B. Ottosson, 2020), as spheregrid.go:14-40 colours its spheres."""
    hr = h * math.pi / 180.0
    a, b = c * math.cos(hr), c * math.sin(hr)
    l_ = (l + 0.3963377774 * a + 0.2158037573 * b) ** 3
    m_ = (l - 0.1055613458 * a - 0.0638541728 * b) ** 3
    s_ = (l - 0.0894841775 * a - 1.2914855480 * b) ** 3
    rgb = (4.0767416621 * l_ - 3.3077115913 * m_ + 0.2309699292 * s_,
           -1.2684380046 * l_ + 2.6097574011 * m_ - 0.3413193965 * s_,
           -0.0041960863 * l_ - 0.7034186147 * m_ + 1.7076147010 * s_)
    return tuple(max(0.0, min(1.0, x)) for x in rgb)


def sphere_grid_scene(grid_size=10, finish="metallic", camera=None):
    """scene.NewSphereGridScene (pkg/scene/spheregrid.go:44-189): a
    grid_size x grid_size grid of spheres over a 9 x 9 area, hue varying
    along both axes; finish is one of matte, glossy (glass over Lambertian),
    mirror, glass, mixed (Mix of Lambertian and metal, 50/50) or metallic."""
    base = CameraConfig(center=(4.5, 6.0, 18.0), look_at=(4.5, 0.8, 4.5), up=(0.0, 1.0, 0.0), width=800,
                        aspect_ratio=16.0 / 9.0, vfov=40.0, aperture=0.02, focus_distance=0.0)
    s = Scene(camera=base.merged(camera))
    s.sampling = SamplingConfig(samples_per_pixel=100, max_depth=40, russian_roulette_min_bounces=12,
                                adaptive_min_samples=0.12, adaptive_threshold=0.015)
    s.add_sphere_light((20.0, 25.0, 20.0), 8.0, (8.0, 7.5, 6.5))
    s.add(NewGroundQuad((0.0, 0.0, 0.0), 10000.0, Lambertian((0.5, 0.5, 0.5))))
    area = 9.0
    spacing = area / float(grid_size - 1)
    radius = max(0.02, min(0.35, spacing * 0.35))
    lo_c, hi_c = 0.05, 0.25
    for i in range(grid_size):
        for j in range(grid_size):
            pos = (i * spacing - area / 2.0 + 4.5, radius, j * spacing - area / 2.0 + 4.5)
            fi, fj = i / float(grid_size - 1), j / float(grid_size - 1)
            hue = math.fmod(fi * 330.0 + fj * 120.0, 360.0)
            chroma = lo_c + 0.8 * (hi_c - lo_c) + 0.2 * (hi_c - lo_c) * fj
            color = _oklch_to_rgb(0.65, chroma, hue)
            if finish == "matte":
                m = Lambertian(color)
            elif finish == "glossy":
                m = Layered(Dielectric(1.5), Lambertian(color))
            elif finish == "mirror":
                m = Metal((0.9, 0.9, 0.9), 0.0)
            elif finish == "glass":
                m = Dielectric(1.5)
            elif finish == "mixed":
                m = Mix(Lambertian(color), Metal(color, 0.1), 0.5)
            else:
                m = Metal(color, 0.05)
            s.add(Sphere(pos, radius, m))
    s.add_gradient_infinite_light((0.5, 0.7, 1.0), (1.0, 1.0, 1.0))
    return s.finalize_size()


def texture_test_scene(camera=None):
    """scene.NewTextureTestScene (pkg/scene/texture_test_scene.go:11-161):
    one shape of each kind, textured with the procedural checkerboard,
    gradient and UV-debug textures, on a checkered ground."""
    base = CameraConfig(center=(0.0, 2.0, 10.0), look_at=(0.0, 1.0, 0.0), up=(0.0, 1.0, 0.0), width=800,
                        aspect_ratio=16.0 / 9.0, vfov=50.0, aperture=0.0, focus_distance=0.0)
    s = Scene(camera=base.merged(camera))
    s.sampling = SamplingConfig(samples_per_pixel=100, max_depth=10, russian_roulette_min_bounces=5,
                                adaptive_min_samples=0.15, adaptive_threshold=0.01)
    checker = TexturedLambertian(NewCheckerboardTexture(256, 256, 32, (0.9, 0.9, 0.9), (0.2, 0.2, 0.8)))
    gradient = TexturedLambertian(NewGradientTexture(256, 256, (1.0, 0.2, 0.2), (0.2, 1.0, 0.2)))
    uv_debug = TexturedLambertian(NewUVDebugTexture(256, 256))
    brick = TexturedLambertian(NewCheckerboardTexture(512, 512, 16, (0.7, 0.3, 0.1), (0.5, 0.2, 0.05)))
    s.add(Sphere((-6.0, 1.0, 0.0), 1.0, checker),
          Cylinder((-4.0, 0.0, 0.0), (-4.0, 2.0, 0.0), 0.6, True, gradient),
          Cone((-2.0, 0.0, 0.0), 0.8, (-2.0, 2.0, 0.0), 0.2, True, uv_debug),
          Box((0.0, 1.0, 0.0), (0.8, 0.8, 0.8), (0.0, 0.0, 0.0), brick),
          Disc((2.0, 1.2, 0.0), (0.0, 0.0, 1.0), 0.9, checker),
          Quad((3.5, 0.0, 0.2), (1.5, 0.0, -0.3), (0.0, 2.0, 0.0), gradient),
          Triangle((5.5, 0.0, 0.0), (7.0, 0.0, 0.0), (6.25, 2.0, 0.0), uv_debug),
          Quad((-10.0, 0.0, -5.0), (20.0, 0.0, 0.0), (0.0, 0.0, 15.0), brick))
    s.add_sphere_light((0.0, 8.0, 5.0), 2.0, (20.0, 20.0, 20.0))
    s.add_gradient_infinite_light((0.3, 0.4, 0.6), (0.2, 0.2, 0.2))
    return s.finalize_size()


def textured_mesh_scene(width=48, max_depth=8, n=12):
    """A triangle mesh with every TriangleMeshOptions field: an n x n grid
    with per-vertex UVs on a UV-debug texture (VertexUVs), per-triangle
    normals tilted away from the geometric ones (Normals), a rotation about
    its centre (Rotation / Center), and a checkerboard ground, under a sphere
    light and a gradient sky."""
    cam = CameraConfig(center=(0.0, 2.0, 4.5), look_at=(0.0, 0.6, 0.0), up=(0.0, 1.0, 0.0), width=width,
                       aspect_ratio=1.0, vfov=45.0)
    s = Scene(camera=cam)
    s.sampling = SamplingConfig(max_depth=max_depth, russian_roulette_min_bounces=16, adaptive_min_samples=1.0,
                                adaptive_threshold=0.0)
    ys, xs = np.mgrid[0:n + 1, 0:n + 1] / float(n)
    verts = np.stack([xs * 2.0 - 1.0, ys * 1.6 + 0.1, 0.15 * np.sin(6.0 * xs)], axis=-1).reshape(-1, 3)
    uvs = np.stack([xs, ys], axis=-1).reshape(-1, 2)
    faces = []
    for j in range(n):
        for i in range(n):
            a, b, c, d = j * (n + 1) + i, j * (n + 1) + i + 1, (j + 1) * (n + 1) + i, (j + 1) * (n + 1) + i + 1
            faces += [(a, b, d), (a, d, c)]
    faces = np.array(faces, dtype=np.uint32)
    e1 = verts[faces[:, 1]] - verts[faces[:, 0]]
    e2 = verts[faces[:, 2]] - verts[faces[:, 0]]
    geo = np.cross(e1, e2)
    tilt = np.stack([0.4 * np.cos(np.arange(len(faces))), 0.3 * np.ones(len(faces)), np.zeros(len(faces))], axis=-1)
    normals = geo / np.linalg.norm(geo, axis=1, keepdims=True) + tilt  # not unit: normalised as NewTriangleWithNormal does
    mesh = TriangleMesh(vertices=verts, faces=faces, material=TexturedLambertian(NewUVDebugTexture(64, 64)),
                        normals=normals, vertex_uvs=uvs, rotation=(0.0, 0.35, 0.1), center=(0.0, 0.9, 0.0))
    s.add(Mesh(mesh),
          Quad((-4.0, 0.0, -4.0), (8.0, 0.0, 0.0), (0.0, 0.0, 8.0),
               TexturedLambertian(NewCheckerboardTexture(128, 128, 16, (0.8, 0.8, 0.8), (0.3, 0.3, 0.3)))))
    s.add_sphere_light((1.5, 3.0, 2.0), 0.5, (12.0, 12.0, 12.0))
    s.add_gradient_infinite_light((0.3, 0.4, 0.6), (0.6, 0.6, 0.6))
    return s.finalize_size()


def spot_scene(width=48, point=False, max_depth=8):
    """The caustic-glass scene's lighting (scene.NewCausticGlassScene,
    caustic_glass.go:36-95: a spot light from (0,5,9) at (-5,2.75,0) with a
    30-degree cone, 5-degree falloff and (for the disc spot) radius 0.7, plus
    a 0.1 uniform infinite light) and its camera, over procedural geometry in
    place of the PLY meshes the reference loads: a floor, a glass sphere, a
    Lambertian cylinder, a metal cone and a layered disc."""
    cam = CameraConfig(center=(-5.5, 7.0, -5.5), look_at=(-4.75, 2.25, 0.0), up=(0.0, 1.0, 0.0), width=width,
                       aspect_ratio=525.0 / 750.0, vfov=45.0)
    s = Scene(camera=cam)
    s.sampling = SamplingConfig(max_depth=max_depth, russian_roulette_min_bounces=16, adaptive_min_samples=1.0,
                                adaptive_threshold=0.0)
    intensity = (139.8113403320, 118.6366500854, 105.3887557983)
    if point:
        s.add_point_spot_light((0.0, 5.0, 9.0), (-5.0, 2.75, 0.0), intensity, 30.0, 5.0, 0.7)
    else:
        s.add_spot_light((0.0, 5.0, 9.0), (-5.0, 2.75, 0.0), intensity, 30.0, 5.0, 0.7)
    s.add_uniform_infinite_light((0.1, 0.1, 0.1))
    white = Lambertian((0.7, 0.7, 0.7))
    s.add(Quad((-15.0, 0.0, -15.0), (30.0, 0.0, 0.0), (0.0, 0.0, 30.0), white),
          Sphere((-5.0, 1.5, 0.0), 1.5, Dielectric(1.25)),
          Cylinder((-2.5, 0.0, 1.5), (-2.5, 2.0, 1.5), 0.6, True, Lambertian((0.6, 0.3, 0.2))),
          Cone((-7.5, 0.0, 1.0), 1.0, (-7.5, 2.5, 1.0), 0.0, True, Metal((0.8, 0.8, 0.8), 0.2)),
          Disc((-4.0, 0.01, -2.5), (0.0, 1.0, 0.0), 1.2, Layered(Dielectric(1.5), Lambertian((0.2, 0.5, 0.3)))))
    return s.finalize_size()


# ---------------------------------------------------------------- icosphere
def icosphere(level):
    """Unit icosphere: the 20-face icosahedron subdivided `level` times,
    midpoints pushed to the sphere.  Returns (vertices float64, faces uint32)."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    for _ in range(level):
        nv = v.shape[0]
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        e.sort(axis=1)
        key = e[:, 0] * nv + e[:, 1]
        uniq, inv = np.unique(key, return_inverse=True)
        a, b = uniq // nv, uniq % nv
        mid = v[a] + v[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        m = inv.reshape(3, -1) + nv  # midpoint ids of edges (01, 12, 20) per face
        v = np.concatenate([v, mid])
        m01, m12, m20 = m[0], m[1], m[2]
        f = np.concatenate([np.stack([f[:, 0], m01, m20], 1), np.stack([f[:, 1], m12, m01], 1),
                            np.stack([f[:, 2], m20, m12], 1), np.stack([m01, m12, m20], 1)])
    return v, f.astype(np.uint32)


def _lattice(ix, iy, iz, seed):
    """Hash of integer lattice points to [-1, 1) (64-bit mix of the three
    coordinates and the seed)."""
    h = (ix.astype(np.uint64) * np.uint64(0x9E3779B97F4A7C15)) ^ (iy.astype(np.uint64) * np.uint64(0xC2B2AE3D27D4EB4F)) \
        ^ (iz.astype(np.uint64) * np.uint64(0x165667B19E3779F9)) ^ np.uint64(seed * 0x27D4EB2F165667C5 & 0xFFFFFFFFFFFFFFFF)
    h ^= h >> np.uint64(33)
    h *= np.uint64(0xFF51AFD7ED558CCD)
    h ^= h >> np.uint64(33)
    h *= np.uint64(0xC4CEB9FE1A85EC53)
    h ^= h >> np.uint64(33)
    return (h >> np.uint64(11)).astype(np.float64) / float(1 << 53) * 2.0 - 1.0


def value_noise(p, seed, octaves=3, base_freq=4.0, gain=0.5):
    """Sum of `octaves` octaves of trilinear lattice value noise with
    smoothstep weights, frequency doubling and amplitude `gain` per octave."""
    total = np.zeros(p.shape[0])
    amp, freq = 1.0, base_freq
    with np.errstate(over="ignore"):
        for o in range(octaves):
            q = p * freq
            i0 = np.floor(q).astype(np.int64)
            fr = q - i0
            w = fr * fr * (3 - 2 * fr)
            acc = np.zeros(p.shape[0])
            for dx in (0, 1):
                for dy in (0, 1):
                    for dz in (0, 1):
                        val = _lattice(i0[:, 0] + dx, i0[:, 1] + dy, i0[:, 2] + dz, seed + o)
                        wx = w[:, 0] if dx else 1 - w[:, 0]
                        wy = w[:, 1] if dy else 1 - w[:, 1]
                        wz = w[:, 2] if dz else 1 - w[:, 2]
                        acc += val * wx * wy * wz
            total += amp * acc
            amp *= gain
            freq *= 2.0
    return total


def icosphere_scene(level=8, width=1024, max_depth=8, noise_seed=7, material_seed=11, amplitude=0.1):
    """The BVH-stress workload: displaced level-`level` icosphere, 50 %
    Lambertian faces (albedo U[0.2,0.8]^3) and 50 % metal faces (albedo
    U[0.5,1]^3, fuzz U[0,0.3]), ground quad, uniform infinite light 1.0.
    Vertices are computed in float64 and rounded to float32 values."""
    v, f = icosphere(level)
    r = 1.0 + amplitude * value_noise(v, noise_seed)
    v = (v * r[:, None]).astype(np.float32).astype(np.float64)
    nf = f.shape[0]
    rng = np.random.default_rng(material_seed)
    metal = rng.random(nf) < 0.5
    rows = np.zeros(nf, dtype=MATERIAL_DTYPE)
    rows["kind"] = np.where(metal, capi.MAT_METAL, capi.MAT_LAMBERTIAN)
    lam_albedo = rng.uniform(0.2, 0.8, size=(nf, 3))
    met_albedo = rng.uniform(0.5, 1.0, size=(nf, 3))
    rows["albedo"] = np.where(metal[:, None], met_albedo, lam_albedo)
    rows["fuzz"] = np.where(metal, rng.uniform(0.0, 0.3, size=nf), 0.0)
    rows["ior"] = 1.0
    mesh = TriangleMesh(vertices=v, faces=f, materials=MaterialTable(rows), material_index=np.arange(nf))
    s = Scene(camera=CameraConfig(center=(0.0, 0.6, 3.4), look_at=(0.0, -0.15, 0.0), up=(0.0, 1.0, 0.0),
                                  width=width, aspect_ratio=1.0, vfov=40.0))
    s.sampling = SamplingConfig(max_depth=max_depth, russian_roulette_min_bounces=16, adaptive_min_samples=1.0)
    s.add(Mesh(mesh), NewGroundQuad((0.0, -1.2, 0.0), 100.0, Lambertian((0.5, 0.5, 0.5))))
    s.add_uniform_infinite_light((1.0, 1.0, 1.0))
    return s.finalize_size()


# ---------------------------------------------------------------- many-sphere jobs
def default_style_scene(seed, width=None, height=None, max_depth=8):
    """One job of the batched workload: ground sphere (0,-1000,0) r 1000,
    feature spheres at (-4,1,0) (0,1,0) (4,1,0) (glass / Lambertian / metal),
    N ~ U[10,500] spheres of radius 0.2 on a jittered grid at y = 0.2 with
    60/25/15 % Lambertian / metal (fuzz U[0,0.5]) / dielectric 1.5, gradient
    sky.  Resolution is drawn from {128^2, 256^2, 512^2, 1024x768} unless
    given."""
    rng = np.random.default_rng(seed)
    if width is None:
        width, height = [(128, 128), (256, 256), (512, 512), (1024, 768)][rng.integers(4)]
    cam = CameraConfig(center=(13.0, 2.0, 3.0), look_at=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0), width=width,
                       aspect_ratio=width / height, vfov=20.0)
    s = Scene(camera=cam)
    s.sampling = SamplingConfig(max_depth=max_depth, russian_roulette_min_bounces=16, adaptive_min_samples=1.0)
    s.add(Sphere((0.0, -1000.0, 0.0), 1000.0, Lambertian((0.5, 0.5, 0.5))))
    c1 = tuple(rng.uniform(0.1, 0.9, 3))
    c2 = tuple(rng.uniform(0.5, 1.0, 3))
    s.add(Sphere((-4.0, 1.0, 0.0), 1.0, Dielectric(1.5)), Sphere((0.0, 1.0, 0.0), 1.0, Lambertian(c1)),
          Sphere((4.0, 1.0, 0.0), 1.0, Metal(c2, 0.0)))
    n = int(rng.integers(10, 501))
    cells = [(a, b) for a in range(-11, 12) for b in range(-11, 12)]
    feats = np.array([[-4.0, 0.0], [0.0, 0.0], [4.0, 0.0]])
    ok = [c for c in cells if np.min(np.hypot(feats[:, 0] - (c[0] + 0.45), feats[:, 1] - (c[1] + 0.45))) > 1.3]
    pick = rng.choice(len(ok), size=min(n, len(ok)), replace=False)
    for k in pick:
        a, b = ok[k]
        x, z = a + 0.9 * rng.random(), b + 0.9 * rng.random()
        u = rng.random()
        if u < 0.60:
            m = Lambertian(tuple(rng.random(3) * rng.random(3)))
        elif u < 0.85:
            m = Metal(tuple(rng.uniform(0.5, 1.0, 3)), float(rng.uniform(0.0, 0.5)))
        else:
            m = Dielectric(1.5)
        s.add(Sphere((x, 0.2, z), 0.2, m))
    s.add_gradient_infinite_light((0.5, 0.7, 1.0), (1.0, 1.0, 1.0))
    return s.finalize_size()


# ---------------------------------------------------------------- ray batches
def ray_batch(scene_vertices, scene_faces, n, seed=13, width=1024, camera=None):
    """A raw ray batch: n/2 coherent camera rays (pixels of a width x width
    image, several jittered samples each) and n/2 incoherent rays from
    area-uniform points on the given triangles in uniform-sphere directions.
    Returns an (n, 8) float32 array in gprt_ray layout."""
    rng = np.random.default_rng(seed)
    half = n // 2
    cam = camera or CameraConfig(center=(0.0, 0.6, 3.4), look_at=(0.0, -0.15, 0.0), up=(0.0, 1.0, 0.0), width=width,
                                 aspect_ratio=1.0, vfov=40.0)
    o = np.array(cam.center, dtype=np.float64)
    w = o - np.array(cam.look_at)
    w /= np.linalg.norm(w)
    u = np.cross(w, np.array(cam.up, dtype=np.float64))
    u /= np.linalg.norm(u)
    vv = np.cross(w, u)
    fd = np.linalg.norm(o - np.array(cam.look_at))
    h = math.tan(math.radians(cam.vfov) / 2)
    vh = 2 * h * fd
    vw = vh * cam.aspect_ratio
    height = cam.height
    du, dv = u * vw / cam.width, vv * vh / height
    p00 = o - w * fd - u * vw / 2 - vv * vh / 2 + (du + dv) / 2
    pix = np.arange(half) % (cam.width * height)
    px, py = pix % cam.width, pix // cam.width
    jit = rng.random((half, 2)) - 0.5
    target = p00 + du * (px + jit[:, 0])[:, None] + dv * (py + jit[:, 1])[:, None]
    d1 = target - o
    d1 /= np.linalg.norm(d1, axis=1, keepdims=True)
    rays = np.zeros((n, 8), dtype=np.float32)
    rays[:half, 0:3] = o
    rays[:half, 3] = 0.001
    rays[:half, 4:7] = d1
    rays[:half, 7] = np.inf
    m = n - half
    tri = scene_faces[rng.integers(0, scene_faces.shape[0], m)]
    a, b, c = scene_vertices[tri[:, 0]], scene_vertices[tri[:, 1]], scene_vertices[tri[:, 2]]
    r1, r2 = rng.random(m), rng.random(m)
    s1 = np.sqrt(r1)
    pts = a * (1 - s1)[:, None] + b * (s1 * (1 - r2))[:, None] + c * (s1 * r2)[:, None]
    z = 1 - 2 * rng.random(m)
    phi = 2 * math.pi * rng.random(m)
    rr = np.sqrt(np.maximum(0, 1 - z * z))
    d2 = np.stack([rr * np.cos(phi), rr * np.sin(phi), z], 1)
    rays[half:, 0:3] = pts
    rays[half:, 3] = 0.001
    rays[half:, 4:7] = d2
    rays[half:, 7] = np.inf
    return rays


# ---------------------------------------------------------------- job streams
def batched_jobs(n=256, seed=17, max_depth=8):
    """The heterogeneous batch: n seeded default-style scenes (resolution from
    {128^2, 256^2, 512^2, 1024x768}) with spp ~ U[1,64], max depth 8.
    Returns [(Scene, spp)]."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        sseed = int(rng.integers(0, 2 ** 31 - 1))
        spp = int(rng.integers(1, 65))
        out.append((default_style_scene(sseed, max_depth=max_depth), spp))
    return out


def serving_requests(n, seed=23, kinds=4):
    """A request stream mixing the workloads: (kind, target spp) per request,
    kind uniform over 0..kinds-1 (0 Cornell 400^2, 1 icosphere 1024^2,
    2 Cornell boxes 512^2, 3 default-style scene), target spp uniform over
    {16, 20, ..., 256} (passes of 4 spp)."""
    rng = np.random.default_rng(seed)
    return [(int(rng.integers(0, kinds)), int(4 * rng.integers(4, 65))) for _ in range(n)]


def poisson_arrivals(n, rate, seed=23):
    """Arrival times (s) of a Poisson process of `rate` requests per second."""
    rng = np.random.default_rng(seed + 1)
    return np.cumsum(rng.exponential(1.0 / rate, n))
