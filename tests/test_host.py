"""CPU tests of the host side: the C ABI loads and exports every symbol of
include/gprt.h; the host scene builder (flattening, world bounds, BVH layout)
agrees with the oracle's restatement of scene.Preprocess; scene builders."""
import ctypes as C
import math
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "gprt.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|void|const \w+\s*\*)\s+(gprt_\w+)\s*\(", txt, re.M)))


def test_library_exports_every_header_symbol(gprt_lib):
    import gprt
    syms = header_symbols()
    assert len(syms) >= 20
    lib = C.CDLL(gprt.capi.LIB_PATH)
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    # the Python binding declares exactly the header's entry points
    assert sorted(gprt.capi.SIGNATURES) == syms
    assert lib.gprt_version() == 1


def _validate(flat):
    import gprt
    info = gprt.capi.SceneInfo()
    err = C.create_string_buffer(256)
    rc = gprt.capi.load().gprt_scene_validate(C.byref(flat.desc), C.byref(info), err, 256)
    return rc, info, err.value.decode()


@pytest.mark.parametrize("name", ["cornell_baseline", "cornell_spheres", "cornell_boxes", "default", "icosphere5",
                                  "spheres17", "quadrics", "spot_disc", "cornell_point",
                                  "cone_test", "cylinder_test", "spheregrid", "texture_test", "textured_mesh"])
def test_host_builder_layout_and_world_bounds(gprt_lib, oracle, name):
    from gprt import scenes
    s = {"cornell_baseline": lambda: scenes.cornell_baseline(64),
         "cornell_spheres": lambda: scenes.cornell_scene(scenes.CORNELL_SPHERES),
         "cornell_boxes": lambda: scenes.cornell_scene(scenes.CORNELL_BOXES),
         "default": lambda: scenes.default_scene(),
         "icosphere5": lambda: scenes.icosphere_scene(level=5, width=64),
         "spheres17": lambda: scenes.default_style_scene(17, 64, 64),
         "quadrics": lambda: scenes.quadric_scene(64),
         "spot_disc": lambda: scenes.spot_scene(48),
         "cornell_point": lambda: scenes.cornell_scene(scenes.CORNELL_BOXES, scenes.CORNELL_POINT_LIGHT),
         "cone_test": lambda: scenes.cone_test_scene(),
         "cylinder_test": lambda: scenes.cylinder_test_scene(),
         "spheregrid": lambda: scenes.sphere_grid_scene(12, "mixed"),
         "texture_test": lambda: scenes.texture_test_scene(),
         "textured_mesh": lambda: scenes.textured_mesh_scene(64)}[name]()
    flat = s.to_desc()
    rc, info, err = _validate(flat)
    assert rc == 0, err
    o = oracle.OracleScene(flat)
    # BVH.Center / BVH.Radius of the reference (bvh.go:39-48) feed the infinite lights
    assert info.world_radius == pytest.approx(o.world_radius, rel=1e-12, abs=1e-12)
    assert np.allclose(np.array(info.world_center), np.array(o.world_center), rtol=1e-12, atol=1e-9)
    assert (info.image_width, info.image_height) == (o.width, o.height)
    assert info.n_nodes >= 1


def test_flat_layout_for_tiny_scenes(gprt_lib):
    """A scene of at most 32 primitives, at most 8 of them spheres, gets one
    leaf per primitive type under the root (a single BVH node): every ray
    tests the same primitives, so a warp's lanes stay converged.  Sphere
    scenes beyond 8 spheres and larger scenes keep a tree."""
    from gprt import scenes
    rc, info, err = _validate(scenes.cornell_baseline(32).to_desc())  # 18 quads
    assert rc == 0, err
    assert info.n_nodes == 1
    rc, info, err = _validate(scenes.cornell_scene(scenes.CORNELL_SPHERES).to_desc())  # quads + 2 spheres
    assert rc == 0, err
    assert info.n_nodes == 1
    rc, info, err = _validate(scenes.default_style_scene(80, 32, 32).to_desc())  # 15 spheres
    assert rc == 0, err
    assert info.n_nodes > 1
    rc, info, err = _validate(scenes.icosphere_scene(level=2, width=32).to_desc())  # 320 triangles
    assert rc == 0, err
    assert info.n_nodes > 1


def test_primitive_counts(gprt_lib):
    from gprt import scenes
    rc, info, err = _validate(scenes.cornell_baseline(64).to_desc())
    assert rc == 0, err
    # 5 walls + light quad + 2 boxes x 6 faces
    assert (info.n_quads, info.n_triangles, info.n_spheres) == (18, 0, 0)
    rc, info, err = _validate(scenes.icosphere_scene(level=3, width=32).to_desc())
    assert rc == 0 and info.n_triangles == 20 * 4 ** 3 and info.n_quads == 1


def test_icosphere_level8_shape():
    from gprt import scenes
    v, f = scenes.icosphere(8)
    assert f.shape == (1310720, 3) and v.shape == (655362, 3)
    assert np.allclose(np.linalg.norm(v, axis=1), 1.0)
    assert f.max() < v.shape[0]


def test_invalid_descriptions_are_rejected(gprt_lib):
    import gprt
    from gprt import scenes
    s = scenes.cornell_baseline(32)
    s.shapes.append(gprt.Quad((0, 0, 0), (1, 0, 0), (2, 0, 0), gprt.Lambertian((1, 1, 1))))  # degenerate
    rc, _, err = _validate(s.to_desc())
    assert rc == gprt.capi.GPRT_E_INVALID and "degenerate" in err
    bad = gprt.TriangleMesh(vertices=np.zeros((3, 3)), faces=np.array([[0, 1, 5]]), material=gprt.Lambertian((1, 1, 1)))
    s2 = scenes.cornell_baseline(32)
    s2.add(gprt.Mesh(bad))
    rc, _, err = _validate(s2.to_desc())
    assert rc == gprt.capi.GPRT_E_INVALID and "out of bounds" in err  # NewTriangleMesh panics (triangle_mesh.go:73-76)


def test_camera_height_and_merge():
    from gprt.scene import CameraConfig
    c = CameraConfig(width=400, aspect_ratio=16 / 9)
    assert c.height == 225  # int(400 / (16/9)), camera.go:91
    base = CameraConfig(center=(278.0, 278.0, -800.0), look_at=(278.0, 278.0, 0.0), up=(0.0, 1.0, 0.0), width=400,
                        aspect_ratio=1.0, vfov=40.0)
    m = base.merged(CameraConfig(width=512))
    # a partly filled override changes only the fields it names (camera.go:320-349)
    assert m.width == 512 and m.vfov == 40.0 and m.look_at == (278.0, 278.0, 0.0) and m.up == (0.0, 1.0, 0.0)
    assert base.merged(CameraConfig(look_at=(1.0, 2.0, 3.0))).look_at == (1.0, 2.0, 3.0)


def test_flat_scene_material_dedup():
    from gprt import scenes
    flat = scenes.cornell_baseline(32).to_desc()
    # white is shared by floor, ceiling, back wall; boxes create their own white
    assert flat.desc.n_shapes == 8 and flat.desc.n_lights == 1
    assert flat.desc.n_materials == 5


def test_oracle_renderer_schedule_and_determinism(oracle):
    from gprt import scenes
    flat = scenes.cornell_baseline(32).to_desc()
    s = oracle.OracleScene(flat)
    r = oracle.OracleRenderer(s, 0, max_spp=50, max_passes=7, seed=3)
    assert [oracle.load().oracle_samples_for_pass(r.h, p) for p in range(1, 8)] == [1, 9, 17, 25, 33, 41, 50]
    r.render_pass(1)
    a = r.image()
    r2 = oracle.OracleRenderer(s, 0, max_spp=50, max_passes=7, seed=3)
    r2.render_pass(1)
    assert np.array_equal(a, r2.image())
    _, lum, lum2, cnt = r.film()
    assert (cnt == 1).all()


def test_mesh_rotation_and_option_counts():
    # rotateVertex (triangle_mesh.go:170-199): X, then Y, then Z, about Center
    import math
    from gprt.scene import Lambertian, Mesh, Scene, TriangleMesh
    m = TriangleMesh(vertices=np.array([[1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [2.0, 0.0, 1.0]]),
                     faces=np.array([[0, 1, 2]]), material=Lambertian((0.5, 0.5, 0.5)),
                     rotation=(0.0, math.pi / 2, 0.0), center=(1.0, 0.0, 0.0))
    v = m.placed_vertices()
    assert np.allclose(v[0], [1.0, 0.0, 0.0]) and np.allclose(v[2], [2.0, 0.0, -1.0])
    s = Scene()
    s.add(Mesh(TriangleMesh(vertices=m.vertices, faces=m.faces, material=m.material, normals=np.zeros((2, 3)))))
    with pytest.raises(ValueError, match="normals must match"):
        s.to_desc()
