"""Scenes from files on the GPU: a PBRT scene (area light on a bilinear
patch, a point light whose sphere is not a shape, boxes, a conductor and a
dielectric) renders as the oracle renders the same loaded description; a
PLY mesh goes straight into the mesh description and renders bit-identically
to the same mesh given from memory, with either BVH builder."""
import numpy as np
import pytest

from test_gpu_render import gpu_render, oracle_render, same_input_stats
from test_loaders import write_ply

pytestmark = pytest.mark.gpu

PBRT_ROOM = '''LookAt 0 2 7  0 1.5 0  0 1 0
Camera "perspective" "float fov" [45]
Film "rgb" "integer xresolution" [48] "integer yresolution" [48]
WorldBegin
LightSource "infinite" "rgb L" [0.05 0.05 0.08]
LightSource "point" "rgb I" [3 3 3] "point3 from" [1.5 3 1]
Material "diffuse" "rgb reflectance" [0.7 0.7 0.7]
Shape "bilinearPatch" "point3 P00" [-4 0 -4] "point3 P01" [4 0 -4] "point3 P10" [-4 0 4] "point3 P11" [4 0 4]
Shape "bilinearPatch" "point3 P00" [-4 0 -3] "point3 P01" [4 0 -3] "point3 P10" [-4 5 -3] "point3 P11" [4 5 -3]
Material "conductor" "rgb eta" [0.9 0.8 0.6] "float roughness" [0.1]
Shape "box" "point3 center" [-1 0.6 -1] "point3 size" [0.6 0.6 0.6] "point3 rotation" [0 0.4 0]
AttributeBegin
  Material "dielectric" "float eta" [1.5]
  Shape "sphere" "float radius" [0.7] "point3 center" [1 0.7 0]
AttributeEnd
AttributeBegin
  AreaLightSource "diffuse" "rgb L" [6 5 4]
  Shape "bilinearPatch" "point3 P00" [-1 4 -1] "point3 P01" [1 4 -1] "point3 P10" [-1 4 1] "point3 P11" [1 4 1]
AttributeEnd
WorldEnd
'''


def _room(depth):
    from gprt import loaders
    s = loaders.parse_pbrt(PBRT_ROOM)
    s.desc.sampling.max_depth = depth
    s.desc.sampling.adaptive_min_samples = 1.0
    s.desc.sampling.adaptive_threshold = 0.0
    return s


@pytest.mark.parametrize("integ", ["pt", "bdpt"])
def test_pbrt_scene_same_inputs_parity(ctx, oracle, integ):
    import gprt
    s = _room(6)
    bd = integ == "bdpt"
    gpu, stats, _ = gpu_render(ctx, s, 8, seed=9, integrator=gprt.BDPTIntegrator() if bd else None)
    r, _ = oracle_render(oracle, s, 8, seed=9, integrator=1 if bd else 0)
    med, frac = same_input_stats(gpu, r.image())
    print(integ, "median rel", med, "frac > 1e-2", frac)
    assert stats.total_samples == 8 * stats.total_pixels
    assert med <= 1e-4, (med, frac)
    assert frac <= (0.03 if bd else 0.02), (med, frac)


@pytest.mark.parametrize("device_bvh", [False, True])
def test_ply_mesh_renders_as_the_in_memory_mesh(ctx, tmp_path, device_bvh):
    import gprt
    from gprt import loaders, scenes
    base = scenes.icosphere_scene(level=5, width=48)
    mesh = base.shapes[0].mesh
    v32 = np.asarray(mesh.vertices, dtype=np.float32)
    path = str(tmp_path / "ico.ply")
    write_ply(path, [tuple(x) for x in v32], [tuple(int(i) for i in f) for f in np.asarray(mesh.faces)])
    ply = loaders.load_ply(path)
    assert ply.vertices.shape == v32.shape and np.array_equal(ply.vertices, v32.astype(np.float64))
    mat = gprt.Lambertian((0.6, 0.5, 0.4))

    def scene(vertices, faces):
        s = scenes.icosphere_scene(level=5, width=48)
        s.shapes[0] = gprt.Mesh(gprt.TriangleMesh(vertices=vertices, faces=faces, material=mat))
        return s

    films = []
    for vs, fs in ((ply.vertices, ply.faces), (v32.astype(np.float64), np.asarray(mesh.faces, dtype=np.uint32))):
        g = gprt.GpuScene(ctx, scene(vs, fs), device_bvh=device_bvh)
        r = gprt.ProgressiveRaytracer(g, gprt.ProgressiveConfig(max_samples_per_pixel=4, max_passes=1, seed=3))
        r.add_samples(4)
        films.append(r.film())
        r.close()
        g.close()
    for a, b in zip(*films):
        assert np.array_equal(a, b)
