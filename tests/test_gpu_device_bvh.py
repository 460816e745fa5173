"""BVH construction on the GPU (GPRT_BUILD_DEVICE).

The device-built linear BVH must hold every primitive exactly once inside
boxes that contain their children (checked on the host copy at creation),
and give the same closest hits as the host-built SAH BVH: the primitive tests
spell out their rounding, so a ray's closest hit does not depend on the tree
except between primitives at the same distance (near-ties)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _both(ctx, scene):
    import gprt
    flat = scene.to_desc()
    return gprt.GpuScene(ctx, flat), gprt.GpuScene(ctx, flat, device_bvh=True)


@pytest.mark.parametrize("name", ["cornell", "spheres", "icosphere6", "quadrics", "textured_mesh"])
def test_device_bvh_hits_match_host_bvh(ctx, name):
    import gprt
    from gprt import scenes
    from test_gpu_intersect import _camera_rays, _rays_in_bounds
    scene = {"cornell": lambda: scenes.cornell_baseline(64), "spheres": lambda: scenes.default_style_scene(17, 64, 64),
             "icosphere6": lambda: scenes.icosphere_scene(level=6, width=64),
             "quadrics": lambda: scenes.quadric_scene(64),
             "textured_mesh": lambda: scenes.textured_mesh_scene(64)}[name]()
    host, dev = _both(ctx, scene)
    info = dev.info
    assert info.n_primitives == host.info.n_primitives and info.n_nodes > 0
    assert np.allclose(info.world_center[:], host.info.world_center[:]) and info.world_radius == host.info.world_radius
    rays = np.concatenate([_camera_rays(scene, 20000, 1),
                           _rays_in_bounds(info.world_center[:], min(info.world_radius, 600.0), 20000, 2)])
    hs, ss = host.primitive_map()
    hd, sd = dev.primitive_map()
    a, b = host.intersect(rays), dev.intersect(rays)
    hit_a, hit_b = a["prim"] != gprt.capi.NO_HIT, b["prim"] != gprt.capi.NO_HIT
    assert np.array_equal(hit_a, hit_b)
    both = hit_a & hit_b
    same = (hs[a["prim"][both]] == hd[b["prim"][both]]) & (ss[a["prim"][both]] == sd[b["prim"][both]])
    # a different primitive only at an exact tie in t
    assert np.all(same | (a["t"][both] == b["t"][both]))
    assert np.array_equal(a["t"][both], b["t"][both])
    host.close()
    dev.close()


@pytest.mark.parametrize("name", ["icosphere5", "textured_mesh"])
def test_device_bvh_render_equals_host_bvh_render(ctx, name):
    """Also covers the mesh normals / UVs each builder applies by final triangle id."""
    import gprt
    from gprt import scenes
    scene = scenes.icosphere_scene(level=5, width=48) if name == "icosphere5" else scenes.textured_mesh_scene(48)
    host, dev = _both(ctx, scene)
    films = []
    for g in (host, dev):
        r = gprt.ProgressiveRaytracer(g, gprt.ProgressiveConfig(max_samples_per_pixel=8, max_passes=1, seed=4))
        r.add_samples(8)
        films.append(r.film())
        r.close()
    rgb_a, rgb_b = films[0][0], films[1][0]
    diff = np.abs(rgb_a - rgb_b).max(axis=1)
    assert (diff > 0).mean() < 1e-3  # ties only
    host.close()
    dev.close()


def test_device_bvh_full_size_icosphere(ctx):
    import gprt
    from gprt import scenes
    scene = scenes.icosphere_scene(level=8, width=256)
    g = gprt.GpuScene(ctx, scene.to_desc(), device_bvh=True)
    assert g.info.n_triangles == 1310720
    r = gprt.ProgressiveRaytracer(g, gprt.ProgressiveConfig(max_samples_per_pixel=2, max_passes=1, seed=1))
    r.add_samples(2)
    r.sync()
    img = r.image()
    assert np.isfinite(img).all() and 0.05 < img.mean() < 1.0
    r.close()
    g.close()
