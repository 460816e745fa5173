"""Hit parity of the GPU BVH traversal against the oracle's BVH.Hit on
seeded ray batches.

Rule: the hit primitive (index in scene.Shapes, box face / mesh triangle)
matches exactly, except near-ties where the two distances agree within the
distance tolerance; hit distances agree within 1e-5 relative.  An FP32 ray
origin carries an absolute error of ~6e-8 x |origin|, so the relative error
is taken against max(t, |origin| / |direction|): for hits far from the
origin this is the plain 1e-5 relative rule.  FP32 rays grazing a
silhouette may legitimately hit in one precision and miss in the other; at
most 1e-4 of the rays may disagree that way.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL = 1e-5


def _rays_in_bounds(center, radius, n, seed):
    rng = np.random.default_rng(seed)
    o = np.array(center) + (rng.random((n, 3)) - 0.5) * radius * 1.2
    z = 1 - 2 * rng.random(n)
    phi = 2 * np.pi * rng.random(n)
    r = np.sqrt(1 - z * z)
    d = np.stack([r * np.cos(phi), r * np.sin(phi), z], 1)
    rays = np.zeros((n, 8), dtype=np.float32)
    rays[:, 0:3] = o
    rays[:, 3] = 0.001
    rays[:, 4:7] = d
    rays[:, 7] = np.inf
    return rays


def _camera_rays(scene, n, seed):
    from gprt import scenes
    cam = scene.camera
    return scenes.ray_batch(np.zeros((3, 3)), np.array([[0, 1, 2]]), 2 * n, seed=seed, camera=cam)[:n]


def _compare(ctx, oracle, scene, rays, any_hit=False):
    import gprt
    flat = scene.to_desc()
    g = gprt.GpuScene(ctx, flat)
    shape_map, sub_map = g.primitive_map()
    hits = g.intersect(rays, any_hit=any_hit)
    o = oracle.OracleScene(flat)
    t_o, shape_o, sub_o, _, nrm_o = o.intersect(rays)
    g_hit = hits["prim"] != gprt.capi.NO_HIT
    o_hit = shape_o >= 0
    if any_hit:
        return g_hit, o_hit
    both = g_hit & o_hit
    pid = hits["prim"][both]
    same = (shape_map[pid] == shape_o[both]) & (sub_map[pid] == sub_o[both])
    o_len = np.linalg.norm(rays[both, 0:3].astype(np.float64), axis=1) / np.linalg.norm(
        rays[both, 4:7].astype(np.float64), axis=1)
    rel = np.abs(hits["t"][both] - t_o[both]) / np.maximum(np.abs(t_o[both]), np.maximum(o_len, 1e-30))
    # conditioning of the hit distance: a perpendicular position error e moves
    # the hit by e / |cos| along a ray at angle acos|cos| to the surface normal,
    # so near-tangent hits (on spheres) are checked with rel * |cos|
    d = rays[both, 4:7].astype(np.float64)
    cosg = np.abs(np.sum(d * nrm_o[both], axis=1)) / np.linalg.norm(d, axis=1)
    rel_c = rel * np.minimum(1.0, np.maximum(cosg, 1e-6))
    near_tie = rel_c <= REL
    bad_prim = ~same & ~near_tie
    # the plain rule (|dt| / t <= 1e-5, no conditioning), reported beside the
    # conditioned one that is asserted
    rel_plain = np.abs(hits["t"][both] - t_o[both]) / np.maximum(np.abs(t_o[both]), 1e-30)
    plain_bad_prim = ~same & ~(rel_plain <= REL)
    return dict(n=len(rays), hit_disagree=int((g_hit != o_hit).sum()), bad_prim=int(bad_prim.sum()),
                rel_bad=int((rel_c[same] > REL).sum()), rel_median=float(np.median(rel)) if rel.size else 0.0,
                rel_max_conditioned=float(rel_c[same].max()) if same.any() else 0.0, hits=int(both.sum()),
                plain_rel_bad=int((rel_plain[same] > REL).sum()), plain_bad_prim=int(plain_bad_prim.sum()))


SCENES = {
    "cornell_baseline": lambda s: s.cornell_baseline(64),
    "cornell_spheres": lambda s: s.cornell_scene(s.CORNELL_SPHERES),
    "default_scene": lambda s: s.default_scene(),
    "icosphere6": lambda s: s.icosphere_scene(level=6, width=64),
    "spheres17": lambda s: s.default_style_scene(17, 64, 64),
    "quadrics": lambda s: s.quadric_scene(64),
    "cone_test": lambda s: s.cone_test_scene(_cam(64)),
    "cylinder_test": lambda s: s.cylinder_test_scene(_cam(64)),
}


def _cam(w):
    from gprt.scene import CameraConfig
    return CameraConfig(width=w)


@pytest.mark.parametrize("name", sorted(SCENES))
def test_closest_hit_parity(ctx, oracle, name):
    from gprt import scenes
    scene = SCENES[name](scenes)
    o = oracle.OracleScene(scene.to_desc())
    rays = np.concatenate([_camera_rays(scene, 20000, 1), _rays_in_bounds(o.world_center, min(o.world_radius, 600.0),
                                                                          20000, 2)])
    r = _compare(ctx, oracle, scene, rays)
    print(name, r)
    assert r["hits"] > 1000
    assert r["hit_disagree"] <= max(2, 1e-4 * r["n"]), r
    assert r["bad_prim"] <= max(2, 1e-4 * r["n"]), r
    assert r["rel_bad"] <= max(2, 1e-4 * r["n"]), r
    assert r["rel_median"] < 1e-6, r


def test_icosphere_raw_batch_parity(ctx, oracle):
    """The raw-batch ray mix (coherent primaries + incoherent surface rays) on
    a level-7 icosphere (327,680 triangles)."""
    from gprt import scenes
    scene = scenes.icosphere_scene(level=7, width=256)
    mesh = scene.shapes[0].mesh
    rays = scenes.ray_batch(mesh.vertices, mesh.faces, 1 << 16, seed=13, width=256)
    r = _compare(ctx, oracle, scene, rays)
    print("icosphere7 raw batch", r)
    assert r["hits"] > 30000
    assert r["hit_disagree"] <= max(3, 1e-4 * r["n"]), r
    assert r["bad_prim"] <= max(3, 1e-4 * r["n"]), r
    assert r["rel_bad"] <= max(3, 1e-4 * r["n"]), r


def test_any_hit_matches_closest_hit_existence(ctx, oracle):
    from gprt import scenes
    scene = scenes.cornell_baseline(64)
    rays = _camera_rays(scene, 5000, 3)
    rays[:, 7] = 500.0  # bounded shadow-style interval
    g_hit, o_hit = _compare(ctx, oracle, scene, rays, any_hit=True)
    assert (g_hit != o_hit).sum() <= 2


def test_edge_cases(ctx, oracle):
    """Empty batch, rays that miss everything, tmax before the first surface,
    axis-parallel rays and rays starting inside a sphere."""
    import gprt
    from gprt import scenes
    scene = scenes.cornell_scene(scenes.CORNELL_SPHERES)
    g = gprt.GpuScene(ctx, scene.to_desc())
    assert g.intersect(np.zeros((0, 8), dtype=np.float32)).shape == (0,)
    rays = np.array([
        [278, 278, -800, 0.001, 0, 0, -1, np.inf],  # away from the box
        [278, 278, -800, 0.001, 0, 0, 1, 100.0],  # stops before the box
        [278, 278, -800, 0.001, 0, 0, 1, np.inf],  # axis-parallel, hits the back wall
        [370, 90, 351, 0.001, 1, 0, 0, np.inf],  # from inside the glass sphere
        [100, 555.999, 300, 0.001, 0, -1, 0, np.inf],  # straight down onto the floor
    ], dtype=np.float32)
    h = g.intersect(rays)
    o = oracle.OracleScene(scene.to_desc())
    t_o, shape_o, sub_o, _, _ = o.intersect(rays)
    shape_map, _ = g.primitive_map()
    for i in range(len(rays)):
        if shape_o[i] < 0:
            assert h["prim"][i] == gprt.capi.NO_HIT
        else:
            assert shape_map[h["prim"][i]] == shape_o[i]
            assert abs(h["t"][i] - t_o[i]) <= 1e-5 * max(abs(t_o[i]), float(np.linalg.norm(rays[i, :3])))


def test_device_pointer_entry_point(ctx):
    """gprt_intersect with device buffers and the context stream."""
    import ctypes as C

    import gprt
    from gprt import scenes
    scene = scenes.cornell_baseline(32)
    g = gprt.GpuScene(ctx, scene.to_desc())
    rays = _camera_rays(scene, 4096, 5)
    host = g.intersect(rays)
    torch = pytest.importorskip("torch")
    d_rays = torch.from_numpy(rays).cuda()
    d_hits = torch.zeros((len(rays), 4), dtype=torch.float32, device="cuda")
    stream = torch.cuda.Stream()  # an explicit stream (NULL would select the context stream)
    stream.wait_stream(torch.cuda.current_stream())
    ctx.check(gprt.capi.load().gprt_intersect(g.h, C.c_void_p(d_rays.data_ptr()), len(rays), gprt.capi.CLOSEST,
                                              C.c_void_p(d_hits.data_ptr()), C.c_void_p(stream.cuda_stream)))
    stream.synchronize()
    out = d_hits.cpu().numpy().view(host.dtype).reshape(-1)
    assert np.array_equal(out, host)
