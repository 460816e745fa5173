"""Image parity of the GPU path tracer and BDPT against the oracle.

Two comparisons:
* same inputs: the oracle draws from the GPU's counter-based sample stream
  (same seed, pixel, sample index), so both render the same paths; per-pixel
  means agree up to FP32-vs-FP64 rounding, except the few paths where a
  rounding difference flips a discrete decision (an edge hit, a Fresnel
  draw).  Tolerance: median relative pixel error <= 1e-6, and at most 0.5 %
  of pixels (BDPT 1 %) off by more than 1e-2 relative (+1e-4 absolute).  On
  GB300 the medians measure 3e-8 - 3.5e-7 and the off-pixel shares at most
  0.22 % (path tracing, cone_test) and 0.54 % (BDPT, cone_test).
* statistics: against the committed 4096-spp oracle reference
  (tests/golden), relative RMSE(gpu_N) <= 1.10 x RMSE(oracle_N), both
  averaged over 4 seeds and taken on the displayed range (radiance clamped
  to [0, 1], as the RGBA8 output is; unclamped caustic fireflies make single
  RMSE estimates swing by +-25 %), and the unclamped mean luminance bias is
  below 3 standard errors.
"""
import os

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def gpu_render(ctx, scene, spp, seed=7, integrator=None, **cfg):
    import gprt
    g = gprt.GpuScene(ctx, scene.to_desc())
    conf = gprt.ProgressiveConfig(max_samples_per_pixel=spp, max_passes=1, seed=seed, **cfg)
    r = gprt.ProgressiveRaytracer(g, conf, integrator or gprt.PathTracingIntegrator())
    img, stats = r.render_pass(1)
    out = r.image()
    film = r.film()
    r.close()
    g.close()
    return out, stats, film


def oracle_render(oracle, scene, spp, seed=7, integrator=0, counter=True, passes=1, initial=1):
    s = oracle.OracleScene(scene.to_desc())
    r = oracle.OracleRenderer(s, integrator, max_spp=spp, max_passes=passes, initial=initial, seed=seed,
                              counter_stream=counter, threads=8)
    for p in range(1, passes + 1):
        r.render_pass(p)
    return r, s


def same_input_stats(gpu, ref):
    d = np.abs(gpu.astype(np.float64) - ref)
    rel = d / (np.abs(ref) + 1e-4)
    return float(np.median(rel)), float((rel > 1e-2).any(axis=-1).mean())


SCENES = {
    "cornell_baseline": lambda s: s.cornell_baseline(48),
    "cornell_spheres": lambda s: _fixed(s.cornell_scene(s.CORNELL_SPHERES, camera=_cam(48))),
    "default_scene": lambda s: _fixed(s.default_scene(camera=_cam(64)), depth=8),
    "icosphere5": lambda s: s.icosphere_scene(level=5, width=48),
    "spheres17": lambda s: s.default_style_scene(17, 48, 48),
    "quadrics": lambda s: s.quadric_scene(48),
    "quadrics_disc_light": lambda s: s.quadric_scene(48, disc_light=True),
    "spot_disc": lambda s: s.spot_scene(40),
    "spot_point": lambda s: s.spot_scene(40, point=True),
    "cornell_point": lambda s: _fixed(s.cornell_scene(s.CORNELL_BOXES, s.CORNELL_POINT_LIGHT, camera=_cam(48)), depth=8),
    "cone_test": lambda s: _untied(_fixed(s.cone_test_scene(_cam(64)), depth=8)),
    "cylinder_test": lambda s: _fixed(s.cylinder_test_scene(_cam(64)), depth=8),
    "spheregrid_mixed": lambda s: _fixed(s.sphere_grid_scene(6, "mixed", _cam(64)), depth=8),
    "spheregrid_glossy": lambda s: _fixed(s.sphere_grid_scene(6, "glossy", _cam(64)), depth=8),
    "texture_test": lambda s: _fixed(s.texture_test_scene(_cam(96)), depth=8),
    "textured_mesh": lambda s: s.textured_mesh_scene(48),
}


def _cam(w):
    from gprt.scene import CameraConfig
    return CameraConfig(width=w)


def _untied(s):
    """The cone test scene with its touching caps lifted by 1e-3: the glass
    cone's base cap lies on the blue frustum's top cap and another glass
    cone's base cap on the ground, so rays meet two surfaces at the same t.
    Such a tie goes to whichever primitive the traversal visits last, and
    two different trees visit in different orders (hit parity allows exact
    ties); same-input image parity needs a scene without them."""
    for k in (4, 6):  # coneGlass, glassConeTouching (cone_scene.go:102-139)
        p = list(s.shapes[k].p)
        p[1] += 1e-3
        s.shapes[k].p = tuple(p)
    return s


def _point_lowered(s):
    """The Cornell point-light scene with the light 1 unit (not 0.001) below
    the ceiling.  At 0.001 the float32 position (555.99902) moves the light
    2.3 % closer to the ceiling, and the ceiling spot it lights (irradiance
    ~ 1/gap^2), which BDPT's light tracing finds, lights most of the room;
    same-input image parity at 1e-2 needs a light whose float32 position
    is well conditioned."""
    s.lights[0].from_ = (278.0, 555.0, 279.5)
    return s


def _fixed(s, depth=None):
    s.sampling.adaptive_min_samples = 1.0
    s.sampling.adaptive_threshold = 0.0
    if depth:
        s.sampling.max_depth = depth
    return s


@pytest.mark.parametrize("name", sorted(SCENES))
def test_pt_same_inputs_parity(ctx, oracle, name):
    from gprt import scenes
    scene = SCENES[name](scenes)
    gpu, stats, _ = gpu_render(ctx, scene, 16, seed=11)
    r, _ = oracle_render(oracle, scene, 16, seed=11)
    med, frac = same_input_stats(gpu, r.image())
    print(name, "median rel", med, "frac > 1e-2", frac)
    assert stats.min_samples == 16 and stats.total_samples == 16 * stats.total_pixels
    assert med <= 1e-6, (med, frac)
    assert frac <= 0.005, (med, frac)


@pytest.mark.parametrize("name", ["cornell_boxes", "cornell_spheres", "default_scene", "quadrics",
                                  "quadrics_disc_light", "spot_disc", "spot_point", "cornell_point", "cone_test",
                                  "spheregrid_mixed", "texture_test", "textured_mesh"])
def test_bdpt_same_inputs_parity(ctx, oracle, name):
    import gprt
    from gprt import scenes
    scene = {"cornell_boxes": lambda: scenes.cornell_boxes_bdpt(width=32, max_depth=6),
             "cornell_spheres": lambda: _fixed(scenes.cornell_scene(scenes.CORNELL_SPHERES, camera=_cam(32)), 6),
             "default_scene": lambda: _fixed(scenes.default_scene(camera=_cam(48)), depth=6),
             "quadrics": lambda: scenes.quadric_scene(32, max_depth=6),
             "quadrics_disc_light": lambda: scenes.quadric_scene(32, max_depth=6, disc_light=True),
             "spot_disc": lambda: scenes.spot_scene(32, max_depth=6),
             "spot_point": lambda: scenes.spot_scene(32, point=True, max_depth=6),
             "cornell_point": lambda: _point_lowered(_fixed(scenes.cornell_scene(
                 scenes.CORNELL_BOXES, scenes.CORNELL_POINT_LIGHT, camera=_cam(32)), 6)),
             "cone_test": lambda: _untied(_fixed(scenes.cone_test_scene(_cam(48)), 6)),
             "spheregrid_mixed": lambda: _fixed(scenes.sphere_grid_scene(5, "mixed", _cam(48)), 6),
             "texture_test": lambda: _fixed(scenes.texture_test_scene(_cam(64)), 6),
             "textured_mesh": lambda: scenes.textured_mesh_scene(32, max_depth=6)}[name]()
    gpu, stats, _ = gpu_render(ctx, scene, 8, seed=5, integrator=gprt.BDPTIntegrator())
    r, _ = oracle_render(oracle, scene, 8, seed=5, integrator=1)
    med, frac = same_input_stats(gpu, r.image())
    print(name, "bdpt median rel", med, "frac > 1e-2", frac)
    assert med <= 1e-6, (med, frac)
    assert frac <= 0.01, (med, frac)


def _rel_rmse(img, ref):
    img, ref = np.clip(img, 0.0, 1.0), np.clip(ref, 0.0, 1.0)
    return float(np.sqrt(np.mean((img - ref) ** 2)) / np.mean(ref))


@pytest.mark.parametrize("name", ["cornell_pt", "cornell_spheres_pt", "spheres_pt", "cornell_boxes_bdpt"])
def test_statistical_parity_against_converged_reference(ctx, name):
    import gprt
    from gprt import scenes
    g = np.load(os.path.join(ROOT, "tests", "golden", name + ".npz"))
    ref = g["ref"].astype(np.float64)
    factory = {"cornell_pt": lambda: scenes.cornell_baseline(width=48),
               "cornell_spheres_pt": lambda: _fixed(scenes.cornell_scene(scenes.CORNELL_SPHERES, camera=_cam(48)), 8),
               "cornell_boxes_bdpt": lambda: scenes.cornell_boxes_bdpt(width=40, max_depth=8),
               "spheres_pt": lambda: scenes.default_style_scene(17, 48, 48)}[name]
    integ = gprt.BDPTIntegrator() if int(g["integrator"]) == 1 else None
    noise = g["noise"].astype(np.float64)
    floor = float(np.mean([_rel_rmse(x, ref) for x in noise]))
    imgs = [gpu_render(ctx, factory(), 64, seed=seed, integrator=integ)[0].astype(np.float64) for seed in (1, 2, 3, 4)]
    errs = [_rel_rmse(x, ref) for x in imgs]
    print(name, "gpu rel rmse", errs, "oracle noise floor", floor)
    assert np.mean(errs) <= 1.10 * floor, (errs, floor)
    # mean bias: |mean(gpu) - mean(ref)| < 3 standard errors of the 4 x 64-spp mean
    lum = lambda im: 0.2126 * im[..., 0] + 0.7152 * im[..., 1] + 0.0722 * im[..., 2]
    se = np.std([lum(x).mean() for x in noise], ddof=1) / 2.0
    bias = np.mean([lum(x).mean() for x in imgs]) - lum(ref).mean()
    print(name, "bias", bias, "se", se)
    assert abs(bias) < 3 * se + 1e-6, (bias, se)


def test_pt_deterministic_and_chunk_invariant(ctx):
    from gprt import scenes
    scene = scenes.cornell_baseline(40)
    a, _, fa = gpu_render(ctx, scene, 12, seed=3)
    b, _, fb = gpu_render(ctx, scene, 12, seed=3)
    c, _, fc = gpu_render(ctx, scene, 12, seed=3, chunk_paths=1000)  # split pixels and layers differently
    assert np.array_equal(fa[0], fb[0]) and np.array_equal(fa[0], fc[0])
    assert np.array_equal(fa[2], fc[2]) and np.array_equal(fa[3], fc[3])
    d, _, _ = gpu_render(ctx, scene, 12, seed=4)
    assert not np.array_equal(a, d)


def test_progressive_passes_schedule(ctx):
    import gprt
    from gprt import scenes
    g = gprt.GpuScene(ctx, scenes.cornell_baseline(32).to_desc())
    r = gprt.ProgressiveRaytracer(g, gprt.ProgressiveConfig(max_samples_per_pixel=50, max_passes=7, seed=1))
    events = list(r.render_progressive(tile_updates=True))
    passes = [e for e in events if isinstance(e, gprt.PassResult)]
    tiles = [e for e in events if isinstance(e, gprt.TileCompletionResult)]
    # getSamplesForPass (progressive.go:98-123): 1, 9, 17, 25, 33, 41, 50
    assert [p.stats.max_samples for p in passes] == [1, 9, 17, 25, 33, 41, 50]
    assert [p.stats.max_samples_used for p in passes] == [1, 9, 17, 25, 33, 41, 50]
    assert passes[-1].is_last and not passes[0].is_last
    assert len(tiles) == 7 and tiles[0].total_tiles == 1
    assert passes[-1].image.shape == (32, 32, 4) and (passes[-1].image[..., 3] == 255).all()


def test_adaptive_sampling_matches_oracle_counts(ctx, oracle):
    """Adaptive stop (tile_renderer.go:77-101) with the reference Cornell
    sampling config (20 % minimum, 0.5 % threshold).  The stop compares a
    float32 (GPU) or float64 (oracle) relative error with the threshold, so a
    pixel right at it may stop one sample apart; on GB300 every count
    matched."""
    import gprt
    from gprt import scenes
    scene = scenes.cornell_scene(scenes.CORNELL_SPHERES, camera=_cam(32))
    g = gprt.GpuScene(ctx, scene.to_desc())
    r = gprt.ProgressiveRaytracer(g, gprt.ProgressiveConfig(max_samples_per_pixel=40, max_passes=3, seed=9))
    for p in (1, 2, 3):
        _, st = r.render_pass(p)
    _, _, _, cnt = r.film()
    orr, _ = oracle_render(oracle, scene, 40, seed=9, passes=3)
    _, _, _, ocnt = orr.film()
    assert st.max_samples_used <= 40 and st.min_samples >= 8
    assert (cnt >= 8).all() and (cnt <= 40).all()
    assert np.mean(cnt == ocnt) >= 0.99, np.mean(cnt == ocnt)


def test_rgba8_and_tiles_follow_vec3_to_color(ctx):
    import gprt
    from gprt import scenes
    g = gprt.GpuScene(ctx, scenes.cornell_baseline(48).to_desc())
    r = gprt.ProgressiveRaytracer(g, gprt.ProgressiveConfig(max_samples_per_pixel=4, max_passes=1, seed=2))
    r.render_pass(1)
    img = r.image().astype(np.float64)
    rgba = r.rgba8()
    want = (255 * np.clip(np.sqrt(img), 0, 1)).astype(np.uint8)
    assert np.abs(rgba[..., :3].astype(int) - want.astype(int)).max() <= 1
    assert (rgba[..., 3] == 255).all()
    assert np.array_equal(r.tile(16, 8, 40, 32), rgba[8:32, 16:40])


def test_errors_are_reported_not_raised_in_c(ctx):
    import gprt
    from gprt import scenes
    s = scenes.cornell_boxes_bdpt(width=16, max_depth=40)
    g = gprt.GpuScene(ctx, s.to_desc())
    with pytest.raises(gprt.capi.GprtError) as e:
        gprt.ProgressiveRaytracer(g, gprt.ProgressiveConfig(max_samples_per_pixel=1, max_passes=1),
                                  gprt.BDPTIntegrator())
    assert e.value.code == gprt.capi.GPRT_E_INVALID
    with pytest.raises(gprt.capi.GprtError):
        gprt.ProgressiveRaytracer(g, gprt.ProgressiveConfig(max_samples_per_pixel=1, max_passes=1, block_size=100))
