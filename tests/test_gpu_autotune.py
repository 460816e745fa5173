"""The autotuner (gprt_autotune) and the kernel variants it chooses between.

Every variant computes the same paths (same sampler, same traversal order,
same per-pixel accumulation order), so any configuration must render the
film bit-identically; the tuner only changes speed."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _film(ctx, g, cfg, spp):
    import gprt
    r = gprt.ProgressiveRaytracer(g, cfg)
    r.add_samples(spp)
    f = r.film()
    r.close()
    return f


def test_variants_render_identically(ctx):
    import gprt
    from gprt import capi, scenes
    for desc in (scenes.icosphere_scene(level=5, width=64).to_desc(),
                 scenes.default_style_scene(3, width=48, height=32).to_desc()):
        _variants_agree(ctx, desc)


def _variants_agree(ctx, desc):
    import gprt
    from gprt import capi
    g = gprt.GpuScene(ctx, desc)
    base = _film(ctx, g, gprt.ProgressiveConfig(max_samples_per_pixel=8, max_passes=1, seed=3), 8)
    for flags, block, chunk in [(capi.JOB_SIMPLE_EXTEND, 64, 0), (capi.JOB_SIMPLE_SHADOW, 256, 5000),
                                (capi.JOB_SIMPLE_EXTEND | capi.JOB_SIMPLE_SHADOW, 128, 20000), (0, 128, 3000),
                                (capi.JOB_SHADE_OCCUPANCY, 256, 0)]:
        f = _film(ctx, g, gprt.ProgressiveConfig(max_samples_per_pixel=8, max_passes=1, seed=3, flags=flags,
                                                  block_size=block, chunk_paths=chunk), 8)
        for a, b in zip(base, f):
            assert np.array_equal(a, b), (flags, block, chunk)
    g.close()


def test_autotune_returns_a_valid_faster_or_equal_config(ctx):
    import gprt
    from gprt import scenes
    g = gprt.GpuScene(ctx, scenes.cornell_baseline(128).to_desc())
    cfg, info = gprt.renderer.autotune(g, spp=4, config=gprt.ProgressiveConfig(max_samples_per_pixel=4, seed=2))
    assert info["candidates"] >= 5
    assert 0 < info["best_ms"] <= info["default_ms"]
    assert cfg.block_size in (64, 128, 256) and cfg.chunk_paths > 0
    a = _film(ctx, g, gprt.ProgressiveConfig(max_samples_per_pixel=4, max_passes=1, seed=2), 4)
    b = _film(ctx, g, gprt.ProgressiveConfig(max_samples_per_pixel=4, max_passes=1, seed=2, flags=cfg.flags,
                                             block_size=cfg.block_size, chunk_paths=cfg.chunk_paths), 4)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    g.close()
