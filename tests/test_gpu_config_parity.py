"""Image parity at the benchmark configurations themselves.

The GPU renders each configuration's whole frame at its real resolution and
sample count -- Cornell 400^2 64 spp (path tracing, depth 8), the reference
Cornell spheres scene 400^2 64 spp (depth 5), the displaced level-8 icosphere
1024^2 16 spp (1,310,720 triangles, uniform sky) and Cornell boxes 512^2
64 spp under BDPT -- and compares fixed windows of it (whole 64x64 tiles of
the reference's tile grid: centre, edge, top, ragged bottom-right corner)
with the oracle's 4096-spp renders of the same windows
(tests/golden/make_golden.py).

Rule (per configuration, over the pixels of all its windows):
* relative RMSE of the GPU image against the 4096-spp reference, averaged over
  GPU_SEEDS seeds, <= 1.10 x the oracle's own relative RMSE at the same spp
  (its noise floor, averaged over 16 oracle seeds; 8 for BDPT), both on
  radiance clamped to [0, 1] (what the RGBA8 output shows) and on unclamped
  radiance (so that a bias confined to bright pixels -- the light, caustics,
  highlights -- is seen too);
* mean-luminance bias of the GPU mean image below 3 standard errors, the
  standard error combining the GPU seeds' mean and the reference's own noise.
The measured values are printed (run with -s) next to the two-seed noise.
"""
import os
import sys

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
import make_golden as mg  # noqa: E402  (the fixture recipe: scene factories, windows, statistics)

GPU_SEEDS = int(os.environ.get("GPRT_PARITY_SEEDS", "16"))


def _luminance_mean(wins):
    lum = np.concatenate([mg.luminance(w.astype(np.float64)).ravel() for w in wins])
    return float(lum.mean())


@pytest.mark.parametrize("name", sorted(mg.config_fixtures()))
def test_config_windows_match_converged_reference(ctx, name):
    import gprt
    factory, integ, spp, tiles, _ = mg.config_fixtures()[name]
    g = np.load(os.path.join(ROOT, "tests", "golden", name + ".npz"))
    bounds = [tuple(b) for b in g["bounds"]]
    refs = [g["ref%d" % k].astype(np.float64) for k in range(len(bounds))]
    assert int(g["spp"]) == spp and int(g["integrator"]) == integ
    gs = gprt.GpuScene(ctx, factory().to_desc())
    assert (gs.width, gs.height) == (int(g["width"]), int(g["height"]))
    errs_c, errs_u, lums, mean_img = [], [], [], None
    for seed in range(1, GPU_SEEDS + 1):
        conf = gprt.ProgressiveConfig(max_samples_per_pixel=spp, max_passes=1, seed=seed)
        r = gprt.ProgressiveRaytracer(gs, conf, gprt.BDPTIntegrator()) if integ else gprt.ProgressiveRaytracer(gs, conf)
        _, stats = r.render_pass(1)
        assert stats.min_samples == spp and stats.total_samples == spp * gs.width * gs.height
        wins = mg.cut(r.image().astype(np.float64), bounds)
        r.close()
        c, u, _ = mg.window_stats(wins, refs)
        errs_c.append(c)
        errs_u.append(u)
        lums.append(_luminance_mean(wins))
        mean_img = wins if mean_img is None else [a + b for a, b in zip(mean_img, wins)]
    gs.close()
    floor_c, floor_u = float(np.mean(g["noise_rmse"])), float(np.mean(g["noise_rmse_unclamped"]))
    gpu_c, gpu_u = float(np.mean(errs_c)), float(np.mean(errs_u))
    # luminance bias: GPU mean over the seeds vs the reference; the oracle
    # noise seeds give the spread of one render's window-mean luminance
    npx = np.array([(b[2] - b[0]) * (b[3] - b[1]) for b in bounds], dtype=np.float64)
    noise_lum = (g["noise_lum"] * npx).sum(axis=1) / npx.sum()  # pixel-weighted over the windows
    sigma = float(np.std(noise_lum, ddof=1))
    se = sigma * np.sqrt(1.0 / GPU_SEEDS + spp / float(g["ref_spp"]))
    bias = float(np.mean(lums)) - _luminance_mean(refs)
    print("%s: rel RMSE clamped gpu %.4f vs floor %.4f (ratio %.3f); unclamped gpu %.4f vs floor %.4f (ratio %.3f); "
          "two-seed noise %.4f / %.4f; bias %.3g = %.2f SE"
          % (name, gpu_c, floor_c, gpu_c / floor_c, gpu_u, floor_u, gpu_u / floor_u, float(np.mean(g["pair_rmse"])),
             float(np.mean(g["pair_rmse_unclamped"])), bias, abs(bias) / se))
    for k, b in enumerate(bounds):  # per window: GPU mean, oracle noise mean, reference
        wl = float(mg.luminance(mean_img[k] / GPU_SEEDS).mean())
        rl = float(mg.luminance(refs[k]).mean())
        sk = float(np.std(g["noise_lum"][:, k], ddof=1))
        sek = sk * np.sqrt(1.0 / GPU_SEEDS + spp / float(g["ref_spp"]))
        print("  window %s: gpu %.5f oracle(%d seeds) %.5f ref %.5f; gpu-ref %.2f SE, oracle-ref %.2f SE"
              % (b, wl, len(g["noise_lum"]), float(g["noise_lum"][:, k].mean()), rl, (wl - rl) / sek,
                 (float(g["noise_lum"][:, k].mean()) - rl) / (sk * np.sqrt(1.0 / len(g["noise_lum"]) + spp / 4096.0))))
    assert gpu_c <= 1.10 * floor_c, (gpu_c, floor_c, errs_c)
    assert gpu_u <= 1.10 * floor_u, (gpu_u, floor_u, errs_u)
    assert abs(bias) < 3.0 * se, (bias, se)
