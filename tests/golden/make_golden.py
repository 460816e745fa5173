"""Generates the converged reference images the GPU image-parity tests use.

Two kinds of fixture, both rendered by the oracle (the float64 restatement of
the reference) with its own per-tile PCG streams:

* small scenes (48^2 / 40^2): the whole 4096-spp image plus four independent
  64-spp renders for the noise floor of the parity rule;
* the benchmark configurations at their real resolutions and sample counts
  (Cornell 400^2 64 spp, reference Cornell spheres 400^2 64 spp, icosphere
  L8 1024^2 16 spp, Cornell boxes BDPT 512^2 64 spp): 4096-spp reference
  windows (whole 64x64 tiles of the reference's tile grid: the centre, an
  edge, the top and the ragged bottom-right corner) and, per noise seed, the
  statistics of an oracle render at the configuration's spp against them
  (relative RMSE on clamped and unclamped radiance, window mean luminance,
  and the RMSE between two noise seeds).  Path tracing has no cross-pixel
  terms, so its windows are rendered alone; BDPT's light-tracing splats come
  from every sample of the frame, so its references and noise renders are
  whole frames (4096 spp in passes of 64) of which the windows are kept.

Run from the repository root:

    python tests/golden/make_golden.py            # all fixtures
    python tests/golden/make_golden.py cornell_pt # one fixture
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "go-progressive-raytracer_gb300"))
sys.path.insert(0, ROOT)

TILE = 64
REF_SPP = 4096
REF_SEED = 4242


def fixtures():
    from gprt import scenes
    return {
        # name: (scene factory, integrator 0=PT 1=BDPT, reference spp)
        "cornell_pt": (lambda: scenes.cornell_baseline(width=48), 0, 4096),
        "cornell_spheres_pt": (lambda: _fixed(scenes.cornell_scene(scenes.CORNELL_SPHERES, camera=_cam(48))), 0, 4096),
        "cornell_boxes_bdpt": (lambda: scenes.cornell_boxes_bdpt(width=40, max_depth=8), 1, 4096),
        "spheres_pt": (lambda: scenes.default_style_scene(17, 48, 48), 0, 4096),
    }


def config_fixtures():
    """The benchmark configurations: name -> (scene factory, integrator,
    spp of the configuration, window tiles (tx, ty) in the 64x64 grid,
    noise seeds)."""
    from gprt import scenes
    return {
        "c0a_cornell_400_pt": (lambda: scenes.cornell_baseline(400), 0, 64, [(3, 3), (0, 3), (3, 0), (6, 6)], 16),
        "c0b_cornell_spheres_400_pt": (lambda: _fixed_spp(scenes.cornell_scene(scenes.CORNELL_SPHERES, camera=_cam(400))),
                                       0, 64, [(3, 3), (0, 3), (3, 0), (6, 6)], 16),
        "c1_icosphere_1024_pt": (lambda: scenes.icosphere_scene(level=8, width=1024), 0, 16,
                                 [(8, 8), (0, 8), (8, 14), (11, 5)], 16),
        "c2_cornell_boxes_512_bdpt": (lambda: scenes.cornell_boxes_bdpt(512), 1, 64,
                                      [(4, 4), (0, 4), (4, 0), (7, 7)], 8),
    }


def _cam(w):
    from gprt.scene import CameraConfig
    return CameraConfig(width=w)


def _fixed_spp(s):
    """Every pixel takes every sample (adaptive stopping off)."""
    s.sampling.adaptive_min_samples = 1.0
    s.sampling.adaptive_threshold = 0.0
    return s


def _fixed(s):
    s = _fixed_spp(s)
    s.sampling.max_depth = 8
    return s


def make(name, threads=None):
    from oracle import client
    importlib_build().build()
    factory, integ, spp = fixtures()[name]
    flat = factory().to_desc()
    threads = threads or os.cpu_count()
    t0 = time.time()
    ref = client.render(flat, integ, spp=spp, seed=4242, threads=threads)
    noise = np.stack([client.render(flat, integ, spp=64, seed=101 + k, threads=threads) for k in range(4)])
    np.savez_compressed(os.path.join(HERE, name + ".npz"), ref=ref.astype(np.float32), noise=noise.astype(np.float32),
                        spp=spp, integrator=integ)
    print("%s: %.1fs, mean %s" % (name, time.time() - t0, ref.mean(axis=(0, 1))))


# ---------------------------------------------------------------- config windows

def window_bounds(width, height, tiles):
    """(x0, y0, x1, y1) of each listed tile of the reference's tile grid
    (NewTileGrid, progressive.go:455-479: 64x64 tiles, clipped at the edge)."""
    out = []
    for tx, ty in tiles:
        x0, y0 = tx * TILE, ty * TILE
        assert x0 < width and y0 < height, (tx, ty)
        out.append((x0, y0, min(x0 + TILE, width), min(y0 + TILE, height)))
    return out


def tile_ids(width, tiles):
    nx = (width + TILE - 1) // TILE
    return [ty * nx + tx for tx, ty in tiles]


def cut(img, bounds):
    return [img[y0:y1, x0:x1] for (x0, y0, x1, y1) in bounds]


def luminance(im):
    return 0.2126 * im[..., 0] + 0.7152 * im[..., 1] + 0.0722 * im[..., 2]


def window_stats(wins, refs):
    """Relative RMSE over the pixels of all windows (clamped to [0, 1] as the
    RGBA8 output is, and unclamped) and the mean luminance of each window."""
    a = np.concatenate([w.reshape(-1, 3) for w in wins]).astype(np.float64)
    r = np.concatenate([w.reshape(-1, 3) for w in refs]).astype(np.float64)
    ac, rc = np.clip(a, 0.0, 1.0), np.clip(r, 0.0, 1.0)
    clamped = float(np.sqrt(np.mean((ac - rc) ** 2)) / np.mean(rc))
    unclamped = float(np.sqrt(np.mean((a - r) ** 2)) / np.mean(r))
    lum = [float(luminance(w.astype(np.float64)).mean()) for w in wins]
    return clamped, unclamped, lum


def _oracle_windows(client, flat, integ, spp, seed, bounds, ids, threads, passes_of=None):
    s = client.OracleScene(flat)
    if integ == 0:
        r = client.OracleRenderer(s, 0, max_spp=spp, max_passes=1, seed=seed, threads=threads)
        r.render_tiles(1, ids)
    else:
        # whole frames (every sample's light-tracing splats), in passes of
        # `passes_of` spp to bound the per-pass splat lists
        npass = max(1, spp // passes_of)
        r = client.OracleRenderer(s, 1, max_spp=spp, max_passes=npass, initial=spp // npass, seed=seed,
                                  threads=threads)
        for p in range(1, npass + 1):
            r.render_pass(p)
    img = r.image()
    r.close()
    s.close()
    return cut(img, bounds)


def make_config(name, threads=None):
    from oracle import client
    importlib_build().build()
    factory, integ, spp, tiles, n_noise = config_fixtures()[name]
    scene = factory()
    flat = scene.to_desc()
    threads = threads or os.cpu_count()
    probe = client.OracleScene(flat)
    width, height = probe.width, probe.height
    probe.close()
    bounds = window_bounds(width, height, tiles)
    ids = tile_ids(width, tiles)
    t0 = time.time()
    refs = _oracle_windows(client, flat, integ, REF_SPP, REF_SEED, bounds, ids, threads, passes_of=64)
    t_ref = time.time() - t0
    rm_c, rm_u, lums, noise_wins = [], [], [], []
    for k in range(n_noise):
        wins = _oracle_windows(client, flat, integ, spp, 101 + k, bounds, ids, threads, passes_of=spp)
        c, u, lum = window_stats(wins, refs)
        rm_c.append(c)
        rm_u.append(u)
        lums.append(lum)
        noise_wins.append(wins)
    # the two-seed noise: RMSE between consecutive pairs of noise seeds
    pair_c, pair_u = [], []
    for k in range(0, n_noise - 1, 2):
        c, u, _ = window_stats(noise_wins[k], noise_wins[k + 1])
        pair_c.append(c)
        pair_u.append(u)
    out = {"width": width, "height": height, "spp": spp, "integrator": integ, "ref_spp": REF_SPP,
           "ref_seed": REF_SEED, "bounds": np.array(bounds, dtype=np.int32),
           "noise_rmse": np.array(rm_c), "noise_rmse_unclamped": np.array(rm_u),
           "noise_lum": np.array(lums), "pair_rmse": np.array(pair_c), "pair_rmse_unclamped": np.array(pair_u)}
    for k, w in enumerate(refs):
        out["ref%d" % k] = w.astype(np.float32)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print("%s: %dx%d, ref %.0fs, total %.0fs; noise floor rel RMSE clamped %.4f unclamped %.4f; "
          "two-seed %.4f / %.4f" % (name, width, height, t_ref, time.time() - t0, np.mean(rm_c), np.mean(rm_u),
                                    np.mean(pair_c), np.mean(pair_u)))


def importlib_build():
    import importlib.util
    spec = importlib.util.spec_from_file_location("oracle_build", os.path.join(ROOT, "oracle", "build.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


if __name__ == "__main__":
    names = sys.argv[1:] or sorted(fixtures()) + sorted(config_fixtures())
    for n in names:
        if n in fixtures():
            make(n)
        else:
            make_config(n)
