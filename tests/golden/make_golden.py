"""Generates the converged reference images the GPU image-parity tests use.

Each fixture is the oracle's (float64 restatement of the reference) render of
a small scene at 4096 samples per pixel with its own per-tile PCG streams,
plus four independent 64-spp oracle renders for the noise floor of the
parity rule.  Run from the repository root:

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


def fixtures():
    from gprt import scenes
    return {
        # name: (scene factory, integrator 0=PT 1=BDPT, reference spp)
        "cornell_pt": (lambda: scenes.cornell_baseline(width=48), 0, 4096),
        "cornell_spheres_pt": (lambda: _fixed(scenes.cornell_scene(scenes.CORNELL_SPHERES, camera=_cam(48))), 0, 4096),
        "cornell_boxes_bdpt": (lambda: scenes.cornell_boxes_bdpt(width=40, max_depth=8), 1, 4096),
        "spheres_pt": (lambda: scenes.default_style_scene(17, 48, 48), 0, 4096),
    }


def _cam(w):
    from gprt.scene import CameraConfig
    return CameraConfig(width=w)


def _fixed(s):
    s.sampling.adaptive_min_samples = 1.0
    s.sampling.adaptive_threshold = 0.0
    s.sampling.max_depth = 8
    return s


def make(name, threads=None):
    from oracle import client
    spec = importlib_build()
    spec.build()
    factory, integ, spp = fixtures()[name]
    flat = factory().to_desc()
    threads = threads or os.cpu_count()
    t0 = time.time()
    ref = client.render(flat, integ, spp=spp, seed=4242, threads=threads)
    noise = np.stack([client.render(flat, integ, spp=64, seed=101 + k, threads=threads) for k in range(4)])
    np.savez_compressed(os.path.join(HERE, name + ".npz"), ref=ref.astype(np.float32), noise=noise.astype(np.float32),
                        spp=spp, integrator=integ)
    print("%s: %.1fs, mean %s" % (name, time.time() - t0, ref.mean(axis=(0, 1))))


def importlib_build():
    import importlib.util
    spec = importlib.util.spec_from_file_location("oracle_build", os.path.join(ROOT, "oracle", "build.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


if __name__ == "__main__":
    names = sys.argv[1:] or sorted(fixtures())
    for n in names:
        make(n)
