"""The allocation-free entry point, gprt_render_noalloc.

It serves callers that cannot allocate device memory at render time (code
recording a CUDA graph, render loops with a device-memory budget fixed at
start-up, hosts sharing the GPU with an allocator they do not own).  It keeps
its path state in a statically sized device array inside the library, so this
test checks that two calls in a row -- the second one reading an array that
still holds the first call's contents -- each give what the job API gives for
the same samples, and that requests beyond the array's size are refused.
The file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_matches_job_api_on_two_calls(ctx):
    torch = pytest.importorskip("torch")
    import gprt
    from gprt import scenes

    lib = gprt.capi.load()
    g = gprt.GpuScene(ctx, scenes.cornell_baseline(48).to_desc())
    spp, seed = 16, 21
    npix = g.width * g.height
    assert npix * spp <= gprt.capi.NOALLOC_MAX_PATHS
    # the existing entry points: a fresh job taking the same samples
    job = gprt.ProgressiveRaytracer(g, gprt.ProgressiveConfig(max_samples_per_pixel=spp, max_passes=1, seed=seed))
    job.add_samples(spp)
    want = job.image().reshape(-1, 3)
    job.close()
    stream = torch.cuda.Stream()  # an explicit stream: NULL would select the library's context stream
    for call in range(2):
        out = torch.full((npix, 3), float("nan"), dtype=torch.float32, device="cuda")
        stream.wait_stream(torch.cuda.current_stream())  # the NaN fill runs on torch's stream
        ctx.check(lib.gprt_render_noalloc(g.h, spp, seed, C.c_void_p(out.data_ptr()), C.c_void_p(stream.cuda_stream)))
        stream.synchronize()
        got = out.cpu().numpy()
        assert np.isfinite(got).all(), call
        # same samples, same summation order: identical up to the tolerance of the other render tests
        assert np.allclose(got, want, rtol=1e-6, atol=1e-7), (call, float(np.abs(got - want).max()))
    g.close()


def test_noalloc_rejects_requests_beyond_its_scratch(ctx):
    torch = pytest.importorskip("torch")
    import gprt
    from gprt import scenes

    lib = gprt.capi.load()
    g = gprt.GpuScene(ctx, scenes.cornell_baseline(128).to_desc())
    npix = g.width * g.height
    spp = gprt.capi.NOALLOC_MAX_PATHS // npix + 1
    out = torch.zeros((npix, 3), dtype=torch.float32, device="cuda")
    rc = lib.gprt_render_noalloc(g.h, spp, 1, C.c_void_p(out.data_ptr()), None)
    assert rc == gprt.capi.GPRT_E_INVALID
    assert b"exceeds" in lib.gprt_last_error(ctx.h)
    g.close()
