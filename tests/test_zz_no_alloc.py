"""The allocation-free entry point, gprt_render_noalloc.

Some callers of this library cannot allocate device memory when they render:
a plugin inside a host application whose own allocator owns the GPU's memory
(a cudaMalloc behind its back can fail, or fragment what it manages), and
render loops whose device-memory budget is fixed when they start.  The entry
point keeps its path state in a statically sized device array inside the
library instead.  These tests call it through the C ABI and check that two
calls in a row -- the second one reading an array that still holds the first
call's contents -- each give what the job API gives for the same samples, on a
closed scene and on one lit by an infinite light (whose shading reads a
hit-first slot order that also lives in the array); that the device status it
writes is 0 for those renders and non-zero, with a NaN image, when a path
exceeds a device bound; and that requests beyond the array's size are refused.
The file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _job_image(g, spp, seed):
    import gprt
    job = gprt.ProgressiveRaytracer(g, gprt.ProgressiveConfig(max_samples_per_pixel=spp, max_passes=1, seed=seed))
    job.add_samples(spp)
    want = job.image().reshape(-1, 3)
    job.close()
    return want


def _noalloc(lib, ctx, g, spp, seed, stream, torch):
    npix = g.width * g.height
    out = torch.full((npix, 3), float("nan"), dtype=torch.float32, device="cuda")
    status = torch.full((1,), 0xABCD, dtype=torch.int32, device="cuda")
    stream.wait_stream(torch.cuda.current_stream())  # the fills run on torch's stream
    ctx.check(lib.gprt_render_noalloc(g.h, spp, seed, C.c_void_p(out.data_ptr()), C.c_void_p(status.data_ptr()),
                                      C.c_void_p(stream.cuda_stream)))
    stream.synchronize()
    return out.cpu().numpy(), int(status.cpu().item())


@pytest.mark.parametrize("name", ["cornell", "icosphere_sky"])
def test_noalloc_matches_job_api_on_two_calls(ctx, name):
    torch = pytest.importorskip("torch")
    import gprt
    from gprt import scenes

    lib = gprt.capi.load()
    scene = {"cornell": lambda: scenes.cornell_baseline(48),
             "icosphere_sky": lambda: scenes.icosphere_scene(level=4, width=40)}[name]()
    g = gprt.GpuScene(ctx, scene.to_desc())
    spp, seed = 16, 21
    assert g.width * g.height * spp <= gprt.capi.NOALLOC_MAX_PATHS
    want = _job_image(g, spp, seed)  # the existing entry points: a fresh job taking the same samples
    stream = torch.cuda.Stream()  # an explicit stream: NULL would select the library's context stream
    for call in range(2):
        got, status = _noalloc(lib, ctx, g, spp, seed, stream, torch)
        assert status == 0, (call, status)
        assert np.isfinite(got).all(), call
        # same samples, same summation order: identical up to the tolerance of the other render tests
        assert np.allclose(got, want, rtol=1e-6, atol=1e-7), (call, float(np.abs(got - want).max()))
    g.close()


def test_noalloc_reports_device_bounds(ctx):
    """A scene built with a 1-entry traversal stack (tests only) makes rays
    overflow it: the call writes the error bits to the status word and NaN to
    the image; a normal scene's next call is clean again (every call clears
    the error word it keeps in the shared array)."""
    torch = pytest.importorskip("torch")
    import gprt
    from gprt import scenes

    lib = gprt.capi.load()
    capped = gprt.GpuScene(ctx, scenes.icosphere_scene(level=4, width=40).to_desc(), test_stack_cap=True)
    stream = torch.cuda.Stream()
    got, status = _noalloc(lib, ctx, capped, 4, 3, stream, torch)
    assert status == 1, status  # bit 0: traversal stack
    assert np.isnan(got).all()
    capped.close()
    g = gprt.GpuScene(ctx, scenes.cornell_baseline(32).to_desc())
    got, status = _noalloc(lib, ctx, g, 4, 3, stream, torch)
    assert status == 0 and np.isfinite(got).all()
    assert np.allclose(got, _job_image(g, 4, 3), rtol=1e-6, atol=1e-7)
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
    rc = lib.gprt_render_noalloc(g.h, spp, 1, C.c_void_p(out.data_ptr()), None, None)
    assert rc == gprt.capi.GPRT_E_INVALID
    assert b"exceeds" in lib.gprt_last_error(ctx.h)
    g.close()
