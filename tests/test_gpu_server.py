"""The batched render server (gprt_server_*).

A job's film must be the same, bit for bit, whether it runs alone through the
plain per-job path (gprt_job_add_samples), alone in the server, or in the
server beside other scenes and resolutions: every sample is keyed by (seed,
pixel, sample index) and each pixel adds its samples in order.  The
tolerance is therefore exact equality."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _plain_film(g, seed, spp):
    import gprt
    r = gprt.ProgressiveRaytracer(g, gprt.ProgressiveConfig(max_samples_per_pixel=spp, max_passes=1, seed=seed))
    r.add_samples(spp)
    f = r.film()
    r.close()
    return f


def _cfg(spp, per_pass, seed):
    import gprt
    passes = max(1, spp // per_pass)
    return gprt.ProgressiveConfig(initial_samples=per_pass, max_samples_per_pixel=spp, max_passes=passes, seed=seed)


def _same(a, b):
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


@pytest.fixture(scope="module")
def scenes(ctx):
    import gprt
    from gprt import scenes as S
    out = {
        "cornell": gprt.GpuScene(ctx, S.cornell_baseline(48).to_desc()),
        "ico": gprt.GpuScene(ctx, S.icosphere_scene(level=4, width=40).to_desc()),
        "spheres_a": gprt.GpuScene(ctx, S.default_style_scene(5, width=64, height=48).to_desc()),
        "spheres_b": gprt.GpuScene(ctx, S.default_style_scene(9, width=32, height=32).to_desc()),
        "textured": gprt.GpuScene(ctx, S.texture_test_scene(gprt.CameraConfig(width=48)).to_desc()),
        "spot": gprt.GpuScene(ctx, S.spot_scene(32).to_desc()),
        "uvmesh": gprt.GpuScene(ctx, S.textured_mesh_scene(40).to_desc()),
    }
    yield out
    for g in out.values():
        g.close()


def test_job_alone_in_server_equals_plain_job(ctx, scenes):
    import gprt
    g = scenes["cornell"]
    plain = _plain_film(g, 3, 8)
    sv = gprt.RenderServer(ctx, step_paths=1 << 16)
    t = sv.submit(g, _cfg(8, 4, 3))
    ev = sv.run_until_idle()
    kinds = [e.kind for e in ev if e.ticket == t]
    assert kinds == ["admitted", "pass", "pass", "done"]
    _same(sv.film(t), plain)
    sv.close()


def test_jobs_in_the_mix_equal_their_plain_films(ctx, scenes):
    import gprt
    jobs = [("cornell", 3, 8, 4), ("ico", 5, 6, 2), ("spheres_a", 7, 12, 4), ("spheres_b", 11, 4, 1),
            ("cornell", 13, 4, 4), ("textured", 17, 4, 2), ("spot", 19, 4, 4), ("uvmesh", 23, 4, 2)]
    # the textured scene samples adaptively (AdaptiveMinSamples 0.15): its
    # reference is the per-job progressive render, the others' fixed spp
    plain = [_progressive(scenes[n], _cfg(spp, per, seed))[0] if n == "textured" else _plain_film(scenes[n], seed, spp)
             for n, seed, spp, per in jobs]
    # a small step capacity forces jobs to share steps and to be split across them
    sv = gprt.RenderServer(ctx, step_paths=3 * 64 * 48)
    tickets = [sv.submit(scenes[n], _cfg(spp, per, seed)) for n, seed, spp, per in jobs]
    ev = sv.run_until_idle()
    done = {e.ticket for e in ev if e.kind == "done"}
    assert done == set(tickets)
    for t, p in zip(tickets, plain):
        _same(sv.film(t), p)
    st = sv.stats()
    assert st["resident_scenes"] == 7  # the two cornell requests share one pooled copy
    assert st["samples"] == sum(int(p[3].sum()) for p in plain)
    sv.close()


def test_device_bound_fails_only_its_job(ctx, scenes):
    """A device bound -- a traversal-stack overflow, forced by a scene built
    with a 1-entry stack (GPRT_BUILD_TEST_STACK_CAP) -- fails the render it
    occurs in and nothing else, as the reference scopes errors to the render
    (progressive.go:165-167, worker_pool.go:21-26).  The kernels set the error
    bits and carry on (no trap): the job API returns GPRT_E_BOUND for path
    tracing and BDPT, raw batches mark the overflowed rays, and in the server
    only the capped job gets a `failed` event while the jobs batched in the
    same steps finish with their solo films, bit for bit."""
    import gprt
    from gprt import capi
    from gprt import scenes as S
    capped = gprt.GpuScene(ctx, S.icosphere_scene(level=4, width=40).to_desc(), test_stack_cap=True)
    for integ in (None, gprt.BDPTIntegrator()):
        conf = gprt.ProgressiveConfig(max_samples_per_pixel=2, max_passes=1, seed=1)
        r = gprt.ProgressiveRaytracer(capped, conf, integ) if integ else gprt.ProgressiveRaytracer(capped, conf)
        with pytest.raises(capi.GprtError) as e:
            r.render_pass(1)
        assert e.value.code == capi.GPRT_E_BOUND
        assert b"traversal stack" in ctx.lib.gprt_last_error(ctx.h)
        r.close()
    # raw batch: camera rays through the sphere overflow, the others do not
    v, f = S.icosphere(4)
    rays = S.ray_batch(v, f, 4096, seed=3)
    with pytest.raises(capi.GprtError) as e:
        capped.intersect(rays)
    assert e.value.code == capi.GPRT_E_BOUND
    normal = gprt.GpuScene(ctx, S.icosphere_scene(level=4, width=40).to_desc())
    assert (normal.intersect(rays)["prim"] != capi.BOUND_HIT).all()
    normal.close()
    # the server: the capped job shares its steps with normal jobs
    jobs = [("cornell", 3, 8, 4), ("spheres_a", 7, 8, 4), ("ico", 5, 4, 2)]
    # the textured scene samples adaptively (AdaptiveMinSamples 0.15): its
    # reference is the per-job progressive render, the others' fixed spp
    plain = [_progressive(scenes[n], _cfg(spp, per, seed))[0] if n == "textured" else _plain_film(scenes[n], seed, spp)
             for n, seed, spp, per in jobs]
    sv = gprt.RenderServer(ctx, step_paths=1 << 16)
    bad = sv.submit(capped, _cfg(4, 2, 9))
    tickets = [sv.submit(scenes[n], _cfg(spp, per, seed)) for n, seed, spp, per in jobs]
    ev = sv.run_until_idle()
    mine = [e for e in ev if e.ticket == bad]
    assert [e.kind for e in mine] == ["admitted", "failed"], mine
    assert mine[-1].status == capi.GPRT_E_BOUND
    done = {e.ticket for e in ev if e.kind == "done"}
    assert done == set(tickets)
    assert not [e for e in ev if e.kind == "failed" and e.ticket != bad]
    for t, p in zip(tickets, plain):
        _same(sv.film(t), p)
    sv.close()
    capped.close()


def test_graphs_and_direct_launches_agree(ctx, scenes):
    import gprt
    from gprt import capi
    out = []
    for flags in (0, capi.SERVER_NO_GRAPHS, capi.JOB_SIMPLE_EXTEND | capi.JOB_SIMPLE_SHADOW,
                  capi.JOB_SHADE_OCCUPANCY):
        sv = gprt.RenderServer(ctx, step_paths=1 << 15, flags=flags)
        ts = [sv.submit(scenes["spheres_a"], _cfg(4, 2, 1)), sv.submit(scenes["ico"], _cfg(4, 2, 2))]
        sv.run_until_idle()
        out.append([sv.film(t) for t in ts])
        st = sv.stats()
        assert (st["graph_launches"] > 0) == (not flags & capi.SERVER_NO_GRAPHS)
        sv.close()
    for other in out[1:]:
        for a, b in zip(out[0], other):
            _same(a, b)


def test_pass_events_follow_the_progressive_schedule(ctx, scenes):
    import gprt
    g = scenes["spheres_b"]
    sv = gprt.RenderServer(ctx)
    # getSamplesForPass: initial 1, max 10 over 4 passes -> 1, 4, 7, 10
    t = sv.submit(g, gprt.ProgressiveConfig(initial_samples=1, max_samples_per_pixel=10, max_passes=4, seed=2))
    ev = [e for e in sv.run_until_idle() if e.ticket == t]
    passes = [e for e in ev if e.kind == "pass"]
    assert [e.samples_per_pixel for e in passes] == [1, 4, 7, 10]
    assert [e.pass_number for e in passes] == [1, 2, 3, 4]
    assert all(b.t_ms >= a.t_ms for a, b in zip(passes, passes[1:]))
    assert passes[0].t_ms >= passes[0].submit_ms
    _same(sv.film(t), _plain_film(g, 2, 10))
    img = sv.rgba8(t)
    assert img.shape == (g.height, g.width, 4) and img[..., 3].min() == 255
    sv.close()


def test_server_tiles_are_windows_of_the_image(ctx, scenes):
    """gprt_server_read_tile: each tile equals the same window of the whole
    RGBA8 image (path tracing and BDPT, ragged edge tiles included), and the
    tile events of a pass cover the image in row-major order."""
    import gprt
    sv = gprt.RenderServer(ctx, step_paths=1 << 16)
    pt = sv.submit(scenes["spheres_a"], _cfg(4, 2, 3))
    bd = sv.submit(scenes["cornell"], _cfg(2, 2, 5), integrator=gprt.BDPTIntegrator())
    sv.run_until_idle()
    for t in (pt, bd):
        full = sv.rgba8(t)
        h, w = full.shape[:2]
        assert np.array_equal(sv.tile(t, 5, 3, w, h), full[3:h, 5:w])
        tiles = list(sv.tiles(t, 2, 2, tile_size=20))
        assert [(r.tile_x, r.tile_y) for r in tiles] == [(x, y) for y in range((h + 19) // 20)
                                                         for x in range((w + 19) // 20)]
        for r in tiles:
            x0, y0 = 20 * r.tile_x, 20 * r.tile_y
            assert np.array_equal(r.tile_image, full[y0:y0 + 20, x0:x0 + 20])
        assert tiles[-1].tile_number == tiles[-1].total_tiles == len(tiles)
    with pytest.raises(gprt.capi.GprtError):
        sv.tile(pt, 0, 0, 0, 1)  # empty tile
    sv.close()


def test_admission_by_budget(ctx, scenes):
    import gprt
    g = scenes["spheres_a"]
    film = g.width * g.height * 24  # sum rgb + lum, lum^2, count
    sv0 = gprt.RenderServer(ctx, step_paths=1 << 12)
    sv0.submit(g, _cfg(2, 2, 1))
    sv0.step()
    used = sv0.stats()["bytes_in_use"]  # path state + pooled scene + one film
    sv0.close()
    budget = used + film // 2  # room for one film, not two
    sv = gprt.RenderServer(ctx, hbm_budget_bytes=budget, step_paths=1 << 12)
    big = sv.submit(scenes["ico"], _cfg(2, 2, 1))  # its pooled BVH never fits
    a = sv.submit(g, _cfg(2, 2, 1))
    b = sv.submit(g, _cfg(2, 2, 2))
    sv.step()
    ev = sv.poll()
    assert any(e.ticket == big and e.kind == "refused" for e in ev)
    assert any(e.ticket == a and e.kind == "admitted" for e in ev)
    assert not any(e.ticket == b for e in ev)
    while sv.step():
        ev += sv.poll()
        if any(e.ticket == a and e.kind == "done" for e in ev):
            break
    ev += sv.poll()
    assert any(e.ticket == a and e.kind == "done" for e in ev)
    assert not any(e.ticket == b for e in ev)  # waits: a's film is still held
    assert sv.stats()["pending_jobs"] == 1
    sv.release(a)
    ev = sv.run_until_idle()
    assert any(e.ticket == b and e.kind == "done" for e in ev)
    _same(sv.film(b), _plain_film(g, 2, 2))
    assert sv.stats()["bytes_in_use"] <= budget
    sv.close()


def test_cancel_and_scene_destroy(ctx, scenes):
    import gprt
    from gprt import scenes as S
    sv = gprt.RenderServer(ctx, max_jobs=1)
    t1 = sv.submit(scenes["spheres_b"], _cfg(64, 1, 1))
    tmp = gprt.GpuScene(ctx, S.default_style_scene(21, width=16, height=16).to_desc())
    t2 = sv.submit(tmp, _cfg(4, 4, 1))  # pending: max_jobs = 1
    sv.step()
    tmp.close()  # destroyed before admission -> cancelled
    sv.cancel(t1)  # running -> cancelled, film released
    ev = sv.poll()
    assert any(e.ticket == t2 and e.kind == "cancelled" for e in ev)
    assert any(e.ticket == t1 and e.kind == "cancelled" for e in ev)
    assert sv.step() == 0
    with pytest.raises(gprt.capi.GprtError):
        sv.film(t1)
    sv.close()


def test_loop_thread_serves_concurrent_submissions(ctx, scenes):
    import time
    import gprt
    sv = gprt.RenderServer(ctx, step_paths=1 << 14)
    sv.start()
    reqs = [("spheres_a", 1, 4), ("ico", 2, 4), ("cornell", 3, 4), ("spheres_b", 4, 8)]
    tickets = []
    for n, seed, spp in reqs:
        tickets.append(sv.submit(scenes[n], _cfg(spp, 2, seed)))
        time.sleep(0.002)  # arrivals while earlier jobs are on the GPU
    ev, deadline = [], time.time() + 60
    while time.time() < deadline and len({e.ticket for e in ev if e.kind == "done"}) < len(tickets):
        ev += sv.poll(timeout_ms=100)
    sv.stop()
    assert {e.ticket for e in ev if e.kind == "done"} == set(tickets)
    for t, (n, seed, spp) in zip(tickets, reqs):
        _same(sv.film(t), _plain_film(scenes[n], seed, spp))
    lat = gprt.latency_summary(ev)
    assert lat["jobs"] == 4 and lat["ttfp_p99_ms"] > 0
    sv.close()


def test_server_autotune_keeps_films_and_picks_a_valid_config(ctx, scenes):
    import gprt
    sv = gprt.RenderServer(ctx, step_paths=1 << 18)
    ts = [sv.submit(scenes["spheres_a"], _cfg(4, 4, 1)), sv.submit(scenes["ico"], _cfg(4, 4, 2))]
    r = sv.autotune()
    assert r["candidates"] >= 5 and 0 < r["chunk_paths"] <= 1 << 18 and r["block_size"] in (64, 128, 256)
    st = sv.stats()
    assert st["step_paths"] == r["chunk_paths"] and st["samples"] == 0  # tuning steps add no samples
    sv.run_until_idle()
    _same(sv.film(ts[0]), _plain_film(scenes["spheres_a"], 1, 4))
    _same(sv.film(ts[1]), _plain_film(scenes["ico"], 2, 4))
    sv.close()


def test_scenes_built_while_the_loop_thread_renders(ctx, scenes):
    # a serving front door: the loop thread renders the jobs already
    # submitted while the host creates the next scenes and submits each as
    # soon as it exists; every film equals the same job rendered alone, and
    # the RGBA8 read-backs (through the server's staging buffers) equal the
    # resolve of that film
    import time
    import gprt
    from gprt import scenes as S
    sv = gprt.RenderServer(ctx, step_paths=1 << 16)
    sv.start()
    keep = sv.submit(scenes["ico"], _cfg(64, 4, 5))  # keeps the loop busy meanwhile
    made, tickets = [], []
    for k in range(6):
        g = gprt.GpuScene(ctx, S.default_style_scene(20 + k, width=32 + 8 * k, height=24 + 8 * k).to_desc())
        made.append(g)
        tickets.append(sv.submit(g, _cfg(4, 2, 11 + k)))
    want = set(tickets + [keep])
    done, deadline = set(), time.perf_counter() + 120
    while done != want:
        assert time.perf_counter() < deadline
        for e in sv.poll(256, timeout_ms=10):
            assert e.kind not in ("failed", "refused", "cancelled")
            if e.kind == "done":
                done.add(e.ticket)
    sv.stop()
    for k, (g, t) in enumerate(zip(made, tickets)):
        _same(sv.film(t), _plain_film(g, 11 + k, 4))
        rgba = sv.rgba8(t)
        r = gprt.ProgressiveRaytracer(g, gprt.ProgressiveConfig(max_samples_per_pixel=4, max_passes=1, seed=11 + k))
        r.add_samples(4)
        assert np.array_equal(rgba, r.rgba8())
        r.close()
        sv.release(t)
    sv.release(keep)
    sv.close()
    for g in made:
        g.close()


def _bdpt_passes_film(g, seed, pass_spp):
    # the per-job BDPT film after the same passes (splats applied after each)
    import gprt
    r = gprt.ProgressiveRaytracer(g, gprt.ProgressiveConfig(max_samples_per_pixel=sum(pass_spp), max_passes=1,
                                                            seed=seed), integrator=gprt.BDPTIntegrator())
    for n in pass_spp:
        r.add_samples(n)
    f = r.film()
    r.close()
    return f


def _close_bdpt(a, b):
    # BDPT t = 1 splats land through float atomics, so their summation order
    # (the last bits of splat-receiving pixels) varies from run to run even
    # for the same job: sums agree to 1e-4 relative, sample counts exactly
    rgb_a, lum_a, lum2_a, cnt_a = a
    rgb_b, lum_b, lum2_b, cnt_b = b
    assert np.array_equal(cnt_a, cnt_b)
    for x, y in ((rgb_a, rgb_b), (lum_a, lum_b), (lum2_a, lum2_b)):
        assert np.allclose(x, y, rtol=1e-4, atol=1e-6 * max(1.0, float(np.abs(y).max())))


def _pass_spp(events, ticket):
    spp = [e.samples_per_pixel for e in events if e.ticket == ticket and e.kind == "pass"]
    return [b - a for a, b in zip([0] + spp[:-1], spp)]


def test_bdpt_served_beside_path_tracing(ctx, scenes):
    # BDPT requests render pass by pass on the server's copy of the scene;
    # the BDPT film equals the per-job render given the same passes, and the
    # path-tracing jobs sharing the server are unchanged
    import gprt
    sv = gprt.RenderServer(ctx, step_paths=1 << 16)
    tb = sv.submit(scenes["cornell"], _cfg(8, 2, 21), integrator=gprt.BDPTIntegrator())
    tp = sv.submit(scenes["spheres_a"], _cfg(4, 2, 22))
    tq = sv.submit(scenes["uvmesh"], _cfg(4, 4, 23))
    ev = sv.run_until_idle()
    kinds = [e.kind for e in ev if e.ticket == tb]
    assert kinds[0] == "admitted" and kinds[-1] == "done" and set(kinds[1:-1]) == {"pass"}
    passes = _pass_spp(ev, tb)
    assert sum(passes) == 8
    _close_bdpt(sv.film(tb), _bdpt_passes_film(scenes["cornell"], 21, passes))
    _same(sv.film(tp), _plain_film(scenes["spheres_a"], 22, 4))
    _same(sv.film(tq), _plain_film(scenes["uvmesh"], 23, 4))
    img = sv.rgba8(tb)
    assert img.shape == (48, 48, 4) and img[..., :3].max() > 0
    for t in (tb, tp, tq):
        sv.release(t)
    sv.close()


def test_bdpt_job_outlives_its_scene_and_can_be_cancelled(ctx):
    import gprt
    from gprt import scenes as S
    desc = S.cornell_baseline(32).to_desc()
    g = gprt.GpuScene(ctx, desc)
    ref = gprt.GpuScene(ctx, desc)
    sv = gprt.RenderServer(ctx, step_paths=1 << 16)
    t = sv.submit(g, _cfg(6, 2, 31), integrator=gprt.BDPTIntegrator())
    t2 = sv.submit(g, _cfg(400, 2, 32), integrator=gprt.BDPTIntegrator())
    ev = []
    for _ in range(2):
        sv.step()
        ev += sv.poll()
    g.close()  # the server renders on its own copy
    for _ in range(3):
        sv.step()
        ev += sv.poll()
    sv.cancel(t2)
    ev += sv.run_until_idle()
    kinds = [e.kind for e in ev if e.ticket == t]
    assert kinds[0] == "admitted" and kinds[-1] == "done"
    assert [e.kind for e in ev if e.ticket == t2][-1] == "cancelled"
    _close_bdpt(sv.film(t), _bdpt_passes_film(ref, 31, _pass_spp(ev, t)))
    sv.release(t)
    st = sv.stats()
    assert st["active_jobs"] == 0
    sv.close()
    ref.close()


def test_bdpt_admission_by_budget(ctx, scenes):
    # a BDPT request holds its film, one chunk's subpath working set and a
    # copy of its scene: refused when that never fits the budget, admitted
    # (and its bytes held until release) when it does
    import gprt
    g = scenes["cornell"]
    sv0 = gprt.RenderServer(ctx, step_paths=1 << 12)
    t = sv0.submit(g, _cfg(4, 2, 1), integrator=gprt.BDPTIntegrator())
    sv0.step()
    st0 = sv0.stats()
    assert st0["active_jobs"] == 1
    with_bdpt = st0["bytes_in_use"]
    sv0.cancel(t)
    bare = sv0.stats()["bytes_in_use"]  # path state and table only
    sv0.close()
    assert with_bdpt > bare
    sv = gprt.RenderServer(ctx, hbm_budget_bytes=bare + (with_bdpt - bare) // 2, step_paths=1 << 12)
    tb = sv.submit(g, _cfg(4, 2, 1), integrator=gprt.BDPTIntegrator())
    tp = sv.submit(scenes["spheres_b"], _cfg(2, 2, 3))
    ev = sv.run_until_idle()
    refused = [e for e in ev if e.ticket == tb and e.kind == "refused"]
    assert refused and refused[0].status == gprt.capi.GPRT_E_ADMISSION
    assert any(e.ticket == tp and e.kind == "done" for e in ev)
    _same(sv.film(tp), _plain_film(scenes["spheres_b"], 3, 2))
    sv.close()


def _adaptive(scene, min_frac=0.25, threshold=0.3):
    scene.sampling.adaptive_min_samples = min_frac
    scene.sampling.adaptive_threshold = threshold
    return scene


def _progressive(g, cfg, integrator=None):
    # the per-job progressive render (gprt_job_render_pass per pass, with the
    # scene's adaptive stop): its film and each pass's average sample count
    import gprt
    r = gprt.ProgressiveRaytracer(g, cfg, integrator) if integrator else gprt.ProgressiveRaytracer(g, cfg)
    avgs = [int(res.stats.average_samples) for res in r.render_progressive()]
    f = r.film()
    r.close()
    return f, avgs


def test_adaptive_sampling_in_the_server_equals_progressive_render(ctx, scenes):
    """A scene with AdaptiveMinSamples < 1 renders in the server as through
    gprt_job_render_pass: per pass every pixel first takes the pass minimum,
    then rounds of one sample per pixel still active (below the pass target
    and not converged, tile_renderer.go:51-101) until none is.  Path-tracing
    films agree bit for bit, BDPT films up to the splat summation order, and
    the pass events report the per-job render's average sample counts;
    fixed-spp jobs in the same steps are unchanged."""
    import gprt
    from gprt import scenes as S
    made = [gprt.GpuScene(ctx, _adaptive(S.cornell_baseline(48)).to_desc()),
            gprt.GpuScene(ctx, _adaptive(S.default_style_scene(5, width=64, height=48)).to_desc()),
            gprt.GpuScene(ctx, _adaptive(S.cornell_boxes_bdpt(32, max_depth=5)).to_desc())]
    cfgs = [_cfg(16, 4, 31), _cfg(24, 6, 32), _cfg(8, 4, 34)]
    integ = [None, None, gprt.BDPTIntegrator()]
    ref = [_progressive(g, c, i) for g, c, i in zip(made, cfgs, integ)]
    # the stop took effect: some pixels ended below the target
    for (film, _), c in zip(ref, cfgs):
        assert film[3].min() < c.max_samples_per_pixel
    sv = gprt.RenderServer(ctx, step_paths=1 << 16)
    fixed = sv.submit(scenes["spheres_b"], _cfg(4, 2, 33))
    ts = [sv.submit(g, c, integrator=i) for g, c, i in zip(made, cfgs, integ)]
    ev = sv.run_until_idle()
    for t, (film, avgs), i in zip(ts, ref, integ):
        kinds = [e.kind for e in ev if e.ticket == t]
        assert kinds[0] == "admitted" and kinds[-1] == "done"
        assert [e.samples_per_pixel for e in ev if e.ticket == t and e.kind == "pass"] == avgs
        if i is None:
            _same(sv.film(t), film)
        else:
            _close_bdpt(sv.film(t), film)
    _same(sv.film(fixed), _plain_film(scenes["spheres_b"], 33, 4))
    sv.close()
    for g in made:
        g.close()


def _plain_rgba8(g, seed, spp):
    import gprt
    r = gprt.ProgressiveRaytracer(g, gprt.ProgressiveConfig(max_samples_per_pixel=spp, max_passes=1, seed=seed))
    r.add_samples(spp)
    img = r.rgba8()
    r.close()
    return img


def test_reused_films_and_reads_while_the_loop_renders(ctx, scenes):
    """Released films go to a cache that later admissions of the same size
    reuse (cleared on reuse), and read-backs run on their own stream while
    the loop thread keeps stepping: every image read at its job's `done`
    event (other jobs still rendering) equals the plain job's, including
    jobs whose film was reused from a released one."""
    import time
    import gprt
    sv = gprt.RenderServer(ctx, step_paths=1 << 14)
    sv.start()
    reqs = [("spheres_a", 31, 4), ("cornell", 32, 4), ("spheres_a", 33, 8), ("cornell", 34, 4),
            ("spheres_b", 35, 4), ("spheres_a", 36, 4)]
    imgs, seeds, done = {}, {}, set()
    deadline = time.time() + 120
    for k, (n, seed, spp) in enumerate(reqs):
        t = sv.submit(scenes[n], _cfg(spp, 2, seed))
        seeds[t] = (n, seed, spp)
        # later requests of a size arrive after an earlier one was read and
        # released, so their film comes from the cache
        while k < 2 and time.time() < deadline and t not in done:
            for e in sv.poll(timeout_ms=50):
                if e.kind == "done":
                    imgs[e.ticket] = sv.rgba8(e.ticket)
                    sv.release(e.ticket)
                    done.add(e.ticket)
    while time.time() < deadline and len(done) < len(reqs):
        for e in sv.poll(timeout_ms=50):
            assert e.kind not in ("failed", "refused", "cancelled")
            if e.kind == "done":
                imgs[e.ticket] = sv.rgba8(e.ticket)
                sv.release(e.ticket)
                done.add(e.ticket)
    sv.stop()
    assert len(done) == len(reqs)
    for t, (n, seed, spp) in seeds.items():
        assert np.array_equal(imgs[t], _plain_rgba8(scenes[n], seed, spp)), (n, seed)
    sv.close()


def test_bdpt_first_passes_of_a_burst_run_together(ctx, scenes):
    """Several BDPT requests arriving together start their first passes in
    the same step (each on its own stream): each film equals the per-job
    render of the same passes, up to the splat summation order."""
    import gprt
    sv = gprt.RenderServer(ctx, step_paths=1 << 16)
    cfgs = [(41, 8, 4), (42, 8, 2), (43, 4, 4)]
    ts = [sv.submit(scenes["cornell"], _cfg(spp, per, seed), integrator=gprt.BDPTIntegrator())
          for seed, spp, per in cfgs]
    tp = sv.submit(scenes["spheres_b"], _cfg(4, 2, 44))
    ev = sv.run_until_idle()
    firsts = [next(i for i, e in enumerate(ev) if e.ticket == t and e.kind == "pass") for t in ts]
    # the three first passes are reported by the first steps, before any later pass
    later = [i for i, e in enumerate(ev) if e.kind == "pass" and e.ticket in ts and i not in firsts]
    assert max(firsts) < min(later)
    for t, (seed, spp, per) in zip(ts, cfgs):
        passes = _pass_spp(ev, t)
        assert sum(passes) == spp
        _close_bdpt(sv.film(t), _bdpt_passes_film(scenes["cornell"], seed, passes))
    _same(sv.film(tp), _plain_film(scenes["spheres_b"], 44, 4))
    sv.close()
