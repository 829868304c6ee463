"""GPU tests of the host API: batching, the reference-shaped engine classes,
error statuses, and that results are the same alone and in a batch.

The FAST path sums its P2G contributions as fixed-point integers, so a
scene's state does not depend on how its particles are grouped into work
items, on the binning schedule, on CTA scheduling or on the other scenes of
a batch: those comparisons are exact (np.array_equal)."""
import ctypes

import numpy as np
import pytest

from snow_gb300 import scenes

gpu = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from snow_gb300 import api
    return api.Context(0)


def _three_scenes():
    return [scenes.small_scene(n=3000, grid_edge=32, seed=81, v0=(0.0, -2.0, 0.0)),
            scenes.small_scene(n=9000, grid_edge=48, seed=82, v0=(1.0, -1.0, 0.0), kind="box",
                               young=6e4, hardening=6.0),
            scenes.small_scene(n=1500, grid_edge=24, seed=83, v0=(0.0, 0.0, 3.0))]


@gpu
@pytest.mark.parametrize("steps", [1, 20])
def test_batch_matches_each_scene_alone(ctx, steps):
    from snow_gb300 import api
    scs = _three_scenes()
    alone = []
    for s in scs:
        a = api.SimScene(ctx, s).upload().init().step(s.dt, steps)
        alone.append(a.download())
    sims = [api.SimScene(ctx, s).upload().init() for s in scs]
    api.Batch(ctx, sims).step(steps, dt=[s.dt for s in scs])
    for s, a, b in zip(scs, alone, (x.download() for x in sims)):
        for k in ("x", "v", "FE", "Jp"):
            assert np.array_equal(a[k], b[k]), k


@gpu
def test_engine_classes_follow_the_reference_call_sequence(ctx):
    from snow_gb300 import api
    s = scenes.small_scene(n=2000, grid_edge=32, seed=91)
    engine = api.MPMPhysicEngine(api.ExplicitTimeUpdate(s, ctx=ctx))
    assert engine.init()
    for _ in range(3):
        engine.update(s.dt)
    st = engine.integration.sim.stats()
    assert st["n"] == s.n and st["nonfinite"] == 0
    assert st["momentum"][1] < 0  # falling


@gpu
def test_error_statuses(ctx):
    from snow_gb300 import api, native as N
    s = scenes.small_scene(n=500, grid_edge=16, seed=92)
    sim = api.SimScene(ctx, s)
    with pytest.raises(N.SnowError) as e:
        sim.step(1e-4, 1)
    assert e.value.status == -7  # SNOW_ESTATE: step before init
    sim.upload().init()
    with pytest.raises(N.SnowError) as e:
        sim.download(fp=True)
    assert e.value.status == -8  # SNOW_EUNSUPPORTED: no F_P in FAST mode
    small = api.Context(0, hbm_budget=1 << 20)
    with pytest.raises(N.SnowError) as e:
        api.SimScene(small, scenes.small_scene(n=20000, grid_edge=64, seed=93), capacity=20000)
    assert e.value.status == -3  # SNOW_EBUDGET
    bad = scenes.small_scene(n=10, grid_edge=16, seed=94)
    bad.grid_dim = (0, 16, 16)
    with pytest.raises(N.SnowError) as e:
        api.SimScene(ctx, bad)
    assert e.value.status == -1  # SNOW_EINVAL


@gpu
def test_rigid_advance_moves_colliders(ctx):
    from snow_gb300 import api
    s = scenes.small_scene(n=500, grid_edge=16, seed=95)
    s.colliders.append(scenes.Collider(pos=(0.5, 0.1, 0.5), type=1, radius=0.05, vel=(0.0, 1.0, 0.0)))
    sim = api.SimScene(ctx, s).upload().init().step(1e-3, 10)
    c = sim.colliders()
    assert abs(c[-1][1] - (0.1 + 10 * 1e-3)) < 1e-6


@gpu
def test_moving_sphere_colliders_in_a_batch(ctx):
    """Two scenes with spheres moving at different velocities through the
    snow: each collider advances by its own dt * v inside the batch, and the
    particles match the same scenes stepped alone."""
    from snow_gb300 import api
    a = scenes.small_scene(n=4000, grid_edge=32, seed=99, v0=(0.0, 0.0, 0.0), center=(0.5, 0.3, 0.5))
    b = scenes.small_scene(n=3000, grid_edge=24, seed=100, v0=(0.0, -1.0, 0.0), center=(0.5, 0.35, 0.5))
    a.colliders.append(scenes.Collider(pos=(0.3, 0.3, 0.5), type=1, radius=0.08, vel=(2.0, 0.0, 0.0)))
    b.colliders.append(scenes.Collider(pos=(0.5, 0.6, 0.5), type=1, radius=0.06, vel=(0.0, -3.0, 0.0),
                                       friction=0.4))
    steps = 15
    alone = [api.SimScene(ctx, s).upload().init().step(s.dt, steps) for s in (a, b)]
    sims = [api.SimScene(ctx, s).upload().init() for s in (a, b)]
    api.Batch(ctx, sims).step(steps, dt=[a.dt, b.dt])
    for s, one, many in zip((a, b), alone, sims):
        want = np.asarray(s.colliders[-1].pos) + steps * s.dt * np.asarray(s.colliders[-1].vel)
        assert np.abs(many.colliders()[-1] - want).max() < 1e-5
        assert np.abs(one.colliders()[-1] - want).max() < 1e-5
        d1, d2 = one.download(), many.download()
        for k in ("x", "v", "FE", "Jp"):
            assert np.array_equal(d1[k], d2[k]), k


@gpu
def test_tunings_change_the_work_split_not_the_physics(ctx):
    """Sort interval, particles per work item and CTAs per SM only change how
    the step is cut into launches: the states are the same bits."""
    from snow_gb300 import api
    scs = _three_scenes()
    steps = 12
    alone = [api.SimScene(ctx, s).upload().init().step(s.dt, steps).download() for s in scs]
    for si, im, cp in [(4, 128, 1), (16, 64, 2), (1, 256, 1)]:
        sims = [api.SimScene(ctx, s).upload().init() for s in scs]
        b = api.Batch(ctx, sims).set_tuning(si, im, cp)
        b.step(steps, dt=[s.dt for s in scs])
        for a, sim in zip(alone, sims):
            got = sim.download()
            for k in ("x", "v", "FE", "Jp"):
                assert np.array_equal(a[k], got[k]), (si, im, cp, k)
        b.close()
        for sim in sims:
            sim.close()
    single = api.SimScene(ctx, scs[0]).upload().init().set_tuning(2, 96, 1).step(scs[0].dt, steps).download()
    for k in ("x", "v", "FE", "Jp"):
        assert np.array_equal(alone[0][k], single[k]), k


@gpu
def test_autotune_picks_a_candidate_and_reuses_the_cache(ctx, tmp_path):
    from snow_gb300 import api, native as N
    scs = _three_scenes()
    sims = [api.SimScene(ctx, s).upload().init() for s in scs]
    b = api.Batch(ctx, sims)
    cache = str(tmp_path / "tuning.json")
    c = b.autotune(dt=[s.dt for s in scs], cache=cache)
    assert not c["cached"] and c["steps_taken"] > 0 and c["ms_per_step"] > 0
    assert c["sort_interval"] in (1, 2, 4, 8, 12, 16, 24, 32) and c["items_max"] in (128, 256) and c["ctas_per_sm"] in (1, 2)
    again = b.autotune(dt=[s.dt for s in scs], cache=cache)
    assert again["cached"] and again["steps_taken"] == 0
    assert {k: again[k] for k in ("sort_interval", "items_max", "ctas_per_sm")} == \
        {k: c[k] for k in ("sort_interval", "items_max", "ctas_per_sm")}
    b.step(3, dt=[s.dt for s in scs])
    for sim in sims:
        assert sim.stats()["nonfinite"] == 0
    bad = N.SnowTuning(0, 256, 2, 0, 0.0)
    assert N.load().snow_batch_set_tuning(b.h, ctypes.byref(bad)) == -1


@gpu
def test_queued_statistics_match_the_waiting_read(ctx):
    from snow_gb300 import api, native as N
    s = scenes.small_scene(n=3000, grid_edge=32, seed=95, v0=(1.0, -2.0, 0.5))
    sim = api.SimScene(ctx, s).upload().init()
    want = []
    for i in range(4):
        sim.step(s.dt, 1)
        sim.stats_enqueue(i % 3)
        want.append(sim.stats())
    # slot 0 was reused by step 3: it holds step 3's statistics
    got = {k: ctx.stats_read(k) for k in range(3)}
    for slot, step in ((0, 3), (1, 1), (2, 2)):
        for key in ("mass", "kinetic_energy", "mean_jp"):
            assert got[slot][key] == want[step][key]
        assert np.array_equal(got[slot]["momentum"], want[step]["momentum"])
    with pytest.raises(N.SnowError) as e:
        ctx.stats_read(0)  # already read
    assert e.value.status == -7


@gpu
def test_bad_time_steps_are_rejected(ctx):
    from snow_gb300 import api, native as N
    s = scenes.small_scene(n=500, grid_edge=16, seed=98)
    sim = api.SimScene(ctx, s).upload().init()
    for dt in (-1e-4, float("nan"), float("inf")):
        with pytest.raises(N.SnowError) as e:
            sim.step(dt, 1)
        assert e.value.status == -1
    sim.step(s.dt, 1)  # the scene is unaffected
    assert sim.stats()["nonfinite"] == 0


@gpu
def test_empty_upload_is_rejected(ctx):
    from snow_gb300 import api, native as N
    s = scenes.small_scene(n=1, grid_edge=16, seed=97)
    s.x, s.v, s.m = s.x[:0], s.v[:0], s.m[:0]
    with pytest.raises(N.SnowError) as e:
        api.SimScene(ctx, s).upload()
    assert e.value.status == -1  # SNOW_EINVAL: a scene holds at least one particle


@gpu
@pytest.mark.parametrize("n", [1, 2])
def test_tiny_scenes_step_in_both_modes(ctx, n):
    """One- and two-particle scenes: upload, init, steps, statistics and
    download work (the reference's smallest scene is one particle)."""
    from snow_gb300 import api, native as N
    s = scenes.small_scene(n=max(n, 1), grid_edge=16, seed=97)
    s.x, s.v, s.m = s.x[:n], s.v[:n], s.m[:n]
    for mode in (N.MODE_FAST, N.MODE_REFERENCE):
        sim = api.SimScene(ctx, s, mode=mode).upload().init().step(s.dt, 5)
        st = sim.stats()
        out = sim.download()
        assert st["n"] == n and st["nonfinite"] == 0
        assert out["x"].shape == (n, 3)
        if n:
            assert np.all(np.isfinite(out["x"])) and out["x"][:, 1].max() < s.x[:, 1].max()  # falling
        sim.close()


@gpu
def test_statistics_do_not_depend_on_block_scheduling(ctx):
    """The statistics kernel sums its per-block records in block order: reads
    of the same state agree to the bit, and with a sum over the downloaded
    particles in FP64."""
    from snow_gb300 import api
    s = scenes.small_scene(n=50000, grid_edge=48, seed=96, v0=(0.5, -1.5, 0.25))
    sim = api.SimScene(ctx, s).upload().init().step(s.dt, 3)
    a, b = sim.stats(), sim.stats()
    for key in ("mass", "kinetic_energy", "mean_jp"):
        assert a[key] == b[key]
    assert np.array_equal(a["momentum"], b["momentum"]) and np.array_equal(a["bbox_min"], b["bbox_min"])
    d = sim.download()
    m = s.m.astype(np.float64)
    assert abs(a["mass"] - m.sum()) <= 1e-6 * m.sum()
    mom = (m[:, None] * d["v"].astype(np.float64)).sum(0)
    assert np.abs(np.asarray(a["momentum"]) - mom).max() <= 1e-5 * np.abs(mom).max()
    assert np.allclose(a["bbox_min"], d["x"].min(0)) and np.allclose(a["bbox_max"], d["x"].max(0))


@gpu
def test_fast_particles_rebin_every_step_with_the_same_physics(ctx):
    """Particles crossing most of a cell per step leave their work items'
    tiles between binnings; snow_scene_step then re-bins every step. The
    states are the same bits as the same scene re-binned every step from the
    start."""
    from snow_gb300 import api
    s = scenes.small_scene(n=6000, grid_edge=48, seed=90, v0=(6.0, -3.0, 2.0), center=(0.45, 0.5, 0.45))
    s.dt = 2e-3  # |v| dt / h = 0.67 cells per step
    a = api.SimScene(ctx, s).upload().init().step(s.dt, 30)
    b = api.SimScene(ctx, s).upload().init().set_tuning(1, 256, 2).step(s.dt, 30)
    da, db = a.download(), b.download()
    assert a.stats()["nonfinite"] == 0
    for k in ("x", "v", "FE", "Jp"):
        assert np.array_equal(da[k], db[k]), k


@gpu
def test_non_finite_particles_are_reported(ctx):
    """A particle uploaded with a NaN velocity: the statistics count it at
    once, and a later step call returns SNOW_ENUMERIC (the device counters are
    read at re-binning points, one interval behind)."""
    from snow_gb300 import api, native as N
    s = scenes.small_scene(n=3000, grid_edge=32, seed=89)
    s.v = s.v.copy()
    s.v[17] = np.nan
    sim = api.SimScene(ctx, s).upload().init()
    assert sim.stats()["nonfinite"] == 1
    status = 0
    for _ in range(40):
        try:
            sim.step(s.dt, 1)
        except N.SnowError as e:
            status = e.status
            break
    assert status == -5  # SNOW_ENUMERIC


@gpu
def test_pinned_and_pageable_host_arrays_give_the_same_state(ctx):
    """Upload reads pinned (page-locked) host arrays in place from the pack
    kernel and download writes them from the unpack kernel; pageable arrays
    go through a device staging buffer. Both routes, and a mix of them,
    give the same bits."""
    import torch

    from snow_gb300 import api
    s = scenes.small_scene(n=5000, grid_edge=32, seed=77, v0=(0.4, -1.5, 0.2))

    def pinned(a):
        t = torch.empty(a.shape, dtype=torch.float32, pin_memory=True).numpy()
        t[...] = a
        return t

    fe0 = np.tile(np.eye(3, dtype=np.float32), (s.n, 1, 1)) * np.float32(1.001)
    ref = api.SimScene(ctx, s).upload(s.x, s.v, s.m, FE=fe0.reshape(-1, 9)).init().step(s.dt, 5).download()
    g = api.SimScene(ctx, s).upload(pinned(s.x), pinned(s.v), s.m, FE=pinned(fe0.reshape(-1, 9))).init()
    g.step(s.dt, 5)
    shapes = dict(x=(s.n, 3), v=(s.n, 3), FE=(s.n, 3, 3), Jp=(s.n,), volume=(s.n,))
    for pin in ({"x", "v", "FE", "Jp", "volume"}, {"x", "FE"}):
        out = {k: pinned(np.zeros(sh, np.float32)) if k in pin else np.zeros(sh, np.float32)
               for k, sh in shapes.items()}
        got = g.download(out=out)
        for k in shapes:
            assert np.array_equal(got[k], ref[k]), k
