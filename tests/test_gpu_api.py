"""GPU tests of the host API: batching, the reference-shaped engine classes,
error statuses, and that results are the same alone and in a batch."""
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
    tol = 1e-5 if steps == 1 else 1e-4
    for s, a, b in zip(scs, alone, (x.download() for x in sims)):
        assert np.abs(a["x"] - b["x"]).max() <= tol * 1.0
        assert np.abs(a["v"] - b["v"]).max() <= tol * max(1.0, np.abs(a["v"]).max())
        assert np.abs(a["FE"] - b["FE"]).max() <= tol
        assert np.abs(a["Jp"] - b["Jp"]).max() <= tol


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
