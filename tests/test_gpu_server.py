"""The serving loop (snow_server_*): admission by HBM budget, resident job
state, continuous batching. A job's result must not depend on which other
jobs shared its batch: it is compared with the same scene stepped alone
through SimScene. The FAST path's P2G sums are fixed-point integers, so the
explicit jobs' states are the same bits alone and served (np.array_equal)
although their binning schedules differ; the semi-implicit solve sums K u in
floats, so a semi-implicit job is compared within a tolerance."""
import numpy as np
import pytest

from snow_gb300 import scenes

gpu = pytest.mark.gpu


def _jobs():
    return [
        scenes.small_scene(n=3000, grid_edge=32, seed=201, v0=(0.5, -1.0, 0.0)),
        scenes.small_scene(n=12000, grid_edge=48, seed=202, v0=(0.0, -2.0, 1.0)),
        scenes.small_scene(n=6000, grid_edge=40, seed=203, v0=(-1.0, 0.0, 0.5)),
        scenes.small_scene(n=1500, grid_edge=24, seed=204, v0=(0.0, 0.0, 0.0)),
    ]


def _alone(s, steps):
    from snow_gb300 import api
    ctx = api.Context(0)
    try:
        sim = api.SimScene(ctx, s).upload().init().step(s.dt, steps)
        return sim.download()
    finally:
        ctx.close()


def _same(a, b):
    for k in ("x", "v", "FE", "Jp"):
        assert np.array_equal(a[k], b[k]), k


def _close(a, b, tol=1e-4):
    assert np.abs(a["x"] - b["x"]).max() <= tol
    assert np.abs(a["v"] - b["v"]).max() <= tol * max(1.0, np.abs(a["v"]).max())
    assert np.abs(a["FE"] - b["FE"]).max() <= tol
    assert np.abs(a["Jp"] - b["Jp"]).max() <= tol


@gpu
def test_job_result_is_the_same_alone_and_in_the_mix():
    from snow_gb300 import api
    jobs = _jobs()
    steps = [20, 13, 27, 7]  # jobs leave the batch at different chunk boundaries
    srv = api.Server(0, chunk_steps=5)
    try:
        ids = [srv.submit(s, steps=k, keep_state=True) for s, k in zip(jobs, steps)]
        srv.drain(120.0)
        res = {r["id"]: r for r in srv.poll()}
        assert sorted(res) == sorted(ids)
        for jid, s, k in zip(ids, jobs, steps):
            r = res[jid]
            assert r["status"] == 0 and r["n"] == s.n and r["steps"] == k
            assert r["stats"]["nonfinite"] == 0
            assert r["latency_s"] >= r["service_s"] >= 0.0
            _same(_alone(s, k), srv.fetch(jid, s.n))
        st = srv.stats()
        assert st["completed"] == len(jobs) and st["failed"] == 0 and st["pending"] == 0
        assert st["particle_steps"] == sum(s.n * k for s, k in zip(jobs, steps))
    finally:
        srv.close()


@gpu
def test_late_arrivals_join_running_jobs():
    import time
    from snow_gb300 import api
    jobs = _jobs()
    srv = api.Server(0, chunk_steps=4)
    try:
        first = srv.submit(jobs[1], steps=4000)
        time.sleep(0.05)  # the first job is running when the others arrive
        late = [srv.submit(s, steps=8, keep_state=True) for s in (jobs[0], jobs[2])]
        srv.drain(120.0)
        res = {r["id"]: r for r in srv.poll()}
        assert all(res[j]["status"] == 0 for j in [first] + late)
        # the late jobs finished long before the 4000-step job
        assert max(res[j]["latency_s"] for j in late) < res[first]["latency_s"]
        for j, s in zip(late, (jobs[0], jobs[2])):
            _same(_alone(s, 8), srv.fetch(j, s.n))
    finally:
        srv.close()


@gpu
def test_admission_keeps_resident_state_within_the_budget():
    from snow_gb300 import api, native as N
    jobs = [scenes.small_scene(n=12000, grid_edge=48, seed=210 + k) for k in range(3)]
    L = N.load()
    fps = [L.snow_scene_footprint(api.params_for(s, N.MODE_FAST), s.n) for s in jobs]
    budget = int(max(fps) * 1.5)  # room for one job at a time
    srv = api.Server(0, hbm_budget=budget, chunk_steps=4)
    try:
        ids = [srv.submit(s, steps=6) for s in jobs]
        too_big = srv.submit(scenes.small_scene(n=2000, grid_edge=160, seed=205), steps=2)
        srv.drain(120.0)
        res = {r["id"]: r for r in srv.poll()}
        assert [res[i]["status"] for i in ids] == [0, 0, 0]
        assert res[too_big]["status"] == -3  # SNOW_EBUDGET: can never fit
        # one at a time: each later job waited for the one before it
        for a, b in zip(ids, ids[1:]):
            assert res[b]["queue_s"] >= res[a]["service_s"] * 0.5
        assert srv.stats()["resident_bytes"] <= budget
    finally:
        srv.close()


@gpu
@pytest.mark.parametrize("policy", ["fifo", "srpt"])
def test_particle_cap_and_policy_order_the_jobs(policy):
    """Under a particle cap that fits one job at a time, SRPT runs a short job
    that arrives behind a long one first; FIFO finishes the long one first.
    Both give the same results as the jobs alone."""
    import time
    from snow_gb300 import api
    long_job = scenes.small_scene(n=12000, grid_edge=48, seed=221)
    short_job = scenes.small_scene(n=3000, grid_edge=32, seed=222)
    srv = api.Server(0, chunk_steps=8, max_active_particles=12000, policy=policy)
    try:
        a = srv.submit(long_job, steps=200, keep_state=True)
        time.sleep(0.02)
        b = srv.submit(short_job, steps=16, keep_state=True)
        srv.drain(120.0)
        res = {r["id"]: r for r in srv.poll()}
        assert res[a]["status"] == 0 and res[b]["status"] == 0
        if policy == "srpt":
            assert res[b]["latency_s"] < res[a]["latency_s"]
        else:
            assert res[b]["latency_s"] > res[a]["latency_s"] - 0.02
        _same(_alone(short_job, 16), srv.fetch(b, short_job.n))
        _same(_alone(long_job, 200), srv.fetch(a, long_job.n))
    finally:
        srv.close()


@gpu
def test_semi_implicit_jobs_serve_beside_explicit_ones():
    """A semi-implicit job (the solve's conditional loop inside the batch
    graph) and explicit jobs in one batch: each matches the same scene stepped
    alone."""
    from snow_gb300 import api
    stiff = scenes.small_scene(n=4000, grid_edge=32, seed=205, v0=(0.0, -1.0, 0.0), young=1.4e7)
    stiff.v = stiff.v + np.random.default_rng(7).normal(scale=0.2, size=stiff.v.shape).astype(np.float32)
    stiff.dt = 5e-4
    stiff.implicit_beta, stiff.implicit_tolerance, stiff.implicit_max_iters = 1.0, 1e-6, 40
    jobs = [stiff, _jobs()[0], _jobs()[3]]
    steps = [12, 9, 6]
    srv = api.Server(0, chunk_steps=4)
    try:
        ids = [srv.submit(s, steps=k, keep_state=True) for s, k in zip(jobs, steps)]
        srv.drain(120.0)
        res = {r["id"]: r for r in srv.poll()}
        for jid, s, k in zip(ids, jobs, steps):
            assert res[jid]["status"] == 0 and res[jid]["stats"]["nonfinite"] == 0
            if s.implicit_beta > 0:
                _close(_alone(s, k), srv.fetch(jid, s.n), tol=2e-4)
            else:
                _same(_alone(s, k), srv.fetch(jid, s.n))
    finally:
        srv.close()
