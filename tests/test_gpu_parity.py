"""GPU parity tests through the C ABI (snow_gb300 on sm_103a) against the
oracle on the same seeded inputs.

Tolerances:
  * SNOW_MODE_REFERENCE vs the FAITHFUL32 oracle (the shaders' arithmetic,
    pinned bit-for-bit to the reference's own shader code): the kernels round
    every operation like the oracle (no FMA); only expf (CUDA's, <= 2 ulp vs
    glibc) differs, which moves the truncated int32 force contributions by a
    count now and then. Density after init is bit-exact (no expf on that
    path); after steps: |dx| <= 1e-6 m, |dv| <= 1e-4 m/s, |dF| <= 1e-5.
  * SNOW_MODE_FAST vs the EXACT64 oracle (FP64, no fixed point, no V
    rounding), one step: per-field relative error <= 1e-5
    (oracle.parity_errors):
        x  : |dx| / max(|x|, 1e-3 m)
        v  : |dv| / max(|v|, 1e-3 m/s)           (strict floor)
        F_E: max|dF| / max|F| per particle
        J_p: |dJ| / |J|
    The strict velocity floor holds where no particle is stopped within the
    step (free flight, first contact). A particle that a collider or the
    snow around it stops has |v'| far below the size S_p of the terms its
    FLIP update adds up (alpha |v_p| + sum_i w_ip (|v*_i| + alpha |p_i/m_i|));
    an FP32 evaluation resolves v' only to a few ulps of S_p, so there the
    asserted bound is |dv| / max(|v|, 1e-3 m/s, S_p) <= 1e-5 (v_flip), with
    S_p from the oracle's own grid of that step. Both are reported. Grid
    forces are compared in a deformed state, where stresses are far above
    the ~1e-7 strain FP32 can resolve in F_E - R.
  * binning: keys and stable permutation bit-exact vs std::stable_sort.
"""
import numpy as np
import pytest

from oracle import oracle as O
from snow_gb300 import scenes
from tests._util import golden_names, load_golden, mat3x3_from_std140

gpu = pytest.mark.gpu

REL_TOL = 1e-5


@pytest.fixture(scope="module")
def ctx():
    from snow_gb300 import api
    return api.Context(0)


def sim(ctx, scene, mode, **kw):
    from snow_gb300 import api
    return api.SimScene(ctx, scene, mode=mode, **kw)


def check_step(got, ref, flip, strict):
    """Asserts the FAST single-step bound (module docstring); `strict` also
    asserts the 1e-3 m/s velocity floor for every particle."""
    e = O.parity_errors(got, ref, flip)
    m = e["max"]
    assert max(m["x"], m["v_flip"], m["FE"], m["Jp"]) <= REL_TOL, e
    if strict:
        assert m["v"] <= REL_TOL, e
    return e


# ---------------------------------------------------------------------------
@gpu
@pytest.mark.parametrize("name", golden_names())
def test_reference_mode_matches_golden_and_faithful_oracle(ctx, name):
    from snow_gb300 import native as N
    s, z = load_golden(name)
    bufs = (z["pxm0"], z["pv0"]) + s.std140()[2:]
    g = sim(ctx, s, N.MODE_REFERENCE).upload_std140(*bufs).init()
    _, pv, _, _ = g.download_std140()
    assert np.array_equal(pv[:, 3], z["pv_init"][:, 3]), "density after init must be bit-exact"
    for k in range(1, int(z["steps"]) + 1):
        g.step(s.dt, 1)
        pxm, pv, fe, fp = g.download_std140()
        assert np.abs(pxm[:, :3] - z[f"pxm_{k}"][:, :3]).max() <= 1e-6
        assert np.abs(pv[:, :3].astype(np.int64) - z[f"pv_{k}"][:, :3]).max() <= 1e4  # 1e-4 m/s
        fe9 = fe.reshape(-1, 4, 4)[:, :3, :3].reshape(-1, 9)
        fp9 = fp.reshape(-1, 4, 4)[:, :3, :3].reshape(-1, 9)
        assert np.abs(fe9 - z[f"fe_{k}"]).max() <= 1e-5
        assert np.abs(fp9 - z[f"fp_{k}"]).max() <= 1e-5


@gpu
def test_reference_mode_kernels_one_by_one(ctx):
    """Each reference-mode kernel against the same oracle phase."""
    from snow_gb300 import native as N
    s = scenes.small_scene(n=3000, grid_edge=32, seed=21, v0=(0.5, -3.0, 0.25))
    bufs = s.std140()
    g = sim(ctx, s, N.MODE_REFERENCE).upload_std140(*bufs).init()
    o = O.OracleSim(s, mode=O.FAITHFUL32).upload_std140(*bufs).init()
    o.step()
    g.step(s.dt, 1)  # leave the identity deformation behind
    for kern, ph in [(N.K_RIGID_ADVANCE, O.PH_RIGID), (N.K_G_RESET, O.PH_RESET), (N.K_P2G, O.PH_P2G)]:
        g.dispatch(kern, s.dt)
        o.phase(ph)
    gd, od = g.grid(), o.grid()
    assert np.abs(gd["mass"] - od["mass"]).max() <= 1e-8 * 2  # exact int sums, 1 count = 1e-8
    assert np.abs(gd["mom"] - od["mom"]).max() <= 64 * 1e-8
    assert np.abs(gd["force"] - od["force"]).max() <= 64 * 1e-6
    g.dispatch(N.K_G_FORCE, s.dt)
    o.phase(O.PH_GRID)
    gd, od = g.grid(), o.grid()
    assert np.abs(gd["vstar"] - od["vstar"]).max() <= 1e-5
    for kern, ph in [(N.K_G2P, O.PH_G2P), (N.K_P_ADVANCE, O.PH_ADVANCE)]:
        g.dispatch(kern, s.dt)
        o.phase(ph)
    a = g.download(fp=True)
    b = o.state()
    assert np.abs(a["x"] - b["x"]).max() <= 1e-6
    assert np.abs(a["v"] - b["v"]).max() <= 1e-4
    assert np.abs(a["FE"] - b["FE"]).max() <= 1e-5


# ---------------------------------------------------------------------------
def _exact_oracle(s, vround=False):
    return O.OracleSim(s, mode=O.EXACT64, vround=vround)


@gpu
@pytest.mark.parametrize("seed,n,edge,v0", [(31, 4000, 32, (0.0, -2.0, 0.0)), (32, 6000, 40, (1.0, -4.0, 0.5)),
                                            (33, 2500, 24, (3.0, 0.0, -2.0))])
def test_fast_single_step_from_rest_within_1e5(ctx, seed, n, edge, v0):
    from snow_gb300 import native as N
    s = scenes.small_scene(n=n, grid_edge=edge, seed=seed, v0=v0)
    g = sim(ctx, s, N.MODE_FAST).upload().init().step(s.dt, 1)
    o = _exact_oracle(s).upload().init()
    flip = o.step_with_flip_scale()
    check_step(g.download(), o.state(), flip, strict=True)


@gpu
def test_fast_single_step_with_sphere_and_moving_colliders_within_1e5(ctx):
    """Grid and particle collider projection (gForceCompute.glsl:72-93,
    particleAdvance.glsl:182-204) for a sphere (type 1) inside the snowball
    and a moving half-plane under it, after the rigid advance of both
    (rigidAdvance.glsl:14-18), against the FP64 oracle."""
    from snow_gb300 import native as N
    s = scenes.small_scene(n=5000, grid_edge=32, seed=34, v0=(0.5, -3.0, 0.2), center=(0.5, 0.3, 0.5))
    s.colliders.append(scenes.Collider(pos=(0.52, 0.28, 0.49), type=1, radius=0.06, vel=(0.0, 0.5, 0.0),
                                       friction=0.3))
    s.colliders.append(scenes.Collider(pos=(0.0, 0.2, 0.0), type=0, normal=(0.0, 1.0, 0.0), vel=(0.0, 1.0, 0.0),
                                       friction=0.1))
    g = sim(ctx, s, N.MODE_FAST).upload().init().step(s.dt, 1)
    o = _exact_oracle(s).upload().init()
    flip = o.step_with_flip_scale()
    check_step(g.download(), o.state(), flip, strict=False)
    assert np.abs(g.colliders() - o.colliders()).max() <= 1e-6


@gpu
def test_fast_step_with_particles_on_the_wide_path_within_1e5(ctx):
    """A snow block moving down at 2 m/s whose bottom layer starts inside a
    static sphere collider: in the first step the collider stops that
    snow, whose stress jumps from nothing to far past what the set-up's
    magnitudes allowed, so its particles' force contributions outgrow the
    fixed-point scales' fast range and are scattered with int64
    contributions rounded in double precision (the wide path;
    snow_phase_times.wide counts them). The step matches the FP64 oracle
    within the single-step bound."""
    from snow_gb300 import native as N
    s = scenes.snow_block_on_sphere(0x5EED0021, 32768, 64, gap=-3.0 / 64, v0=(0.0, -2.0, 0.0))
    g = sim(ctx, s, N.MODE_FAST).upload().init()
    y0 = g.download()
    g.phase_times(reset=True)
    y1 = g.step(s.dt, 1).download()
    wide = g.phase_times(reset=True)["wide"]
    o = _oracle_from_gpu_state(s, y0)
    flip = o.step_with_flip_scale()
    check_step(y1, o.state(), flip, strict=False)
    assert wide > 100, wide


def _deformed_restart(ctx, warm_steps, seed=41):
    """The FP64 oracle advanced `warm_steps` through an impact on the floor,
    then both the oracle and a FAST GPU scene restarted from its state
    (rounded to float32, with the initial volumes carried over)."""
    from snow_gb300 import native as N
    s = scenes.small_scene(n=4000, grid_edge=32, seed=seed, v0=(0.5, -6.0, 0.3), center=(0.5, 0.22, 0.5))
    warm = _exact_oracle(s).upload().init().step(n=warm_steps).state()
    s2 = scenes.Scene(**{k: getattr(s, k) for k in ("grid_pos", "grid_dim", "grid_spacing", "young", "poisson",
                                                    "hardening", "crit_compression", "crit_stretch", "alpha",
                                                    "gravity", "dt", "colliders")})
    s2.x = warm["x"].astype(np.float32)
    s2.v = warm["v"].astype(np.float32)
    s2.m = s.m.copy()
    fe = warm["FE"].astype(np.float32)
    fp = warm["FP"].astype(np.float32)
    rho = warm["rho"]
    assert np.abs(fe - np.eye(3)).max() > 1e-4, "the warm-up must deform the snow"
    o = _exact_oracle(s2).upload(FE=fe.astype(np.float64), FP=fp.astype(np.float64)).set_density(rho)
    g = sim(ctx, s2, N.MODE_FAST).upload(FE=fe.reshape(-1, 9), FP=fp.reshape(-1, 9))
    g.set_volume((s2.m / rho).astype(np.float32)).init()
    return s2, o, g


def _oracle_from_gpu_state(scene, y):
    """The FP64 oracle restarted from a FAST scene's downloaded state y (the
    colliders must be static: their advanced positions are not carried
    over). Only det F_P enters a step, so F_P = diag(J_p, 1, 1); the
    densities come from the particles' initial volumes."""
    n = len(y["x"])
    fp = np.zeros((n, 3, 3))
    fp[:, 0, 0] = y["Jp"]
    fp[:, 1, 1] = fp[:, 2, 2] = 1.0
    s3 = scenes.Scene(**{k: getattr(scene, k) for k in ("grid_pos", "grid_dim", "grid_spacing", "young",
                                                        "poisson", "hardening", "crit_compression", "crit_stretch",
                                                        "alpha", "gravity", "dt")})
    assert all(tuple(c.vel) == (0.0, 0.0, 0.0) for c in scene.colliders)
    s3.colliders = list(scene.colliders)
    s3.x, s3.v, s3.m = y["x"], y["v"], scene.m.copy()
    rho = np.where(y["volume"] > 0, s3.m.astype(np.float64) / np.maximum(y["volume"], 1e-30), 0.0)
    return _exact_oracle(s3).upload(FE=y["FE"].astype(np.float64), FP=fp).set_density(rho)


def _uneven_batch(n_scenes=8, seed=0x5EED0103):
    """Scenes drawn as the 64-scene batched workload draws them, at sizes the
    oracle steps in seconds: particle counts log-uniform in [2k, 30k],
    sphere or box, per-scene E0 ~ U[4.8e4, 1.4e5] and xi ~ U[5, 10], initial
    velocity |v| <= 4 m/s in a random direction, dt = 1e-4, grids of uneven
    edge (including edges that are not a multiple of the 4-node block)."""
    rng = np.random.default_rng(seed)
    edges = [48, 64, 50, 96, 72, 64, 41, 80, 56, 88][:n_scenes]
    out = []
    for i, edge in enumerate(edges):
        n = int(round(np.exp(rng.uniform(np.log(2000), np.log(30000)))))
        kind = "sphere" if i % 2 == 0 else "box"
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        v0 = tuple(float(c) for c in d * rng.uniform(0.5, 4.0))
        center = tuple(float(c) for c in 0.5 + rng.uniform(-0.05, 0.05, size=3))
        out.append(scenes.small_scene(n=n, grid_edge=edge, seed=seed * 100 + i, v0=v0, kind=kind, center=center,
                                      young=float(rng.uniform(4.8e4, 1.4e5)),
                                      hardening=float(rng.uniform(5.0, 10.0))))
    return out


@gpu
@pytest.mark.parametrize("warm", [0, 5])
def test_fast_batched_step_matches_the_oracle_per_scene(ctx, warm):
    """Eight uneven scenes advanced together by snow_batch_step (one launch
    per phase for all scenes, CUDA graph), each checked against the FP64
    oracle on its own: one step from the initial state (warm = 0), or one
    step after five batched steps, the oracle restarted from the GPU state
    (warm SVD frames, re-binned particles)."""
    from snow_gb300 import api, native as N
    scs = _uneven_batch()
    sims = [sim(ctx, s, N.MODE_FAST).upload().init() for s in scs]
    batch = api.Batch(ctx, sims)
    dts = [s.dt for s in scs]
    if warm:
        batch.step(warm, dts)
        oracles = [_oracle_from_gpu_state(s, g.download()) for s, g in zip(scs, sims)]
    else:
        oracles = [_exact_oracle(s).upload().init() for s in scs]
    flips = [o.step_with_flip_scale() for o in oracles]
    batch.step(1, dts)
    for s, g, o, flip in zip(scs, sims, oracles, flips):
        check_step(g.download(), o.state(), flip, strict=True)
    batch.close()
    for g in sims:
        g.close()


@gpu
@pytest.mark.parametrize("warm_steps", [5, 20])
def test_fast_single_step_from_deformed_state_within_1e5(ctx, warm_steps):
    s2, o, g = _deformed_restart(ctx, warm_steps)
    flip = o.step_with_flip_scale()
    g.step(s2.dt, 1)
    check_step(g.download(), o.state(), flip, strict=False)


@gpu
def test_fast_step_with_warm_svd_frames_within_1e5(ctx):
    """The FAST advance starts each particle's Jacobi eigen-solve from the
    frame of its previous SVD. Step the GPU once from a deformed state (the
    frames become warm), restart the FP64 oracle from the GPU's state after
    that step, and compare the next step of both."""
    s2, o, g = _deformed_restart(ctx, 20, seed=61)
    g.step(s2.dt, 1)
    o2 = _oracle_from_gpu_state(s2, g.download())
    flip = o2.step_with_flip_scale()
    g.step(s2.dt, 1)
    check_step(g.download(), o2.state(), flip, strict=False)


@gpu
def test_fast_grid_after_p2g_and_grid_update(ctx):
    from snow_gb300 import native as N
    s2, o, g = _deformed_restart(ctx, 20, seed=51)
    for kern, ph in [(N.K_RIGID_ADVANCE, O.PH_RIGID), (N.K_G_RESET, O.PH_RESET), (N.K_P2G, O.PH_P2G)]:
        g.dispatch(kern, s2.dt)
        o.phase(ph)
    gd, od = g.grid(), o.grid()
    mscale = od["mass"].max()
    assert np.abs(gd["mass"] - od["mass"]).max() <= REL_TOL * mscale
    assert abs(gd["mass"].sum() - s2.m.astype(np.float64).sum()) <= 1e-5 * s2.m.sum()
    pscale = np.abs(od["mom"]).max()
    assert np.abs(gd["mom"] - od["mom"]).max() <= REL_TOL * pscale
    # A node's force sums ~500 particle contributions that largely cancel;
    # its FP32 sum is good to ~1e-5 of the largest force, so the grid force
    # (an intermediate, not a particle field) is held to 1e-4 of it.
    fscale = np.abs(od["force"]).max()
    assert np.abs(gd["force"] - od["force"]).max() <= 1e-4 * fscale, (np.abs(gd["force"] - od["force"]).max(), fscale)
    g.dispatch(N.K_G_FORCE, s2.dt)
    o.phase(O.PH_GRID)
    # v* = p/m + dt (f/m + g). The P2G sums are fixed point: a node's m, p
    # and f carry an absolute rounding error (~1e-7 of the largest
    # contribution per contribution), so v* = p/m divides it by the node's
    # own mass. What a node hands its particles is its momentum m v*
    # (weighted by w, which is small wherever m is): m_i v*_i is compared with
    # the FP64 grid's to 1e-5 of the largest, and v* itself where the node
    # holds >= 10% of the peak node mass.
    vs = o.grid()["vstar"]
    gvs = g.grid()["vstar"]
    mref = od["mass"][:, None]
    pscale_v = np.abs(mref * vs).max()
    assert np.abs(mref * (gvs - vs)).max() <= REL_TOL * pscale_v, np.abs(mref * (gvs - vs)).max() / pscale_v
    heavy = od["mass"] >= 0.1 * mscale
    vscale = np.abs(vs[heavy]).max()
    assert np.abs(gvs[heavy] - vs[heavy]).max() <= REL_TOL * vscale, np.abs(gvs[heavy] - vs[heavy]).max() / vscale


@gpu
@pytest.mark.parametrize("which", ["small", "cfg1"])
def test_fast_short_horizon_bulk_statistics(ctx, which):
    """100 steps of a snowball (a small one, and the plain CPU-checkable
    workload itself: 32,768 particles in a 64^3 grid dropped at 2 m/s):
    trajectories diverge, bulk quantities agree with the FP64 oracle."""
    from snow_gb300 import native as N
    if which == "cfg1":
        s = scenes.cfg1_snowball()
    else:
        s = scenes.small_scene(n=8000, grid_edge=48, seed=61, v0=(0.0, -2.0, 0.0), center=(0.5, 0.3, 0.5))
    g = sim(ctx, s, N.MODE_FAST).upload().init().step(s.dt, 100)
    o = _exact_oracle(s).upload().init().step(n=100)
    st = g.stats()
    ref = o.state()
    m = s.m.astype(np.float64)
    com = (m[:, None] * ref["x"]).sum(0) / m.sum()
    mom = (m[:, None] * ref["v"]).sum(0)
    ke = 0.5 * (m * (ref["v"] ** 2).sum(1)).sum()
    assert st["nonfinite"] == 0
    assert np.abs(st["center_of_mass"] - com).max() <= 1e-4
    assert np.abs(st["momentum"] - mom).max() <= 1e-3 * np.abs(mom).max() + 1e-9
    assert abs(st["kinetic_energy"] - ke) <= 1e-3 * ke
    assert abs(st["mean_jp"] - ref["Jp"].mean()) <= 1e-4
    assert np.abs(st["bbox_min"] - ref["x"].min(0)).max() <= 1e-3
    assert np.abs(st["bbox_max"] - ref["x"].max(0)).max() <= 1e-3


@gpu
def test_reference_mode_cfg1_100_steps_tracks_the_faithful_oracle(ctx):
    """REFERENCE mode (the shaders' FP32 + int32 fixed-point arithmetic) on
    the plain CPU-checkable workload for its 100 steps, against the FP32
    fixed-point restatement: per-particle state stays within float rounding
    of the shader arithmetic (exp differs by ~2 ulp), far tighter than the
    FAST bound."""
    from snow_gb300 import native as N
    s = scenes.cfg1_snowball()
    g = sim(ctx, s, N.MODE_REFERENCE).upload_std140(*s.std140()).init().step(s.dt, 100)
    o = O.OracleSim(s, mode=O.FAITHFUL32).upload_std140(*s.std140()).init().step(n=100)
    got, ref = g.download(), o.state()
    assert np.abs(got["x"] - ref["x"]).max() <= 1e-5
    assert np.abs(got["v"] - ref["v"]).max() <= 1e-3 * max(1.0, np.abs(ref["v"]).max())
    assert np.abs(got["Jp"] - ref["Jp"]).max() <= 1e-4


# ---------------------------------------------------------------------------
@gpu
@pytest.mark.parametrize("steps", [0, 7])
def test_cell_keys_and_binning_bit_exact(ctx, steps):
    from snow_gb300 import native as N
    s = scenes.small_scene(n=20000, grid_edge=64, seed=71, v0=(1.0, -3.0, 2.0))
    g = sim(ctx, s, N.MODE_FAST).upload().init()
    if steps:
        g.step(s.dt, steps)
    x = g.download()["x"]
    keys, perm = g.cell_keys()
    lin, blk, cperm = O.cell_keys(x, s.grid_pos, s.grid_dim, s.grid_spacing)
    assert np.array_equal(keys, blk)
    assert np.array_equal(perm, cperm)


@gpu
def test_binning_edge_cases(ctx):
    """Particles outside the grid (clamped keys), duplicates, a single
    particle and a grid whose edge is not a multiple of the block size."""
    from snow_gb300 import native as N
    rng = np.random.default_rng(5)
    s = scenes.unit_box_scene(37, dt=1e-4)
    x = rng.uniform(-0.1, 1.1, size=(3001, 3)).astype(np.float32)
    x[1000:1010] = x[999]
    s.x, s.v, s.m = x, np.zeros_like(x), np.full(len(x), 1e-6, np.float32)
    g = sim(ctx, s, N.MODE_FAST).upload()
    g.init()
    keys, perm = g.cell_keys()
    _, blk, cperm = O.cell_keys(x, s.grid_pos, s.grid_dim, s.grid_spacing)
    assert np.array_equal(keys, blk) and np.array_equal(perm, cperm)
    one = scenes.unit_box_scene(16, dt=1e-4)
    one.x, one.v, one.m = x[:1].clip(0.3, 0.7), np.zeros((1, 3), np.float32), np.ones(1, np.float32) * 1e-4
    g1 = sim(ctx, one, N.MODE_FAST).upload().init().step(1e-4, 3)
    assert g1.stats()["nonfinite"] == 0
