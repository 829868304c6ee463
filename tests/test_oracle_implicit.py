"""The oracle's semi-implicit velocity update (CPU only).

The reference declares SemiImplicitTimeUpdate and leaves it empty
(src/snow/simulation/timeUpdate/semiimplicittimeupdate.cpp:3-5), so there is
nothing of the reference's to pin it to. These tests pin the oracle's
restatement of Stomakhin et al. 2013 (eq. 9) by its defining properties:
K is the derivative of the explicit force (central differences of the force
with the deformation applied), K is symmetric and annihilates translations,
and the solve returns v with (M + beta dt^2 K) v = M v* to its tolerance."""
import numpy as np
import pytest

from oracle import oracle as O
from snow_gb300 import scenes


def _stiff_oracle(seed=5, n=1500, young=1.4e7):
    s = scenes.small_scene(n=n, grid_edge=24, seed=seed, young=young)
    rng = np.random.default_rng(seed)
    FE = np.eye(3)[None] + 3e-3 * rng.normal(size=(n, 3, 3))
    FP = np.eye(3)[None] + 1e-2 * rng.normal(size=(n, 3, 3))
    o = O.OracleSim(s, O.EXACT64, vround=False, qround=False).upload(FE=FE, FP=FP).init()
    o.phase(O.PH_RESET)
    o.phase(O.PH_P2G)
    return s, o, rng


def _active_field(o, rng):
    act = o.grid()["mass"] > 0
    return rng.normal(size=(o.G, 3)) * act[:, None]


def test_hessian_is_symmetric_and_annihilates_translations():
    _, o, rng = _stiff_oracle()
    u, w = _active_field(o, rng), _active_field(o, rng)
    a, b = np.sum(w * o.hessian(u)), np.sum(u * o.hessian(w))
    assert abs(a - b) <= 1e-10 * max(abs(a), abs(b))
    act = o.grid()["mass"] > 0
    shift = np.tile([0.3, -1.2, 0.7], (o.G, 1)) * act[:, None]
    ku = o.hessian(u)
    # the stencil of a particle can reach massless nodes only with zero weight and gradient
    assert np.abs(o.hessian(shift)).max() <= 1e-9 * np.abs(ku).max()


def test_hessian_is_the_derivative_of_the_force():
    _, o, rng = _stiff_oracle()
    u = _active_field(o, rng)
    ku = o.hessian(u)
    scale = np.abs(ku).max()
    errs = []
    for eps in (1e-3, 1e-4):
        fd = -(o.force_at(u, eps) - o.force_at(u, -eps)) / (2 * eps)
        errs.append(np.abs(fd - ku).max() / scale)
    assert errs[-1] <= 1e-6, errs
    assert errs[0] <= 1e-5, errs


def test_undeformed_force_is_the_explicit_force():
    _, o, rng = _stiff_oracle()
    f0 = o.force_at(np.zeros((o.G, 3)), 0.0)
    f = o.grid()["force"]
    # only the polar rotation differs (exact here, the shaders' approximate SVD there)
    assert np.abs(f0 - f).max() <= 1e-3 * np.abs(f).max()


def _solve(beta, tol=1e-10, max_iters=200, dt=5e-3, young=1.4e7):
    """One P2G and grid update of a snowball with random particle velocities
    (a rough v*, on which the implicit term acts strongly), then the solve."""
    s = scenes.small_scene(n=3000, grid_edge=32, seed=5, young=young)
    s.v = np.random.default_rng(3).normal(size=(s.n, 3)).astype(np.float32)
    o = O.OracleSim(s, O.EXACT64, vround=False, qround=False).upload().init()
    o.phase(O.PH_RESET)
    o.phase(O.PH_P2G)
    o.phase(O.PH_GRID, dt)
    g = o.grid()
    vstar, m = g["vstar"].copy(), g["mass"]
    o.set_implicit(beta, tol, max_iters)
    o.phase(O.PH_IMPLICIT, dt)
    v = o.grid()["vstar"]
    return o, m, vstar, v, o.solver_report()


def test_solve_satisfies_the_implicit_system():
    beta, dt = 1.0, 5e-3
    o, m, vstar, v, rep = _solve(beta, dt=dt)
    c = beta * float(np.float32(dt)) ** 2
    live = m > 0
    sq = np.sqrt(np.where(live, m, 0.0))[:, None]
    # the residual of the mass-scaled system M^-1/2 ((M + c K) v - M v*)
    res = np.where(live[:, None], (m[:, None] * (v - vstar) + c * o.hessian(v)) / np.where(sq > 0, sq, 1), 0)
    scale = np.linalg.norm(sq * vstar)
    assert rep["initial_residual"] > 0.1  # the implicit term matters in this scene
    assert 1 < rep["iterations"] < 100
    assert rep["residual"] <= 1e-10
    assert np.linalg.norm(res) <= 1e-8 * scale
    # K u sums to zero over the grid: the solve keeps the total momentum
    assert np.abs((m[:, None] * (v - vstar)).sum(0)).max() <= 1e-8 * np.abs(m[:, None] * vstar).sum()
    # backward Euler on a positive-definite K would not raise the kinetic energy
    assert np.sum(m[:, None] * v * v) <= np.sum(m[:, None] * vstar * vstar) * (1 + 1e-9)


def test_zero_beta_keeps_the_explicit_velocity():
    o, m, vstar, v, rep = _solve(0.0)
    assert np.array_equal(v, vstar)
    assert rep["iterations"] == 0


@pytest.mark.parametrize("beta", [0.5, 1.0])
def test_implicit_steps_stay_finite(beta):
    s = scenes.small_scene(n=2000, grid_edge=24, seed=11, young=1.4e7)
    o = O.OracleSim(s, O.EXACT64).upload().init().set_implicit(beta, 1e-6, 100)
    o.step(5e-3, 3)
    st = o.state()
    assert np.all(np.isfinite(st["x"])) and np.all(np.isfinite(st["v"]))
    assert o.solver_report()["residual"] <= 1e-6
