"""Known-answer and property tests of the oracle (CPU only).

The reference ships no tests; its only worked numbers are the comment
examples in shader/compute/lame/lame.include.glsl:8-9 (mu) and :22-23
(lambda, whose comment uses (1.9 - 2nu) where the code uses (1 - 2nu); the
values below follow the code)."""
import numpy as np
import pytest

from oracle import oracle as O
from snow_gb300 import scenes


def test_lame_comment_examples():
    mu, _ = O.lame(1.4e5, 0.2, 10.0, 1.1)
    assert abs(mu - 21459.63) < 0.02
    mu, _ = O.lame(1.4e5, 0.2, 10.0, 0.9)
    assert abs(mu - 158566.43) < 0.05


def test_lame_lambda_follows_code():
    _, lam = O.lame(1.4e5, 0.2, 10.0, 1.1)
    assert abs(lam - 14306.42) < 0.02
    _, lam = O.lame(1.4e5, 0.2, 10.0, 0.9)
    assert abs(lam - 105710.96) < 0.1


def _test_matrices(rng, n=400):
    a = rng.normal(size=(n, 3, 3))
    near_i = np.eye(3) + 1e-3 * rng.normal(size=(n, 3, 3))
    rot = np.linalg.qr(rng.normal(size=(n, 3, 3)))[0]
    degenerate = np.einsum("nij,njk->nik", rot, np.diag([2.0, 1.0, 0.0])[None])
    inverted = near_i.copy()
    inverted[:, :, 0] *= -1
    return np.concatenate([a, near_i, rot, degenerate, inverted, np.tile(np.eye(3), (4, 1, 1))])


@pytest.mark.parametrize("fp64", [True, False])
def test_svd_reconstruction_and_orthogonality(fp64):
    a = _test_matrices(np.random.default_rng(0))
    w, s, v = O.svd(a, fp64=fp64, vround=False)
    rec = np.einsum("nij,njk,nlk->nil", w, s, v)
    # The shader's constants (GAMMA, CSTAR, SSTAR) carry ~10 digits, so the
    # accumulated quaternion is unit only to ~1e-9 and V is orthogonal to
    # ~1e-8 even in FP64: that is the algorithm, not rounding.
    tol = 1e-7 if fp64 else 3e-5
    scale = np.maximum(np.abs(a).max((1, 2)), 1.0)
    assert (np.abs(rec - a).max((1, 2)) / scale).max() < tol
    for q in (w, v):
        e = np.abs(np.einsum("nji,njk->nik", q, q) - np.eye(3)).max()
        assert e < (1e-7 if fp64 else 3e-6)
        assert np.allclose(np.linalg.det(q), 1.0, atol=1e-5)
    # S is upper triangular (QR factor); its diagonal is sorted by magnitude.
    assert np.abs(np.tril(s, -1)).max() < (1e-12 if fp64 else 1e-5)
    d = np.abs(np.diagonal(s, axis1=1, axis2=2))
    assert np.all(d[:, 0] + 1e-6 >= d[:, 1]) and np.all(d[:, 1] + 1e-6 >= d[:, 2])


def test_svd_vround_matches_shader_rounding():
    a = _test_matrices(np.random.default_rng(1), 50)
    w, s, v = O.svd(a, fp64=True, vround=True)
    # V entries are multiples of 1e-5 before the sort (which only permutes
    # and negates columns).
    assert np.abs(v * 1e5 - np.round(v * 1e5)).max() < 1e-6


def test_exact64_conserves_mass_and_momentum():
    s = scenes.small_scene(n=3000, grid_edge=32, seed=3, v0=(0.3, -2.0, 0.1))
    o = O.OracleSim(s, mode=O.EXACT64).upload().init()
    o.phase(O.PH_RIGID)
    o.phase(O.PH_RESET)
    o.phase(O.PH_P2G)
    g = o.grid()
    m = s.m.astype(np.float64)
    assert abs(g["mass"].sum() - m.sum()) / m.sum() < 1e-12
    p_expect = (m[:, None] * s.v.astype(np.float64)).sum(0)
    assert np.allclose(g["mom"].sum(0), p_expect, rtol=1e-12, atol=1e-15)
    # sum_i grad w_ip = 0 for interior particles: the stress forces cancel.
    fsum = np.abs(g["force"].sum(0)).max()
    assert fsum <= 1e-10 * max(np.abs(g["force"]).sum(), 1e-30)


def test_faithful32_close_to_exact64():
    s = scenes.small_scene(n=2000, grid_edge=32, seed=5)
    a = O.OracleSim(s, mode=O.FAITHFUL32).upload_std140(*s.std140()).init().step()
    b = O.OracleSim(s, mode=O.EXACT64).upload().init().step()
    sa, sb = a.state(), b.state()
    assert np.abs(sa["x"] - sb["x"]).max() < 1e-6
    assert np.abs(sa["v"] - sb["v"]).max() < 2e-3
    assert np.abs(sa["FE"] - sb["FE"]).max() < 1e-4


def test_cell_keys_and_stable_binning():
    s = scenes.small_scene(n=5000, grid_edge=40, seed=2)
    lin, blk, perm = O.cell_keys(s.x, s.grid_pos, s.grid_dim, s.grid_spacing)
    c = np.trunc((s.x - np.float32(0.0)) / np.float32(s.grid_spacing)).astype(np.int64)
    c = np.clip(c, 0, np.array(s.grid_dim) - 1)
    assert np.array_equal(lin, c[:, 0] + c[:, 1] * 40 + c[:, 2] * 40 * 40)
    bx = (40 + 3) // 4
    b = ((c[:, 2] >> 2) * bx + (c[:, 1] >> 2)) * bx + (c[:, 0] >> 2)
    assert np.array_equal(blk, b * 64 + (c[:, 0] & 3) + 4 * (c[:, 1] & 3) + 16 * (c[:, 2] & 3))
    assert np.array_equal(perm, np.argsort(blk, kind="stable"))
