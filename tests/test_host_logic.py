"""Host-only logic, run without a GPU: the C ABI's defaults of defines.hpp,
the reference world's walls, the device footprint bound the serving loop
admits jobs by, parameter validation, and the bench's oracle check."""
import ctypes

import pytest


@pytest.fixture(scope="module")
def L():
    import shutil
    import os
    if shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"):
        pytest.skip("nvcc unavailable")
    from snow_gb300 import build, native
    build.build()
    lib = native.load()
    lib.snow_scene_footprint.restype = ctypes.c_size_t
    return lib


def _params(L, **kw):
    from snow_gb300 import native as N
    p = N.SnowParams()
    L.snow_params_default(ctypes.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def test_defaults_follow_defines_hpp(L):
    from snow_gb300 import native as N
    p = _params(L)
    # defines.hpp:14-54
    assert [round(v, 4) for v in p.grid_pos] == [0.5125, 0.5125, 1.5125]
    assert list(p.grid_dim) == [201, 201, 201]
    assert abs(p.grid_spacing - 0.05) < 1e-7
    assert p.young == pytest.approx(6e6) and p.poisson == pytest.approx(0.2)
    assert p.hardening == pytest.approx(30.0) and p.alpha == pytest.approx(0.95)
    assert p.mode == N.MODE_FAST and p.implicit_beta == 0.0
    walls = (N.SnowCollider * 6)()
    assert L.snow_default_walls(ctypes.byref(p), walls) == 6
    # half-planes 4 nodes inside each face, normals pointing inwards
    assert all(w.type == 0 for w in walls)
    assert sum(abs(sum(w.normal)) for w in walls) == pytest.approx(6.0)


def test_footprint_bounds_grow_with_particles_and_the_solver(L):
    from snow_gb300 import native as N
    p = _params(L, grid_dim=(128, 128, 128), grid_spacing=1.0 / 128)
    small = L.snow_scene_footprint(ctypes.byref(p), 100000)
    large = L.snow_scene_footprint(ctypes.byref(p), 1000000)
    assert 0 < small < large
    # per particle: streams, binning scratch, staging (~300 B)
    assert 250 * 900000 <= large - small <= 400 * 900000
    imp = _params(L, grid_dim=(128, 128, 128), grid_spacing=1.0 / 128, implicit_beta=1.0)
    nb = 32 ** 3
    extra = L.snow_scene_footprint(ctypes.byref(imp), 100000) - small
    assert nb * 64 * 60 <= extra <= nb * 64 * 60 + 8192  # solver planes per pool block + scalars
    ref = _params(L, grid_dim=(128, 128, 128), grid_spacing=1.0 / 128, mode=N.MODE_REFERENCE)
    assert L.snow_scene_footprint(ctypes.byref(ref), 100000) > 0


@pytest.mark.parametrize("field,value", [("grid_spacing", 0.0), ("implicit_beta", 1.5), ("implicit_beta", -0.1),
                                         ("implicit_max_iters", 129), ("implicit_tolerance", float("nan")),
                                         ("mode", 7)])
def test_invalid_parameters_have_no_footprint(L, field, value):
    p = _params(L)
    setattr(p, field, value)
    assert L.snow_scene_footprint(ctypes.byref(p), 1000) == 0


def test_bench_oracle_check_on_an_oracle_state():
    """The bench's full-size check (one FP64 oracle step restarted from a
    state, against a given next state) on CPU, with the oracle's own FP32-
    rounded steps standing in for the GPU's: within 1e-5, and the reported
    fields are the parity tests' (x, v with the strict floor, v against the
    FLIP update's scale, F_E, J_p)."""
    import numpy as np
    import bench
    from oracle import oracle as O
    from snow_gb300 import scenes
    s = scenes.small_scene(n=2000, grid_edge=24, seed=3, v0=(0.0, -2.0, 0.0))
    o = O.OracleSim(s, mode=O.EXACT64).upload().init().step(n=3)

    def f32(st, vol=None):
        d = dict(x=st["x"].astype(np.float32), v=st["v"].astype(np.float32), FE=st["FE"].astype(np.float32),
                 Jp=np.linalg.det(st["FP"]).astype(np.float32))
        if vol:
            d["volume"] = (s.m / st["rho"]).astype(np.float32)
        return d

    y0 = f32(o.state(), vol=True)
    y1 = f32(o.step().state())
    r = bench.oracle_check(s, (y0, y1))
    assert set(r["max"]) == {"x", "v", "v_flip", "FE", "Jp"}
    assert r["within_tolerance"] and r["strict_v_within_tolerance"] and max(r["max"].values()) < 1e-6, r["max"]
