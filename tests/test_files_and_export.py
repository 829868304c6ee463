"""Particle input from `x,y,z` files (the reference's
ParticleSystem::initParticlesFromFile) and headless position export. CPU
only, except the last test."""
import numpy as np
import pytest

from snow_gb300 import export, scenes


def test_xyz_file_places_particles_like_the_reference(tmp_path):
    p = tmp_path / "bunny.voxel"
    p.write_text("0.5,1.0,-2\n1e-1, 2.5 ,3\n-0.25,0,7.5e1\n")
    x, v, m = scenes.particles_from_xyz(str(p), pos=(1.0, 2.0, 3.0), scale=(2.0, 0.5, 1.0))
    want = np.array([[2.0, 2.5, 1.0], [1.2, 3.25, 6.0], [0.5, 2.0, 78.0]], np.float32)
    assert x.dtype == np.float32 and np.array_equal(x, want)
    assert np.all(v == 0) and np.all(m == np.float32(6.25e-3))


def test_xyz_parsing_follows_stof():
    assert scenes._stof("  1.5abc") == np.float32(1.5)
    assert scenes._stof("-2e-3,") == np.float32(-2e-3)
    with pytest.raises(ValueError):
        scenes._stof("abc")


def test_line_without_comma_repeats_its_number(tmp_path):
    p = tmp_path / "one.xyz"
    p.write_text("4.25\n")
    x, _, _ = scenes.particles_from_xyz(str(p))
    assert np.array_equal(x, np.array([[4.25, 4.25, 4.25]], np.float32))


def test_malformed_line_raises(tmp_path):
    p = tmp_path / "bad.xyz"
    p.write_text("1,2,3\nx,y,z\n")
    with pytest.raises(ValueError):
        scenes.particles_from_xyz(str(p))


def test_missing_file_yields_no_particles(tmp_path, capsys):
    x, v, m = scenes.particles_from_xyz(str(tmp_path / "nope.voxel"))
    assert x.shape == (0, 3) and v.shape == (0, 3) and m.shape == (0,)
    assert "not found" in capsys.readouterr().err


def test_add_particles_appends():
    s = scenes.unit_box_scene(32)
    scenes.add_particles(s, np.ones((2, 3)), np.zeros((2, 3)), np.full(2, 0.5))
    scenes.add_particles(s, np.zeros((1, 3)), np.ones((1, 3)), [1.0])
    assert s.n == 3 and s.m.tolist() == [0.5, 0.5, 1.0] and s.v[2].tolist() == [1.0, 1.0, 1.0]


@pytest.mark.parametrize("fmt", ["npy", "xyz"])
def test_exported_positions_read_back_exactly(tmp_path, fmt):
    rng = np.random.default_rng(3)
    x = rng.random((500, 3)).astype(np.float32) * np.float32(3.7) - np.float32(1.1)
    path = export.write_positions(str(tmp_path / f"f.{fmt}"), x)
    back = np.load(path) if fmt == "npy" else scenes.particles_from_xyz(path)[0]
    assert np.array_equal(back, x)


@pytest.mark.gpu
def test_exporter_writes_every_n_steps(tmp_path):
    from snow_gb300 import api
    ctx = api.Context(0)
    try:
        s = scenes.small_scene(n=2000, grid_edge=32, seed=31)
        sim = api.SimScene(ctx, s).upload().init()
        ex = export.PositionExporter(sim, str(tmp_path), every=4, fmt="xyz")
        files = ex.run(10, s.dt)
        assert [f[-10:] for f in files] == ["000000.xyz", "000004.xyz", "000008.xyz"]
        last = scenes.particles_from_xyz(files[-1])[0]
        ref = api.SimScene(ctx, s).upload().init().step(s.dt, 8).download()["x"]
        assert np.abs(last - ref).max() <= 1e-5
    finally:
        ctx.close()
