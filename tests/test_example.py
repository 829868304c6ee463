"""The C++ drop-in example (examples/cuda_explicit_time_update.cpp) builds
against include/snow_mpm.h and the library with a plain C++ compiler; on a
GPU it runs the reference's default world for 100 steps."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _build(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ unavailable")
    from snow_gb300 import build
    lib = build.build()
    exe = str(tmp_path / "explicit_step")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "examples", "cuda_explicit_time_update.cpp"),
                           "-L", os.path.dirname(lib), "-lsnow_gb300", "-Wl,-rpath," + os.path.dirname(lib),
                           "-o", exe])
    return exe


def test_example_compiles_and_links(tmp_path):
    assert os.path.exists(_build(tmp_path))


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["", "--semi-implicit"])
def test_example_runs_the_default_world(tmp_path, mode):
    out = subprocess.run([_build(tmp_path), "100"] + ([mode] if mode else []), capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "nonfinite 0" in out.stdout
    if mode:
        assert "semi-implicit" in out.stdout and "last solve" in out.stdout
