"""CPU checks of the C ABI: the library builds for sm_103a, loads without a
GPU and exports every function include/snow_mpm.h declares; the Python
bindings cover the same list. No compute calls."""
import ctypes
import os
import re
import shutil

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "snow_mpm.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    return sorted(set(re.findall(r"\b(snow_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib_path():
    if shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"):
        pytest.skip("nvcc unavailable")
    from snow_gb300 import build
    return build.build()


def test_header_declares_the_documented_entry_points():
    names = declared_functions()
    for must in ("snow_scene_create", "snow_scene_upload", "snow_scene_init", "snow_scene_step", "snow_dispatch",
                 "snow_scene_download", "snow_batch_step", "snow_scene_cell_keys"):
        assert must in names


def test_library_exports_every_declared_symbol(lib_path):
    lib = ctypes.CDLL(lib_path)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_bindings_cover_the_header():
    from snow_gb300 import native
    assert sorted(native.EXPORTS) == declared_functions()


def test_struct_layouts_match_the_header():
    from snow_gb300 import native
    # snow_collider is the reference's cx, cv, cn vec4 triple: 48 bytes
    assert ctypes.sizeof(native.SnowCollider) == 48
    assert ctypes.sizeof(native.SnowParams) == 4 * (3 + 3 + 1 + 6 + 3 + 2 + 3)


def test_ctypes_structs_match_the_c_compiler_layout(tmp_path):
    """Every struct of the header, laid out by gcc, against its ctypes twin:
    size and each field's offset."""
    if shutil.which("gcc") is None:
        pytest.skip("gcc unavailable")
    import subprocess
    from snow_gb300 import native as N
    pairs = {"snow_params": N.SnowParams, "snow_collider": N.SnowCollider, "snow_stats": N.SnowStats,
             "snow_phase_times": N.SnowPhaseTimes, "snow_tuning": N.SnowTuning,
             "snow_server_config": N.SnowServerConfig, "snow_job_desc": N.SnowJobDesc,
             "snow_job_result": N.SnowJobResult, "snow_server_report": N.SnowServerStats,
             "snow_solver_report": N.SnowSolverReport}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "snow_mpm.h"', "int main(void) {"]
    for cname, ct in pairs.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in ct._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("  return 0;\n}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = {}
    for line in subprocess.check_output([str(exe)], text=True).splitlines():
        a, b, v = line.split()
        got[(a, b)] = int(v)
    for cname, ct in pairs.items():
        assert got[(cname, "size")] == ctypes.sizeof(ct), cname
        for fname, _ in ct._fields_:
            assert got[(cname, fname)] == getattr(ct, fname).offset, (cname, fname)
