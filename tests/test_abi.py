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
    assert ctypes.sizeof(native.SnowParams) == 4 * (3 + 3 + 1 + 6 + 3 + 2)
