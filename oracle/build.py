"""ORACLE / TEST INFRASTRUCTURE ONLY -- builds the CPU checkers.

  * oracle/_build/liboracle.so : this project's restatement (snow_oracle.cpp).
  * oracle/_ref/liboracle_ref.so : the reference's GLSL compute shaders
    compiled as C++ (ref_translate.py). Translated from the reference tree
    when it is present; otherwise rebuilt from translated sources already in
    oracle/_ref/ (they travel with the working tree); otherwise skipped.
Both are compiled with -ffp-contract=off so x86-64 and AArch64 hosts give the
same FP32 results.
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
# The reference tree whose shaders are translated: $SNOW_REFERENCE_TREE, else
# the read-only checkout this recipe was written against.
REFERENCE_TREE = os.environ.get("SNOW_REFERENCE_TREE", "/root/reference")

CXXFLAGS = ["-O2", "-std=gnu++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-strict-aliasing"]


def _stale(target: str, sources) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    so = os.path.join(BUILD, "liboracle.so")
    srcs = [os.path.join(HERE, "snow_oracle.cpp"), os.path.join(HERE, "glsl_builtins.hpp")]
    if force or _stale(so, srcs):
        subprocess.check_call(["g++", *CXXFLAGS, "-shared", srcs[0], "-o", so])
    return so


def build_ref(force: bool = False):
    """Returns the path of liboracle_ref.so, or None when neither the
    reference tree nor translated sources are available."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("ref_translate", os.path.join(HERE, "ref_translate.py"))
    rt = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(rt)
    so = os.path.join(REF_OUT, "liboracle_ref.so")
    deps = [os.path.join(HERE, f) for f in ("ref_driver.cpp", "glsl_compat.hpp", "glsl_builtins.hpp",
                                            "ref_translate.py")]
    if os.path.isdir(os.path.join(REFERENCE_TREE, "shader", "compute")):
        if force or _stale(so, deps):
            rt.build(REFERENCE_TREE, REF_OUT, compile_=True)
        return so
    translated = [os.path.join(REF_OUT, f"{n}.cpp") for n in rt.SHADERS]
    if all(os.path.exists(t) for t in translated):
        if force or _stale(so, deps + translated):
            rt.compile_sources(REF_OUT)
        return so
    return None


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_ref(force=True))
