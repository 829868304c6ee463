"""ORACLE / TEST INFRASTRUCTURE ONLY -- the recipe that compiles the snow
reference's own GLSL compute shaders as C++ for the host cores.

The reference runs its MPM step as GLSL 4.40 compute shaders
(shader/compute/mpm/*.glsl and their #includes). No OpenGL stack exists
on these machines, so instead of running the shaders through an OpenGL
implementation this recipe turns each shader into a C++ translation unit and compiles it against
oracle/glsl_compat.hpp, which gives the GLSL types and built-ins their GLSL
meaning. The kernel bodies are not edited: only declarations change.

Mechanical rewrites (nothing else):
  * #include "shader/..." is expanded from the reference tree. The missing
    "shader/compute/lame/snow.include.glsl" (included by p2gTransfer.glsl:41,
    absent from the tree) is resolved to lame/lame.include.glsl, the only
    file that defines the mu()/lambda() it calls.
  * comments and "#version" / "layout(local_size...) in;" lines are removed
    (the local size is kept for the dispatch loop).
  * "uniform T name;" becomes a namespace-scope variable set per dispatch.
  * "layout(std140, binding = B) buffer Blk { T name[ ]; };" becomes a
    namespace-scope pointer "T* name" bound to binding point B per dispatch.
  * "inout T name" parameters become "T& name".
  * float literals without a suffix get "f" (GLSL literals are float; C++
    literals would be double).
  * everything else (globals with initialisers, functions, main) becomes the
    body of a struct Invocation, one instance per invocation, so each
    invocation gets fresh private globals as in GLSL.

Outputs go only to oracle/_ref/ (git-ignored): one .cpp per shader and, when
compiled, liboracle_ref.so together with oracle/ref_driver.cpp.

Usage: python oracle/ref_translate.py [--reference DIR] [--out DIR] [--compile]
"""
from __future__ import annotations

import argparse
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference tree: --reference DIR, else $SNOW_REFERENCE_TREE, else the
# read-only checkout this recipe was written against.
DEFAULT_REF = os.environ.get("SNOW_REFERENCE_TREE", "/root/reference")
SHADERS = [
    "gReset", "rigidAdvance", "gMassCompute", "pVolumeCompute",
    "p2gTransfer", "gForceCompute", "g2pTransfer", "particleAdvance",
]
INCLUDE_REMAP = {
    "shader/compute/lame/snow.include.glsl": "shader/compute/lame/lame.include.glsl",
}
UNIFORM_ASSIGN = {
    ("vec3", "gGridPos"): "gGridPos = vec3(u->gGridPos[0], u->gGridPos[1], u->gGridPos[2]);",
    ("ivec3", "gGridDim"): "gGridDim = ivec3(u->gGridDim[0], u->gGridDim[1], u->gGridDim[2]);",
}
SCALAR_UNIFORMS = {"gridSpacing", "young", "poisson", "hardening", "critComp",
                   "critStretch", "dt", "indexSize", "gNumColliders"}


def expand_includes(path: str, ref_root: str, seen=None) -> str:
    seen = set() if seen is None else seen
    with open(path) as f:
        src = f.read()
    out = []
    for line in src.splitlines():
        m = re.match(r'\s*#include\s+"([^"]+)"', line)
        if m:
            inc = INCLUDE_REMAP.get(m.group(1), m.group(1))
            inc_path = os.path.join(ref_root, inc)
            if not os.path.exists(inc_path):
                raise FileNotFoundError(f"{path}: include {m.group(1)} not found")
            if inc_path in seen:
                continue
            seen.add(inc_path)
            out.append(expand_includes(inc_path, ref_root, seen))
        else:
            out.append(line)
    return "\n".join(out)


def strip_comments(src: str) -> str:
    """Remove comments the way the C preprocessor does: scanning left to
    right, whichever of // or /* comes first wins (SVD.include.glsl ends in
    "//* ... *//", a line comment)."""
    out = []
    i, n = 0, len(src)
    while i < n:
        if src.startswith("//", i):
            j = src.find("\n", i)
            i = n if j < 0 else j
        elif src.startswith("/*", i):
            j = src.find("*/", i + 2)
            out.append(" ")
            i = n if j < 0 else j + 2
        else:
            out.append(src[i])
            i += 1
    return "".join(out)


_FLOAT_LIT = re.compile(
    r"(?<![\w.])((?:\d+\.\d*|\.\d+)(?:[eE][+-]?\d+)?|\d+[eE][+-]?\d+)(?![\w.])")


def suffix_float_literals(src: str) -> str:
    # Literals already carrying an f suffix do not match: the lookahead
    # rejects a following word character.
    return _FLOAT_LIT.sub(lambda m: m.group(1) + "f", src)


def translate(name: str, ref_root: str) -> str:
    path = os.path.join(ref_root, "shader", "compute", "mpm", name + ".glsl")
    src = strip_comments(expand_includes(path, ref_root))
    src = re.sub(r"^\s*#version[^\n]*", "", src, flags=re.M)

    m = re.search(r"layout\s*\(\s*local_size_x\s*=\s*(\d+)\s*,\s*local_size_y\s*=\s*(\d+)"
                  r"\s*,\s*local_size_z\s*=\s*(\d+)\s*\)\s*in\s*;", src)
    if not m:
        raise ValueError(f"{name}: no local_size layout")
    local = tuple(int(g) for g in m.groups())
    src = src[:m.start()] + src[m.end():]

    buffers = []  # (binding, type, var)

    def _buf(mm):
        buffers.append((int(mm.group(1)), mm.group(3), mm.group(4)))
        return ""

    src = re.sub(r"layout\s*\(\s*std140\s*,\s*binding\s*=\s*(\d+)\s*\)\s*buffer\s+(\w+)\s*\{\s*"
                 r"(\w+)\s+(\w+)\s*\[\s*\]\s*;\s*\}\s*;", _buf, src)

    uniforms = []  # (type, name)

    def _uni(mm):
        uniforms.append((mm.group(1), mm.group(2)))
        return ""

    src = re.sub(r"\buniform\s+(\w+)\s+(\w+)\s*;", _uni, src)
    src = re.sub(r"\binout\s+(\w+)\s+(\w+)", r"\1& \2", src)
    src = suffix_float_literals(src)
    for bad in (r"\bout\s+\w+\s+\w+\s*[,)]", r"\bbuffer\b", r"\buniform\b", r"\blayout\b"):
        if re.search(bad, src):
            raise ValueError(f"{name}: untranslated construct matching {bad!r}")

    ns = f"ref_{name}"
    lines = [
        "// Generated by oracle/ref_translate.py from the snow reference's",
        f"// shader/compute/mpm/{name}.glsl (and its includes). Do not edit; do not commit.",
        '#include "glsl_compat.hpp"',
        f"namespace {ns} {{",
        "using namespace glslc;",
    ]
    for t, n in uniforms:
        lines.append(f"{t} {n};")
    for b, t, v in buffers:
        lines.append(f"{t}* {v} = nullptr;  // binding {b}")
    lines.append("struct Invocation {")
    lines.append("uvec3 gl_GlobalInvocationID;")
    lines.append(src)
    lines.append("};")
    lines.append(f"}}  // namespace {ns}")
    lines.append("")
    lines.append(f'extern "C" void snowref_dispatch_{name}(const RefBindings* b, const RefUniforms* u,')
    lines.append("    unsigned gx, unsigned gy, unsigned gz, int threads) {")
    lines.append(f"  using namespace {ns};")
    lines.append("  using namespace glslc;")
    for b, t, v in buffers:
        lines.append(f"  {v} = static_cast<{t}*>(b->ptr[{b}]);")
    for t, n in uniforms:
        if (t, n) in UNIFORM_ASSIGN:
            lines.append("  " + UNIFORM_ASSIGN[(t, n)])
        elif n in SCALAR_UNIFORMS:
            lines.append(f"  {n} = u->{n};")
        else:
            raise ValueError(f"{name}: unknown uniform {t} {n}")
    lx, ly, lz = local
    lines += [
        f"  const unsigned long long X = (unsigned long long)gx * {lx}ull;",
        f"  const unsigned long long Y = (unsigned long long)gy * {ly}ull;",
        f"  const unsigned long long Z = (unsigned long long)gz * {lz}ull;",
        "  const long long total = (long long)(X * Y * Z);",
        "  #pragma omp parallel for schedule(static) num_threads(threads > 0 ? threads : 1) if (threads > 1)",
        "  for (long long t = 0; t < total; ++t) {",
        "    Invocation inv;",
        "    inv.gl_GlobalInvocationID.x = (uint)((unsigned long long)t % X);",
        "    inv.gl_GlobalInvocationID.y = (uint)(((unsigned long long)t / X) % Y);",
        "    inv.gl_GlobalInvocationID.z = (uint)((unsigned long long)t / (X * Y));",
        "    inv.main();",
        "  }",
        "}",
        "",
    ]
    return "\n".join(lines)


CXXFLAGS = ["-O2", "-std=gnu++17", "-fPIC", "-fopenmp", "-ffp-contract=off",
            "-fno-strict-aliasing", "-w"]


def build(ref_root: str, out_dir: str, compile_: bool = True) -> str:
    os.makedirs(out_dir, exist_ok=True)
    cpps = []
    for name in SHADERS:
        code = translate(name, ref_root)
        p = os.path.join(out_dir, f"{name}.cpp")
        with open(p, "w") as f:
            f.write(code)
        cpps.append(p)
    so = os.path.join(out_dir, "liboracle_ref.so")
    if compile_:
        compile_sources(out_dir)
    return so


def compile_sources(out_dir: str) -> str:
    """Compile the translated sources already in out_dir (no reference tree
    needed) together with ref_driver.cpp into liboracle_ref.so."""
    cpps = [os.path.join(out_dir, f"{n}.cpp") for n in SHADERS]
    missing = [c for c in cpps if not os.path.exists(c)]
    if missing:
        raise FileNotFoundError(f"translated shaders missing: {missing}")
    so = os.path.join(out_dir, "liboracle_ref.so")
    objs = []
    procs = []
    for src in cpps + [os.path.join(HERE, "ref_driver.cpp")]:
        obj = os.path.join(out_dir, os.path.basename(src)[:-4] + ".o")
        objs.append(obj)
        procs.append(subprocess.Popen(["g++", *CXXFLAGS, "-I", HERE, "-c", src, "-o", obj]))
    for p in procs:
        if p.wait() != 0:
            raise RuntimeError("compiling the translated reference shaders failed")
    subprocess.check_call(["g++", "-shared", "-fopenmp", *objs, "-o", so])
    return so


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=DEFAULT_REF)
    ap.add_argument("--out", default=os.path.join(HERE, "_ref"))
    ap.add_argument("--compile", action="store_true")
    a = ap.parse_args(argv)
    so = build(a.reference, a.out, a.compile)
    print(so if a.compile else a.out)


if __name__ == "__main__":
    sys.exit(main())
