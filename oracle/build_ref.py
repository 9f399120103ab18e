#!/usr/bin/env python3
"""Build recipe for ``oracle/_ref/libdpm_ref.so``: the reference itself, on the CPU.

Test infrastructure only (the checker, never the product).  It compiles the
reference's own sources where they lie -- ``src/cell.cpp``, ``src/Tissue2D.cpp``,
``src/Tissue3D.cpp``, ``src/readKernel.cpp`` unmodified, plus the kernel text of
``shaders/Cell2D_kernel.cl`` and ``shaders/Cell3D_Kernel.cl`` -- against the
project-written CPU OpenCL shim in ``oracle/clshim``.

The kernel text gets one mechanical rewrite so that C++ accepts it: OpenCL
vector literals ``(float3)(a, b, c)`` become constructor calls
``float3(a, b, c)``.  The rewritten text is written only into ``oracle/_ref/``
(git-ignored) and wrapped in a namespace nested inside ``clc`` (see
``clshim/clc_prelude.hpp``).  Each kernel found by ``__kernel void NAME`` is
registered with the shim, together with a checksum of the original ``.cl``
file, which ``cl::Program::build`` compares against the text the reference
reads at run time.

Usage: ``python oracle/build_ref.py [--reference DIR]``.  Without a reference
tree (the GPU machines have none) it prints a notice and exits 0.
"""
from __future__ import annotations

import argparse
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
DEFAULT_REFERENCE = "/root/reference"

KERNEL_FILES = (("Cell2D_kernel.cl", "k2d"), ("Cell3D_Kernel.cl", "k3d"))
HOST_SOURCES = ("cell.cpp", "Tissue2D.cpp", "Tissue3D.cpp", "readKernel.cpp")

_VEC_LITERAL = re.compile(r"\((float|uint|int)([234])\)\(")
_KERNEL_NAME = re.compile(r"__kernel\s+void\s+(\w+)\s*\(")


def fnv1a(data: bytes) -> int:
    h = 1469598103934665603
    for c in data:
        h ^= c
        h = (h * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


def rewrite_kernel(src_path: str, namespace: str) -> str:
    raw = open(src_path, "rb").read()
    text = raw.decode("utf-8")
    body = _VEC_LITERAL.sub(lambda m: f"{m.group(1)}{m.group(2)}(", text)
    names = _KERNEL_NAME.findall(text)
    if not names:
        raise RuntimeError(f"no kernels found in {src_path}")
    lines = [
        "// Generated by oracle/build_ref.py from the reference kernel text; do not edit.",
        '#include "clc_prelude.hpp"',
        f"namespace clc {{ namespace {namespace} {{",
        f'#line 1 "{os.path.basename(src_path)}"',
        body,
        f"}} }} // namespace clc::{namespace}",
    ]
    for n in names:
        lines.append(f"CLSHIM_REGISTER(clc::{namespace}, {n})")
    lines.append(
        f"static cl::shim::SourceRegistrar clshim_src_{namespace}(0x{fnv1a(raw):016x}ull);"
    )
    return "\n".join(lines) + "\n"


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("DPM_REFERENCE_DIR", DEFAULT_REFERENCE))
    ap.add_argument("--cxx", default=os.environ.get("CXX", "g++"))
    args = ap.parse_args(argv)
    ref = args.reference
    if not os.path.isdir(os.path.join(ref, "src")) or not os.path.isdir(os.path.join(ref, "shaders")):
        print(f"build_ref: no reference tree at {ref}; oracle/_ref not built")
        return 0
    os.makedirs(OUT, exist_ok=True)
    gen = []
    for fname, ns in KERNEL_FILES:
        out = os.path.join(OUT, fname.replace(".cl", ".cpp"))
        with open(out, "w") as f:
            f.write(rewrite_kernel(os.path.join(ref, "shaders", fname), ns))
        gen.append(out)
    srcs = [os.path.join(ref, "src", s) for s in HOST_SOURCES]
    lib = os.path.join(OUT, "libdpm_ref.so")
    cmd = [
        args.cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-fno-strict-aliasing",
        "-fPIC", "-shared", "-w",
        "-I", os.path.join(HERE, "clshim"),
        "-I", os.path.join(ref, "include"),
        *srcs, *gen, os.path.join(HERE, "ref_driver.cpp"),
        "-o", lib,
    ]
    print("build_ref:", " ".join(cmd))
    subprocess.run(cmd, check=True)
    # The reference opens its kernel files relative to the working directory
    # (src/Tissue2D.cpp:38, src/Tissue3D.cpp:36); record where they are.
    with open(os.path.join(OUT, "reference_dir.txt"), "w") as f:
        f.write(os.path.abspath(ref) + "\n")
    print("build_ref: wrote", lib)
    return 0


if __name__ == "__main__":
    sys.exit(main())
