"""Build of the native libraries, in-tree, for sm_103a.

* ``libdpm_gb300.so``: the CUDA kernels, the runtime and the C ABI of
  ``include/dpm_gb300.h`` (nvcc, one ``-gencode`` for sm_103a).
* ``clDPM*.so``: the pybind11 module with the reference's Python API
  (``Cell2D``, ``Tissue2D``, ``Cell3D``, ``Tissue3D``), linked against the
  library above.  pybind11's headers come from PyTorch's include tree, which
  is present wherever PyTorch is, or from the pybind11 package.

Translation units are compiled in parallel; a unit is rebuilt only when its
source or a header is newer than its object file.
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libdpm_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    p = os.path.join(home, "bin", "nvcc")
    return p if os.path.exists(p) else "nvcc"


def _newest(paths) -> float:
    return max((os.path.getmtime(p) for p in paths), default=0.0)


def _headers():
    return (glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.hpp"))
            + glob.glob(os.path.join(CSRC, "host", "*.hpp"))
            + glob.glob(os.path.join(ROOT, "include", "*.h")))


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r


def pybind_includes():
    incs = []
    try:
        import torch.utils.cpp_extension as ce  # noqa: F401
        import torch
        tinc = os.path.join(os.path.dirname(torch.__file__), "include")
        if os.path.isdir(os.path.join(tinc, "pybind11")):
            incs.append(tinc)
    except Exception:
        pass
    if not incs:
        try:
            import pybind11
            incs.append(pybind11.get_include())
        except Exception:
            pass
    if not incs:
        raise RuntimeError("pybind11 headers not found (neither in PyTorch nor pybind11)")
    return incs + [sysconfig.get_paths()["include"]]


# The step kernels' plain float divisions and square roots (shape forces,
# geometry, winding face terms) need only the parity tolerance, so they take
# the approximate forms; every operation that must match the reference or a
# host rebuild bit for bit is written with explicit round-to-nearest
# intrinsics (__fdiv_rn, __fadd_rn, ...), which these flags leave alone, and
# denormals are kept.  The dispersion, the sort and the runtime keep IEEE
# division and square root throughout.
FAST_MATH_SOURCES = {"dpm2d_kernels.cu", "dpm2d_step_s1.cu", "dpm2d_step_s2.cu",
                     "dpm2d_step_s4.cu", "dpm2d_step_s8.cu", "dpm2d_step_s8_att.cu",
                     "dpm3d_kernels.cu"}


def _device_math(src: str) -> list:
    if os.path.basename(src) in FAST_MATH_SOURCES:
        return ["-prec-div=false", "-prec-sqrt=false"]
    return []


def build_library(verbose: bool = False, jobs: int = 8) -> str:
    os.makedirs(BUILD, exist_ok=True)
    cu = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    cpp = []
    hdr_time = _newest(_headers())
    jobs_list = []
    objs = []
    for src in cu + cpp:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), hdr_time):
            continue
        if src.endswith(".cu"):
            cmd = [nvcc(), *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-Xcompiler", "-ffp-contract=off", *_device_math(src),
                   "-I", os.path.join(ROOT, "include"), "-c", src, "-o", obj]
        else:
            cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-I", os.path.join(ROOT, "include"),
                   "-I", os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include"),
                   "-c", src, "-o", obj]
        jobs_list.append(cmd)
    if jobs_list:
        with ThreadPoolExecutor(max_workers=jobs) as ex:
            list(ex.map(lambda c: _run(c, verbose), jobs_list))
    if jobs_list or not os.path.exists(LIB):
        tmp = LIB + f".tmp{os.getpid()}"
        cuda_lib = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "lib64")
        _run([nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart",
              "-Xlinker", f"-rpath,{cuda_lib}"], verbose)
        os.replace(tmp, LIB)
    return LIB


def build_module(verbose: bool = False) -> str:
    """The clDPM module: the host classes (csrc/host/*.cpp) and their bindings."""
    srcs = sorted(glob.glob(os.path.join(CSRC, "host", "*.cpp")))
    if not srcs:
        return ""
    suffix = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    out = os.path.join(PKG, "clDPM" + suffix)
    deps = srcs + [LIB] + _headers()
    if os.path.exists(out) and os.path.getmtime(out) >= _newest(deps):
        return out
    tmp = out + f".tmp{os.getpid()}"
    incs = []
    for i in pybind_includes():
        incs += ["-I", i]
    # no FMA contraction: host geometry and dispersion reproduce the
    # reference's separately rounded float operations on x86 and Arm alike
    _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fvisibility=hidden",
          "-ffp-contract=off", *incs,
          "-I", os.path.join(ROOT, "include"), "-I", os.path.join(CSRC, "host"), *srcs,
          "-o", tmp, "-L", PKG, "-ldpm_gb300", "-Wl,-rpath,$ORIGIN"], verbose)
    os.replace(tmp, out)
    return out


def build(verbose: bool = False) -> None:
    build_library(verbose)
    build_module(verbose)


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(LIB)
