"""ORACLE build recipe — test infrastructure only.

* ``build_oracle()`` compiles this directory's C restatement
  (myers_oracle.c) into ``oracle/_build/liborc.so`` with gcc. It runs here
  and on the GPU host (the .so is rebuilt there; nothing compiled on one
  machine is used on the other).
* ``build_ref_cuda()`` compiles the reference's OWN CUDA kernels
  (csrc/gpu_kernels.cu with csrc/gpu_myers.cuh), where they lie, into
  ``oracle/_ref/ref_gpu_kernels.cubin`` for sm_103a with nvcc, so that
  ``oracle/ref_cuda.py`` can time them on the same GB300 with the launch
  geometry of bitlev/gpu.py (CuPy, the reference's own launcher, is not
  installable offline). The cubin is device code, the same on x86 and Arm
  hosts, so one built here serves the GPU host too.
* ``build_ref()`` compiles the reference's OWN CPU sources, where they lie in
  the read-only reference checkout, into ``oracle/_ref/`` (git-ignored):
  ``libmyers.so`` (csrc/myers.c), the CPython extension ``_edpy`` that
  bitlev's CPU API imports (csrc/edpy.c, which includes myers.c) and
  ``libgpucheck.so`` (csrc/gpu_hostcheck.cpp, the reference's host build of
  its GPU device functions).  No reference source is copied: gcc reads the
  files in place.  Portable flags only (no -march/-mcpu=native), unlike the
  reference's Makefile:1-46 which tunes for the build machine.

Usage:  python oracle/build_oracle.py [oracle|ref|all]
"""
from __future__ import annotations

import os
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
# the reference checkout: BLG_REFERENCE_ROOT, else a sibling directory
# named "reference" next to this repository
REF_SRC = os.environ.get("BLG_REFERENCE_ROOT") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")
CC = os.environ.get("CC", "gcc")
CXX = os.environ.get("CXX", "g++")


def _run(cmd):
    subprocess.run(cmd, check=True)


def _stale(target, *sources) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def oracle_lib_path() -> str:
    return os.path.join(BUILD, "liborc.so")


def build_oracle(force: bool = False) -> str:
    src = os.path.join(HERE, "myers_oracle.c")
    out = oracle_lib_path()
    if force or _stale(out, src):
        os.makedirs(BUILD, exist_ok=True)
        tmp = out + f".{os.getpid()}.tmp"
        _run([CC, "-O2", "-fPIC", "-shared", "-std=c11", "-pthread", "-Wall", "-Wextra",
              "-o", tmp, src])
        os.replace(tmp, out)
    return out


def ref_available() -> bool:
    return os.path.exists(os.path.join(REF_SRC, "csrc", "myers.c"))


def ref_paths() -> dict:
    suffix = sysconfig.get_config_var("EXT_SUFFIX")
    return {"libmyers": os.path.join(REF_OUT, "libmyers.so"),
            "edpy": os.path.join(REF_OUT, "_edpy" + suffix),
            "gpucheck": os.path.join(REF_OUT, "libgpucheck.so")}


def ref_cuda_cubin() -> str:
    return os.path.join(REF_OUT, "ref_gpu_kernels.cubin")


def build_ref_cuda(force: bool = False) -> str:
    """Compile the reference's CUDA kernels in place into a sm_103a cubin."""
    if not ref_available():
        raise FileNotFoundError(f"reference checkout not found at {REF_SRC}")
    csrc = os.path.join(REF_SRC, "csrc")
    src = os.path.join(csrc, "gpu_kernels.cu")
    out = ref_cuda_cubin()
    if force or _stale(out, src, os.path.join(csrc, "gpu_myers.cuh")):
        os.makedirs(REF_OUT, exist_ok=True)
        nvcc = os.environ.get("NVCC") or "/usr/local/cuda/bin/nvcc"
        tmp = out + f".{os.getpid()}.tmp"
        # the reference's NVRTC options are -std=c++17 -I<csrc> (bitlev/gpu.py:44-51)
        _run([nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
              f"-I{csrc}", "-o", tmp, src])
        os.replace(tmp, out)
    return out


def build_ref(force: bool = False) -> dict:
    """Compile the reference's CPU sources in place into oracle/_ref/."""
    if not ref_available():
        raise FileNotFoundError(f"reference checkout not found at {REF_SRC}")
    csrc = os.path.join(REF_SRC, "csrc")
    paths = ref_paths()
    os.makedirs(REF_OUT, exist_ok=True)
    myers = os.path.join(csrc, "myers.c")
    if force or _stale(paths["libmyers"], myers):
        _run([CC, "-O3", "-fPIC", "-shared", "-std=c11", "-o", paths["libmyers"], myers])
    edpy = os.path.join(csrc, "edpy.c")
    if force or _stale(paths["edpy"], edpy, myers):
        inc = sysconfig.get_paths()["include"]
        _run([CC, "-O3", "-fPIC", "-shared", "-std=c11", f"-I{inc}", f"-I{csrc}",
              "-o", paths["edpy"], edpy])
    hc = os.path.join(csrc, "gpu_hostcheck.cpp")
    if force or _stale(paths["gpucheck"], hc, os.path.join(csrc, "gpu_myers.cuh")):
        _run([CXX, "-O2", "-fPIC", "-shared", "-std=c++17", "-Wno-unknown-pragmas",
              f"-I{csrc}", "-o", paths["gpucheck"], hc])
    return paths


if __name__ == "__main__":
    what = sys.argv[1] if len(sys.argv) > 1 else "all"
    if what in ("oracle", "all"):
        print(build_oracle(force=True))
    if what in ("ref", "all"):
        print(build_ref(force=True))
        print(build_ref_cuda(force=True))
