"""In-tree build of the CUDA library ``libbitlev_gb300.so`` (sm_103a only).

Each translation unit is compiled by nvcc in parallel, then linked into one
shared library beside this file. The CUDA runtime is linked statically, so
ctypes needs no libcudart on the library path. The host-compiled device
header check (``libblg_hostcheck.so``) is built with g++ for the CPU tests.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
INCLUDE = os.path.join(ROOT, "include")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libbitlev_gb300.so")
HOSTCHECK = os.path.join(HERE, "libblg_hostcheck.so")
PROBE = os.path.join(HERE, "libblg_probe.so")

CU_SOURCES = ["blg_api.cu", "blg_kernels.cu", "blg_noalloc.cu", "blg_pairs_sched.cu", "blg_mlp.cu", "blg_batch.cu",
              "blg_pairs_tile.cu", "blg_search_band.cu", "blg_matches.cu"]
HEADERS = ["blg_device.cuh", "blg_internal.h", "blg_kernels.cuh", "blg_context.h", "blg_sched.h", "blg_batch.h", "blg_tma.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = [os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]
    for c in cand:
        if c and os.path.exists(c):
            return c
    raise FileNotFoundError("nvcc not found (set NVCC or put CUDA's bin on PATH)")


def _newest_input() -> float:
    files = [os.path.join(CSRC, f) for f in CU_SOURCES + HEADERS]
    files.append(os.path.join(INCLUDE, "bitlev_gb300.h"))
    files.append(os.path.abspath(__file__))
    return max(os.path.getmtime(f) for f in files if os.path.exists(f))


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(OBJ, os.path.splitext(os.path.basename(src))[0] + ".o")
    cmd = [nvcc(), "-c", "-O3", "-std=c++17", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC",
           "--expt-relaxed-constexpr", "--extended-lambda", f"-I{INCLUDE}", *extra,
           "-o", obj, os.path.join(CSRC, src)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if os.environ.get("BLG_BUILD_VERBOSE"):
        sys.stderr.write(r.stdout + r.stderr)
    return obj


def build(force: bool = False, extra: list[str] | None = None) -> str:
    """Compile every CUDA translation unit for sm_103a and link the library."""
    extra = list(extra or [])
    if os.environ.get("BLG_PTXAS_VERBOSE"):
        extra += ["-Xptxas", "-v"]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _newest_input() and not extra:
        return LIB
    os.makedirs(OBJ, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(CU_SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), CU_SOURCES))
    tmp = LIB + f".{os.getpid()}.tmp"
    cmd = [nvcc(), "-shared", *ARCH, "-o", tmp, *objs, "-Xcompiler", "-fPIC", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


def build_probe(force: bool = False) -> str:
    """The integer-pipe throughput probe (bench.py's roofline denominator)."""
    src = os.path.join(CSRC, "blg_probe.cu")
    if not force and os.path.exists(PROBE) and os.path.getmtime(PROBE) >= os.path.getmtime(src):
        return PROBE
    tmp = PROBE + f".{os.getpid()}.tmp"
    r = subprocess.run([nvcc(), "-O3", "-std=c++17", *ARCH, "-lineinfo", "-shared", "-Xcompiler",
                        "-fPIC", "-o", tmp, src], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for blg_probe.cu:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, PROBE)
    return PROBE


def packer_path() -> str:
    import sysconfig
    return os.path.join(HERE, "_blgpack" + (sysconfig.get_config_var("EXT_SUFFIX") or ".so"))


def build_packer(force: bool = False) -> str | None:
    """gcc build of the native str/bytes packer (csrc/blg_pack.c, a CPython
    extension). Returns None when this Python has no development headers:
    the package then packs with its numpy/bytes code (same layout, same
    errors, slower)."""
    import sysconfig
    src = os.path.join(CSRC, "blg_pack.c")
    out = packer_path()
    if not force and os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
        return out
    inc = sysconfig.get_paths().get("include")
    if not inc or not os.path.exists(os.path.join(inc, "Python.h")):
        return None
    tmp = out + f".{os.getpid()}.tmp"
    cc = os.environ.get("CC", "gcc")
    r = subprocess.run([cc, "-O2", "-shared", "-fPIC", "-Wall", f"-I{inc}", "-o", tmp, src],
                       capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(f"native packer not built (numpy packing is used):\n{r.stderr}\n")
        return None
    os.replace(tmp, out)
    return out


def build_hostcheck(force: bool = False) -> str:
    """g++ build of the device header's host path (blg_hostcheck.cpp)."""
    src = os.path.join(CSRC, "blg_hostcheck.cpp")
    deps = [src, os.path.join(CSRC, "blg_device.cuh")]
    if (not force and os.path.exists(HOSTCHECK)
            and os.path.getmtime(HOSTCHECK) >= max(os.path.getmtime(d) for d in deps)):
        return HOSTCHECK
    tmp = HOSTCHECK + f".{os.getpid()}.tmp"
    cxx = os.environ.get("CXX", "g++")
    subprocess.run([cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-Wall", "-Wextra",
                    "-o", tmp, src], check=True)
    os.replace(tmp, HOSTCHECK)
    return HOSTCHECK


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
