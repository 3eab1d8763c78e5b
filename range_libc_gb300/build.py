"""Build recipe of the CUDA library (librangelibc_gb300.so), in-tree.

nvcc compiles each translation unit of ``csrc/`` for sm_103a in parallel and
links them into ``_build/librangelibc_gb300.so``.  Host code is compiled
with ``-ffp-contract=off`` and device code with ``-fmad=false`` so that no
multiply-add is contracted (the ray-casting arithmetic is bit-exact against
the reference's plain IEEE C++).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
# per-architecture build folder: x86-64 objects must never be linked on an aarch64 host
BUILD = os.path.join(HERE, "_build", platform.machine() or "unknown")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
LIB_NAME = "librangelibc_gb300.so"
LIB_PATH = os.path.join(BUILD, LIB_NAME)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["rlc_map.cu", "rlc_cast.cu", "rlc_cddt.cu", "rlc_api.cu", "rlc_mlp.cu", "rlc_png.cu"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build range_libc_gb300")
    return cand


def common_flags() -> list[str]:
    return ARCH + [
        "-O3", "-lineinfo", "-std=c++17", "-fmad=false",
        "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden",
        "-I", INCLUDE, "-I", CSRC,
    ]


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(INCLUDE, "rangelibc.h"))
    objs = []
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc(), "-c", s, "-o", o] + common_flags())

    def run(cmd):
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        for err in ex.map(run, jobs):
            if verbose and err:
                print(err, file=sys.stderr)
    if force or jobs or _stale(LIB_PATH, objs):
        run([nvcc(), "-shared", "-o", LIB_PATH] + objs + ARCH +
            ["-cudart", "shared", "-Xlinker", f"-soname,{LIB_NAME}"])
    build_fast(verbose, force)
    return LIB_PATH


FAST_SRC = os.path.join(CSRC, "rlc_py.c")


def fast_module_path() -> str:
    return os.path.join(BUILD, "_rlcfast" + (sysconfig.get_config_var("EXT_SUFFIX") or ".so"))


def build_fast(verbose: bool = False, force: bool = False):
    """The CPython entry points of the per-call methods (csrc/rlc_py.c) beside the library, linked
    to it; None where Python's headers or a C compiler are absent (the ctypes path serves then)."""
    inc = sysconfig.get_paths().get("include")
    cc = shutil.which("gcc") or shutil.which("cc")
    if not inc or not os.path.exists(os.path.join(inc, "Python.h")) or not cc:
        return None
    out = fast_module_path()
    if not force and not _stale(out, [FAST_SRC, os.path.join(INCLUDE, "rangelibc.h"), LIB_PATH]):
        return out
    cmd = [cc, "-O2", "-shared", "-fPIC", "-I", inc, "-I", INCLUDE, FAST_SRC, "-o", out,
           "-L", BUILD, "-lrangelibc_gb300", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        if verbose:
            print(f"CPython entry points not built:\n{r.stderr}", file=sys.stderr)
        return None
    return out


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
