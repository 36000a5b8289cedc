"""In-tree build of the native libraries (nvcc + gcc, no cmake).

    python -m rajzel_gb300.build          # build everything that is stale

Products (all git-ignored, rebuilt on each machine):
    rajzel_gb300/librajzel_gb300.so     CUDA kernels + the C ABI of include/rajzel_gb300.h
    rajzel_gb300/librajzel_compat.so    reference-signature shim (eikonal(), grad_obj(), ...)
    rajzel_gb300/librz_selftest.so      device self-tests of the arithmetic kernels (tests only)
    rajzel_gb300/rajzel_gpu             driver: runs a RAJZEL parameter directory (INVMAT 0/1/2)
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "librajzel_gb300.so")
COMPAT = os.path.join(PKG, "librajzel_compat.so")
SELFTEST = os.path.join(PKG, "librz_selftest.so")
DRIVER = os.path.join(PKG, "rajzel_gpu")
C_SOURCES = ["rz_io.c"]  # host C compiled into the library

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall"]
CU_SOURCES = ["rz_shot.cu", "rz_aux.cu", "rz_api.cu", "rz_noalloc.cu", "rz_fatt.cu", "rz_fp64.cu"]
HEADERS = ["rz_device.cuh", "rz_internal.h"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "rajzel_gb300.h")]
    objs, jobs = [], []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if _stale(o, [s] + hdrs):
            jobs.append([nvcc(), *NVFLAGS, "-c", s, "-o", o])
    selftest_src = os.path.join(CSRC, "rz_selftest.cu")
    selftest_obj = os.path.join(BUILD, "rz_selftest.o")
    if os.path.exists(selftest_src) and _stale(selftest_obj, [selftest_src] + hdrs):
        jobs.append([nvcc(), *NVFLAGS, "-c", selftest_src, "-o", selftest_obj])
    inc = os.path.join(ROOT, "include")
    for src in C_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".c", ".o"))
        objs.append(o)
        if _stale(o, [s, os.path.join(inc, "rajzel_io.h")]):
            jobs.append(["gcc", "-O2", "-std=gnu99", "-fPIC", "-Wall", "-ffp-contract=off", "-I", inc, "-c", s, "-o", o])
    if jobs:
        with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            list(ex.map(_run, jobs))
    if _stale(LIB, objs):
        _run([nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lpthread"])
    if os.path.exists(selftest_src) and _stale(SELFTEST, [selftest_obj]):
        _run([nvcc(), *ARCH, "-shared", "-o", SELFTEST, selftest_obj])
    compat_src = os.path.join(CSRC, "rz_compat.c")
    if os.path.exists(compat_src) and _stale(COMPAT, [compat_src, LIB, os.path.join(ROOT, "include", "rajzel_compat.h")]):
        _run(["gcc", "-O2", "-std=gnu99", "-fPIC", "-shared", "-I", os.path.join(ROOT, "include"), "-o", COMPAT,
              compat_src, "-L", PKG, "-lrajzel_gb300", "-Wl,-rpath,$ORIGIN", "-lm"])
    driver_src = os.path.join(CSRC, "rz_main.c")
    if os.path.exists(driver_src) and _stale(DRIVER, [driver_src, LIB]):
        _run(["gcc", "-O2", "-std=gnu99", "-Wall", "-ffp-contract=off", "-I", inc, "-o", DRIVER, driver_src, "-L",
              PKG, "-lrajzel_gb300", "-Wl,-rpath,$ORIGIN", "-lm"])
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
