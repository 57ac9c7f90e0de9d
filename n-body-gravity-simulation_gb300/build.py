"""Builds the engine's shared library for sm_103a with nvcc.

    python n-body-gravity-simulation_gb300/build.py [--force] [--verbose-ptxas] [--checks]

Compiles every csrc/*.cu and csrc/*.cpp in parallel into _build/ and links
nbody_gb300/libnbody_gb300.so (static CUDA runtime, one -gencode:
compute_103a/sm_103a).  The C++ compat layer (compat/src/*.cpp against
compat/include) is linked into nbody_gb300/libnbody_compat.so on top of it.
Objects are rebuilt only when a source or header is newer.

--checks builds nbody_gb300/libnbody_gb300_checks.so instead (objects in
_build_checks/, no compat layer): the same engine with -DNB_DEVICE_CHECKS=1,
whose kernels test every index they use against its bound and record the
first failure (nb_debug_device_checks); select it with NBODY_GB300_LIB.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
COMPAT = os.path.join(PKG, "compat")
OUT_DIR = os.path.join(PKG, "nbody_gb300")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(OUT_DIR, "libnbody_gb300.so")
CHECKS_LIB = os.path.join(OUT_DIR, "libnbody_gb300_checks.so")
COMPAT_LIB = os.path.join(OUT_DIR, "libnbody_compat.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              "-I" + os.path.join(REPO, "include")]


def nvcc() -> str:
    exe = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return exe


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, obj: str, headers, extra, verbose: bool, force: bool):
    if not force and not _newer(obj, [src, *headers]):
        return obj, ""
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", src, "-o", obj]
    if verbose and src.endswith(".cu"):
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj, (r.stdout + r.stderr)


def build(force: bool = False, verbose_ptxas: bool = False, jobs: int | None = None,
          checks: bool = False) -> str:
    build_dir = os.path.join(PKG, "_build_checks") if checks else BUILD
    lib = CHECKS_LIB if checks else LIB
    extra = ["-DNB_DEVICE_CHECKS=1"] if checks else []
    os.makedirs(build_dir, exist_ok=True)
    headers = sorted(glob.glob(os.path.join(CSRC, "*.h")) +
                     glob.glob(os.path.join(CSRC, "*.cuh")) +
                     glob.glob(os.path.join(REPO, "include", "*.h")))
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")) +
                     glob.glob(os.path.join(CSRC, "*.cpp")))
    compat_headers = sorted(glob.glob(os.path.join(COMPAT, "include", "*.hpp")))
    compat_sources = [] if checks else sorted(glob.glob(os.path.join(COMPAT, "src", "*.cpp")))
    jobs = jobs or min(16, (os.cpu_count() or 4))
    logs = []
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        futs = []
        for s in sources:
            o = os.path.join(build_dir, os.path.basename(s) + ".o")
            futs.append(ex.submit(_compile, s, o, headers, extra, verbose_ptxas, force))
        cfuts = []
        for s in compat_sources:
            o = os.path.join(BUILD, "compat_" + os.path.basename(s) + ".o")
            cfuts.append(ex.submit(_compile, s, o, headers + compat_headers,
                                   ["-I" + os.path.join(COMPAT, "include")], False, force))
        objs = []
        for f in futs:
            o, log = f.result()
            objs.append(o)
            if log.strip():
                logs.append(log)
        cobjs = []
        for f in cfuts:
            o, log = f.result()
            cobjs.append(o)
            if log.strip():
                logs.append(log)
    os.makedirs(OUT_DIR, exist_ok=True)
    if force or _newer(lib, objs):
        tmp = lib + ".tmp"
        cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, lib)
    if cobjs and (force or _newer(COMPAT_LIB, cobjs + [LIB])):
        tmp = COMPAT_LIB + ".tmp"
        cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *cobjs, "-L" + OUT_DIR, "-lnbody_gb300",
               "-Xlinker", "-rpath=$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compat link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, COMPAT_LIB)
    if verbose_ptxas:
        print("\n".join(logs))
    return lib


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose-ptxas", action="store_true")
    ap.add_argument("--checks", action="store_true", help="the device-checked library")
    a = ap.parse_args(argv)
    print(build(force=a.force, verbose_ptxas=a.verbose_ptxas, checks=a.checks))
    return 0


if __name__ == "__main__":
    sys.exit(main())
