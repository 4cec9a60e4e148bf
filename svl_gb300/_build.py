"""In-tree build of the native parts: the CUDA/C++ library (product) and the
CPU oracle (test infrastructure).  Plain nvcc/g++ invocations, compiled in
parallel, one -gencode (sm_103a)."""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "svl_gb300"
CSRC = PKG / "csrc"
LIBDIR = PKG / "lib"
BUILD = ROOT / "_build"
LIB = LIBDIR / "libsvl_gb300.so"
ORACLE_SRC = ROOT / "oracle" / "svl_oracle.cpp"
ORACLE_LIB = ROOT / "oracle" / "_build" / "libsvl_oracle.so"

NVCC = os.environ.get("NVCC", shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "--expt-relaxed-constexpr"] + GENCODE
CXX = os.environ.get("CXX", "g++")
CXX_FLAGS = ["-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-Wall", "-Wno-unused-function"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s\n%s" % (" ".join(map(str, cmd)), r.stdout, r.stderr))
    return r.stdout + r.stderr


def _stale(target: Path, sources) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(s).stat().st_mtime > t for s in sources)


def build_library(force: bool = False, verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.hpp")) + list(CSRC.glob("*.cuh")) + [ROOT / "include" / "svl_gb300.h"]
    jobs = []
    objs = []
    for src in sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp")):
        obj = BUILD / (src.name + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            if src.suffix == ".cu":
                cmd = [NVCC, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
            else:
                cmd = [CXX, *CXX_FLAGS, "-I/usr/local/cuda/include", "-c", str(src), "-o", str(obj)]
            jobs.append(cmd)
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            for out in ex.map(_run, jobs):
                if verbose and out.strip():
                    print(out)
    if force or jobs or _stale(LIB, objs):
        _run([NVCC, "-shared", *GENCODE, "-o", str(LIB), *map(str, objs), "-lcudart", "-Xlinker", "-lpthread"])
    return LIB


def build_oracle(force: bool = False) -> Path:
    ORACLE_LIB.parent.mkdir(parents=True, exist_ok=True)
    hdr = ROOT / "include" / "svl_gb300.h"
    if force or _stale(ORACLE_LIB, [ORACLE_SRC, hdr]):
        _run([CXX, "-O2", "-fPIC", "-shared", "-std=c++17", "-fopenmp", "-ffp-contract=off",
              str(ORACLE_SRC), "-o", str(ORACLE_LIB)])
    return ORACLE_LIB


def build_all(force: bool = False, verbose: bool = False):
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_library, force, verbose)
        f2 = ex.submit(build_oracle, force)
        return f1.result(), f2.result()
