"""Builds the sm_103a shared library ``supermc_gb300/_build/libsupermc_gb300.so``.

Plain nvcc, one object per translation unit compiled in parallel, then one
link; no CMake and no torch extension machinery.  The library depends only on
the CUDA runtime.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libsupermc_gb300.so")
HOST = os.path.join(HERE, "host")
HOST_SOURCES = ["ParameterReader.cpp", "MakeDensity.cpp", "MCnucl.cpp", "main.cpp"]
EXE = os.path.join(OUT_DIR, "superMC")
# one event through the MCnucl call surface (host/MCnucl.h), for its test
MCNUCL_SOURCES = ["ParameterReader.cpp", "MakeDensity.cpp", "MCnucl.cpp", "mcnucl_event.cpp"]
MCNUCL_EXE = os.path.join(OUT_DIR, "mcnucl_event")
SOURCES = ["smc_capi.cu", "k_sample_pair.cu", "k_grid.cu", "k_kln.cu", "k_kln_cells.cu", "k_average.cu", "smc_noalloc.cu", "k_grid_tc.cu", "k_adjoint.cu", "smc_output.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
         "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build supermc_gb300")


def _stale(obj: str, deps: list[str]) -> bool:
    return not os.path.exists(obj) or any(os.path.getmtime(d) > os.path.getmtime(obj) for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "supermc.h"))
    cc = nvcc()
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([cc, *ARCH, *FLAGS, "-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            results = list(ex.map(lambda cmd: subprocess.run(cmd, capture_output=True, text=True), jobs))
        for cmd, r in zip(jobs, results):
            if verbose or r.returncode:
                sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            if r.returncode:
                raise RuntimeError(f"nvcc failed for {cmd[-3]}")
    if force or jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        r = subprocess.run([cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"], capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
        os.replace(tmp, LIB)
    build_host(force)
    return LIB


def _host_exe(exe: str, sources: list[str], force: bool) -> str:
    srcs = [os.path.join(HOST, f) for f in sources]
    deps = srcs + [os.path.join(HOST, h) for h in os.listdir(HOST) if h.endswith(".h")] + [LIB]
    if not force and not _stale(exe, deps):
        return exe
    cxx = shutil.which("g++") or "g++"
    tmp = exe + ".tmp"
    r = subprocess.run([cxx, "-O2", "-std=c++17", "-Wall", "-o", tmp, *srcs, "-L" + OUT_DIR, "-lsupermc_gb300",
                        "-Wl,-rpath,$ORIGIN"], capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError("host build failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, exe)
    return exe


def build_host(force: bool = False) -> str:
    """The C++ drop-in driver ``_build/superMC`` (ParameterReader,
    MakeDensity, MCnucl, main over the C ABI) and ``_build/mcnucl_event``
    (one event through the MCnucl call surface), linked to the library."""
    _host_exe(MCNUCL_EXE, MCNUCL_SOURCES, force)
    return _host_exe(EXE, HOST_SOURCES, force)


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
