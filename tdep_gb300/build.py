"""In-tree build of the native parts.

libtdep_gb300.so : CUDA kernels for sm_103a + host C++ (readers, mesh, phonons, C-ABI)
thermal_conductivity : C++ host driver over the C-ABI (mirror of the reference program)
liboracle.so : the CPU restatement used by the tests and the CPU baseline (oracle/)

Translation units compile in parallel; nothing is rebuilt when outputs are newer than
their sources. Run `python -m tdep_gb300.build` or call build_all().
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "tdep_gb300"
CSRC = PKG / "csrc"
LIBDIR = PKG / "lib"
BINDIR = PKG / "bin"
OBJDIR = PKG / "_build"
ORACLE = ROOT / "oracle"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CXXFLAGS = ["-O2", "-fPIC", "-std=c++17", "-Wall", "-Wno-unused-function"]
NVCCFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"] + ARCH

HOST_SRC = ["host/crystal.cpp", "host/qmesh.cpp", "host/phonons.cpp", "host/mcgrid.cpp", "host/problem.cpp",
            "host/h5write.cpp", "host/gridout.cpp", "host/forcemap.cpp"]
CUDA_SRC = ["k_triplets.cu", "k_threephonon.cu", "k_fourphonon.cu", "k_misc.cu", "tdg_api.cu", "tdg_noalloc.cu", "k_tcgemm.cu", "k_largecell.cu", "k_offdiag.cu", "autotune.cu", "k_threephonon_tc.cu", "k_bte_adjoint.cu", "k_harmonic.cu"]
HEADERS = ["host/common.hpp", "host/crystal.hpp", "tdg_internal.cuh", "dev_common.cuh", "tc_common.cuh",
           "k3_parts.cuh", "host/h5write.hpp"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build tdep_gb300")


def _stale(out: Path, deps) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def _run(cmd) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(map(str, cmd)) + "\n" + r.stdout + r.stderr)


def _common_deps():
    return [CSRC / h for h in HEADERS] + [ROOT / "include" / "tdep_gb300.h", Path(__file__)]


def build_library(verbose: bool = False) -> Path:
    nvcc = _nvcc()
    OBJDIR.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    jobs = []
    objs = []
    for src in HOST_SRC:
        s = CSRC / src
        o = OBJDIR / (Path(src).stem + ".o")
        objs.append(o)
        if _stale(o, [s] + _common_deps()):
            jobs.append(["g++"] + CXXFLAGS + ["-c", str(s), "-o", str(o)])
    for src in CUDA_SRC:
        s = CSRC / src
        o = OBJDIR / (Path(src).stem + ".cu.o")
        objs.append(o)
        if _stale(o, [s] + _common_deps()):
            jobs.append([nvcc] + NVCCFLAGS + ["-c", str(s), "-o", str(o)])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for cmd in jobs:
                if verbose:
                    print(" ".join(cmd), file=sys.stderr)
            list(ex.map(_run, jobs))
    lib = LIBDIR / "libtdep_gb300.so"
    if _stale(lib, objs):
        _run([nvcc, "-shared"] + ARCH + ["-o", str(lib)] + [str(o) for o in objs] + ["-lpthread"])
    return lib


def build_driver() -> Path:
    BINDIR.mkdir(exist_ok=True)
    exe = BINDIR / "thermal_conductivity"
    src = CSRC / "tc_main.cpp"
    lib = LIBDIR / "libtdep_gb300.so"
    if _stale(exe, [src, lib] + _common_deps()):
        _run(["g++"] + CXXFLAGS + [str(src), "-o", str(exe), f"-L{LIBDIR}", "-ltdep_gb300",
                                   "-Wl,-rpath,$ORIGIN/../lib"])
    return exe


def build_oracle() -> Path:
    out = ORACLE / "lib" / "liboracle.so"
    out.parent.mkdir(exist_ok=True)
    src = ORACLE / "oracle.cpp"
    if _stale(out, [src, ROOT / "include" / "tdep_gb300.h"]):
        _run(["g++", "-O2", "-fPIC", "-std=c++17", "-fopenmp", "-shared", str(src), "-o", str(out)])
    return out


def build_all(verbose: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=2) as ex:
        f_lib = ex.submit(build_library, verbose)
        f_orc = ex.submit(build_oracle)
        f_lib.result()
        f_orc.result()
    build_driver()


if __name__ == "__main__":
    build_all(verbose="-v" in sys.argv)
    print("built", LIBDIR / "libtdep_gb300.so")
