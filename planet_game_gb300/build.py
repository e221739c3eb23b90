"""In-tree build of the GB300 library.

``build_library()`` compiles the CUDA kernels for sm_103a with nvcc and the host
C++ (mesh builder, hierarchy, C-ABI) with g++ under ``-ffp-contract=off``, then links
``planet_game_gb300/lib/libplanetsim_gb300.so``. It is incremental (a target is rebuilt
when any of its sources is newer) and compiles its translation units in parallel. No
cmake, no torch extension machinery. (The checker's own build is ``oracle/build.py``.)
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIB_DIR = PKG / "lib"
OBJ_DIR = PKG / "lib" / "obj"
LIBRARY = LIB_DIR / "libplanetsim_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))

CU_SOURCES = ["multigrid.cu", "krylov.cu", "operators.cu", "column.cu", "noalloc.cu", "persistent.cu",
              "persistent_f32.cu", "persistent_f64.cu", "coarse_tail.cu",
              "newton.cu", "nonsym.cu", "insolation.cu", "multirhs.cu", "coarse_cluster.cu"]
CPP_SOURCES = ["solver.cpp", "multirhs.cpp", "autotune.cpp", "capi.cpp", "profile.cpp", "host/icosphere.cpp", "host/agglomerate.cpp", "host/ilu_pattern.cpp", "host/tail_blocks.cpp", "host/shared_columns.cpp", "host/hierarchy.cpp", "host/insolation.cpp",
               "serve_core.cpp", "serve.cpp"]
# Files compiled without FMA contraction (reference operation order).
NO_FMAD = {"column.cu", "newton.cu", "nonsym.cu", "insolation.cu"}


def _nvcc() -> str:
    exe = shutil.which("nvcc") or str(CUDA_HOME / "bin" / "nvcc")
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found; the GB300 library needs the CUDA toolkit")
    return exe


def _headers() -> list[Path]:
    return sorted(CSRC.rglob("*.hpp")) + sorted(CSRC.rglob("*.cuh")) + [ROOT / "include" / "planetsim_gb300.h"]


def _stale(target: Path, sources: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources)


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + proc.stdout + proc.stderr)


def _compile_jobs(verbose_ptxas: bool = False) -> list[tuple[Path, list[str], list[Path]]]:
    headers = _headers()
    jobs = []
    for name in CU_SOURCES:
        src = CSRC / name
        obj = OBJ_DIR / (name.replace("/", "_") + ".o")
        cmd = [_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler",
               "-ffp-contract=off", "--expt-relaxed-constexpr", "-I", str(CSRC), "-c", str(src), "-o", str(obj)]
        if name in NO_FMAD:
            cmd.insert(1, "--fmad=false")
        if verbose_ptxas:
            cmd.insert(1, "-Xptxas=-v")
        jobs.append((obj, cmd, [src, *headers]))
    for name in CPP_SOURCES:
        src = CSRC / name
        obj = OBJ_DIR / (name.replace("/", "_") + ".o")
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-pthread", "-I", str(CSRC),
               "-I", str(CUDA_HOME / "include"), "-c", str(src), "-o", str(obj)]
        jobs.append((obj, cmd, [src, *headers]))
    return jobs


def build_library(force: bool = False, verbose_ptxas: bool = False) -> Path:
    """Compile and link the GB300 library; returns its path."""
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    jobs = _compile_jobs(verbose_ptxas)
    todo = [(o, c) for o, c, deps in jobs if force or verbose_ptxas or _stale(o, deps)]
    if todo:
        with ThreadPoolExecutor(max_workers=max(2, min(len(todo), os.cpu_count() or 4))) as pool:
            list(pool.map(lambda oc: _run(oc[1]), todo))
    objs = [o for o, _, _ in jobs]
    if force or todo or _stale(LIBRARY, objs):
        tmp = LIBRARY.with_suffix(".so.tmp")
        _run([_nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart", "-lpthread"])
        os.replace(tmp, LIBRARY)
    return LIBRARY


if __name__ == "__main__":
    print(build_library(force="--force" in sys.argv, verbose_ptxas="--ptxas" in sys.argv))
