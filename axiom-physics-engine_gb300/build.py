"""Builds the GB300 step library and the CPU oracle in-tree.

    python axiom-physics-engine_gb300/build.py          # both
    python axiom-physics-engine_gb300/build.py --lib    # only the CUDA library

CUDA sources are compiled for sm_103a only, with --fmad=false so that every fp32
expression rounds exactly as written (the kernels are bit-identical to the oracle's
scalar evaluation).  Objects compile in parallel; the library links with nvcc.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "lib"
BUILD = ROOT / "_build" / platform.machine()
ORACLE = ROOT / "oracle"

LIB_NAME = "libaxiom_gb300.so"
ORACLE_LIB = ORACLE / "liboracle.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "--fmad=false", "-lineinfo", "-std=c++17",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
    "-I", str(ROOT / "include"),
]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I", str(ROOT / "include")]
# The oracle is also the timed CPU baseline: -O3, OpenMP, still no FP contraction.  No
# -march=native: the same source builds on x86 and Arm hosts and must give the same bits
# on both, so no host-specific instruction selection enters it.
ORACLE_CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fopenmp", "-I", str(ROOT / "include")]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the library")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"command failed ({res.returncode}): {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")


def _stamp(target: Path) -> Path:
    return target.with_name(f".{target.name}.{platform.machine()}")


def _stale(target: Path, deps: list[Path], stamped: bool = True) -> bool:
    """True when target is missing, older than a dependency, or built on another machine."""
    if not target.exists() or (stamped and not _stamp(target).exists()):
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted((ROOT / "include").glob("*.h"))


def library_path() -> Path:
    return LIBDIR / LIB_NAME


def build_library(force: bool = False, jobs: int | None = None) -> Path:
    """Compiles every csrc/*.cu (nvcc, sm_103a) and csrc/*.cpp (g++) and links the .so."""
    nvcc = _nvcc()
    BUILD.mkdir(parents=True, exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    hdrs = _headers()
    jobs_list = []
    objs = []
    for src in sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp")):
        obj = BUILD / (src.name + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + hdrs, stamped=False):
            if src.suffix == ".cu":
                cmd = [nvcc] + NVCC_FLAGS + ["-c", str(src), "-o", str(obj)]
            else:
                cmd = ["g++"] + CXX_FLAGS + ["-c", str(src), "-o", str(obj)]
            jobs_list.append(cmd)
    if jobs_list:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
            list(ex.map(_run, jobs_list))
    lib = library_path()
    if force or jobs_list or _stale(lib, objs):
        # every symbol resolved at link time: a missing definition fails the build, not the load
        _run([nvcc] + ARCH + ["-shared", "-Xlinker", "--no-undefined", "-o", str(lib)] + [str(o) for o in objs])
        _stamp(lib).write_text(platform.machine() + "\n")
    return lib


def build_oracle(force: bool = False) -> Path:
    """Compiles the CPU oracle (test infrastructure) into oracle/liboracle.so, with the
    seeded scene generators (axiom_scene.h) so that a CPU-only run needs no GPU library."""
    srcs = [ORACLE / "oracle_world.cpp", CSRC / "scene.cpp"]
    deps = srcs + sorted(ORACLE.glob("*.h")) + sorted((ROOT / "include").glob("*.h")) + [CSRC / "host_math.h"]
    if force or _stale(ORACLE_LIB, deps):
        _run(["g++"] + ORACLE_CXX_FLAGS + ["-shared", "-o", str(ORACLE_LIB)] + [str(s) for s in srcs])
        _stamp(ORACLE_LIB).write_text(platform.machine() + "\n")
    return ORACLE_LIB


def main(argv: list[str] | None = None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--lib", action="store_true", help="only the CUDA library")
    ap.add_argument("--oracle", action="store_true", help="only the oracle")
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args(argv)
    if not a.oracle:
        print(build_library(a.force))
    if not a.lib:
        print(build_oracle(a.force))
    return 0


if __name__ == "__main__":
    sys.exit(main())
