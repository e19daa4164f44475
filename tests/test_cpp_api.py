"""The C++ world API (include/axiom_world.hpp) compiled into a program and run.

``tests/cpp/world_api_main.cpp`` drives PhysicsWorld::create / createBodies / step /
readState / pairs / contacts / saveSnapshot / loadSnapshot / writeState on a mixed scene
(spheres, boxes with given mass and inertia, capsules, ground plane; 60 steps at dt 1/120 s)
and checks, itself, that the wrapper steps to the same bits as raw ``axiom_world_*`` calls,
that a snapshot resumes bit for bit, and that errors come back as the engine's
``core::ErrorCode`` values (the reference's ``core::Result`` convention,
include/axiom/core/result.hpp:16, error_code.hpp:21-57).  It prints the final state as float
bits.  Linked with the CPU oracle it runs here; linked with the CUDA library it runs on the
GPU and must print exactly what the oracle-linked program prints.

``tests/cpp/batch_api_main.cpp`` drives PhysicsWorldBatch (CUDA library only) and checks
that every world of a batch ends bit-identical to a PhysicsWorld holding the same bodies.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

import pytest

import build as axbuild

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "world_api_main.cpp"
BATCH_SRC = ROOT / "tests" / "cpp" / "batch_api_main.cpp"

pytestmark = pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")


def _compile(lib: Path, out: Path, src: Path = SRC) -> Path:
    """Builds a program against one library exporting axiom_c.h (lib = path of the .so)."""
    name = lib.name[len("lib"):-len(".so")]
    cmd = ["g++", "-std=c++20", "-O2", "-Wall", "-Wextra", "-Werror", f"-I{ROOT / 'include'}", str(src),
           f"-L{lib.parent}", f"-l{name}", f"-Wl,-rpath,{lib.parent}", "-o", str(out)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


def _run(exe: Path) -> str:
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, f"{exe.name} failed: {r.stderr.strip()}"
    return r.stdout


@pytest.fixture(scope="module")
def oracle_output(tmp_path_factory) -> str:
    exe = _compile(axbuild.build_oracle(), tmp_path_factory.mktemp("cpp") / "api_oracle")
    return _run(exe)


def test_cpp_api_on_oracle(oracle_output):
    lines = oracle_output.splitlines()
    assert lines[0] == "bodies 77 dynamic 76 static 1"
    counts = dict(zip(lines[1].split()[0::2], map(int, lines[1].split()[1::2])))
    assert counts["contacts"] > 0 and counts["pairs"] > 0 and counts["colours"] > 0
    assert counts["sweeps"] == 10
    assert lines[2] == "bad_shape_code 300"  # core::ErrorCode::InvalidShape
    state = lines[3:]
    assert len(state) == 77 and all(len(s.split()) == 14 for s in state)


def test_cpp_api_links_against_cuda_library(lib, tmp_path):
    """Every C-ABI call the header makes resolves in the CUDA library (link only, no GPU)."""
    _compile(axbuild.build_library(), tmp_path / "api_gpu")
    _compile(axbuild.build_library(), tmp_path / "batch_gpu", BATCH_SRC)


@pytest.mark.gpu
def test_cpp_api_gpu_matches_oracle(gpu_lib, oracle_output, tmp_path):
    exe = _compile(axbuild.build_library(), tmp_path / "api_gpu")
    assert _run(exe) == oracle_output


@pytest.mark.gpu
def test_cpp_batch_api_matches_single_worlds(gpu_lib, tmp_path):
    exe = _compile(axbuild.build_library(), tmp_path / "batch_gpu", BATCH_SRC)
    out = _run(exe)
    assert out.startswith("batch worlds 6 ")


@pytest.mark.skipif(not os.environ.get("AXIOM_REFERENCE"), reason="needs AXIOM_REFERENCE (a reference checkout)")
def test_cpp_api_with_engine_result(oracle_output, tmp_path):
    """With AXIOM_GB300_ENGINE_RESULT the header takes core::Result and core::ErrorCode from
    the engine's own include/axiom/core/result.hpp and error_code.hpp (compiled where they
    lie in the reference checkout); the program must build and print what the standalone
    build prints."""
    ref = Path(os.environ["AXIOM_REFERENCE"]) / "include"
    lib = axbuild.build_oracle()
    exe = tmp_path / "api_engine_result"
    cmd = ["g++", "-std=c++20", "-O2", "-Wall", "-Wextra", "-DAXIOM_GB300_ENGINE_RESULT", f"-I{ref}",
           f"-I{ROOT / 'include'}", str(SRC), f"-L{lib.parent}", "-loracle", f"-Wl,-rpath,{lib.parent}",
           "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    assert _run(exe) == oracle_output
