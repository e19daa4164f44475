"""Shared fixtures.  CPU tests (default) need no GPU; tests marked ``gpu`` need one."""
from __future__ import annotations

import ctypes
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "axiom-physics-engine_gb300"
sys.path.insert(0, str(PKG))
sys.path.insert(0, str(ROOT))

import axiom_gb300 as ax  # noqa: E402
import build as axbuild  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def lib():
    """The CUDA library (built in-tree).  Loading it needs no GPU."""
    axbuild.build_library()
    return ax.load_library()


ORACLE_EXTRA = {
    "oracle_set_threads": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_int32]),
    "oracle_aabb_intersects": (ctypes.c_int32, [ctypes.POINTER(ctypes.c_float)] * 4),
    "oracle_aabb_from_center": (None, [ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                                       ctypes.c_float, ctypes.POINTER(ctypes.c_float),
                                       ctypes.POINTER(ctypes.c_float)]),
    "oracle_vec3_ops": (None, [ctypes.POINTER(ctypes.c_float)] * 5),
    "oracle_quat_rotate": (None, [ctypes.POINTER(ctypes.c_float)] * 3),
    "oracle_quat_mul": (None, [ctypes.POINTER(ctypes.c_float)] * 3),
    "oracle_quat_normalize": (None, [ctypes.POINTER(ctypes.c_float)] * 2),
    "oracle_quat_from_axis_angle": (None, [ctypes.POINTER(ctypes.c_float), ctypes.c_float,
                                           ctypes.POINTER(ctypes.c_float)]),
}


@pytest.fixture(scope="session")
def oracle():
    """The CPU oracle (test infrastructure), exporting the same C ABI."""
    path = axbuild.build_oracle()
    o = ctypes.CDLL(str(path))
    ax._bind(o, ax.WORLD_FUNCS)
    ax._bind(o, ORACLE_EXTRA)
    return o


@pytest.fixture(scope="session")
def gpu_lib(lib):
    """The CUDA library on a machine with a GPU; skips the test elsewhere."""
    import torch  # device query only

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return lib
