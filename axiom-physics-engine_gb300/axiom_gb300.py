"""Python mirror of the GB300 rigid-body step API, bound to the C ABI of include/axiom_c.h.

The reference engine (itsakeyfut/axiom-physics-engine) intends a C++
``PhysicsWorld::step(dt)`` (reference CLAUDE.md:160-177) over bodies described by
``gui::RigidBodyData`` (include/axiom/gui/body_inspector.hpp:57-90) and configured by
``gui::PhysicsWorldConfig`` (include/axiom/gui/physics_panel.hpp:34-43).  This module
exposes the same vocabulary to Python: :class:`PhysicsWorld` with ``create`` /
``add_bodies`` / ``step`` / state and contact getters, raising :class:`AxiomError`
carrying the reference's ``core::ErrorCode`` value where the C++ API returns a failed
``core::Result`` (include/axiom/core/result.hpp:16).

The same binding drives the CPU oracle (``oracle/liboracle.so``, test infrastructure),
which exports the identical ``axiom_world_*`` symbols.  There is no fallback: if the
CUDA library is missing or no GPU is present, loading or creating a world fails.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
DEFAULT_LIB = PKG / "lib" / "libaxiom_gb300.so"

# core::ErrorCode values (reference include/axiom/core/error_code.hpp:21-57)
ERROR_NAMES = {
    0: "Success", 100: "DivisionByZero", 200: "OutOfMemory", 201: "InvalidAllocation",
    202: "NullPointer", 300: "InvalidShape", 301: "GJKFailedToConverge",
    302: "EPAFailedToConverge", 400: "InvalidRigidBody", 401: "ConstraintSolverFailure",
    503: "GPU_INVALID_OPERATION", 504: "GPU_TIMEOUT", 505: "GPU_OPERATION_FAILED",
    600: "InvalidParameter", 601: "OutOfRange",
}

ERR_INVALID_SHAPE, ERR_GJK_FAILED, ERR_EPA_FAILED = 300, 301, 302
ERR_INVALID_RIGID_BODY, ERR_SOLVER_FAILURE = 400, 401
ERR_INVALID_PARAMETER, ERR_OUT_OF_RANGE = 600, 601
ERR_GPU_INVALID_OPERATION, ERR_GPU_TIMEOUT, ERR_GPU_OPERATION_FAILED = 503, 504, 505
# step statuses after which the step has completed (the state advanced)
STEP_COMPLETED = (0, ERR_GJK_FAILED, ERR_EPA_FAILED)

BODY_STATIC, BODY_DYNAMIC, BODY_KINEMATIC = 0, 1, 2
SHAPE_SPHERE, SHAPE_BOX, SHAPE_CAPSULE, SHAPE_CYLINDER, SHAPE_MESH, SHAPE_CONVEX, SHAPE_PLANE = 0, 1, 2, 3, 4, 5, 6
CONVEX_MAX_VERTICES = 64
WARM_NONE, WARM_PREVIOUS, WARM_LEARNED = 0, 1, 2
MLP_PARAM_COUNT = 128 * 16 + 128 + 128 * 128 + 128 + 128 * 128 + 128 + 3 * 128 + 3


class AxiomError(RuntimeError):
    def __init__(self, code: int, what: str = ""):
        self.code = int(code)
        super().__init__(f"{what}: {ERROR_NAMES.get(self.code, 'Unknown')} ({self.code})")


class WorldConfig(ctypes.Structure):
    _fields_ = [
        ("gravity", ctypes.c_float * 3), ("time_step", ctypes.c_float),
        ("velocity_iterations", ctypes.c_uint32), ("position_iterations", ctypes.c_uint32),
        ("residual_tolerance", ctypes.c_float), ("max_iterations", ctypes.c_uint32),
        ("baumgarte", ctypes.c_float), ("linear_slop", ctypes.c_float),
        ("aabb_margin", ctypes.c_float), ("restitution_threshold", ctypes.c_float),
        ("warm_start", ctypes.c_uint32), ("warm_start_factor", ctypes.c_float),
        ("pair_capacity", ctypes.c_uint32), ("contact_capacity", ctypes.c_uint32),
        ("device", ctypes.c_int32),
        # PhysicsWorldConfig::allowSleep and thresholds (physics_panel.hpp:39-42)
        ("allow_sleep", ctypes.c_uint32), ("sleep_linear_threshold", ctypes.c_float),
        ("sleep_angular_threshold", ctypes.c_float), ("sleep_time_threshold", ctypes.c_float),
        ("speculative_contacts", ctypes.c_uint32),  # continuous collision (off by default)
        ("temporal_colouring", ctypes.c_uint32),  # keep last step's colours (off by default)
    ]


_F = ctypes.POINTER(ctypes.c_float)
_U = ctypes.POINTER(ctypes.c_uint32)
_U8 = ctypes.POINTER(ctypes.c_uint8)


class BodySoA(ctypes.Structure):
    _fields_ = [
        ("type", _U), ("shape", _U), ("position", _F), ("rotation", _F),
        ("linear_velocity", _F), ("angular_velocity", _F), ("shape_extents", _F),
        ("mass", _F), ("inertia", _F), ("friction", _F), ("restitution", _F),
        ("density", _F), ("linear_damping", _F), ("angular_damping", _F),
        ("filter_category", _U), ("filter_mask", _U), ("filter_group", ctypes.POINTER(ctypes.c_int16)),
        ("allow_sleep", _U8), ("is_sleeping", _U8), ("convex_hull", _U),
        ("rolling_friction", _F),  # MaterialInfo::rollingFriction (carried, not applied)
    ]


class StepStats(ctypes.Structure):
    _fields_ = [(name, ctypes.c_uint32) for name in (
        "total_bodies", "active_bodies", "sleeping_bodies", "static_bodies", "dynamic_bodies",
        "kinematic_bodies", "contact_point_count", "constraint_count", "island_count")] + [
        (name, ctypes.c_float) for name in (
            "total_step_time", "broadphase_time", "narrowphase_time", "solver_time",
            "integration_time")] + [
        (name, ctypes.c_uint32) for name in ("pair_count", "manifold_count", "colour_count",
                                             "iterations")] + [
        ("residual", ctypes.c_float), ("status", ctypes.c_int32), ("colour_rounds", ctypes.c_uint32),
        ("gjk_failures", ctypes.c_uint32), ("epa_failures", ctypes.c_uint32)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class ContactPoint(ctypes.Structure):
    _fields_ = [
        ("body_a", ctypes.c_uint32), ("body_b", ctypes.c_uint32),
        ("position", ctypes.c_float * 3), ("normal", ctypes.c_float * 3),
        ("penetration_depth", ctypes.c_float), ("impulse", ctypes.c_float * 3),
        ("colour", ctypes.c_uint32), ("point_index", ctypes.c_uint32),
    ]


CONTACT_DTYPE = np.dtype([
    ("body_a", np.uint32), ("body_b", np.uint32), ("position", np.float32, 3),
    ("normal", np.float32, 3), ("penetration_depth", np.float32), ("impulse", np.float32, 3),
    ("colour", np.uint32), ("point_index", np.uint32),
])
assert CONTACT_DTYPE.itemsize == ctypes.sizeof(ContactPoint)


# World snapshot records (include/axiom_c.h): header, bodies by id, warm-start entries.
class SnapshotHeader(ctypes.Structure):
    _fields_ = [("magic", ctypes.c_char * 8), ("version", ctypes.c_uint32), ("body_count", ctypes.c_uint32),
                ("contact_count", ctypes.c_uint32), ("flags", ctypes.c_uint32), ("hull_count", ctypes.c_uint32),
                ("hull_vertex_count", ctypes.c_uint32), ("total_bytes", ctypes.c_uint64), ("config", WorldConfig)]


SNAPSHOT_BODY_DTYPE = np.dtype([
    ("type", np.uint32), ("shape", np.uint32), ("flags", np.uint32), ("island", np.uint32),
    ("position", np.float32, 3), ("rotation", np.float32, 4), ("linear_velocity", np.float32, 3),
    ("angular_velocity", np.float32, 3), ("shape_extents", np.float32, 3), ("inv_mass", np.float32),
    ("inv_inertia", np.float32, 3), ("friction", np.float32), ("restitution", np.float32),
    ("linear_damping", np.float32), ("angular_damping", np.float32), ("filter_category", np.uint32),
    ("filter_mask", np.uint32), ("filter_group", np.int32), ("sleep_time", np.float32),
    ("rolling_friction", np.float32), ("reserved", np.uint32, 3),
])
SNAPSHOT_CONTACT_DTYPE = np.dtype([("body_lo", np.uint32), ("body_hi", np.uint32), ("point", np.uint32),
                                   ("impulse", np.float32, 3)])
assert SNAPSHOT_BODY_DTYPE.itemsize == 144 and SNAPSHOT_CONTACT_DTYPE.itemsize == 24

# Debug feed records (debug::PhysicsDebugDraw) and the PhysicsDebugFlags bits that select them
DEBUG_SHAPES, DEBUG_AABBS, DEBUG_CONTACTS, DEBUG_VELOCITIES, DEBUG_ISLANDS = 1, 2, 4, 16, 128
DEBUG_ALL = DEBUG_SHAPES | DEBUG_AABBS | DEBUG_CONTACTS | DEBUG_VELOCITIES | DEBUG_ISLANDS
DEBUG_BODY_DTYPE = np.dtype([
    ("position", np.float32, 3), ("rotation", np.float32, 4), ("shape", np.uint32),
    ("shape_extents", np.float32, 3), ("aabb_min", np.float32, 3), ("aabb_max", np.float32, 3),
    ("linear_velocity", np.float32, 3), ("angular_velocity", np.float32, 3), ("is_awake", np.uint32),
    ("island_index", np.uint32),
])
DEBUG_CONTACT_DTYPE = np.dtype([("position", np.float32, 3), ("normal", np.float32, 3),
                                ("penetration_depth", np.float32), ("body_a", np.uint32), ("body_b", np.uint32)])
assert DEBUG_BODY_DTYPE.itemsize == 100 and DEBUG_CONTACT_DTYPE.itemsize == 36


def parse_snapshot(data: bytes) -> tuple[SnapshotHeader, np.ndarray, np.ndarray, list[np.ndarray]]:
    """(header, body records, warm-start entries, convex hull points) of a snapshot."""
    h = SnapshotHeader.from_buffer_copy(data[: ctypes.sizeof(SnapshotHeader)])
    off = ctypes.sizeof(SnapshotHeader)
    bodies = np.frombuffer(data, SNAPSHOT_BODY_DTYPE, h.body_count, off)
    off += SNAPSHOT_BODY_DTYPE.itemsize * h.body_count
    contacts = np.frombuffer(data, SNAPSHOT_CONTACT_DTYPE, h.contact_count, off)
    off += SNAPSHOT_CONTACT_DTYPE.itemsize * h.contact_count
    counts = np.frombuffer(data, np.uint32, h.hull_count, off)
    off += 4 * h.hull_count
    pts = np.frombuffer(data, np.float32, 3 * h.hull_vertex_count, off).reshape(-1, 3)
    hulls = np.split(pts, np.cumsum(counts)[:-1]) if h.hull_count else []
    return h, bodies, contacts, hulls


class SceneStruct(ctypes.Structure):
    _fields_ = [("n", ctypes.c_uint32), ("type", _U), ("shape", _U), ("position", _F),
                ("rotation", _F), ("linear_velocity", _F), ("angular_velocity", _F),
                ("shape_extents", _F), ("mass", _F), ("inertia", _F), ("friction", _F),
                ("restitution", _F), ("density", _F), ("linear_damping", _F),
                ("angular_damping", _F), ("structures", ctypes.c_uint32)]


class KernelProfile(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 32), ("launches", ctypes.c_uint64),
                ("ranges", ctypes.c_uint64), ("total_ms", ctypes.c_double)]


WORLD_FUNCS = {
    "axiom_world_config_default": (None, [ctypes.POINTER(WorldConfig)]),
    "axiom_world_create": (ctypes.c_int32, [ctypes.POINTER(WorldConfig), ctypes.POINTER(ctypes.c_void_p)]),
    "axiom_world_destroy": (ctypes.c_int32, [ctypes.c_void_p]),
    "axiom_world_add_bodies": (ctypes.c_int32, [ctypes.c_void_p, ctypes.POINTER(BodySoA), ctypes.c_uint32, _U]),
    "axiom_world_body_count": (ctypes.c_int32, [ctypes.c_void_p, _U]),
    "axiom_world_check_bodies": (ctypes.c_int32, [ctypes.c_void_p, ctypes.POINTER(BodySoA), ctypes.c_uint32]),
    "axiom_world_step": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_float, ctypes.POINTER(StepStats)]),
    "axiom_world_read_state": (ctypes.c_int32, [ctypes.c_void_p, _F, _F, _F, _F]),
    "axiom_world_write_state": (ctypes.c_int32, [ctypes.c_void_p, _F, _F, _F, _F]),
    "axiom_world_read_aabbs": (ctypes.c_int32, [ctypes.c_void_p, _F, _F]),
    "axiom_world_read_sleep": (ctypes.c_int32, [ctypes.c_void_p, _U8, _F, _U]),
    "axiom_world_add_convex_hull": (ctypes.c_int32, [ctypes.c_void_p, _F, ctypes.c_uint32, _U]),
    "axiom_world_add_triangle_mesh": (ctypes.c_int32, [ctypes.c_void_p, _F, ctypes.c_uint32, _U, ctypes.c_uint32,
                                                       ctypes.c_float, ctypes.c_float, _U]),
    "axiom_world_snapshot_size": (ctypes.c_int32, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)]),
    "axiom_world_save_snapshot": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64,
                                                   ctypes.POINTER(ctypes.c_uint64)]),
    "axiom_world_load_snapshot": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64]),
    "axiom_world_read_debug": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint32,
                                                ctypes.c_void_p, ctypes.c_uint32, _U, _U]),
    "axiom_world_set_sleeping": (ctypes.c_int32, [ctypes.c_void_p, _U, ctypes.c_uint32, ctypes.c_int32]),
    "axiom_world_read_pairs": (ctypes.c_int32, [ctypes.c_void_p, _U, ctypes.c_uint32, _U]),
    "axiom_world_read_contacts": (ctypes.c_int32, [ctypes.c_void_p, ctypes.POINTER(ContactPoint),
                                                   ctypes.c_uint32, _U]),
    "axiom_world_set_warm_start_model": (ctypes.c_int32, [ctypes.c_void_p, _F, ctypes.c_uint32]),
    "axiom_world_set_recording": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_int32]),
    "axiom_world_read_samples": (ctypes.c_int32, [ctypes.c_void_p, _F, _F, _U, ctypes.c_uint32, _U]),
    "axiom_world_set_profiling": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_int32]),
    "axiom_world_set_profiling_groups": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_uint32]),
    "axiom_world_reset_profile": (ctypes.c_int32, [ctypes.c_void_p]),
    "axiom_world_read_profile": (ctypes.c_int32, [ctypes.c_void_p, ctypes.POINTER(KernelProfile),
                                                  ctypes.c_uint32, _U]),
    "axiom_version": (ctypes.c_char_p, []),
}
SCENE_FUNCS = {
    "axiom_scene_sphere_drop": (ctypes.c_int32, [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_float,
                                                 ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                                 ctypes.c_float, ctypes.POINTER(ctypes.POINTER(SceneStruct))]),
    "axiom_scene_sphere_lattice": (ctypes.c_int32, [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32,
                                                    ctypes.c_uint32, ctypes.c_float, ctypes.c_float,
                                                    ctypes.c_float, ctypes.c_float,
                                                    ctypes.POINTER(ctypes.POINTER(SceneStruct))]),
    "axiom_scene_sphere_pile": (ctypes.c_int32, [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32,
                                                 ctypes.c_uint32, ctypes.c_float, ctypes.c_float,
                                                 ctypes.c_float, ctypes.c_float,
                                                 ctypes.POINTER(ctypes.POINTER(SceneStruct))]),
    "axiom_scene_mixed": (ctypes.c_int32, [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_float,
                                           ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                           ctypes.POINTER(ctypes.POINTER(SceneStruct))]),
    "axiom_scene_towers": (ctypes.c_int32, [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_float,
                                            ctypes.POINTER(ctypes.POINTER(SceneStruct))]),
    "axiom_scene_free": (None, [ctypes.POINTER(SceneStruct)]),
    "axiom_scene_as_soa": (None, [ctypes.POINTER(SceneStruct), ctypes.POINTER(BodySoA)]),
    "axiom_rng_u32": (None, [ctypes.c_uint64, ctypes.c_uint32, _U]),
    "axiom_rng_float": (None, [ctypes.c_uint64, ctypes.c_uint32, _F]),
    "axiom_rng_float_range": (None, [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_float, ctypes.c_float, _F]),
}


MLP_FUNCS = {
    "axiom_mlp_create": (ctypes.c_int32, [ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p)]),
    "axiom_mlp_destroy": (ctypes.c_int32, [ctypes.c_void_p]),
    "axiom_mlp_set_params": (ctypes.c_int32, [ctypes.c_void_p, _F, ctypes.c_uint32]),
    "axiom_mlp_get_params": (ctypes.c_int32, [ctypes.c_void_p, _F, ctypes.c_uint32]),
    "axiom_mlp_forward": (ctypes.c_int32, [ctypes.c_void_p, _F, ctypes.c_uint32, _F]),
    "axiom_mlp_gradients": (ctypes.c_int32, [ctypes.c_void_p, _F, _F, ctypes.c_uint32, _F, _F]),
    "axiom_mlp_train": (ctypes.c_int32, [ctypes.c_void_p, _F, _F, ctypes.c_uint32, ctypes.c_uint32,
                                         ctypes.c_uint32, ctypes.c_float, ctypes.c_uint64, _F]),
}


_U64 = ctypes.POINTER(ctypes.c_uint64)
BATCH_FUNCS = {
    "axiom_batch_create": (ctypes.c_int32, [ctypes.POINTER(WorldConfig), ctypes.POINTER(ctypes.c_void_p)]),
    "axiom_batch_destroy": (ctypes.c_int32, [ctypes.c_void_p]),
    "axiom_batch_set_worlds": (ctypes.c_int32, [ctypes.c_void_p, ctypes.POINTER(BodySoA), _U, ctypes.c_uint32]),
    "axiom_batch_step": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_float, ctypes.POINTER(StepStats)]),
    "axiom_batch_read_world_stats": (ctypes.c_int32, [ctypes.c_void_p, _U, _U64, _F]),
    "axiom_batch_read_phase_ns": (ctypes.c_int32, [ctypes.c_void_p, _U64]),
    "axiom_batch_read_state": (ctypes.c_int32, [ctypes.c_void_p, _F, _F, _F, _F]),
    "axiom_batch_set_launch": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32]),
    "axiom_batch_autotune": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_uint32, _U, _U]),
    "axiom_batch_inject_queue_fault": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32]),
    "axiom_batch_set_stage": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_uint32]),
    "axiom_batch_get_launch": (ctypes.c_int32, [ctypes.c_void_p, _U, _U, _U]),
    "axiom_scene_batch": (ctypes.c_int32, [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_float, ctypes.c_float,
                                           ctypes.c_uint32, ctypes.c_uint32, ctypes.c_float, _U,
                                           ctypes.POINTER(ctypes.POINTER(SceneStruct))]),
}


def _bind(lib: ctypes.CDLL, funcs: dict) -> ctypes.CDLL:
    for name, (res, args) in funcs.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


_LIB_CACHE: dict[str, ctypes.CDLL] = {}


def load_library(path: str | os.PathLike | None = None) -> ctypes.CDLL:
    """Loads the CUDA step library (built in-tree by build.py).  Raises if absent."""
    p = Path(path) if path else Path(os.environ.get("AXIOM_GB300_LIB", DEFAULT_LIB))
    key = str(p.resolve())
    if key not in _LIB_CACHE:
        if not p.exists():
            raise FileNotFoundError(f"{p} not built: run axiom-physics-engine_gb300/build.py "
                                    "(the GPU step has no CPU fallback)")
        lib = ctypes.CDLL(str(p))
        _bind(lib, WORLD_FUNCS)
        _bind(lib, SCENE_FUNCS)
        _bind(lib, MLP_FUNCS)
        _bind(lib, BATCH_FUNCS)
        _LIB_CACHE[key] = lib
    return _LIB_CACHE[key]


def _check(code: int, what: str) -> None:
    if code != 0:
        raise AxiomError(code, what)


def _fptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(_F)


def _uptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(_U)


def default_config(lib: ctypes.CDLL | None = None, **overrides) -> WorldConfig:
    """gui::PhysicsWorldConfig defaults plus the solver controls, with overrides."""
    lib = lib or load_library()
    cfg = WorldConfig()
    lib.axiom_world_config_default(ctypes.byref(cfg))
    for k, v in overrides.items():
        if k == "gravity":
            cfg.gravity[:] = list(v)
        else:
            setattr(cfg, k, v)
    return cfg


SCENE_FIELDS = ("type", "shape", "position", "rotation", "linear_velocity", "angular_velocity",
                "shape_extents", "mass", "inertia", "friction", "restitution", "density",
                "linear_damping", "angular_damping")
# gui::FilterInfo: category / mask bits and group index (defaults 0x0001 / 0xFFFF / 0)
FILTER_FIELDS = ("filter_category", "filter_mask", "filter_group")
# gui::SleepInfo: allowSleep (default 1) and isSleeping (default 0)
SLEEP_FIELDS = ("allow_sleep", "is_sleeping")
# hull id (PhysicsWorld.add_convex_hull) of each SHAPE_CONVEX body
BODY_FIELDS = SCENE_FIELDS + FILTER_FIELDS + SLEEP_FIELDS + ("convex_hull", "rolling_friction")
_DTYPE = {"type": np.uint32, "shape": np.uint32, "filter_category": np.uint32, "filter_mask": np.uint32,
          "filter_group": np.int16, "allow_sleep": np.uint8, "is_sleeping": np.uint8, "convex_hull": np.uint32}
_WIDTH = {"position": 3, "rotation": 4, "linear_velocity": 3, "angular_velocity": 3,
          "shape_extents": 3, "inertia": 3}


class Bodies:
    """Host SoA body description (fields of gui::RigidBodyData), numpy-owned."""

    def __init__(self, **fields):
        n = None
        self.arrays: dict[str, np.ndarray] = {}
        for name in BODY_FIELDS:
            v = fields.get(name)
            if v is None:
                continue
            dt = _DTYPE.get(name, np.float32)
            a = np.ascontiguousarray(np.asarray(v, dtype=dt))
            w = _WIDTH.get(name, 1)
            a = a.reshape(-1, w) if w > 1 else a.reshape(-1)
            if n is None:
                n = a.shape[0]
            elif a.shape[0] != n:
                raise ValueError(f"field {name} has {a.shape[0]} rows, expected {n}")
            self.arrays[name] = a
        for req in ("type", "shape", "position", "shape_extents"):
            if req not in self.arrays:
                raise ValueError(f"missing required body field {req}")
        self.n = int(n or 0)

    def soa(self) -> BodySoA:
        s = BodySoA()
        for name in BODY_FIELDS:
            a = self.arrays.get(name)
            if a is None:
                ptr = None
            elif a.dtype == np.uint32:
                ptr = _uptr(a)
            elif a.dtype == np.int16:
                ptr = a.ctypes.data_as(ctypes.POINTER(ctypes.c_int16))
            elif a.dtype == np.uint8:
                ptr = a.ctypes.data_as(_U8)
            else:
                ptr = _fptr(a)
            setattr(s, name, ptr)
        return s

    def subset(self, idx) -> "Bodies":
        return Bodies(**{k: v[idx] for k, v in self.arrays.items()})


class Scene:
    """A seeded benchmark scene generated by the library's host code (axiom_scene.h)."""

    def __init__(self, lib: ctypes.CDLL, ptr):
        self._lib = lib
        self._ptr = ptr
        s = ptr.contents
        self.n = int(s.n)
        self.structures = int(s.structures)
        self.bodies = Bodies(**{
            name: np.ctypeslib.as_array(getattr(s, name), shape=(self.n * _WIDTH.get(name, 1),)).copy()
            for name in SCENE_FIELDS})

    def __del__(self):
        try:
            if self._ptr:
                self._lib.axiom_scene_free(self._ptr)
                self._ptr = None
        except Exception:
            pass

    @staticmethod
    def _make(lib, fn_name, *args) -> "Scene":
        out = ctypes.POINTER(SceneStruct)()
        _check(getattr(lib, fn_name)(*args, ctypes.byref(out)), fn_name)
        return Scene(lib, out)

    @classmethod
    def sphere_drop(cls, seed=1, count=1000, radius=0.5, size=(20.0, 40.0, 20.0), friction=0.5, lib=None):
        lib = lib or load_library()
        return cls._make(lib, "axiom_scene_sphere_drop", seed, count, radius, *size, friction)

    @classmethod
    def sphere_lattice(cls, seed=3, dims=(128, 64, 128), spacing=0.49, radius=0.25, jitter=0.002,
                       friction=0.5, lib=None):
        lib = lib or load_library()
        return cls._make(lib, "axiom_scene_sphere_lattice", seed, *dims, spacing, radius, jitter, friction)

    @classmethod
    def sphere_pile(cls, seed=3, dims=(128, 64, 128), spacing=0.49, radius=0.25, jitter=0.002,
                    friction=0.5, lib=None):
        """The lattice held by four wall planes touching its outer spheres (a dense pile that
        keeps its ~6 contacts per body); walls and ground are the last five bodies."""
        lib = lib or load_library()
        return cls._make(lib, "axiom_scene_sphere_pile", seed, *dims, spacing, radius, jitter, friction)

    @classmethod
    def mixed(cls, seed=2, count=100_000, size=(200.0, 100.0, 200.0), friction=0.5, lib=None):
        lib = lib or load_library()
        return cls._make(lib, "axiom_scene_mixed", seed, count, *size, friction)

    @classmethod
    def towers(cls, seed=5, count=2048, friction=0.6, lib=None):
        lib = lib or load_library()
        return cls._make(lib, "axiom_scene_towers", seed, count, friction)


class PhysicsWorld:
    """One world on one GPU (or on the CPU oracle when given ``liboracle.so``)."""

    def __init__(self, config: WorldConfig | None = None, lib: ctypes.CDLL | None = None, **overrides):
        self.lib = lib or load_library()
        self.config = config if config is not None else default_config(self.lib, **overrides)
        self._h = ctypes.c_void_p()
        _check(self.lib.axiom_world_create(ctypes.byref(self.config), ctypes.byref(self._h)),
               "axiom_world_create")
        self.last_stats: StepStats | None = None

    @classmethod
    def create(cls, config: WorldConfig | None = None, lib=None, **overrides) -> "PhysicsWorld":
        return cls(config, lib, **overrides)

    def close(self) -> None:
        if self._h:
            self.lib.axiom_world_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def add_bodies(self, bodies: Bodies) -> int:
        first = ctypes.c_uint32()
        soa = bodies.soa()
        _check(self.lib.axiom_world_add_bodies(self._h, ctypes.byref(soa), bodies.n, ctypes.byref(first)),
               "axiom_world_add_bodies")
        return int(first.value)

    def add_convex_hull(self, points) -> int:
        """Registers a convex hull (points [k][3] in the body frame); returns its id."""
        pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
        hid = ctypes.c_uint32()
        _check(self.lib.axiom_world_add_convex_hull(self._h, _fptr(pts), len(pts), ctypes.byref(hid)),
               "axiom_world_add_convex_hull")
        return int(hid.value)

    def add_triangle_mesh(self, vertices, triangles, friction: float = 0.5, restitution: float = 0.5) -> int:
        """Static triangle mesh (world-space vertices [v][3], triangles [t][3]); returns the
        id of the first triangle body (one static body per triangle)."""
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
        t = np.ascontiguousarray(triangles, np.uint32).reshape(-1, 3)
        first = ctypes.c_uint32()
        _check(self.lib.axiom_world_add_triangle_mesh(self._h, _fptr(v), len(v), _uptr(t), len(t), friction,
                                                      restitution, ctypes.byref(first)),
               "axiom_world_add_triangle_mesh")
        return int(first.value)

    def body_count(self) -> int:
        n = ctypes.c_uint32()
        _check(self.lib.axiom_world_body_count(self._h, ctypes.byref(n)), "axiom_world_body_count")
        return int(n.value)

    def step(self, dt: float = 0.0, check: bool = True) -> StepStats:
        """One step.  With check, a status that means the step did not complete raises;
        GJKFailedToConverge / EPAFailedToConverge (a completed step with pairs whose
        contact is approximate) are left to the caller in the returned stats."""
        st = StepStats()
        code = self.lib.axiom_world_step(self._h, float(dt), ctypes.byref(st))
        self.last_stats = st
        if check and code not in STEP_COMPLETED:
            _check(code, "axiom_world_step")
        return st

    def read_state(self, out: dict[str, np.ndarray] | None = None) -> dict[str, np.ndarray]:
        """Body state; out (optional) holds caller-owned float32 arrays to fill, e.g. pinned."""
        n = self.body_count()
        if out is None:
            out = {"position": np.empty((n, 3), np.float32), "rotation": np.empty((n, 4), np.float32),
                   "linear_velocity": np.empty((n, 3), np.float32),
                   "angular_velocity": np.empty((n, 3), np.float32)}
        for k, w in (("position", 3), ("rotation", 4), ("linear_velocity", 3), ("angular_velocity", 3)):
            a = out[k]
            if a.dtype != np.float32 or not a.flags.c_contiguous or a.size != n * w:
                raise ValueError(f"read_state: out[{k!r}] must be a contiguous float32 array of {n} x {w}")
        _check(self.lib.axiom_world_read_state(self._h, _fptr(out["position"]), _fptr(out["rotation"]),
                                               _fptr(out["linear_velocity"]), _fptr(out["angular_velocity"])),
               "axiom_world_read_state")
        return out

    def write_state(self, position=None, rotation=None, linear_velocity=None, angular_velocity=None) -> None:
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float32)
                for a in (position, rotation, linear_velocity, angular_velocity)]
        _check(self.lib.axiom_world_write_state(self._h, *[_fptr(a) for a in arrs]),
               "axiom_world_write_state")

    def read_aabbs(self) -> tuple[np.ndarray, np.ndarray]:
        n = self.body_count()
        mn = np.empty((n, 3), np.float32)
        mx = np.empty((n, 3), np.float32)
        _check(self.lib.axiom_world_read_aabbs(self._h, _fptr(mn), _fptr(mx)), "axiom_world_read_aabbs")
        return mn, mx

    def read_sleep(self) -> dict[str, np.ndarray]:
        """Per body: sleeping flag, sleep time (s) and island label (gui::SleepInfo)."""
        n = self.body_count()
        sl = np.zeros(n, np.uint8)
        st = np.zeros(n, np.float32)
        isl = np.zeros(n, np.uint32)
        _check(self.lib.axiom_world_read_sleep(self._h, sl.ctypes.data_as(_U8), _fptr(st), _uptr(isl)),
               "axiom_world_read_sleep")
        return {"sleeping": sl, "sleep_time": st, "island": isl}

    def save_snapshot(self) -> bytes:
        """Everything needed to resume this world bit for bit (layout in include/axiom_c.h)."""
        size = ctypes.c_uint64()
        _check(self.lib.axiom_world_snapshot_size(self._h, ctypes.byref(size)), "axiom_world_snapshot_size")
        buf = ctypes.create_string_buffer(size.value)
        written = ctypes.c_uint64()
        _check(self.lib.axiom_world_save_snapshot(self._h, buf, size.value, ctypes.byref(written)),
               "axiom_world_save_snapshot")
        return buf.raw[: written.value]

    def load_snapshot(self, data: bytes) -> None:
        """Replaces this world's bodies, configuration and warm start with the snapshot's."""
        buf = ctypes.create_string_buffer(bytes(data), len(data))
        _check(self.lib.axiom_world_load_snapshot(self._h, buf, len(data)), "axiom_world_load_snapshot")
        n = ctypes.c_uint32()
        self.lib.axiom_world_body_count(self._h, ctypes.byref(n))

    def read_debug(self, flags: int = DEBUG_ALL) -> tuple[np.ndarray, np.ndarray]:
        """Debug-draw records of every body and of the last step's contact points."""
        nb, nc = ctypes.c_uint32(), ctypes.c_uint32()
        _check(self.lib.axiom_world_read_debug(self._h, flags, None, 0, None, 0, ctypes.byref(nb), ctypes.byref(nc)),
               "axiom_world_read_debug")
        bodies = np.zeros(nb.value, DEBUG_BODY_DTYPE)
        contacts = np.zeros(nc.value, DEBUG_CONTACT_DTYPE)
        _check(self.lib.axiom_world_read_debug(self._h, flags, bodies.ctypes.data, nb.value, contacts.ctypes.data,
                                               nc.value, ctypes.byref(nb), ctypes.byref(nc)),
               "axiom_world_read_debug")
        return bodies, contacts[: nc.value]

    def set_sleeping(self, ids, sleeping: bool) -> None:
        """Wakes (False) or puts to sleep (True) the listed bodies."""
        a = np.ascontiguousarray(ids, np.uint32).reshape(-1)
        _check(self.lib.axiom_world_set_sleeping(self._h, _uptr(a), a.size, int(bool(sleeping))),
               "axiom_world_set_sleeping")

    def read_pairs(self) -> np.ndarray:
        cnt = ctypes.c_uint32()
        _check(self.lib.axiom_world_read_pairs(self._h, None, 0, ctypes.byref(cnt)), "axiom_world_read_pairs")
        out = np.empty((cnt.value, 2), np.uint32)
        _check(self.lib.axiom_world_read_pairs(self._h, _uptr(out), cnt.value, ctypes.byref(cnt)),
               "axiom_world_read_pairs")
        return out

    def read_contacts(self) -> np.ndarray:
        cnt = ctypes.c_uint32()
        _check(self.lib.axiom_world_read_contacts(self._h, None, 0, ctypes.byref(cnt)),
               "axiom_world_read_contacts")
        out = np.zeros(cnt.value, dtype=CONTACT_DTYPE)
        ptr = out.ctypes.data_as(ctypes.POINTER(ContactPoint))
        _check(self.lib.axiom_world_read_contacts(self._h, ptr, cnt.value, ctypes.byref(cnt)),
               "axiom_world_read_contacts")
        return out[: cnt.value]

    def set_profiling(self, enable: bool = True) -> None:
        _check(self.lib.axiom_world_set_profiling(self._h, int(bool(enable))), "axiom_world_set_profiling")

    PROFILE_GROUPS = ("integrate_velocities", "radix_sort", "broadphase_gather", "broadphase_sweep",
                      "narrowphase", "colouring", "solver_prepare", "warm_start_apply", "pgs_colour",
                      "store_impulses", "integrate_positions", "sleep_islands")

    def set_profiling_groups(self, groups) -> None:
        """Times only the named kernel groups (others keep launch counts only)."""
        mask = 0
        for g in groups:
            mask |= 1 << self.PROFILE_GROUPS.index(g)
        _check(self.lib.axiom_world_set_profiling_groups(self._h, mask), "axiom_world_set_profiling_groups")

    def reset_profile(self) -> None:
        _check(self.lib.axiom_world_reset_profile(self._h), "axiom_world_reset_profile")

    def read_profile(self) -> dict[str, dict]:
        """Per kernel group: launches, timed ranges and summed device milliseconds."""
        cnt = ctypes.c_uint32()
        _check(self.lib.axiom_world_read_profile(self._h, None, 0, ctypes.byref(cnt)), "axiom_world_read_profile")
        arr = (KernelProfile * max(cnt.value, 1))()
        _check(self.lib.axiom_world_read_profile(self._h, arr, cnt.value, ctypes.byref(cnt)),
               "axiom_world_read_profile")
        return {arr[i].name.decode(): {"launches": int(arr[i].launches), "ranges": int(arr[i].ranges),
                                       "ms": float(arr[i].total_ms)} for i in range(cnt.value)}

    def set_recording(self, enable: bool = True) -> None:
        _check(self.lib.axiom_world_set_recording(self._h, int(bool(enable))), "axiom_world_set_recording")

    def read_samples(self) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        """Features [n][14], targets [n][3] and keys (a, b, point) [n][3] of the last step."""
        cnt = ctypes.c_uint32()
        _check(self.lib.axiom_world_read_samples(self._h, None, None, None, 0, ctypes.byref(cnt)),
               "axiom_world_read_samples")
        n = cnt.value
        f = np.zeros((n, 14), np.float32)
        t = np.zeros((n, 3), np.float32)
        k = np.zeros((n, 3), np.uint32)
        _check(self.lib.axiom_world_read_samples(self._h, _fptr(f), _fptr(t), _uptr(k), n, ctypes.byref(cnt)),
               "axiom_world_read_samples")
        return f, t, k

    def set_warm_start_model(self, params: np.ndarray) -> None:
        p = np.ascontiguousarray(params, dtype=np.float32).reshape(-1)
        _check(self.lib.axiom_world_set_warm_start_model(self._h, _fptr(p), p.size),
               "axiom_world_set_warm_start_model")


class BatchScene:
    """Batched-world scene: bodies of all worlds and each world's size (axiom_scene_batch)."""

    def __init__(self, seed=4, worlds=4096, median=256.0, sigma=1.0, min_bodies=16, max_bodies=8192,
                 friction=0.5, lib=None):
        lib = lib or load_library()
        self.sizes = np.zeros(worlds, np.uint32)
        out = ctypes.POINTER(SceneStruct)()
        _check(lib.axiom_scene_batch(seed, worlds, median, sigma, min_bodies, max_bodies, friction,
                                     _uptr(self.sizes), ctypes.byref(out)), "axiom_scene_batch")
        self.scene = Scene(lib, out)
        self.bodies = self.scene.bodies
        self.offsets = np.concatenate([[0], np.cumsum(self.sizes.astype(np.int64))])

    def world(self, w: int) -> Bodies:
        return self.bodies.subset(slice(int(self.offsets[w]), int(self.offsets[w + 1])))


class Batch:
    """Independent worlds stepped together by one persistent kernel (axiom_batch_*)."""

    def __init__(self, config: WorldConfig | None = None, lib=None, **overrides):
        self.lib = lib or load_library()
        self.config = config if config is not None else default_config(self.lib, **overrides)
        self._h = ctypes.c_void_p()
        _check(self.lib.axiom_batch_create(ctypes.byref(self.config), ctypes.byref(self._h)), "axiom_batch_create")
        self.sizes = None

    def close(self):
        if self._h:
            self.lib.axiom_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_worlds(self, bodies: Bodies, sizes) -> None:
        self.sizes = np.ascontiguousarray(sizes, np.uint32)
        soa = bodies.soa()
        _check(self.lib.axiom_batch_set_worlds(self._h, ctypes.byref(soa), _uptr(self.sizes), len(self.sizes)),
               "axiom_batch_set_worlds")

    def step(self, dt: float = 0.0, check: bool = True) -> StepStats:
        st = StepStats()
        code = self.lib.axiom_batch_step(self._h, float(dt), ctypes.byref(st))
        if check and code not in STEP_COMPLETED:
            _check(code, "axiom_batch_step")
        return st

    def world_stats(self) -> dict:
        n = len(self.sizes)
        counts = np.zeros((n, 8), np.uint32)
        ns = np.zeros(n, np.uint64)
        res = np.zeros(n, np.float32)
        _check(self.lib.axiom_batch_read_world_stats(self._h, _uptr(counts), ns.ctypes.data_as(_U64), _fptr(res)),
               "axiom_batch_read_world_stats")
        names = ("pairs", "manifolds", "points", "colours", "rounds", "iterations", "flags", "gjk")
        out = {k: counts[:, i] for i, k in enumerate(names)}
        out["step_ns"] = ns
        out["residual"] = res
        return out

    PHASES = ("integrate_sort", "sweep", "narrow_analytic", "gjk_epa", "colouring", "solver", "store_positions")

    def phase_ns(self) -> np.ndarray:
        """[worlds, 7] device ns of each phase of the last step (names in PHASES)."""
        out = np.zeros((len(self.sizes), len(self.PHASES)), np.uint64)
        _check(self.lib.axiom_batch_read_phase_ns(self._h, out.ctypes.data_as(_U64)), "axiom_batch_read_phase_ns")
        return out

    def read_state(self) -> dict[str, np.ndarray]:
        n = int(self.sizes.sum())
        pos = np.empty((n, 3), np.float32)
        rot = np.empty((n, 4), np.float32)
        lin = np.empty((n, 3), np.float32)
        ang = np.empty((n, 3), np.float32)
        _check(self.lib.axiom_batch_read_state(self._h, _fptr(pos), _fptr(rot), _fptr(lin), _fptr(ang)),
               "axiom_batch_read_state")
        return {"position": pos, "rotation": rot, "linear_velocity": lin, "angular_velocity": ang}

    def set_launch(self, block: int, ctas_per_sm: int) -> None:
        _check(self.lib.axiom_batch_set_launch(self._h, block, ctas_per_sm), "axiom_batch_set_launch")

    def set_stage(self, stage_bodies: int) -> None:
        """Worlds of at most stage_bodies bodies solve with their bodies in shared memory."""
        _check(self.lib.axiom_batch_set_stage(self._h, stage_bodies), "axiom_batch_set_stage")

    def launch(self) -> tuple[int, int, int]:
        """(threads per world, CTAs per SM, staged bodies) of the persistent kernel."""
        b, c, s = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        _check(self.lib.axiom_batch_get_launch(self._h, ctypes.byref(b), ctypes.byref(c), ctypes.byref(s)),
               "axiom_batch_get_launch")
        return int(b.value), int(c.value), int(s.value)

    def inject_queue_fault(self, kind: int, value: int) -> None:
        """Corrupts the next step's work queue on the host (kind 1: the counter starts at
        `value`; kind 2: entry `value` names no world), for failure-detection tests."""
        _check(self.lib.axiom_batch_inject_queue_fault(self._h, kind, value), "axiom_batch_inject_queue_fault")

    def autotune(self, cache_path: str | None = None, trial_steps: int = 2) -> tuple[int, int]:
        b = ctypes.c_uint32()
        c = ctypes.c_uint32()
        path = cache_path.encode() if cache_path else None
        _check(self.lib.axiom_batch_autotune(self._h, path, trial_steps, ctypes.byref(b), ctypes.byref(c)),
               "axiom_batch_autotune")
        return int(b.value), int(c.value)


def canonical_pairs(pairs: np.ndarray) -> np.ndarray:
    """Pairs as a sorted (P, 2) array, for set comparison."""
    if len(pairs) == 0:
        return pairs.reshape(0, 2)
    keys = pairs[:, 0].astype(np.uint64) << np.uint64(32) | pairs[:, 1].astype(np.uint64)
    return pairs[np.argsort(keys, kind="stable")]


def canonical_contacts(c: np.ndarray) -> np.ndarray:
    """Contacts sorted by (body_a, body_b, point_index)."""
    order = np.lexsort((c["point_index"], c["body_b"], c["body_a"]))
    return c[order]
