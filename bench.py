"""Benchmark of the GB300 rigid-body step (body-steps/s on the 1M-sphere pile).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Workload: 1,048,576 spheres (r 0.25 m, rho 1000) on a seeded jittered 128x64x128 cubic
lattice (spacing 0.49 m, jitter +-0.002 m) on a ground plane, held by four wall planes
that touch its outer spheres: a dense pile that keeps its ~6 contacts per body through
the run.  dt 1/120 s, 10 PGS sweeps with previous-step warm start, linear slop 0.02 m
(the lattice's 6-14 mm overlaps lie inside it, so the pile starts at rest instead of
being pushed apart by the position bias), temporally coherent colouring (a contact that
persists keeps last step's colour), fp32.  A step is one full broadphase ->
narrowphase -> colouring -> PGS -> integration pass over the pile.

value      bodies x K / device time of the K steps (CUDA events the library records on
           its own stream around every step), state resident in HBM.  Inside the timed
           steps only the PGS colour launches are bracketed by profiler events (for the
           roofline); stage_ms comes from up to 5 further steps with every stage timed.
e2e        the same metric through the C ABI with host buffers: every step writes the
           body state from host memory, steps, and reads the state back; e2e.link is the
           host link alone (the same pinned arrays copied each way with plain copies), the
           floor of those transfers.
roofline   the PGS colour kernel (the dominant kernel): algorithmic bytes per launch /
           mean launch duration (CUDA events around each launch, on the library stream),
           196 B per contact point and sweep; step_frac applies the whole-step byte count
           280 N + 228 P + 196 I P (N bodies, P contact points, I sweeps) to the step time.
learned_vs_plain  PGS sweeps, solver ms and final residual to the 1e-4 residual on a
           box-tower scene, previous-step warm start against the trained network (the
           committed weight file), both from the same settled state.
cpu_baseline  the CPU oracle (this project's restatement of the step; the reference has
           no step of its own) on the first timed steps of the same pile, all host cores.

--impl reference times that CPU oracle as the reference arm on the full pile with the same
--steps / --warmup (one JSON line, rank 0); it loads only the oracle library.
With --gpus N > 1 (torchrun) every rank steps its own replica of the pile: the single
world does not shard, so the run is N independent replicas ("scaling": "weak").
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "axiom-physics-engine_gb300"
sys.path.insert(0, str(PKG))

import numpy as np  # noqa: E402

METRIC = "body-steps/s at 1M spheres; PGS iters+ms to 1e-4 residual, learned vs plain"
UNIT = "body-steps/s"
DIMS = (128, 64, 128)
SEED = 3
DT = 1.0 / 120.0
ITERS = 10
SLOP = 0.02
CPU_MAX_STEPS = 10  # the CPU baseline times at most this many of the timed steps

# Algorithmic bytes of the step (sphere form; N bodies, P contact points, I sweeps):
#   integrate velocity + AABB 64 N, Morton 32 N, radix sort 64 N, sweep 32 N + 8 P,
#   narrowphase 68 P, warm-start match 32 P, colouring 12 P + 8 N, solver preparation 108 P,
#   PGS 196 P per sweep (read 2 x (v 12 + w 12), constants 76, impulses 12; write impulses
#   12 and 2 x (v 12 + w 12)), integrate position 80 N.
STEP_BYTES_PER_BODY = 280
STEP_BYTES_PER_POINT = 228
PGS_BYTES_PER_POINT_SWEEP = 196
# The same PGS update as the kernel's records move it (single-point sphere manifold):
#   hdr 16 + normal 16 + rA 16 + rB 16 + kt 8 + impulses 16 read, impulses 16 written,
#   two 32-byte solver bodies read and, for each dynamic body, written (a plane manifold
#   writes only its sphere).
PGS_PADDED_BYTES_READ = 88 + 64
PGS_PADDED_BYTES_WRITE_FIXED = 16
PGS_PADDED_BYTES_PER_DYNAMIC_BODY = 32
# DRAM bytes the PGS colour kernel moves per manifold and sweep: ncu dram__bytes_read.sum +
# dram__bytes_write.sum (warm caches) of the first five colour launches of a sweep on the
# 128x32x128 walled pile (1.57 M manifolds), divided by those colours' manifolds; scaled to
# a launch of this workload by its manifold-sweeps
PGS_DRAM_BYTES_PER_MANIFOLD_SWEEP = 94.5

# Learned-vs-plain evaluation: box towers (base 4-16, 4-32 levels, friction 0.6), dt 1/60,
# PGS to residual 1e-4; the trained network is the committed weight file
WARMSTART_WEIGHTS = PKG / "weights" / "warmstart_towers.npy"
EVAL_TOWERS, EVAL_SEED, EVAL_SETTLE, EVAL_STEPS = 256, 11, 5, 8


def peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []
        self._first = threading.Event()

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
            # nvidia-smi takes a moment to start; a timed region shorter than that would
            # otherwise see no sample, so the region starts once sampling is live
            self._first.wait(timeout=5.0)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())
            self._first.set()
        self._first.set()

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env() -> tuple[int, int, int]:
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def load_oracle(path):
    """The CPU oracle library alone: the step and the seeded scene generators."""
    import axiom_gb300 as ax

    o = ctypes.CDLL(str(path))
    ax._bind(o, ax.WORLD_FUNCS)
    ax._bind(o, ax.SCENE_FUNCS)
    o.oracle_set_threads.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    o.oracle_set_threads.restype = ctypes.c_int32
    return o


def pile_config(lib, **kw):
    import axiom_gb300 as ax

    cfg = dict(time_step=DT, velocity_iterations=ITERS, linear_slop=SLOP, temporal_colouring=1)
    cfg.update(kw)
    return ax.default_config(lib, **cfg)


def pile_scene(lib, dims=DIMS):
    import axiom_gb300 as ax

    return ax.Scene.sphere_pile(seed=SEED, dims=dims, lib=lib)


def oracle_world(oracle, threads: int):
    import axiom_gb300 as ax

    w = ax.PhysicsWorld(pile_config(oracle), lib=oracle)
    oracle.oracle_set_threads(w.handle, threads)
    return w


def run_reference(args) -> int:
    """The reference arm: the CPU oracle alone (no GPU library is loaded) on the full pile,
    the same warm-up and timed steps as the GPU arm, all host cores."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    import build as axbuild

    oracle = load_oracle(axbuild.build_oracle())
    threads = os.cpu_count() or 1
    steps, warmup = max(1, args.steps), max(3, args.warmup)
    dims = tuple(int(x) for x in args.dims.split(","))
    sc = pile_scene(oracle, dims)
    w = oracle_world(oracle, threads)
    w.add_bodies(sc.bodies)
    for _ in range(warmup):
        w.step(DT)
    manifolds = []
    t0 = time.perf_counter()
    for _ in range(steps):
        manifolds.append(w.step(DT).manifold_count)
    secs = time.perf_counter() - t0
    v = sc.n * steps / secs
    sample = (f"the whole pile ({sc.n} bodies incl. walls and ground), {steps} steps after {warmup} "
              f"warm-up, {secs:.1f} s")
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": steps, "warmup": warmup, "ms_per_step": secs / steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded DeterministicRNG lattice)",
        "config": {"workload": workload_name(dims), "bodies": sc.n, "lattice": list(dims), "dt": DT,
                   "pgs_iterations": ITERS, "linear_slop_m": SLOP, "temporal_colouring": 1,
                   "manifolds_min_max": [min(manifolds), max(manifolds)]},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference engine has no rigid-body step (src/collision, src/dynamics are "
                "empty); its arm is this project's CPU oracle of the same step",
    }
    print(json.dumps(line), flush=True)
    return 0


def workload_name(dims) -> str:
    return "sphere_pile_1M" if tuple(dims) == DIMS else "sphere_pile_%dx%dx%d" % tuple(dims)


def learned_vs_plain(lib) -> dict:
    """Sweeps, solver ms and final residual to the 1e-4 PGS residual on a box-tower scene,
    plain previous-step warm start against the trained network, both arms stepping the
    same steps from the same settled state (warmstart.evaluate)."""
    import warmstart

    if not WARMSTART_WEIGHTS.exists():
        return {"unavailable": f"no trained weight file {WARMSTART_WEIGHTS.name}"}
    params = np.load(WARMSTART_WEIGHTS).astype(np.float32)
    ev = warmstart.evaluate(lib, params, towers=EVAL_TOWERS, seed=EVAL_SEED, steps=EVAL_STEPS, settle=EVAL_SETTLE)
    out = {"scene": f"{EVAL_TOWERS} box towers (seed {EVAL_SEED}, {ev['bodies']} bodies), dt 1/60, "
                    f"{EVAL_STEPS} steps after {EVAL_SETTLE} settling steps, residual 1e-4",
           "weights": WARMSTART_WEIGHTS.name}
    for name in ("plain", "learned"):
        out[f"sweeps_{name}"] = ev[name]["mean_iterations"]
        out[f"ms_{name}"] = ev[name]["mean_solver_ms"]
        out[f"max_residual_{name}"] = ev[name]["max_residual"]
    out["sweep_reduction"] = ev["iteration_reduction"]
    out["time_reduction"] = ev["time_reduction"]
    return out


def max_over_ranks(values: list[float], world: int) -> list[float]:
    """Element-wise maximum over the ranks (gloo all-reduce): a replicated job's time is its
    slowest rank's.  The identity for one rank."""
    if world <= 1:
        return [float(v) for v in values]
    import torch
    import torch.distributed as dist

    t = torch.tensor(values, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t]


def run_gpu(args) -> int:
    rank, world, local = dist_env()
    import torch

    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    torch.cuda.set_device(local)
    import build as axbuild

    lib_path = library_path(axbuild)
    import axiom_gb300 as ax

    lib = ax.load_library(lib_path)
    dims = tuple(int(x) for x in args.dims.split(","))
    sc = pile_scene(lib, dims)
    w = ax.PhysicsWorld(pile_config(lib, device=local), lib=lib)
    w.add_bodies(sc.bodies)
    n_bodies = sc.n
    warmup = max(3, args.warmup)
    for _ in range(warmup):
        w.step(DT)
    # every leg below replays the same steps from this snapshot: the timed steps, the stage
    # breakdown, the e2e leg and the CPU baseline
    start = w.save_snapshot()

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            import torch.distributed as dist

            dist.barrier()

    # ---- device-resident timed region ----
    # only the PGS colour launches are timed with events here (their per-launch duration
    # feeds the roofline); the per-stage breakdown comes from a separate pass below, so
    # that the events of every other stage do not slow the timed steps
    w.set_profiling_groups(["pgs_colour"])
    w.reset_profile()
    barrier()
    step_ms, stats = [], []
    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            st = w.step(DT)
            step_ms.append(st.total_step_time)
            stats.append(st)
        barrier()
        wall = time.perf_counter() - t0
    prof = w.read_profile()
    w.set_profiling(False)
    # per-stage breakdown: the first steps of the timed region again, every kernel group timed
    breakdown_steps = max(1, min(args.steps, 5))
    w.load_snapshot(start)
    w.set_profiling(True)
    w.reset_profile()
    for _ in range(breakdown_steps):
        w.step(DT)
    stage_prof = w.read_profile()
    w.set_profiling(False)
    dev_s, wall = max_over_ranks([sum(step_ms) / 1e3, wall], world)
    value = n_bodies * args.steps * world / dev_s

    # ---- roofline of the PGS colour kernel and of the whole step ----
    pg = prof["pgs_colour"]
    launches = max(pg["launches"], 1)
    pgs_s = pg["ms"] / 1e3
    point_sweeps = sum(st.contact_point_count * st.iterations for st in stats)
    manifold_sweeps = sum(st.manifold_count * st.iterations for st in stats)
    bytes_per_launch = PGS_BYTES_PER_POINT_SWEEP * point_sweeps / launches
    launch_s = pgs_s / launches
    achieved = bytes_per_launch / launch_s / 1e9
    # the kernel's own record layout: plane manifolds (spheres against the ground and the
    # walls, counted in the last timed step) write one body, the others two
    contacts = w.read_contacts()
    plane_ids = np.nonzero(sc.bodies.arrays["shape"] == ax.SHAPE_PLANE)[0]
    plane_manifolds = int(np.isin(contacts["body_a"], plane_ids).sum())
    per_colour = np.bincount(contacts["colour"][contacts["point_index"] == 0]).tolist()
    padded = (manifold_sweeps * (PGS_PADDED_BYTES_READ + PGS_PADDED_BYTES_WRITE_FIXED
                                 + 2 * PGS_PADDED_BYTES_PER_DYNAMIC_BODY)
              - plane_manifolds * PGS_PADDED_BYTES_PER_DYNAMIC_BODY * sum(st.iterations for st in stats))
    step_bytes = sum(STEP_BYTES_PER_BODY * n_bodies + STEP_BYTES_PER_POINT * st.contact_point_count
                     + PGS_BYTES_PER_POINT_SWEEP * st.iterations * st.contact_point_count for st in stats)
    pk = peaks()
    traffic = PGS_DRAM_BYTES_PER_MANIFOLD_SWEEP * manifold_sweeps / launches
    gpu_launches = sum(v["launches"] for v in prof.values())

    # ---- end to end through the C ABI with host buffers: the timed steps again ----
    # host state in pinned (page-locked) memory, as a caller streaming states would hold it
    w.load_snapshot(start)
    nb = w.body_count()
    host = {k: torch.empty((nb, c), dtype=torch.float32, pin_memory=True).numpy()
            for k, c in (("position", 3), ("rotation", 4), ("linear_velocity", 3), ("angular_velocity", 3))}
    w.read_state(out=host)
    h2d = sum(host[k].nbytes for k in host)
    e2e_steps = 0 if args.no_e2e else args.steps
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        w.write_state(**host)
        w.step(DT)
        w.read_state(out=host)
    barrier()
    e2e_wall = max_over_ranks([max(time.perf_counter() - t0, 1e-9)], world)[0]
    e2e = n_bodies * e2e_steps * world / e2e_wall if e2e_steps else None
    link = copy_rates(host) if e2e_steps else None

    lvp = None
    if rank == 0 and not args.no_learned:
        lvp = learned_vs_plain(lib)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        # the oracle resumes the GPU world's snapshot and steps the first timed steps
        oracle = load_oracle(axbuild.build_oracle())
        threads = os.cpu_count() or 1
        o = oracle_world(oracle, threads)
        o.load_snapshot(start)
        oracle.oracle_set_threads(o.handle, threads)
        csteps = max(1, min(args.steps, CPU_MAX_STEPS))
        t0 = time.perf_counter()
        for _ in range(csteps):
            o.step(DT)
        secs = time.perf_counter() - t0
        cpu = {"value": n_bodies * csteps / secs, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"the whole pile ({n_bodies} bodies) resumed from the GPU's snapshot before the "
                         f"timed region, its first {csteps} timed steps, {secs:.1f} s"}

    if rank == 0:
        man = [st.manifold_count for st in stats]
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": warmup, "ms_per_step": dev_s / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded DeterministicRNG lattice)",
            "config": {
                "workload": workload_name(dims),
                "bodies": n_bodies, "lattice": list(dims), "walls": 4,
                "spacing_m": 0.49, "radius_m": 0.25, "jitter_m": 0.002, "dt": DT,
                "pgs_iterations": ITERS, "warm_start": "previous", "linear_slop_m": SLOP,
                "pairs_first_last": [stats[0].pair_count, stats[-1].pair_count],
                "manifolds_first_last": [stats[0].manifold_count, stats[-1].manifold_count],
                "manifolds_min_max": [min(man), max(man)],
                "contact_points_mean": float(np.mean([st.contact_point_count for st in stats])),
                "colours": stats[-1].colour_count, "colour_rounds": stats[-1].colour_rounds,
                "colour_rounds_first": stats[0].colour_rounds, "manifolds_per_colour_last": per_colour,
                "colouring": "temporally coherent (previous colours kept, new contacts recoloured)",
                "l2": "working set > L2 (pairs + manifold + solver arrays ~1.5 GB per step)",
                "parallelism": f"replicas{world}", "wall_ms_per_step": wall / args.steps * 1e3,
                "stage_ms": {k: round(v["ms"] / breakdown_steps, 4) for k, v in stage_prof.items()},
            },
            "roofline": {"bound": "hbm", "kernel": "kSolveColour (PGS colour batch)",
                         "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                         "frac": achieved / pk["hbm_gbs"], "peak_source": pk["source"],
                         "traffic": traffic, "bytes_per_launch": bytes_per_launch,
                         "launch_ms": launch_s * 1e3, "launches_timed": pg["launches"],
                         "bytes_per_point_sweep": PGS_BYTES_PER_POINT_SWEEP,
                         "frac_padded_records": padded / pgs_s / 1e9 / pk["hbm_gbs"],
                         "step_bytes_per_step": step_bytes / args.steps,
                         "step_frac": step_bytes / dev_s / 1e9 / pk["hbm_gbs"] / world},
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": h2d,
                    "steps": e2e_steps, "wall_ms_per_step": e2e_wall / e2e_steps * 1e3 if e2e_steps else None,
                    "link": link},
            "learned_vs_plain": lvp,
            "gpu_launches": gpu_launches,
            "clocks": clocks.summary(),
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return 0


def copy_rates(host: dict) -> dict:
    """The host link alone: the same pinned arrays copied to device tensors and back with
    plain cudaMemcpyAsync (torch), CUDA events around 10 repetitions after 3 — the floor of
    the end-to-end step's transfers."""
    import torch

    src = [torch.from_numpy(a) for a in host.values()]
    dev = [torch.empty_like(t, device="cuda") for t in src]
    nbytes = sum(t.numel() * t.element_size() for t in src)

    def timed(fn, reps=10):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            fn()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    h2d = timed(lambda: [d.copy_(t, non_blocking=True) for d, t in zip(dev, src)])
    d2h = timed(lambda: [t.copy_(d, non_blocking=True) for d, t in zip(dev, src)])
    return {"h2d_gbs": nbytes / h2d / 1e6, "d2h_gbs": nbytes / d2h / 1e6, "copy_ms_per_step": h2d + d2h}


def library_path(axbuild) -> Path:
    """The step library: $AXIOM_GB300_LIB when set (a build elsewhere), else the in-tree
    build, compiled first if missing."""
    env = os.environ.get("AXIOM_GB300_LIB")
    if env:
        return Path(env)
    p = axbuild.library_path()
    if not p.exists():
        axbuild.build_library()
    return p


def run_batch(args) -> int:
    """4,096 independent worlds (lognormal body counts, median 256, sigma 1, clipped to
    [16, 8192]; random box/sphere stacks on their own planes) in one persistent launch."""
    import tempfile

    import torch

    torch.cuda.set_device(0)
    import build as axbuild

    import axiom_gb300 as ax

    lib = ax.load_library(library_path(axbuild))
    bs = ax.BatchScene(seed=4, worlds=4096, median=256.0, sigma=1.0, min_bodies=16, max_bodies=8192, lib=lib)
    batch = ax.Batch(ax.default_config(lib, time_step=1 / 60, velocity_iterations=10), lib=lib)
    batch.set_worlds(bs.bodies, bs.sizes)
    for _ in range(max(3, args.warmup)):
        batch.step(1 / 60, check=False)
    tune = Path(tempfile.gettempdir()) / "axiom_batch_autotune.txt"
    block, ctas = batch.autotune(str(tune), trial_steps=2)
    stage = batch.launch()[2]
    torch.cuda.synchronize()
    step_ms, per_world = [], []
    with ClockSampler(0) as clocks:
        for _ in range(args.steps):
            st = batch.step(1 / 60, check=False)
            step_ms.append(st.total_step_time)
            per_world.append(batch.world_stats()["step_ns"].astype(np.float64) / 1e6)
    pw = np.concatenate(per_world)
    n = bs.bodies.n
    value = n * args.steps / (sum(step_ms) / 1e3)
    ws = batch.world_stats()
    ph = batch.phase_ns().astype(np.float64)  # last step, [worlds, phases]
    big = int(np.argmax(bs.sizes))
    phases = {
        "cta_time_share": {k: float(ph[:, i].sum() / ph.sum()) for i, k in enumerate(batch.PHASES)},
        "largest_world_ms": {k: float(ph[big, i] / 1e6) for i, k in enumerate(batch.PHASES)},
    }
    line = {
        "metric": "aggregate body-steps/s, 4096 batched worlds", "value": value, "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": sum(step_ms) / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded DeterministicRNG stacks)",
        "config": {"workload": "batched_worlds_4096", "worlds": 4096, "bodies": n,
                   "body_count_median": float(np.median(bs.sizes)), "body_count_max": int(bs.sizes.max()),
                   "dt": 1 / 60, "pgs_iterations": 10, "launch": {"block": block, "ctas_per_sm": ctas, "staged_bodies": stage},
                   "graph": "whole step captured once, replayed per step",
                   "manifolds": int(ws["manifolds"].sum()), "gjk_pairs": int(ws["gjk"].sum())},
        "per_world_step_ms": {"p50": float(np.percentile(pw, 50)), "p99": float(np.percentile(pw, 99)),
                              "max": float(pw.max())},
        "phases": phases,
        "clocks": clocks.summary(),
    }
    print(json.dumps(line), flush=True)
    return 0


SCENES = {
    # falling spheres: 1,000 spheres r 0.5 m in a 20x40x20 m box onto a ground plane, 10 sweeps
    "drop1k": dict(builder="sphere_drop", kw=dict(seed=1, count=1000, radius=0.5, size=(20.0, 40.0, 20.0)),
                   iters=10, steps=120, cpu_steps=120),
    # mixed convex shapes: 100,000 bodies (40 % spheres, 40 % boxes, 20 % capsules) in a
    # 200x100x200 m box, 20 sweeps; box-box and box-capsule pairs through GJK/EPA
    "mixed100k": dict(builder="mixed", kw=dict(seed=2, count=100_000, size=(200.0, 100.0, 200.0)),
                      iters=20, steps=240, cpu_steps=6),
}


def run_scene(args) -> int:
    """One of the configurations beside the 1M pile: device body-steps/s over the
    configured step count, and the CPU oracle on the same scene (all host cores)."""
    import torch

    torch.cuda.set_device(0)
    import build as axbuild

    import axiom_gb300 as ax

    spec = SCENES[args.workload]
    lib = ax.load_library(library_path(axbuild))
    sc = getattr(ax.Scene, spec["builder"])(lib=lib, **spec["kw"])
    cfg = dict(time_step=DT, velocity_iterations=spec["iters"])
    w = ax.PhysicsWorld(ax.default_config(lib, **cfg), lib=lib)
    w.add_bodies(sc.bodies)
    warm = max(3, args.warmup)
    for _ in range(warm):
        w.step(DT)
    start = w.save_snapshot()
    steps = spec["steps"]
    step_ms, stats = [], []
    torch.cuda.synchronize()
    with ClockSampler(0) as clocks:
        for _ in range(steps):
            st = w.step(DT)
            step_ms.append(st.total_step_time)
            stats.append(st)
    value = sc.n * steps / (sum(step_ms) / 1e3)
    # per-stage breakdown: the timed steps again (at most 60), every kernel group timed
    w.load_snapshot(start)
    w.set_profiling(True)
    w.reset_profile()
    replay = min(steps, 60)
    for _ in range(replay):
        w.step(DT)
    stage = {k: round(v["ms"] / replay, 4) for k, v in w.read_profile().items()}
    w.set_profiling(False)
    cpu = None
    if not args.no_cpu:
        oracle = load_oracle(axbuild.build_oracle())
        o = ax.PhysicsWorld(ax.default_config(oracle, **cfg), lib=oracle)
        threads = os.cpu_count() or 1
        oracle.oracle_set_threads(o.handle, threads)
        o.add_bodies(sc.bodies)
        for _ in range(warm):
            o.step(DT)
        t0 = time.perf_counter()
        for _ in range(spec["cpu_steps"]):
            o.step(DT)
        secs = time.perf_counter() - t0
        cpu = {"value": sc.n * spec["cpu_steps"] / secs, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"the same scene, {spec['cpu_steps']} steps after {warm} warm-up"}
    line = {
        "metric": f"body-steps/s, {args.workload}", "value": value, "unit": UNIT, "n_gpus": 1, "steps": steps,
        "warmup": warm, "ms_per_step": sum(step_ms) / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded DeterministicRNG scene)",
        "config": {"workload": args.workload, "bodies": sc.n, "dt": DT, "pgs_iterations": spec["iters"],
                   "pairs_first_last": [stats[0].pair_count, stats[-1].pair_count],
                   "manifolds_first_last": [stats[0].manifold_count, stats[-1].manifold_count],
                   "ms_per_step_min_max": [min(step_ms), max(step_ms)],
                   "stage_ms_first_steps": stage, "stage_steps": replay},
        "cpu_baseline": cpu,
        "clocks": clocks.summary(),
    }
    print(json.dumps(line), flush=True)
    return 0


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)  # the 60-step run of the 1M-pile configuration
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-vs-plain leg")
    ap.add_argument("--dims", default=",".join(map(str, DIMS)),
                    help="lattice size x,y,z of the pile (default: the 1M-sphere pile)")
    ap.add_argument("--workload", default="lattice", choices=["lattice", "batch", *SCENES],
                    help="lattice: the walled 1M-sphere pile (headline); batch: 4096 batched worlds; "
                         "drop1k / mixed100k: the 1,000-sphere drop and the 100k mixed-shape scene")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batch":
        return run_batch(args)
    if args.workload in SCENES:
        return run_scene(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
