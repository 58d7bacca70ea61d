#!/usr/bin/env python
"""Benchmark: particle-steps/s of the explicit GIMP MPM step on one GB300.

Workload: the 3D Newtonian dam break (domain 4 x 2 x 2 m, cellsize 0.01 m, psep 0.005 m,
water column 1.0 x 1.96 x 0.765 m against the x = 0 wall, 11,997,600 particles, gravity
-9.81 in z, zero-velocity node walls two cells deep), seeded synthetic lattice input.
A step is one full explicit step (sort, P2G, fold + nodal solve + BCs, G2P + update +
constitutive) over all particles.  State stays resident in HBM; the particle and grid state
(1.1 GB + 0.5 GB) is far larger than L2, so no explicit L2 flush is needed between steps.

The timed window lies in the developed flow: the run is first advanced (untimed) to the
middle of the configuration's run -- step 1000 of the dam break's 2000, where the column is
collapsing and particles change cell every step -- and the K steps after the W warm-up
steps from there are timed.  The same K steps taken from rest are reported beside them
(`rest_state`), with the share of particles that change cell per step in both windows.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

With N > 1 (torchrun) every rank advances an independent replica: the step has no
partition without a halo exchange, so this is replicas only and value = all ranks'
particle-steps / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/sec, 1 GB300: plain MPM vs DP surrogate at <=1e-3 rel stress err"
UNIT = "particle-steps/s"

# algorithmic bytes (FP32 SoA state read once and written once per step)
P2G_BYTES_PER_PARTICLE = 64        # key, offsets, v, sigma, m, rho, info
P2G_BYTES_PER_NODE = 28            # m, p(3), f(3) accumulated per active node
G2P_BYTES_PER_PARTICLE = 168       # full particle state read + written (models 1-2)
G2P_BYTES_PER_NODE = 24            # v(3), a(3) read per active node
SOLVE_BYTES_PER_NODE = 52          # m, p, f read; v, a written
STEP_BYTES_PER_PARTICLE = 168
STEP_BYTES_PER_NODE = 104
# multi-body Drucker-Prager + Grady-Kipp (the Brazilian disc): the plastic strain, eqps,
# damage and smax fields add 68 B per particle; per active node the centre-of-mass fields
# plus two body slots (accumulated, solved, read back)
DP_BYTES_PER_PARTICLE = 236
MB_P2G_BYTES_PER_NODE = 84           # COM + two body slots, 28 B each
MB_SOLVE_BYTES_PER_NODE = 156
MB_G2P_BYTES_PER_NODE = 72
MB_STEP_BYTES_PER_NODE = 312
# per step the end-to-end loop reads back the conservation partials (16 slots x 8 FP64) and
# the four status words
STATS_D2H_BYTES = 16 * 8 * 8 + 4 * 4
# the step's device scalars (dt, dt at the nodes, gravity x3, damping, friction, BC time, grid-BC
# switch, body count, initial volume, step index: 12 four-byte words), copied host-to-device
# every step
STEP_SCALARS_H2D_BYTES = 12 * 4


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Dist:
    def __init__(self, world, local):
        self.world = world
        self.pg = None
        if world > 1:
            import torch
            import torch.distributed as dist
            self.torch, self.dist = torch, dist
            backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(local)
            dist.init_process_group(backend)

    def barrier(self):
        if self.world > 1:
            self.dist.barrier()

    def _reduce(self, x: float, op) -> float:
        t = self.torch.tensor([x], dtype=self.torch.float64,
                              device="cuda" if self.dist.get_backend() == "nccl" else "cpu")
        self.dist.all_reduce(t, op=op)
        return float(t.item())

    def max(self, x: float) -> float:
        return x if self.world == 1 else self._reduce(x, self.dist.ReduceOp.MAX)

    def sum(self, x: float) -> float:
        return x if self.world == 1 else self._reduce(x, self.dist.ReduceOp.SUM)

    def close(self):
        if self.world > 1:
            self.dist.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        rows = [r.split(",") for r in open(self.path).read().strip().splitlines() if r.strip()]
        os.unlink(self.path)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                smax = float(r[2])
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic():
    """Per-launch DRAM bytes of the dominant kernels from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        return json.load(open(path))
    except Exception:
        return {}


WORKLOADS = {
    "dam_break": "dam_break_3d_newtonian",
    "brazilian_disc": "brazilian_disc_dp_gk_rigid_platens",
    "impact_batch": "impact_batch_sphere_on_dp_gk_slab",
}
# steps of each configuration's run; the timed window starts half-way through it
RUN_STEPS = {"dam_break": 2000, "brazilian_disc": 5000, "impact_batch": 500}

# the CPU legs step the full workload, timing at most this many steps after one warm-up step
CPU_MAX_TIMED_STEPS = 3


def cpu_scene(workload: str = "dam_break", args=None):
    """The CPU legs' workload: the GPU run's own scene (same particles, grid and materials),
    bounded by the number of steps timed, not by a smaller sample.  Returns the scene and a
    description."""
    from graphyt_gb300 import scenes
    if workload == "brazilian_disc":
        return scenes.brazilian_disc(scale=args.scale if args else 1.0), "the full Brazilian disc"
    if workload == "impact_batch":
        return (scenes.impact_batch(n_inst=args.instances if args else 256, seed=0),
                "the full impact batch")
    scale = args.scale if args else 1.0
    return (scenes.dam_break(scale=scale, height=args.column_height if args else 0.765),
            "the full dam break" if scale == 1.0 else f"the dam break at scale {scale}")


def run_cpu(nsteps: int, warmup: int, prefer_reference: bool = True, workload: str = "dam_break", args=None,
            scene=None):
    """Time the reference's CPU step (oracle/_ref when built, else the FP64 restatement) on
    the same workload as the GPU run, from rest, over at most CPU_MAX_TIMED_STEPS steps after
    one warm-up step (a CPU step of 12 M particles takes seconds).  Returns (particle-steps/s,
    kind, threads, sample description)."""
    from oracle import oracle as O
    kind = "ref" if (prefer_reference and O.available("ref")) else "port"
    if not O.available(kind):
        O.build()
    if scene is None:
        sc, what = cpu_scene(workload, args)
    else:
        sc, what = scene, f"the GPU run's {workload} scene"
    nsteps = max(1, min(nsteps, CPU_MAX_TIMED_STEPS))
    warmup = max(1, min(warmup, 1))
    o = O.Oracle(sc, kind, mode=1)
    o.run(warmup)
    t0 = time.perf_counter()
    o.run(nsteps)
    dt = time.perf_counter() - t0
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    o.close()
    sample = (f"{what}: {sc.n} particles, {sc.num_nodes()} nodes, {nsteps} timed steps after {warmup} "
              f"from rest")
    return sc.n * nsteps / dt, ("reference" if kind == "ref" else "port"), threads, sample


def bench_reference(args, rank):
    if rank != 0:
        return
    value, kind, threads, sample = run_cpu(args.steps, args.warmup, workload=args.workload, args=args)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOADS[args.workload], "sample": sample, "same_config": True},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind, "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def bench_surrogate(solver, args, step, n_job, names):
    """The learned surrogate against the plain return mapping from the same state: train on the
    logged returns (timed on the host clock), then time K steps of each arm (CUDA events, graph
    replay) after W warm-up steps, both from the state at `step`, and compare the stress,
    velocity and plastic strain they reach."""
    import numpy as np
    from graphyt_gb300 import _lib as L
    lib, h = solver.lib, solver.h
    dt = solver.dt
    logged = solver.dp_log_count()
    solver.dp_log_end()
    t0 = time.perf_counter()
    loss = solver.train_surrogate(steps=args.surrogate_train_steps, batch=4096, lr=1e-3, seed=0)
    solver.Synchronise()
    train_s = time.perf_counter() - t0
    fd, path = tempfile.mkstemp(suffix=".gystate")
    os.close(fd)
    solver.save(path)

    def arm():
        k = step
        for _ in range(args.warmup):
            solver.iterate_GPU(k * dt, k)
            k += 1
        solver.Synchronise()
        ms = C.c_float()
        L.check(lib.gy_time_steps(h, k * dt, k, args.steps, C.byref(ms)), h, "timed steps")
        solver.Synchronise()
        return ms.value / args.steps, {f: solver._get_particles(f) for f in ("stress", "vel", "eqps")}

    ms_plain, plain = arm()
    solver.load(path)
    solver.set_surrogate(True, tol=1e-4)
    c0 = solver.surrogate_counts()
    ms_surr, surr = arm()
    c1 = solver.surrogate_counts()
    solver.set_surrogate(False)
    solver.load(path)
    os.unlink(path)

    def rel(a, b):
        d = np.linalg.norm(b)
        return float(np.linalg.norm(a - b) / d) if d > 0 else float(np.linalg.norm(a))

    kept, fb = c1["kept"] - c0["kept"], c1["fallback"] - c0["fallback"]
    return {"metric": "particle-steps/s, plain return mapping vs learned surrogate, same state and steps",
            "plain_ms_per_step": ms_plain, "plain_value": n_job / (ms_plain / 1e3),
            "surrogate_ms_per_step": ms_surr, "surrogate_value": n_job / (ms_surr / 1e3),
            "rel_l2_vs_plain": {f: rel(surr[f], plain[f]) for f in plain},
            "deferred_per_step": (kept + fb) / max(args.warmup + args.steps, 1),
            "kept_fraction": kept / max(kept + fb, 1), "tol_x_cohesion": 1e-4,
            "logged_returns": logged, "train_steps": args.surrogate_train_steps, "train_batch": 4096,
            "train_s": train_s, "train_loss": loss, "first_step": step}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--workload", default="dam_break", choices=list(WORKLOADS),
                    help="dam_break: the headline 3D Newtonian dam break; brazilian_disc: the multi-body "
                         "Drucker-Prager + Grady-Kipp disc between rigid platens; impact_batch: independent "
                         "sphere-on-slab impacts of uneven sizes advanced as one grid")
    ap.add_argument("--instances", type=int, default=256, help="impact_batch: number of instances")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--sort-every", type=int, default=1)
    ap.add_argument("--temperature", type=float, default=0.0,
                    help="initial temperature of every particle; nonzero runs the heat conduction terms")
    ap.add_argument("--column-height", type=float, default=0.765,
                    help="dam break water column height in m (1.5 gives the configuration's 24 M particles)")
    ap.add_argument("--full-sort", action="store_true", help="full radix sort every step (no incremental re-sort)")
    ap.add_argument("--p2g-lanes", type=int, default=3, choices=[3, 9],
                    help="single-body P2G lanes per run of equal cell: 3 z-plane lanes or 9 x-column lanes")
    ap.add_argument("--autotune", dest="autotune", action="store_true", default=None,
                    help="run Solver.autotune before the timed window (default: on for impact_batch)")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false")
    ap.add_argument("--surrogate", action="store_true",
                    help="brazilian_disc: also train the learned Drucker-Prager surrogate on the returns the plain "
                         "solver logs up to the timed window, and time the surrogate step beside the plain one")
    ap.add_argument("--surrogate-train-steps", type=int, default=20000)
    ap.add_argument("--preroll", type=int, default=-1,
                    help="untimed steps before the warm-up (default: half the configuration's run)")
    ap.add_argument("--save-state", metavar="PATH",
                    help="write a checkpoint of the state reached after the preroll (Solver.save)")
    ap.add_argument("--load-state", metavar="PATH",
                    help="start the timed window from a checkpoint written with --save-state and the same "
                         "--preroll (no rest-state window, no preroll): the developed flow with few launches "
                         "before it, for profiling")
    ap.add_argument("--no-secondary", action="store_true",
                    help="the default dam-break run (one GPU) also measures the Brazilian disc and the batch "
                         "after its own line's measurements and reports them under secondary_workloads; "
                         "this skips them")
    args = ap.parse_args()
    explicit_workload = any(a == "--workload" or a.startswith("--workload=") for a in sys.argv[1:])
    if args.preroll < 0:
        args.preroll = RUN_STEPS[args.workload] // 2
    args.warmup = max(args.warmup, 3)
    rank, world, local = dist_env()
    if args.impl == "reference":
        bench_reference(args, rank)
        return

    from graphyt_gb300 import build as gbuild
    if not os.path.exists(gbuild.LIB):
        gbuild.build()

    dist = Dist(world, local)
    line = measure(args, rank, world, local, dist)
    if (rank == 0 and world == 1 and not explicit_workload and not args.no_secondary and args.workload == "dam_break"
            and not args.load_state):
        # the configuration's other single-GPU workloads, measured the same way after the
        # headline (fewer timed steps, no CPU leg); their own lines come from --workload
        sec = {}
        for wl in ("brazilian_disc", "impact_batch"):
            a2 = argparse.Namespace(**vars(args))
            a2.workload, a2.scale, a2.temperature, a2.surrogate = wl, 1.0, 0.0, False
            a2.steps, a2.no_cpu_baseline, a2.autotune = min(args.steps, 10), True, None
            a2.preroll, a2.save_state, a2.load_state = RUN_STEPS[wl] // 2, None, None
            a2.sort_every, a2.full_sort, a2.p2g_lanes = 1, False, 3
            try:
                r = measure(a2, rank, world, local, dist)
            except Exception as e:  # the headline line is printed whatever happens here
                sec[wl] = {"error": f"{type(e).__name__}: {e}"[:300]}
                continue
            sec[wl] = {k: r.get(k) for k in ("value", "unit", "ms_per_step", "steps", "phase_ms_per_step", "e2e",
                                             "roofline", "gpu_launches", "clocks", "autotune")}
            sec[wl]["config"] = {k: r["config"].get(k) for k in ("workload", "particles", "nodes", "model",
                                                                  "instances", "active_nodes")
                                 if k in r["config"]}
            sec[wl]["window"] = r["window"]
        line["secondary_workloads"] = sec
    if rank == 0:
        print(json.dumps(line), flush=True)
    dist.close()


def measure(args, rank, world, local, dist):
    """One workload's measurements; the JSON line's dict on rank 0 (None elsewhere)."""
    from graphyt_gb300 import _lib as L
    from graphyt_gb300 import graphyt, scenes

    if args.workload == "dam_break":
        sc = scenes.dam_break(scale=args.scale, height=args.column_height)
    elif args.workload == "brazilian_disc":
        sc = scenes.brazilian_disc(scale=args.scale)
    else:
        # one process per GPU: the instances split across the ranks (instance i on rank
        # i mod N), each rank stepping its share as one grid -- no exchange between ranks
        sc = scenes.impact_batch(n_inst=args.instances, seed=0, shard=(rank, world) if world > 1 else None)
    if args.temperature:
        # a linear profile along x, so the conduction terms have gradients to carry
        x = sc.pos[:, 0]
        sc.temp = args.temperature * (1.0 + (x - x.min()) / max(x.max() - x.min(), 1e-30))
    n = sc.n
    solver = graphyt.from_scene(sc, device=local, options=dict(sort_every=args.sort_every, full_sort=int(args.full_sort),
                                                               p2g_lanes=args.p2g_lanes))
    lib, h = solver.lib, solver.h
    dt = solver.dt
    import numpy as np
    step = 0

    def advance(k):
        """k untimed steps."""
        nonlocal step
        for _ in range(k):
            solver.iterate_GPU(step * dt, step)
            step += 1
        solver.Synchronise()

    def timed(k):
        """Device time of k steps as the library runs them (graph replay), CUDA events on the
        handle's stream around them."""
        nonlocal step
        ms = C.c_float()
        L.check(lib.gy_time_steps(h, step * dt, step, k, C.byref(ms)), h, "timed steps")
        step += k
        return ms.value

    def phases(k):
        """Per-phase ms per step over k kernel-by-kernel steps (events between the phases)."""
        nonlocal step
        L.check(lib.gy_set_phase_timing(h, 1), h)
        L.check(lib.gy_steps(h, step * dt, step, k, 0), h, "phase-timed steps")
        step += k
        solver.Synchronise()
        ph = (C.c_float * 5)()
        nph = C.c_int64()
        L.check(lib.gy_get_phase_times(h, ph, C.byref(nph)), h)
        L.check(lib.gy_set_phase_timing(h, 0), h)
        return [ph[q] / max(nph.value, 1) for q in range(4)]

    def mover_fraction():
        """Share of the particles whose cell changes in one step."""
        c0 = solver._get_particles_int("cellid")
        advance(1)
        return float(np.mean(c0 != solver._get_particles_int("cellid")))

    if args.surrogate:
        # the plain solver logs its Drucker-Prager returns up to the timed window
        solver.dp_log_begin(cap=50_000_000, every=1)
    names = ["sort", "p2g", "grid", "g2p_update"]
    rest = None
    if args.load_state:
        solver.load(args.load_state)
        step = args.preroll
    else:
        advance(args.warmup)
        # the same window from rest: few particles change cell, so the re-sort is cheapest here
        rest_ms = timed(args.steps)
        rest_phase = phases(args.steps)
        rest_movers = mover_fraction()
        rest = (rest_ms, rest_phase, rest_movers)
    # the developed flow: advance to the middle of the configuration's run, warm up, time
    tuned = None
    if args.autotune or (args.autotune is None and args.workload == "impact_batch"):
        # the autotuner's candidates run as real steps of the run, before the timed window
        res = solver.autotune(step0=step, steps=4)
        step = res["next_step"]
        tuned = {k: res[k] for k in ("sort_every", "full_sort", "p2g_lanes")}
        tuned["candidates_ms_per_step"] = {f"sort_every={a},full_sort={b}": v for (a, b), v in res["ms_per_step"].items()}
        tuned["p2g_lanes_ms_per_step"] = {str(k): v for k, v in res["lanes_ms_per_step"].items()}
    advance(max(0, args.preroll - step))
    if args.save_state:
        solver.save(args.save_state)
    surrogate = None
    if args.surrogate:
        surrogate = bench_surrogate(solver, args, step, float(n) * world, names)
    advance(args.warmup)
    dist.barrier()
    sampler = ClockSampler(local)
    if rank == 0:
        sampler.start()
    launches0 = lib.gy_kernel_launches()
    step_timed0 = step
    ms_timed = timed(args.steps)
    launches = lib.gy_kernel_launches() - launches0
    clocks = sampler.stop() if rank == 0 else None
    solver.Synchronise()
    ms_max = dist.max(ms_timed)
    ms_per_step = ms_max / args.steps
    sharded = args.workload == "impact_batch" and world > 1
    n_job = dist.sum(float(n)) if sharded else float(n) * world  # particles the job steps
    value = n_job * args.steps / (ms_max / 1e3)
    per_step = phases(args.steps)
    movers = mover_fraction()

    st = solver.stats()
    n_active = int(st["active_nodes"])

    # end to end through the public API: per step the parameter block goes host->device
    # with the launch and the step's FP64 conservation sums (summed by the step's G2P into
    # partial slots) come back device->host with the status words
    prm = solver.params
    dist.barrier()
    t0 = time.perf_counter()
    for k in range(args.steps):
        solver.iterate_GPU(step * dt, step, prm)
        step += 1
        solver.stats()
    e2e_s = dist.max(time.perf_counter() - t0)
    e2e_value = n_job * args.steps / e2e_s

    # roofline of the dominant kernel
    multi = args.workload != "dam_break"
    algo = {
        "sort": 0.0,
        "p2g": P2G_BYTES_PER_PARTICLE * n + (MB_P2G_BYTES_PER_NODE if multi else P2G_BYTES_PER_NODE) * n_active,
        "grid": (MB_SOLVE_BYTES_PER_NODE if multi else SOLVE_BYTES_PER_NODE) * n_active,
        "g2p_update": (DP_BYTES_PER_PARTICLE if multi else G2P_BYTES_PER_PARTICLE) * n
                      + (MB_G2P_BYTES_PER_NODE if multi else G2P_BYTES_PER_NODE) * n_active,
    }
    dom = max(range(4), key=lambda k: per_step[k] if names[k] != "sort" else -1)
    peak, peak_kind = measured_peak()
    achieved = algo[names[dom]] / (per_step[dom] / 1e3) / 1e9
    traffic = profiled_traffic().get(names[dom]) if not multi else None
    roofline = {"bound": "hbm", "kernel": names[dom], "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
                "algorithmic_bytes": algo[names[dom]]}
    step_bytes = ((DP_BYTES_PER_PARTICLE if multi else STEP_BYTES_PER_PARTICLE) * n
                  + (MB_STEP_BYTES_PER_NODE if multi else STEP_BYTES_PER_NODE) * n_active)
    whole = step_bytes / (ms_per_step / 1e3) / 1e9

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, kind, threads, sample = run_cpu(2, 1, workload=args.workload, args=args, scene=sc)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": kind, "sample": sample}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "strong" if sharded else "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOADS[args.workload],
                       "particles": int(n_job) if sharded else n, "nodes": sc.num_nodes(),
                       **({"instances": args.instances, "instance_particles": [min(i.n for i in sc.instances),
                                                                              max(i.n for i in sc.instances)],
                           "dt_shared": sc.dt} if sc.instances else {}),
                       **({"column_height_m": args.column_height} if not multi else {}),
                       **({"heat_conduction": True} if args.temperature else {}),
                       "active_nodes": n_active, "cellsize": sc.cellsize, "psep": sc.psep,
                       "model": {"dam_break": "newtonian", "brazilian_disc": "drucker_prager+grady_kipp, 3 bodies",
                                 "impact_batch": "drucker_prager+grady_kipp slab + elastic sphere per instance, "
                                                 "2 bodies"}[args.workload],
                       "sort_every": args.sort_every, "p2g_lanes": args.p2g_lanes, "sort": "full" if args.full_sort else "incremental", "l2": "state larger than L2 (no flush needed)",
                       "parallelism": ("instances sharded" if sharded else "replicas") if world > 1 else "single"},
            "window": {"first_timed_step": step_timed0, "of_run_steps": RUN_STEPS[args.workload],
                       "movers_per_step": movers},
            "phase_ms_per_step": dict(zip(names, per_step)),
            "rest_state": {"first_timed_step": args.warmup, "ms_per_step": rest[0] / args.steps,
                           "value": n_job * args.steps / (dist.max(rest[0]) / 1e3),
                           "phase_ms_per_step": dict(zip(names, rest[1])), "movers_per_step": rest[2]}
                          if rest else None,
            "roofline": roofline,
            "step_roofline": {"achieved": whole, "peak": peak, "unit": "GB/s", "frac": whole / peak,
                              "bytes_per_step": step_bytes},
            "cpu_baseline": cpu,
            **({"surrogate": surrogate} if surrogate else {}),
            **({"autotune": tuned} if tuned else {}),
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": STEP_SCALARS_H2D_BYTES,
                    "d2h_bytes_per_step": STATS_D2H_BYTES},
            "gpu_launches": int(launches),
            "clocks": clocks,
        }
    else:
        line = None
    solver.close()
    return line


if __name__ == "__main__":
    main()
