#!/usr/bin/env python
"""Benchmark of the simulation step on the 256^3 APIC workload.

Workload (fill256_apic): 256^3 MAC grid in the unit cube, solid walls on all
six faces; fluid fills every interior cell with centre y < 0.5 (8 jittered
particles per cell, seed 0, 65.5M particles, FP32 SoA, APIC C as 9 FP32);
a solid sphere of radius 0.15 at (0.5 + 0.1 sin(pi t), 0.6, 0.5); a disc source
of radius 4 cells at y = 0.95 emitting 8 jittered particles per covered cell
per step with velocity (0, -1, 0); an 8x8x8-cell sink box at the floor corner
(0, 0, 0); dt = 1/480 s; PCG to relative residual 1e-6 (max 2000 iterations)
from zero pressure, as the reference starts.  All inputs are synthetic and
seeded; no dataset is involved.

A "step" is one Simulator::simulate(dt).  `value` is steps/s with the state
resident in HBM (8.6 GB of particle state, far larger than the 129 MB L2, so
no L2 flush is needed between steps); `e2e` is the same metric through the C
ABI with the renderer hand-off of every step (fsim_fill_gfx into pinned host
memory, SimulationManager::getParticleGfxData) inside the timed region.

--impl reference times the reference's algorithm on the host cores: the FP64
oracle (oracle/fsim_oracle.c, a bit-exact restatement of the reference's
Simulator pinned by tests/golden) with all OpenMP threads, on the same
workload.  Each of its steps takes tens of seconds, so it times min(K, 2)
steps after one warm-up step and says so in its line.

Multi-GPU: the step does not shard (every PCG iteration needs halo exchange and
global reductions), so --gpus N runs N independent replicas, one per GPU, and
`value` sums their steps/s ("replicas only").
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
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "fill256_apic"


# ---------------------------------------------------------------- workload
def workload_scene(res: int = 256):
    from fluid_simulator_gb300.scenes import GridSpec, fill_below

    grid = GridSpec(res)
    return grid, fill_below(grid, 0.5, seed=0)


def obstacles_at(t: float, dt: float, h: float, N):
    """Sphere moving in x, disc source, corner sink box (fsim obstacle structs)."""
    x = 0.5 + 0.1 * math.sin(math.pi * t)
    xp = 0.5 + 0.1 * math.sin(math.pi * (t - dt))
    return [
        N.obstacle(N.OBS_SPHERE, (x, 0.6, 0.5), r=0.15, prev_pos=(xp, 0.6, 0.5), speed=((x - xp) / dt, 0.0, 0.0)),
        N.obstacle(N.OBS_DISC_SOURCE, (0.5, 0.95, 0.5), r=4 * h, spawn_speed=-1.0),
        N.obstacle(N.OBS_BOX_SINK, (4 * h, 4 * h, 4 * h), size=(8 * h, 8 * h, 8 * h)),
    ]


# ---------------------------------------------------------------- helpers
class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 50 ms from before the
    warm-up steps to the end of the timed region; each sample carries its
    timestamp, so the summary can tell the timed window from the rest of the
    loaded period."""

    def __init__(self, path: str, gpu: int):
        self.path = path
        self.proc = None
        self.gpu = gpu
        self.t_load = self.t0 = self.t1 = None

    def __enter__(self):
        q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)  # let the first samples come before the load starts
        self.t_load = time.time()
        return self

    def timed(self, start: bool):
        if start:
            self.t0 = time.time()
        else:
            self.t1 = time.time()

    def __exit__(self, *exc):
        if self.proc is not None:
            import signal

            time.sleep(0.1)
            self.proc.send_signal(signal.SIGINT)  # nvidia-smi ends its loop and flushes
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.proc.wait()
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        import datetime

        rows = []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 10:
                continue
            try:
                ts = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                rows.append((ts, float(parts[2]), float(parts[3]),
                             {nm for nm, val in zip(names, parts[6:10]) if val.lower() == "active"}))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        t_end = self.t1 if self.t1 is not None else rows[-1][0]
        timed = [r for r in rows if self.t0 is not None and self.t0 <= r[0] <= t_end]
        loaded = [r for r in rows if self.t_load is not None and self.t_load <= r[0] <= t_end] or rows
        use = timed if len(timed) >= 3 else loaded
        return {"sm_mhz": statistics.median(r[1] for r in use), "sm_max_mhz": max(r[2] for r in use),
                "reasons": sorted(set().union(*(r[3] for r in use))),
                "samples": len(use), "samples_timed": len(timed),
                "window": "timed region" if use is timed else "warm-up and timed steps"}


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def cudart():
    for name in ("libcudart.so.13", "libcudart.so"):
        try:
            return C.CDLL(name)
        except OSError:
            pass
    import glob

    return C.CDLL(sorted(glob.glob("/usr/local/cuda/lib64/libcudart.so*"))[0])


class Events:
    """CUDA events on the library's stream (cudart through ctypes)."""

    def __init__(self, rt, stream):
        self.rt, self.stream = rt, stream
        self.a, self.b = C.c_void_p(), C.c_void_p()
        rt.cudaEventCreate(C.byref(self.a))
        rt.cudaEventCreate(C.byref(self.b))

    def start(self):
        self.rt.cudaEventRecord(self.a, C.c_void_p(self.stream))

    def stop_ms(self):
        self.rt.cudaEventRecord(self.b, C.c_void_p(self.stream))
        self.rt.cudaEventSynchronize(self.b)
        ms = C.c_float()
        self.rt.cudaEventElapsedTime(C.byref(ms), self.a, self.b)
        return ms.value


# algorithmic bytes (FP32 SoA, each array counted once per stage; sort traffic excluded)
BYTES_PER_PARTICLE = {0: 84, 1: 96, 2: 156}   # PIC, FLIP, APIC per step
BYTES_P2G_PER_PARTICLE = {0: 24, 1: 24, 2: 60}  # read pos, v (+C)
BYTES_P2G_PER_CELL = 17                        # write 3 face v + flag + avgPNum
BYTES_G2P_PER_PARTICLE = {0: 24, 1: 36, 2: 60}
BYTES_G2P_PER_CELL = {0: 12, 1: 24, 2: 12}
BYTES_GRID_PER_CELL = 150
BYTES_PCG_PER_FLUID_CELL_ITER = 60
# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) of one k_p2g / k_g2p launch per
# particle, from full ncu captures of the same scene at 128^3 (8.0M particles; cells per particle
# are the same at 256^3, so the per-particle figure scales to the 256^3 launch)
DRAM_BYTES_PER_PARTICLE = {"p2g": (679.849984e6 + 32.129536e6) / 7999554,
                           "g2p": (170.228736e6 + 425.340672e6) / 7999554}


def dist_setup(n_gpus: int):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist  # only for the barrier / max over replicas

        dist.init_process_group("gloo")
    return rank, world, local, dist


def dist_max(dist, x: float) -> float:
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


# ---------------------------------------------------------------- our arm
def run_fsim(args):
    from fluid_simulator_gb300 import native as N

    rank, world, local, dist = dist_setup(args.gpus)
    rt = cudart()
    rt.cudaSetDevice(local)
    res = args.res
    grid, pos = workload_scene(res)
    h = grid.h
    dt = 1.0 / 480.0 if res == 256 else 1.0 / (480.0 * res / 256.0)
    precond = {"mg": N.PRECOND_MG, "rbic": N.PRECOND_RBIC}[args.precond]
    p = N.default_params(transfer=N.APIC, resolution=res, tol=1e-6, tol_mode=N.TOL_REL_L2, max_iters=2000,
                         spawning=True, despawning=True, timing=True, precision=N.PREC_MIXED,
                         warm_start=N.WARM_ZERO, precond=precond, mg_sweeps=args.mg_sweeps,
                         mg_coarse_sweeps=args.mg_coarse_sweeps, mg_cluster_sweeps=args.mg_cluster_sweeps,
                         refine_digits=args.refine_digits, mg_boundary_sweeps=args.mg_boundary_sweeps)
    sim = N.Simulation(res, p)
    sim.set_particles(pos)
    del pos
    t = 0.0

    def step():
        nonlocal t
        sim.set_obstacles(obstacles_at(t, dt, h, N))
        st = sim.step(dt)
        t += dt
        return st

    clk = ClockSampler(os.path.join(args.out_dir, f"clocks_rank{rank}.csv"), local)
    with clk:
        for _ in range(args.warmup):
            step()
        stream = sim.lib.fsim_stream(sim.ctx)
        ev = Events(rt, stream)
        stats = []
        barrier(dist)
        sim.synchronize()
        clk.timed(True)
        ev.start()
        for _ in range(args.steps):
            stats.append(step())
        ms = ev.stop_ms()
        clk.timed(False)
    sim.synchronize()
    barrier(dist)
    ms_max = dist_max(dist, ms)
    clocks = clk.summary()

    # end to end through the C ABI with the renderer hand-off in pinned host memory:
    # each step's records are published asynchronously (fsim_fill_gfx_async) and
    # land in host memory while the next step runs; the timed region ends after
    # the last copy (fsim_gfx_wait)
    n_cap = int(sim.n * 1.2) + 1_000_000
    # pinned host memory from the CUDA allocator (a registered ctypes array made
    # the copy rate vary from run to run with the host's page layout)
    gfx_ptr = C.c_void_p()
    if rt.cudaHostAlloc(C.byref(gfx_ptr), C.c_size_t(n_cap * C.sizeof(N.ParticleGfx)), 0) != 0:
        raise RuntimeError("cudaHostAlloc of the gfx buffer failed")
    gfx = (N.ParticleGfx * n_cap).from_address(gfx_ptr.value)
    # every copy is inside the window; the last one is waited for at its end, so
    # longer windows measure the steady state (the tail is one copy, ~7 ms)
    e2e_steps = max(1, min(args.steps, 20))
    d2h = 0
    h2d = 0

    def e2e_step():
        nonlocal t, d2h, h2d
        obs = obstacles_at(t, dt, h, N)
        h2d += len(obs) * C.sizeof(N.Obstacle)
        sim.set_obstacles(obs)
        sim.step(dt)
        t += dt
        got = C.c_int64()
        if sim.lib.fsim_fill_gfx_async(sim.ctx, gfx, n_cap, C.byref(got)) != 0:
            raise RuntimeError("fsim_fill_gfx_async failed")
        d2h += got.value * C.sizeof(N.ParticleGfx)

    # one untimed warm-up step per staging slot (their one-time allocation)
    for _ in range(2):
        e2e_step()
    sim.lib.fsim_gfx_wait(sim.ctx)
    d2h = h2d = 0
    barrier(dist)
    ev.start()
    for _ in range(e2e_steps):
        e2e_step()
    if sim.lib.fsim_gfx_wait(sim.ctx) != 0:
        raise RuntimeError("fsim_gfx_wait failed")
    e2e_ms = ev.stop_ms()
    barrier(dist)
    e2e_ms = dist_max(dist, e2e_ms)
    # one publish alone (gfx kernel + copy to the pinned host buffer), for the copy's own rate
    pub = []
    for _ in range(3):
        sim.synchronize()
        t0 = time.perf_counter()
        got = C.c_int64()
        sim.lib.fsim_fill_gfx_async(sim.ctx, gfx, n_cap, C.byref(got))
        sim.lib.fsim_gfx_wait(sim.ctx)
        pub.append(time.perf_counter() - t0)
    pub_s = min(pub)
    pub_bytes = got.value * C.sizeof(N.ParticleGfx)
    del gfx
    rt.cudaFreeHost(gfx_ptr)

    # per-stage breakdown (library events)
    def mean(key):
        return statistics.mean(getattr(s, key) for s in stats)

    np_mean = mean("num_particles")
    its = mean("pcg_iterations")
    ms_step = ms_max / args.steps
    value = world * args.steps / (ms_max / 1000.0)
    peak, peak_kind = load_peaks()
    ncell = res ** 3
    nfluid_est = mean("num_active_bricks") * 256
    # roofline of the dominant kernel class: the PCG iteration (three kernels) at 60 B/fluid cell
    pcg_ms_per_it = (mean("ms_solve") - mean("ms_pcg_setup")) / max(1.0, its)
    g2p_bytes = np_mean * BYTES_G2P_PER_PARTICLE[2] + ncell * BYTES_G2P_PER_CELL[2]
    p2g_bytes = np_mean * BYTES_P2G_PER_PARTICLE[2] + ncell * BYTES_P2G_PER_CELL
    kernels = {
        "g2p": {"ms": mean("ms_g2p_kernel"), "bytes": g2p_bytes},
        "p2g": {"ms": mean("ms_p2g_kernel"), "bytes": p2g_bytes},
    }
    for k in kernels.values():
        k["gbs"] = k["bytes"] / (k["ms"] / 1e3) / 1e9 if k["ms"] > 0 else None
        k["frac"] = k["gbs"] / peak if k["gbs"] else None
    dominant = "g2p" if kernels["g2p"]["ms"] >= kernels["p2g"]["ms"] else "p2g"
    dk = kernels[dominant]
    step_bytes = np_mean * BYTES_PER_PARTICLE[2] + ncell * BYTES_GRID_PER_CELL + \
        its * nfluid_est * BYTES_PCG_PER_FLUID_CELL_ITER
    line = {
        "metric": "steps/s (256^3 APIC step, PCG to 1e-6 relative residual)",
        "value": round(value, 4),
        "unit": "steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_step, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 (FP64 PCG scalars and solution)",
        "data": "synthetic (seeded dam-break fill, no dataset)",
        "config": {"workload": WORKLOAD, "grid": [res, res, res], "transfer": "APIC",
                   "particles": int(np_mean), "dt": dt, "pcg_tol": "1e-6 relative L2",
                   "obstacles": "moving sphere r=0.15, disc source r=4 cells, 8^3 sink box",
                   "parallelism": f"replicas x{world}", "l2": "state 8.6 GB > L2; no flush needed",
                   "warm_start": "zero", "precond": args.precond},
        "particle_steps_per_s": round(np_mean * value, 1),
        "pcg_iterations_mean": round(its, 2),
        "pcg_refinements_mean": round(mean("reliable_updates"), 2),
        "stage_ms": {k: round(mean(k), 3) for k in ("ms_simulate_particles", "ms_p2g", "ms_p2g_kernel", "ms_prep",
                                                   "ms_pcg_setup", "ms_solve", "ms_extrapolate", "ms_g2p")},
        "pcg_ms_per_iteration": round(pcg_ms_per_it, 4),
        "step_roofline": {"bytes": step_bytes, "achieved_gbs": round(step_bytes / (ms_step / 1e3) / 1e9, 1),
                          "frac": round(step_bytes / (ms_step / 1e3) / 1e9 / peak, 4)},
        "roofline": {"kernel": f"k_{dominant}", "bound": "hbm", "achieved": round(dk["gbs"], 1), "peak": peak,
                     "unit": "GB/s", "frac": round(dk["frac"], 4),
                     "traffic": (round(DRAM_BYTES_PER_PARTICLE[dominant] * np_mean)
                                 if DRAM_BYTES_PER_PARTICLE[dominant] else None),
                     "traffic_source": "ncu capture at 128^3 scaled per particle",
                     "algorithmic_bytes": round(dk["bytes"]),
                     "peak_source": peak_kind,
                     "all": {k: {kk: (round(vv, 4) if isinstance(vv, float) else vv) for kk, vv in v.items()}
                             for k, v in kernels.items()}},
        "clocks": clocks,
        "e2e": {"value": round(world * e2e_steps / (e2e_ms / 1000.0), 4), "unit": "steps/s",
                "h2d_bytes_per_step": h2d // e2e_steps, "d2h_bytes_per_step": d2h // e2e_steps,
                "steps": e2e_steps,
                "path": "fsim_set_obstacles + fsim_step + fsim_fill_gfx_async(pinned host) per step, fsim_gfx_wait",
                "d2h_gbs_window": round(d2h / (e2e_ms / 1e3) / 1e9, 1),
                "publish_alone_ms": round(pub_s * 1e3, 3),
                "publish_alone_d2h_gbs": round(pub_bytes / pub_s / 1e9, 1)},
        "gpu_launches": int(sum(s.kernel_launches for s in stats)),
    }
    # the studies are single-GPU diagnostics outside the timed region: N = 1 only
    if args.precision_study and world == 1:
        line["pcg_precision"] = precision_study(sim, N)
    if args.ws_steps > 0 and world == 1:
        line["pcg_warm_start"] = warm_start_study(sim, dt, t, h, N, args)
    if args.render and world == 1:
        line["render"] = render_study(sim, N, h, peak)
    sim.close()
    if args.parity and rank == 0 and world == 1:
        line["parity_drift"] = {"dam32_flip_vs_oracle_fixture": drift_dam32(N), "dam128_vs_oracle_fixture": drift_dam128(N)}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(res, dt)
        line["cpu_baseline"]["configs"] = cpu_baseline_configs()
    if rank == 0:
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- drift curves
DRIFT_GOLDEN = os.path.join(ROOT, "tests", "golden", "drift_dam128.npz")
DRIFT32_GOLDEN = os.path.join(ROOT, "tests", "golden", "drift_dam32.npz")


def _traj_stats(sim, N):
    """Fluid cells, mean kinetic energy, centroid, max speed (the oracle fixture's columns)."""
    p, v, _ = sim.particles()
    v64 = v.astype(np.float64)
    sp2 = (v64 * v64).sum(axis=1)
    return np.array([float((sim.grid(N.F_FLAGS) == N.WATER).sum()), 0.5 * float(sp2.mean()),
                     *p.astype(np.float64).mean(axis=0), float(np.sqrt(sp2.max()))]), p, v


def _curve(a, every):
    return [float(f"{x:.3g}") for x in np.asarray(a)[every - 1::every]]


def drift_dam32(N, every=5):
    """32^3 FLIP dam break (dt 1/120, 100 steps) on the GPU against the oracle's
    free-running trajectory in tests/golden/drift_dam32.npz (single-threaded FP64
    oracle = the reference's results; generated by tests/golden/make_drift.py),
    with the GPU's step rate (library CUDA-event step time after 3 warm-up steps)."""
    from fluid_simulator_gb300.scenes import GridSpec, dam_break

    if not os.path.exists(DRIFT32_GOLDEN):
        return {"unavailable": "tests/golden/drift_dam32.npz missing"}
    gold = np.load(DRIFT32_GOLDEN)
    res, dt, steps, sample = 32, float(gold["dt"]), int(gold["steps"]), int(gold["sample_every"])
    tracked = gold["tracked"]
    pos = dam_break(GridSpec(res), seed=0)
    p = N.default_params(transfer=N.FLIP, resolution=res, tol=1e-6, tol_mode=N.TOL_ABS_MAX, max_iters=200,
                         timing=True)
    sim = N.Simulation(res, p, track_ids=True)
    sim.set_particles(pos)
    h = sim.h
    stats, tp, tv, gpu_ms = [], [], [], []
    for s_ in range(1, steps + 1):
        gpu_ms.append(sim.step(dt).ms_total)
        row, pp, vv = _traj_stats(sim, N)
        stats.append(row)
        if s_ % sample == 0:
            tp.append(pp[tracked])
            tv.append(vv[tracked])
    sim.close()
    stats, tp, tv = np.array(stats), np.array(tp), np.array(tv)
    rs, rp, rv = gold["flip_stats"], gold["flip_pos"], gold["flip_vel"]
    dpos = np.sqrt(((tp.astype(np.float64) - rp) ** 2).sum(axis=2)) / h
    vs = np.maximum(np.sqrt((rv.astype(np.float64) ** 2).sum(axis=2)).max(axis=1), 1e-9)
    dvel = np.sqrt(((tv.astype(np.float64) - rv) ** 2).sum(axis=2).mean(axis=1)) / vs
    ke = np.abs(stats[:, 1] - rs[:, 1]) / np.maximum(rs[:, 1], 1e-12)
    g_ms = float(np.median(gpu_ms[3:]))
    return {"workload": "dam32_flip (32^3, FLIP 0.95, dt 1/120, 51840 particles)", "steps": steps,
            "gpu_steps_per_s": round(1e3 / g_ms, 1), "gpu_ms_per_step": round(g_ms, 3),
            "tracked_particles": int(tracked.size), "sampled_every": sample,
            "position_rms_cells": [float(f"{x:.3g}") for x in np.sqrt((dpos ** 2).mean(axis=1))],
            "position_max_cells": [float(f"{x:.3g}") for x in dpos.max(axis=1)],
            "velocity_rms_rel": [float(f"{x:.3g}") for x in dvel],
            "kinetic_energy_rel": _curve(ke, every),
            "fluid_cells_diff": [int(x) for x in (stats[:, 0] - rs[:, 0])[every - 1::every]]}


def drift_dam128(N, every=10):
    """128^3 dam break (dt 1/240, 200 steps) in PIC, FLIP 0.95 and APIC on the GPU,
    against the oracle's free-running trajectories in tests/golden/drift_dam128.npz
    (single-threaded FP64 oracle = the reference's results; generated by
    tests/golden/make_drift.py).  'fp64_threads' is the same comparison between
    two FP64 runs of the reference algorithm that differ only in the order of
    P2G's additions (1 vs 8 OpenMP threads): the drift rounding alone causes."""
    from fluid_simulator_gb300.scenes import GridSpec, dam_break

    if not os.path.exists(DRIFT_GOLDEN):
        return {"unavailable": "tests/golden/drift_dam128.npz missing"}
    gold = np.load(DRIFT_GOLDEN)
    res, dt, steps = 128, float(gold["dt"]), int(gold["steps"])
    sample = int(gold["sample_every"])
    tracked = gold["tracked"]
    pos = dam_break(GridSpec(res), seed=0)
    h = 1.0 / res
    out = {"workload": "dam128 (128^3, dt 1/240, 3830400 particles)", "steps": steps, "sampled_every": every,
           "tracked_particles": int(tracked.size), "tracked_every": sample}

    def compare(stats, tpos, tvel, ref):
        rs, rp, rv = gold[f"{ref}_stats"], gold[f"{ref}_pos"], gold[f"{ref}_vel"]
        ke = np.abs(stats[:, 1] - rs[:, 1]) / np.maximum(rs[:, 1], 1e-12)
        cen = np.sqrt(((stats[:, 2:5] - rs[:, 2:5]) ** 2).sum(axis=1)) / h
        cells = (stats[:, 0] - rs[:, 0]) / np.maximum(rs[:, 0], 1)
        dpos = np.sqrt(((tpos.astype(np.float64) - rp) ** 2).sum(axis=2)) / h
        vs = np.maximum(np.sqrt((rv.astype(np.float64) ** 2).sum(axis=2)).max(axis=1), 1e-9)
        dvel = np.sqrt(((tvel.astype(np.float64) - rv) ** 2).sum(axis=2).mean(axis=1)) / vs
        return {"kinetic_energy_rel": _curve(ke, every), "centroid_cells": _curve(cen, every),
                "fluid_cells_rel": _curve(cells, every),
                "tracked_position_rms_cells": [float(f"{x:.3g}") for x in np.sqrt((dpos ** 2).mean(axis=1))],
                "tracked_velocity_rms_rel": [float(f"{x:.3g}") for x in dvel]}

    for name, transfer in (("pic", N.PIC), ("flip", N.FLIP), ("apic", N.APIC)):
        p = N.default_params(transfer=transfer, resolution=res, tol=1e-6, tol_mode=N.TOL_ABS_MAX, max_iters=200,
                             timing=True)
        sim = N.Simulation(res, p, track_ids=True)
        sim.set_particles(pos)
        stats, tp, tv, its, ms = [], [], [], [], []
        for s in range(1, steps + 1):
            st = sim.step(dt)
            its.append(st.pcg_iterations)
            ms.append(st.ms_total)
            row, pp, vv = _traj_stats(sim, N)
            stats.append(row)
            if s % sample == 0:
                tp.append(pp[tracked])
                tv.append(vv[tracked])
        sim.close()
        out[name] = compare(np.array(stats), np.array(tp), np.array(tv), name)
        out[name]["gpu_pcg_iterations_mean"] = round(float(np.mean(its)), 2)
        g_ms = float(np.median(ms[3:]))
        out[name]["gpu_steps_per_s"] = round(1e3 / g_ms, 1)
        out[name]["gpu_particle_steps_per_s"] = round(pos.shape[0] * 1e3 / g_ms, 1)
        out[name]["oracle_pcg_iterations_mean"] = round(float(gold[f"{name}_stats"][:, 6].mean()), 2)
    ref = gold["flip_threads8_stats"]
    out["fp64_threads"] = compare(ref, gold["flip_threads8_pos"], gold["flip_threads8_vel"], "flip")
    return out


# ---------------------------------------------------------------- renderer
def render_study(sim, N, h, peak):
    """One 1000 x 1000 frame of the simulation's particles through the headless
    renderer (fsim_render_ctx: gfx publish + every FluidSurfaceGfx pass), with the
    reference GUI's settings scaled from its 40-unit box to the unit box."""
    W = H = 1000
    r = N.Renderer(W, H)
    eye = (1.9, 1.3, 2.3)
    yaw, pitch = N.look_at_angles(eye, (0.5, 0.3, 0.5))
    cam = N.camera(eye, yaw, pitch, fov=40.0, aspect=1.0, near=0.05, far=20.0)
    s = 1.0 / 40.0
    prm = N.default_render_params(particle_radius=h / 4, smoothing_size=2.4 * s, transparency_blur_size=2.4 * s,
                                  noise_scale=0.956 / s)
    for l in range(prm.num_lights):
        for k in range(3):
            prm.lights[l].position[k] *= s
            prm.lights[l].power_density[k] *= s * s
    for _ in range(2):
        r.frame_sim(sim, cam, prm)
    sim.synchronize()
    frames, kernel_ms = 5, []
    t0 = time.perf_counter()
    for f in range(frames):
        prm.noise_offset = 0.317 * 10.0 * f / 60.0
        r.frame_sim(sim, cam, prm)
        ms, launches = r.stats()
        kernel_ms.append(ms)
    sim.synchronize()
    wall_ms = (time.perf_counter() - t0) * 1e3 / frames
    n = sim.n
    covered = int((r.read(N.IMG_RAW_DEPTH) < 1.0).sum())
    r.close()
    # algorithmic bytes: two particle passes over the 20-byte records (surface
    # splat and spray splat, each also adding thickness) + the image passes
    # (~120 B per pixel)
    alg = 2 * 20 * n + 120 * W * H
    k = statistics.median(kernel_ms)
    return {"image": [W, H], "particles": n, "covered_pixels": covered, "ms_per_frame_kernels": round(k, 3),
            "ms_per_frame_wall": round(wall_ms, 3), "launches_per_frame": launches,
            "algorithmic_bytes": alg, "achieved_gbs": round(alg / (k / 1e3) / 1e9, 1),
            "frac": round(alg / (k / 1e3) / 1e9 / peak, 4),
            "note": "wall time includes fsim_fill_gfx (device) and the Python call"}


# ---------------------------------------------------------------- precision study
def precision_study(sim, N, seed: int = 11):
    """Pressure projection alone at 256^3: cell types from APIC dam-break
    snapshots (after 30 and 60 steps) and from seeded random masks
    (Gaussian-filtered N(0, 1) noise, sigma 6 cells, 40-70 % fluid, solid
    walls); rhs the divergence of a seeded N(0, 1) face-velocity field smoothed
    with sigma 3 cells.  Solvers: FP32 PCG with FP64 dots and scalars
    (FSIM_PREC_FP32) and FP32 inner solves with FP64-residual refinement
    (FSIM_PREC_MIXED), multigrid-preconditioned, at relative residuals 1e-4,
    1e-6 and 1e-8, against the all-FP64 PCG (FSIM_PREC_FP64, red-black IC)
    solved to 1e-10.  Error = max over fluid cells of |p - p_fp64| / max |p_fp64|;
    time-to-tolerance = the solve's CUDA-event time."""
    from fluid_simulator_gb300 import warmstart as W
    from fluid_simulator_gb300.scenes import GridSpec, dam_break

    res = sim.shape[0]
    dt = 1.0 / float(res * res)  # dt / (rho h^2) = 1: rhs in the solver's units
    problems = []
    p = N.default_params(transfer=N.APIC, resolution=res, tol=1e-6, tol_mode=N.TOL_REL_L2, max_iters=2000)
    ds = N.Simulation(res, p)
    ds.set_particles(dam_break(GridSpec(res), seed=0))
    for s in range(60):
        ds.step(1.0 / 480.0)
        if s + 1 in (30, 60):
            problems.append((f"dam256_step{s + 1}", ds.grid(N.F_FLAGS)))
    ds.close()
    masks, _ = W.mask_problems(res, 2, seed)
    problems += [(f"mask_seed{seed}_{i}", masks[i]) for i in range(2)]
    rng = np.random.default_rng(seed + 1)
    out = {"grid": [res] * 3, "reference": "FP64 PCG (red-black IC), relative residual 1e-10",
           "preconditioner": "multigrid", "problems": {}}
    keep = sim.params
    for name, flags in problems:
        rhs = np.where(flags == N.WATER, W.random_divergence(rng, 1, res)[0], 0.0).astype(np.float64)
        sim.set_grid(N.F_FLAGS, flags)
        ref, st = sim.solve_pressure(rhs, dt, precision=N.PREC_FP64, tol_mode=N.TOL_REL_L2, tol=1e-10,
                                     max_iters=40000)
        fluid = W.solver_fluid(flags)
        scale = max(float(np.abs(ref[fluid]).max()), 1e-300)
        row = {"fluid_cells": int(fluid.sum()), "fp64": {"iterations": st.pcg_iterations, "ms": round(st.ms_solve, 2),
                                                         "residual_rel": float(f"{st.residual_rel:.3g}")}}
        for pname, prec in (("mixed", N.PREC_MIXED), ("fp32", N.PREC_FP32)):
            for tol in (1e-4, 1e-6, 1e-8):
                pp, st = sim.solve_pressure(rhs, dt, precision=prec, tol_mode=N.TOL_REL_L2, tol=tol, max_iters=400)
                row[f"{pname}_{tol:.0e}"] = {
                    "iterations": st.pcg_iterations, "ms": round(st.ms_solve, 3), "converged": bool(st.converged),
                    "residual_rel": float(f"{st.residual_rel:.3g}"),
                    "err_vs_fp64": float(f"{float(np.abs(pp - ref)[fluid].max()) / scale:.3g}")}
        out["problems"][name] = row
    sim.set_params(keep)
    return out


# ---------------------------------------------------------------- learned warm start
WARMSTART_WEIGHTS = os.path.join(ROOT, "fluid_simulator_gb300", "weights", "warmstart_c5.npz")
# FSIM_WARM_ZERO / _PREVIOUS / _LEARNED / _LEARNED_RESIDUAL
STARTS = (("zero", 0), ("previous", 1), ("learned", 3), ("learned_residual", 4))
PRECONDS = (("rbic", 0), ("mg", 1))                      # FSIM_PRECOND_RBIC (the plain solver) / _MG


def compare_starts(sim, dt, N, stages_fn, problems: int, max_iters: int = 20000):
    """On `problems` consecutive solves of a running simulation, the pressure
    solve (relative residual 1e-6) from the zero start (the reference's), the
    previous step's pressure and the network's judged guess, each with the
    red-black IC preconditioner (the plain solver) and the multigrid one.
    Times are the library's CUDA events from the solve's first to last kernel,
    inference included.  The step then continues from the previous-pressure
    multigrid solve."""
    rec = {(pn, sn): [] for pn, _ in PRECONDS for sn, _ in STARTS}
    base = sim.params
    for k in range(problems + 1):
        stages_fn()
        p_prev = sim.grid(N.F_PRESSURE)
        for pn, pc in PRECONDS:
            base.precond, base.tol_mode, base.residual_tol, base.max_iters = pc, N.TOL_REL_L2, 1e-6, max_iters
            sim.set_params(base)
            for sn, start in STARTS:
                sim.set_grid(N.F_PRESSURE, p_prev)
                st = sim.solve_current(dt, start, apply=False)
                if k > 0:  # the first problem also pays one-time allocations and graph captures
                    rec[(pn, sn)].append((st.ms_solve, st.pcg_iterations, st.guess_used, st.ms_guess,
                                          st.residual_rel, st.converged))
        base.precond = N.PRECOND_MG
        sim.set_params(base)
        sim.set_grid(N.F_PRESSURE, p_prev)
        sim.solve_current(dt, N.WARM_PREVIOUS, apply=True)
        sim.stage(N.STAGE_EXTRAPOLATE, dt)
        sim.stage(N.STAGE_G2P, dt)
    out = {}
    for pn, _ in PRECONDS:
        row = {}
        for sn, _ in STARTS:
            r = rec[(pn, sn)]
            row[sn] = {"ms": round(statistics.mean(x[0] for x in r), 3),
                       "iterations": round(statistics.mean(x[1] for x in r), 2),
                       "residual_rel_max": float(f"{max(x[4] for x in r):.3g}"),
                       "converged": all(x[5] == 1 for x in r)}
        for sn, mode in (("learned", 3), ("learned_residual", 4)):
            lr = rec[(pn, sn)]
            row[sn]["guess_used_frac"] = round(sum(1 for x in lr if x[2] == mode) / len(lr), 3)
            row[sn]["fallback_rate"] = round(1.0 - row[sn]["guess_used_frac"], 3)
            row[sn]["ms_inference"] = round(statistics.mean(x[3] for x in lr), 3)
            row[f"speedup_{sn}_vs_zero"] = round(row["zero"]["ms"] / row[sn]["ms"], 3)
            row[f"speedup_{sn}_vs_previous"] = round(row["previous"]["ms"] / row[sn]["ms"], 3)
        row["speedup_previous_vs_zero"] = round(row["zero"]["ms"] / row["previous"]["ms"], 3)
        out[pn] = row
    return out


def warm_start_study(sim, dt, t, h, N, args):
    """PCG time-to-1e-6 from the learned start against the plain (zero) start:
    on this benchmark's 256^3 APIC scene, and inside 128^3 / 256^3 APIC dam-break
    runs (the evaluation of the network's training protocol).  The network's
    parameters are the committed result of that protocol
    (fluid_simulator_gb300/weights/warmstart_c5.npz, produced on the GPU by
    python -m fluid_simulator_gb300.warmstart protocol)."""
    from fluid_simulator_gb300 import warmstart as W
    from fluid_simulator_gb300.scenes import GridSpec, dam_break

    if not os.path.exists(WARMSTART_WEIGHTS):
        return {"unavailable": "fluid_simulator_gb300/weights/warmstart_c5.npz not present"}
    net = W.load_net(WARMSTART_WEIGHTS)
    meta = json.loads(str(np.load(WARMSTART_WEIGHTS)["meta"]))
    out = {"tol": "1e-6 relative L2", "problems": args.ws_steps,
           "training": {k: meta[k] for k in ("pool", "iters", "batch", "lr", "loss", "loss_first_100",
                                             "loss_last_100", "train_seconds") if k in meta}}
    tt = [t]
    stages = (N.STAGE_SPAWN, N.STAGE_ADVECT, N.STAGE_PUSH_OUT, N.STAGE_P2G, N.STAGE_OBSTACLES, N.STAGE_WALLS,
              N.STAGE_POST_P2G)

    def bench_stages():
        sim.set_obstacles(obstacles_at(tt[0], dt, h, N))
        for stg in stages:
            sim.stage(stg, dt)
        tt[0] += dt

    sim.set_net(net)
    out["fill256_apic"] = compare_starts(sim, dt, N, bench_stages, args.ws_steps)
    sim.set_net(None)
    for res, dtr, warm in ((128, 1.0 / 240.0, 40), (256, 1.0 / 480.0, 40)):
        p = N.default_params(transfer=N.APIC, resolution=res, tol=1e-6, tol_mode=N.TOL_REL_L2, max_iters=20000,
                             timing=True)
        ds = N.Simulation(res, p)
        ds.set_particles(dam_break(GridSpec(res), seed=0))
        for _ in range(warm):
            ds.step(dtr)
        ds.set_net(net)

        def dam_stages():
            for stg in (N.STAGE_ADVECT, N.STAGE_PUSH_OUT, N.STAGE_P2G, N.STAGE_OBSTACLES, N.STAGE_WALLS,
                        N.STAGE_POST_P2G):
                ds.stage(stg, dtr)

        out[f"dam{res}_apic"] = compare_starts(ds, dtr, N, dam_stages, args.ws_steps)
        out[f"dam{res}_apic"]["after_steps"] = warm
        ds.set_net(None)
        ds.close()
    net.close()
    return out


# ---------------------------------------------------------------- CPU leg
def cpu_baseline(res: int, dt: float, steps: int = 1, warm: int = 0):
    """The reference's algorithm (FP64 oracle, all host threads) on the same workload."""
    from oracle import oracle as O

    O.build_port()
    grid, pos = workload_scene(res)
    h = grid.h
    p = O.make_params(res, transfer=O.APIC, tol=1e-6, max_iters=2000, spawning=True, despawning=True)
    o = O.Oracle(p, pos.astype(np.float64), lib="port")
    del pos
    cores = os.cpu_count() or 1
    o.set_threads(cores)
    t = 0.0
    times = []
    its = []
    for k in range(warm + steps):
        x = 0.5 + 0.1 * math.sin(math.pi * t)
        xp = 0.5 + 0.1 * math.sin(math.pi * (t - dt))
        o.set_obstacles([
            O.obstacle(O.OBS_SPHERE, (x, 0.6, 0.5), r=0.15, prev_pos=(xp, 0.6, 0.5), speed=((x - xp) / dt, 0, 0)),
            O.obstacle(O.OBS_DISC_SOURCE, (0.5, 0.95, 0.5), r=4 * h, spawn_speed=-1.0),
            O.obstacle(O.OBS_BOX_SINK, (4 * h, 4 * h, 4 * h), size=(8 * h, 8 * h, 8 * h))])
        t0 = time.perf_counter()
        its.append(o.step(dt))
        t1 = time.perf_counter()
        if k >= warm:
            times.append(t1 - t0)
        t += dt
    n = o.n
    o.close()
    sec = sum(times) / len(times)
    return {"value": round(1.0 / sec, 5), "unit": "steps/s", "cores": cores, "kind": "port",
            "sample": f"{steps} full step(s) of {WORKLOAD} ({n} particles) after {warm} warm-up, "
                      f"FP64 oracle, OpenMP x{cores}, MIC(0) PCG iterations {its[warm:]}",
            "seconds_per_step": round(sec, 3)}


def cpu_baseline_configs():
    """The oracle (FP64, all host threads) on the smaller dam-break
    configurations: 32^3 FLIP (dt 1/120; 20 steps after 3) and 128^3 APIC
    (dt 1/240; 2 steps after 1), from the seeded start."""
    from fluid_simulator_gb300.scenes import GridSpec, dam_break
    from oracle import oracle as O

    O.build_port()
    threads = os.cpu_count() or 1
    out = {}
    for name, res, transfer, dt, warm, steps in (("dam32_flip", 32, O.FLIP, 1.0 / 120.0, 3, 20),
                                                 ("dam128_apic", 128, O.APIC, 1.0 / 240.0, 1, 2)):
        pos = dam_break(GridSpec(res), seed=0)
        o = O.Oracle(O.make_params(res, transfer=transfer, tol=1e-6, max_iters=200), pos.astype(np.float64),
                     lib="port")
        o.set_threads(threads)
        for _ in range(warm):
            o.step(dt)
        t0 = time.perf_counter()
        for _ in range(steps):
            o.step(dt)
        sec = (time.perf_counter() - t0) / steps
        o.close()
        out[name] = {"steps_per_s": round(1.0 / sec, 3), "threads": threads,
                     "sample": f"{steps} steps after {warm} from the seeded start"}
    return out


def run_solve_case(args):
    """Pressure solves alone on the benchmark's cell types (fluid below y = 0.5
    in the 256^3 box, solid walls) with a seeded random-divergence rhs and no
    particles: the solver's kernels at the benchmark size with a few hundred MB
    on the device, for counter captures.  Prints one JSON line."""
    from fluid_simulator_gb300 import native as N
    from fluid_simulator_gb300 import warmstart as W

    res = args.res
    p = N.default_params(transfer=N.APIC, resolution=res, tol=1e-6, tol_mode=N.TOL_REL_L2, max_iters=2000,
                         timing=True, precond={"mg": N.PRECOND_MG, "rbic": N.PRECOND_RBIC}[args.precond])
    sim = N.Simulation(res, p)
    c = (np.arange(res) + 0.5) / res
    flags = np.full((res, res, res), N.AIR, np.uint8)
    flags[:, c < 0.5, :] = N.WATER
    flags[0], flags[-1] = N.SOLID, N.SOLID
    flags[:, 0], flags[:, -1] = N.SOLID, N.SOLID
    flags[:, :, 0], flags[:, :, -1] = N.SOLID, N.SOLID
    rhs = np.where(flags == N.WATER, W.random_divergence(np.random.default_rng(3), 1, res)[0], 0.0)
    sim.set_grid(N.F_FLAGS, flags)
    dt = 1.0 / float(res * res)
    rec = []
    for _ in range(args.solve_case):
        _, st = sim.solve_pressure(rhs, dt, precision=N.PREC_MIXED, tol_mode=N.TOL_REL_L2, tol=1e-6, max_iters=2000)
        rec.append((st.ms_solve, st.pcg_iterations))
    sim.close()
    print(json.dumps({"solve_case": {"grid": [res] * 3, "precond": args.precond, "fluid_cells": int((flags == 0).sum()),
                                     "ms": [round(x[0], 3) for x in rec], "iterations": [x[1] for x in rec]}}),
          flush=True)


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return
    res = args.res
    dt = 1.0 / 480.0 if res == 256 else 1.0 / (480.0 * res / 256.0)
    steps = max(1, min(args.steps, 2))
    cb = cpu_baseline(res, dt, steps=steps, warm=1 if args.warmup > 0 else 0)
    line = {
        "impl": "reference",
        "metric": "steps/s (256^3 APIC step, PCG to 1e-6 relative residual)",
        "value": cb["value"],
        "unit": "steps/s",
        "n_gpus": world,
        "steps": steps,
        "warmup": 1 if args.warmup > 0 else 0,
        "ms_per_step": round(1000.0 * cb["seconds_per_step"], 1),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded dam-break fill, no dataset)",
        "config": {"workload": WORKLOAD, "grid": [res, res, res], "transfer": "APIC",
                   "note": f"reference algorithm on host cores; {steps} timed step(s) of the requested "
                           f"{args.steps} (each takes tens of seconds)"},
        "cpu_baseline": cb,
        "e2e": {"value": cb["value"], "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="fsim", choices=["fsim", "reference"])
    ap.add_argument("--res", type=int, default=256, help="grid resolution (256 = the benchmark workload)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--precond", default="mg", choices=["mg", "rbic"],
                    help="pressure preconditioner: multigrid V-cycle or red-black incomplete Cholesky")
    ap.add_argument("--out-dir", default=os.path.join(ROOT, "bench_out"),
                    help="where the clock samples of the timed region are written")
    ap.add_argument("--mg-sweeps", type=int, default=0,
                    help="multigrid smoothing sweeps before and after the coarse correction (0: library default)")
    ap.add_argument("--mg-coarse-sweeps", type=int, default=0,
                    help="multigrid sweeps on the coarser levels (0: as --mg-sweeps)")
    ap.add_argument("--mg-boundary-sweeps", type=int, default=0,
                    help="extra red-black sweeps on the finest level's free-surface band "
                         "(0: 3 on grids of 2^23 cells or more, else none; -1: none)")
    ap.add_argument("--mg-cluster-sweeps", type=int, default=0,
                    help="multigrid sweeps on the levels run by the cluster kernel (0: library default)")
    ap.add_argument("--precision-study", type=int, default=1,
                    help="solve the last step's pressure problem in FP64 / mixed / FP32 and report errors (0: skip)")
    ap.add_argument("--ws-steps", type=int, default=6,
                    help="problems per scene of the zero / previous / learned warm-start comparison (0: skip)")
    ap.add_argument("--render", type=int, default=1, help="time one 1000x1000 frame of the headless renderer")
    ap.add_argument("--solve-case", type=int, default=0,
                    help="only K pressure solves of the benchmark's cell types (no particles), for counter captures")
    ap.add_argument("--parity", type=int, default=1,
                    help="free-running drift curves against the oracle: 32^3 FLIP (100 steps, oracle run live) "
                         "and 128^3 PIC / FLIP / APIC (200 steps, oracle trajectories from tests/golden) (0: skip)")
    ap.add_argument("--refine-digits", type=int, default=0,
                    help="mixed-precision refinement every 10^k residual drop (0: library default 3)")
    args = ap.parse_args()
    os.makedirs(args.out_dir, exist_ok=True)
    if args.solve_case > 0:
        run_solve_case(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_fsim(args)


if __name__ == "__main__":
    main()
