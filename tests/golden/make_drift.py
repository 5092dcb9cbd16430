"""Generates tests/golden/drift_dam128.npz: the oracle's free-running
trajectories of the 128^3 dam break (dt = 1/240, 200 steps; PIC, FLIP 0.95,
APIC), the reference side of the drift curve that bench.py reports; and
(`python tests/golden/make_drift.py dam32`, a few seconds) drift_dam32.npz, the
same for the 32^3 FLIP dam break (dt = 1/120, 100 steps).

The oracle (oracle/fsim_oracle.c) runs single-threaded, where it equals the
reference's own Simulator bit for bit (pinned by tests/golden/golden.json), so
these are the reference's trajectories on the seeded dam break.  A second
FLIP run with 8 OpenMP threads (same inputs; its P2G adds in a different order)
records how far two FP64 runs of the reference drift apart by rounding alone.

Per step (after Simulator::simulate): fluid-cell count, mean kinetic energy
0.5 |v|^2, particle centroid, max |v| and the PCG iteration count; every
SAMPLE_EVERY steps the positions and velocities (FP32) of TRACKED particles
with evenly spaced indices (the oracle keeps the particle order: nothing is
deleted in this scene).

    python tests/golden/make_drift.py            (~20 minutes on 8 cores)
    python tests/golden/make_drift.py dam32      (the 32^3 fixture only)
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

RES = 128
DT = 1.0 / 240.0
STEPS = 200
SAMPLE_EVERY = 20
TRACKED = 1024
OUT = os.path.join(HERE, "drift_dam128.npz")


def stats_of(o, its):
    from oracle import oracle as O

    pos, vel, _ = o.particles()
    return np.array([float((o.grid(O.F_FLAGS) == O.WATER).sum()), 0.5 * float((vel * vel).sum(axis=1).mean()),
                     *pos.mean(axis=0), float(np.sqrt((vel * vel).sum(axis=1)).max()), float(its)]), pos, vel


def run(transfer: int, threads: int, res: int = RES, dt: float = DT, steps: int = STEPS,
        sample_every: int = SAMPLE_EVERY, tracked: int = TRACKED):
    from fluid_simulator_gb300.scenes import GridSpec, dam_break
    from oracle import oracle as O

    O.build_port()
    pos = dam_break(GridSpec(res), seed=0)
    o = O.Oracle(O.make_params(res, transfer=transfer, tol=1e-6, max_iters=200), pos.astype(np.float64),
                 lib="port")
    o.set_threads(threads)
    n = o.n
    idx = np.linspace(0, n - 1, tracked).round().astype(np.int64)
    stats, tp, tv = [], [], []
    for s in range(1, steps + 1):
        its = o.step(dt)
        st, p, v = stats_of(o, its)
        stats.append(st)
        if s % sample_every == 0:
            tp.append(p[idx].astype(np.float32))
            tv.append(v[idx].astype(np.float32))
    o.close()
    return np.array(stats), np.array(tp), np.array(tv), idx


def main():
    from oracle import oracle as O

    jobs = {"pic": (O.PIC, 1), "flip": (O.FLIP, 1), "apic": (O.APIC, 1), "flip_threads8": (O.FLIP, 8)}
    out = {"dt": np.array(DT), "steps": np.array(STEPS), "sample_every": np.array(SAMPLE_EVERY),
           "stat_names": np.array(["fluid_cells", "kinetic_energy", "centroid_x", "centroid_y", "centroid_z",
                                   "max_speed", "pcg_iterations"])}
    ctx = __import__("multiprocessing").get_context("spawn")
    with cf.ProcessPoolExecutor(max_workers=len(jobs), mp_context=ctx) as ex:
        futs = {k: ex.submit(run, *v) for k, v in jobs.items()}
        for k, f in futs.items():
            stats, tp, tv, idx = f.result()
            out[f"{k}_stats"] = stats
            out[f"{k}_pos"] = tp
            out[f"{k}_vel"] = tv
            out["tracked"] = idx
            print(k, "done", stats[-1], flush=True)
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


def main_dam32():
    """32^3 FLIP dam break, dt 1/120, 100 steps, single-threaded oracle; every
    5th step the positions and velocities of 1024 evenly spaced particles."""
    from oracle import oracle as O

    steps, every = 100, 5
    stats, tp, tv, idx = run(O.FLIP, 1, res=32, dt=1.0 / 120.0, steps=steps, sample_every=every, tracked=1024)
    path = os.path.join(HERE, "drift_dam32.npz")
    np.savez_compressed(path, dt=np.array(1.0 / 120.0), steps=np.array(steps), sample_every=np.array(every),
                        stat_names=np.array(["fluid_cells", "kinetic_energy", "centroid_x", "centroid_y",
                                             "centroid_z", "max_speed", "pcg_iterations"]),
                        flip_stats=stats, flip_pos=tp, flip_vel=tv, tracked=idx)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "dam32":
        main_dam32()
    else:
        main()
