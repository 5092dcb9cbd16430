"""Generate the golden fixtures under tests/golden/ from the reference itself.

Runs the reference's own Simulator sources (oracle/_ref/libfsim_ref.so, built
by `make -C oracle ref` from the sources in the reference checkout) with one
OpenMP thread on seeded dam-break inputs and records, per step, SHA-256
digests of every FP64 grid field and particle array plus the PCG iteration
count, and the full FP64 arrays of a few early states.  The CPU oracle
(oracle/fsim_oracle.c) must reproduce every digest bit for bit
(tests/test_oracle_golden.py); the CUDA path is then checked against the
oracle.

Usage:  python tests/golden/make_golden.py   (needs the reference checkout)
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from fluid_simulator_gb300.scenes import GridSpec, dam_break, dam_break_2d  # noqa: E402
from oracle import oracle as O  # noqa: E402

GRID_FIELDS = {"flags": O.F_FLAGS, "avgPNum": O.F_AVGPNUM, "vx": O.F_VX, "vy": O.F_VY, "vz": O.F_VZ,
               "v2x": O.F_V2X, "v2y": O.F_V2Y, "v2z": O.F_V2Z, "wx": O.F_WX, "wy": O.F_WY, "wz": O.F_WZ}


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()[:32]


def obstacles_at(step: int, dt: float, plane_z=None):
    """Moving sphere, moving box and a sink (the obstacle case); in 2D mode
    (plane_z set) all three sit on the particles' plane and the box spans z."""
    t = step * dt
    sx = 0.55 + 0.1 * np.sin(np.pi * t * 4)
    sxp = 0.55 + 0.1 * np.sin(np.pi * (t - dt) * 4)
    if plane_z is not None:
        z = plane_z
        return [O.obstacle(O.OBS_SPHERE, (sx, 0.3, z), r=0.12, prev_pos=(sxp, 0.3, z),
                           speed=((sx - sxp) / dt, 0, 0)),
                O.obstacle(O.OBS_BOX, (0.3, 0.15, z), size=(0.1, 0.2, 4 * z), speed=(0, 0.5, 0)),
                O.obstacle(O.OBS_SINK, (0.1, 0.1, z), r=0.08)]
    return [O.obstacle(O.OBS_SPHERE, (sx, 0.3, 0.5), r=0.12, prev_pos=(sxp, 0.3, 0.5), speed=((sx - sxp) / dt, 0, 0)),
            O.obstacle(O.OBS_BOX, (0.3, 0.15, 0.3), size=(0.1, 0.2, 0.15), speed=(0, 0, 0.5)),
            O.obstacle(O.OBS_SINK, (0.1, 0.1, 0.8), r=0.08)]


CASES = {
    # name: (resolution, transfer, block_hi, seed, steps, dt, obstacles)
    "dam16_pic": (16, O.PIC, (0.5, 0.6, 1.0), 0, 4, 1 / 120, False),
    "dam16_flip": (16, O.FLIP, (0.5, 0.6, 1.0), 0, 4, 1 / 120, False),
    "dam16_apic": (16, O.APIC, (0.5, 0.6, 1.0), 0, 4, 1 / 120, False),
    "obs32_flip": (32, O.FLIP, (0.5, 0.7, 1.0), 3, 6, 1 / 120, True),
    "obs32_apic": (32, O.APIC, (0.5, 0.7, 1.0), 3, 6, 1 / 120, True),
    "dam32_flip": (32, O.FLIP, (0.4, 0.6, 1.0), 0, 10, 1 / 120, False),
    # non-cubic 3D grid (32 x 24 x 16 cells)
    "box32x24x16_flip": (32, O.FLIP, (0.5, 0.5, 0.5), 1, 6, 1 / 120, False, {"dims": (1.0, 0.75, 0.5)}),
    # 2D mode: 32 x 32 x 3 cells, cellD.z = 0.1 (not the x / y cell size)
    "dam2d32_flip": (32, O.FLIP, (0.4, 0.6), 0, 8, 1 / 120, False, {"dims": (1.0, 1.0, 0.3), "two_d": True}),
    "obs2d32_apic": (32, O.APIC, (0.5, 0.7), 3, 6, 1 / 120, True, {"dims": (1.0, 1.0, 0.3), "two_d": True}),
}

# cases whose first steps are stored as full FP64 arrays
FULL = {"dam16_flip": 2, "dam16_apic": 1}


def case_setup(name: str):
    """(grid, FP32 positions, oracle params, plane z or None) of a case."""
    res, tr, hi, seed, steps, dt, obst = CASES[name][:7]
    extra = CASES[name][7] if len(CASES[name]) > 7 else {}
    dims, two_d = extra.get("dims", (1.0, 1.0, 1.0)), extra.get("two_d", False)
    grid = GridSpec(res, dims, two_d)
    if two_d:
        pos = dam_break_2d(grid, (0.0, 0.0), hi, seed=seed)
    else:
        pos = dam_break(grid, (0.0, 0.0, 0.0), hi, seed=seed)
    params = O.make_params(res, transfer=tr, despawning=obst, dims=dims, two_d=two_d)
    return grid, pos, params, (dims[2] / 2 if two_d else None)


def run_case(lib: str, name: str, full_steps: int = 0):
    steps, dt, obst = CASES[name][4:7]
    grid, pos, params, plane = case_setup(name)
    o = O.Oracle(params, pos.astype(np.float64), lib=lib)
    o.set_threads(1)
    rec = {"n0": int(pos.shape[0]), "steps": []}
    arrays = {"pos0": pos}
    for s in range(steps):
        if obst:
            o.set_obstacles(obstacles_at(s, dt, plane))
        its = o.step(dt)
        p, v, c = o.particles()
        step = {"its": int(its), "n": int(o.n), "fluid": int(o.fluid_count())}
        for k, f in GRID_FIELDS.items():
            g = o.grid(f)
            step[k] = digest(g)
            if s < full_steps:
                arrays[f"s{s}_{k}"] = g
        step["pos"], step["vel"], step["c"] = digest(p), digest(v), digest(c)
        if s < full_steps:
            arrays[f"s{s}_pos"], arrays[f"s{s}_vel"], arrays[f"s{s}_c"] = p, v, c
        rec["steps"].append(step)
    o.close()
    return rec, arrays


def main():
    if O.build_ref() is None:
        sys.exit("reference sources not found; fixtures are generated from the reference itself")
    out = {"generator": "tests/golden/make_golden.py", "library": "oracle/_ref/libfsim_ref.so",
           "threads": 1, "cases": {}}
    for name in CASES:
        rec, arrays = run_case("ref", name, FULL.get(name, 0))
        out["cases"][name] = rec
        if name in FULL:
            np.savez_compressed(os.path.join(HERE, f"{name}_full.npz"), **arrays)
        print(name, [s["its"] for s in rec["steps"]], rec["steps"][-1]["n"])
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
