"""Shared helpers of the parity tests: build identical GPU / oracle instances
from one seeded FP32 particle set and compare their state.

Tolerances (written here once, used by every parity test):
  * cell marks, per-cell particle counts, cell indices: bit-exact
  * grid velocities after P2G, v2, extrapolated v2, avgPNum: |gpu - ref| <=
    REL_GRID * max(|ref|, FLOOR) elementwise-scaled by the field's max norm
  * pressure: |gpu - ref| <= REL_PRESSURE * max|ref|
  * particle velocities / APIC C after one G2P from identical grids:
    |gpu - ref| <= REL_PARTICLE * max|ref| (+ FLOOR)
"""
from __future__ import annotations

import numpy as np

from fluid_simulator_gb300 import native as N
from oracle import oracle as O

REL_GRID = 1e-5
REL_PRESSURE = 1e-4
REL_PARTICLE = 1e-5
FLOOR = 1e-6

TRANSFER_O = {N.PIC: O.PIC, N.FLIP: O.FLIP, N.APIC: O.APIC}


def make_pair(pos, resolution, transfer, *, vel=None, c=None, lib="port", threads=0, tol=1e-6,
              max_iters=200, gpu_tol=None, gpu_tol_mode=N.TOL_ABS_MAX, gpu_max_iters=None, dims=(1.0, 1.0, 1.0),
              two_d=False, **kw):
    """(gpu Simulation, oracle) on identical FP32 particles."""
    pos = np.ascontiguousarray(pos, np.float32)
    p = N.default_params(transfer=transfer, resolution=resolution, tol=tol if gpu_tol is None else gpu_tol,
                         tol_mode=gpu_tol_mode, max_iters=max_iters if gpu_max_iters is None else gpu_max_iters,
                         **kw)
    g = N.Simulation(resolution, p, track_ids=True, dims=dims, two_d=two_d)
    g.set_particles(pos, vel, None if c is None else np.asarray(c, np.float32).reshape(-1, 9))
    okw = {k: v for k, v in kw.items() if k in ("spawning", "despawning", "stop_particles", "gravity",
                                                "flip_ratio", "top_solid", "pressure_enabled", "grid_solver",
                                                "push_apart")}
    op = O.make_params(resolution, transfer=TRANSFER_O[transfer], tol=tol, max_iters=max_iters, dims=dims,
                       two_d=two_d, **okw)
    o = O.Oracle(op, pos.astype(np.float64),
                 None if vel is None else np.asarray(vel, np.float32).astype(np.float64),
                 None if c is None else np.asarray(c, np.float32).astype(np.float64), lib=lib)
    if threads:
        o.set_threads(threads)
    return g, o


def ref_counts(pos, shape, h):
    cell = np.floor(np.asarray(pos, np.float64) / h).astype(np.int64)
    counts = np.zeros(shape, np.int64)
    np.add.at(counts, (cell[:, 0], cell[:, 1], cell[:, 2]), 1)
    return counts


def assert_close_field(gpu, ref, rel, name, floor=FLOOR):
    gpu = np.asarray(gpu, np.float64)
    ref = np.asarray(ref, np.float64)
    scale = max(float(np.abs(ref).max()), floor)
    err = float(np.abs(gpu - ref).max())
    assert err <= rel * scale, f"{name}: max abs err {err:.3e} > {rel:.1e} * {scale:.3e}"
    return err / scale


def sync_oracle_particles_from_gpu(g, o):
    """Give the oracle the GPU's FP32 particle state (promoted to FP64)."""
    pos, vel, c = g.particles()
    o.set_particles(pos.astype(np.float64), vel.astype(np.float64), c.astype(np.float64))
    return pos, vel, c


def inject_grid_from_oracle(g, o, fields):
    m = {N.F_FLAGS: O.F_FLAGS, N.F_AVGPNUM: O.F_AVGPNUM, N.F_VX: O.F_VX, N.F_VY: O.F_VY, N.F_VZ: O.F_VZ,
         N.F_V2X: O.F_V2X, N.F_V2Y: O.F_V2Y, N.F_V2Z: O.F_V2Z}
    for f in fields:
        vals = o.grid(m[f])
        if f != N.F_FLAGS:
            vals = vals.astype(np.float32)
            o.set_grid(m[f], vals.astype(np.float64))  # both sides hold the same FP32 values
        g.set_grid(f, vals)
