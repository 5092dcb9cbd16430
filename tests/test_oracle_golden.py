"""Pins the CPU oracle (oracle/fsim_oracle.c) to the reference.

tests/golden/golden.json holds SHA-256 digests of every grid field and
particle array after each step, produced by the reference's own Simulator
sources (tests/golden/make_golden.py).  With one thread the oracle must
reproduce every digest bit for bit, on this machine and on the aarch64 GPU host
(the oracle is compiled without floating-point contraction).  Where the
reference library is built (oracle/_ref), the two are also compared directly.
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")

import sys  # noqa: E402

sys.path.insert(0, GOLDEN)
import make_golden as MG  # noqa: E402


def load_golden():
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        return json.load(f)


@pytest.mark.parametrize("case", list(MG.CASES))
def test_oracle_reproduces_reference_digests(port_lib, case):
    gold = load_golden()["cases"][case]
    rec, arrays = MG.run_case("port", case, MG.FULL.get(case, 0))
    assert rec["n0"] == gold["n0"]
    for s, (got, want) in enumerate(zip(rec["steps"], gold["steps"])):
        for k in want:
            assert got[k] == want[k], f"{case} step {s}: {k} differs from the reference"


@pytest.mark.parametrize("case", list(MG.FULL))
def test_oracle_full_arrays(port_lib, case):
    ref = np.load(os.path.join(GOLDEN, f"{case}_full.npz"))
    rec, arrays = MG.run_case("port", case, MG.FULL[case])
    for k in ref.files:
        assert np.array_equal(ref[k], arrays[k]), k


def test_golden_inputs_are_the_seeded_scene():
    """The fixtures' inputs are the dam-break seeding rule (scenes.dam_break)."""
    from fluid_simulator_gb300.scenes import GridSpec, dam_break

    ref = np.load(os.path.join(GOLDEN, "dam16_flip_full.npz"))
    pos = dam_break(GridSpec(16), (0, 0, 0), (0.5, 0.6, 1.0), seed=0)
    assert np.array_equal(ref["pos0"], pos)


@pytest.mark.skipif(not O.have_ref(), reason="reference library not built here")
@pytest.mark.parametrize("transfer", [O.PIC, O.FLIP, O.APIC])
def test_oracle_equals_reference_stagewise(port_lib, transfer):
    """Stage by stage, the oracle equals the reference's own member functions."""
    from fluid_simulator_gb300.scenes import GridSpec, dam_break

    pos = dam_break(GridSpec(32), (0, 0, 0), (0.5, 0.7, 1.0), seed=5).astype(np.float64)
    p = O.make_params(32, transfer=transfer, despawning=True)
    a = O.Oracle(p, pos, lib="ref")
    b = O.Oracle(p, pos, lib="port")
    a.set_threads(1)
    dt = 1 / 120
    obs = MG.obstacles_at(2, dt)
    a.set_obstacles(obs)
    b.set_obstacles(obs)
    for _ in range(2):
        a.step(dt)
        b.step(dt)
    stages = [O.STAGE_ADVECT, O.STAGE_PUSH_OUT, O.STAGE_P2G, O.STAGE_MARK, O.STAGE_OBSTACLES, O.STAGE_WALLS,
              O.STAGE_POST_P2G, O.STAGE_SOLVE, O.STAGE_EXTRAPOLATE, O.STAGE_G2P]
    for st in stages:
        ia, ib = a.stage(st, dt), b.stage(st, dt)
        assert ia == ib
        for f in (O.F_FLAGS, O.F_AVGPNUM, O.F_VX, O.F_VY, O.F_VZ, O.F_V2X, O.F_V2Y, O.F_V2Z):
            assert np.array_equal(a.grid(f), b.grid(f)), (st, f)
        pa, pb = a.particles(), b.particles()
        for x, y in zip(pa, pb):
            assert np.array_equal(x, y), st
        if st == O.STAGE_SOLVE:
            pr_a, pr_b = a.grid(O.F_PRESSURE), b.grid(O.F_PRESSURE)
            m = ~np.isnan(pr_a)
            assert np.allclose(pr_a[m], pr_b[m], rtol=0, atol=1e-9 * np.abs(pr_b).max())


@pytest.mark.skipif(not O.have_ref(), reason="reference library not built here")
@pytest.mark.parametrize("pressure_enabled", [False, True])
def test_sor_oracle_equals_reference(port_lib, pressure_enabled):
    """BasicMacGrid's SOR: the oracle equals the reference's own solver bit for bit."""
    from fluid_simulator_gb300.scenes import GridSpec, dam_break

    pos = dam_break(GridSpec(32), (0, 0, 0), (0.5, 0.7, 1.0), seed=7).astype(np.float64)
    p = O.make_params(32, transfer=O.FLIP, max_iters=25, grid_solver=1, pressure_enabled=pressure_enabled)
    a = O.Oracle(p, pos, lib="ref")
    b = O.Oracle(p, pos, lib="port")
    dt = 1 / 120
    for _ in range(3):
        assert a.step(dt) == b.step(dt) == 25
    for st in (O.STAGE_ADVECT, O.STAGE_PUSH_OUT, O.STAGE_P2G, O.STAGE_MARK, O.STAGE_OBSTACLES, O.STAGE_WALLS,
               O.STAGE_POST_P2G, O.STAGE_SOLVE):
        assert a.stage(st, dt) == b.stage(st, dt)
    for f in (O.F_FLAGS, O.F_V2X, O.F_V2Y, O.F_V2Z):
        assert np.array_equal(a.grid(f), b.grid(f)), f
    for x, y in zip(a.particles(), b.particles()):
        assert np.array_equal(x, y)


def test_oracle_threads_agree_within_rounding(port_lib):
    """Multi-threaded oracle (timed CPU baseline) differs only by summation order."""
    from fluid_simulator_gb300.scenes import GridSpec, dam_break

    pos = dam_break(GridSpec(32), seed=0).astype(np.float64)
    p = O.make_params(32, transfer=O.FLIP)
    a = O.Oracle(p, pos, lib="port")
    a.set_threads(1)
    b = O.Oracle(p, pos, lib="port")
    b.set_threads(4)
    for _ in range(3):
        a.step(1 / 120)
        a.set_threads(1)
        b.set_threads(4)
        b.step(1 / 120)
    va, vb = a.particles()[1], b.particles()[1]
    assert np.abs(va - vb).max() <= 1e-9 * max(1.0, np.abs(va).max())
    a.set_threads(1)
