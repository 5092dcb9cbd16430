"""The reference-shaped C++ facade (include/fsim_facade.hpp).

The demo program tests/facade/facade_demo.cpp drives the library the way the
reference's SimulationManager drives Simulator / BridsonSolverGrid /
HashedParticles.  It must compile against the facade (CPU test) and, on a GPU,
give the same particles as the same run through the C ABI from Python.
"""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DEMO = os.path.join(ROOT, "tests", "facade", "facade_demo.cpp")
GLM = os.path.join(ROOT, "oracle", "glmshim")  # vector-math header used to compile tests only
INC = os.path.join(ROOT, "include")
LIBDIR = os.path.join(ROOT, "fluid_simulator_gb300")


def test_reference_manager_compiles_against_facade(tmp_path):
    """The reference's own SimulationManager (src/Simulator/manager), byte for
    byte, compiles against the facade: its two files are placed unmodified in a
    scratch tree whose simulator headers (simulator.h, basicMacGrid.h,
    bridsonSolverGrid.h, hashedParticles.h -- the four simulationManager.h
    includes -- and util/interpolation.h, which the .cpp includes) each forward
    to include/fsim_facade.hpp.  Needs the reference checkout (CPU only)."""
    import shutil

    from oracle import oracle as O

    ref = O.reference_dir()
    if ref is None:
        pytest.skip("reference checkout not present")
    mgr = os.path.join(ref, "src", "Simulator", "manager")
    (tmp_path / "manager").mkdir()
    for f in ("simulationManager.h", "simulationManager.cpp"):
        shutil.copyfile(os.path.join(mgr, f), tmp_path / "manager" / f)
        assert (tmp_path / "manager" / f).read_bytes() == open(os.path.join(mgr, f), "rb").read()
    for shim in ("simulator/simulator.h", "simulator/macGrid/basicMacGrid.h", "simulator/macGrid/bridsonSolverGrid.h",
                 "simulator/particles/hashedParticles.h", "simulator/util/interpolation.h"):
        path = tmp_path / shim
        path.parent.mkdir(parents=True, exist_ok=True)
        path.write_text('#pragma once\n#include "fsim_facade.hpp"\n')
    r = subprocess.run(["g++", "-std=c++20", "-fsyntax-only", f"-I{GLM}", f"-I{INC}",
                        str(tmp_path / "manager" / "simulationManager.cpp")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_facade_compiles():
    r = subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-fsyntax-only", f"-I{GLM}",
                        f"-I{INC}", DEMO], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("transfer,mode", [(1, ""), (2, ""), (1, "basic"), (2, "2d")])
def test_facade_matches_c_abi(gpu, tmp_path, transfer, mode):
    from fluid_simulator_gb300 import native as N
    from fluid_simulator_gb300.scenes import GridSpec, dam_break, dam_break_2d

    exe = tmp_path / "facade_demo"
    r = subprocess.run(["g++", "-std=c++17", "-O2", f"-I{GLM}", f"-I{INC}", DEMO, "-o", str(exe), f"-L{LIBDIR}",
                        "-lfsim", f"-Wl,-rpath,{LIBDIR}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    res, steps, dt = 32, 6, 1.0 / 120.0
    basic, two_d = mode == "basic", mode == "2d"
    dims = (1.0, 1.0, 0.3) if two_d else (1.0, 1.0, 1.0)
    zc = dims[2] / 2 if two_d else 0.5
    grid = GridSpec(res, dims, two_d)
    pos = dam_break_2d(grid, seed=3) if two_d else dam_break(grid, seed=3)
    inp = tmp_path / "pos.bin"
    out = tmp_path / "out.bin"
    pos.astype(np.float32).tofile(inp)
    r = subprocess.run([str(exe), str(res), str(steps), repr(dt), str(transfer), str(inp), str(out)] +
                       ([mode] if mode else []), capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr + r.stdout
    raw = out.read_bytes()
    n = int(np.frombuffer(raw[:8], np.int64)[0])
    body = np.frombuffer(raw[8:8 + 4 * 15 * n], np.float32)
    fp, fv, fc = body[:3 * n].reshape(n, 3), body[3 * n:6 * n].reshape(n, 3), body[6 * n:].reshape(n, 9)
    its = int(np.frombuffer(raw[8 + 4 * 15 * n:8 + 4 * 15 * n + 4], np.int32)[0])
    fdens = np.frombuffer(raw[8 + 4 * 15 * n + 4:], np.float32)
    assert fdens.shape == (n,)

    h = 1.0 / res
    p = N.default_params(transfer=transfer, resolution=res, flip_ratio=0.95, gravity=-9.81, max_iters=200,
                         tol=1e-6, tol_mode=N.TOL_ABS_MAX, precision=N.PREC_MIXED, warm_start=N.WARM_ZERO,
                         top_solid=True, particle_r=h / 4, pressure_enabled=False, timing=True,
                         precond=N.PRECOND_MG, grid_solver=N.SOLVER_SOR if basic else N.SOLVER_PCG)
    sim = N.Simulation(res, p, dims=dims, two_d=two_d)
    sim.set_particles(pos)
    st = None
    for s in range(steps):
        x = 0.6 + 0.01 * s
        xp = 0.6 + 0.01 * (s - 1) if s > 0 else 0.6
        sim.set_obstacles([N.obstacle(N.OBS_SPHERE, (x, 0.3, zc), r=0.15, prev_pos=(xp, 0.3, zc),
                                      speed=((x - xp) / dt, 0.0, 0.0))])
        st = sim.step(dt)
    gp, gv, gc = sim.particles()
    gdens = sim.gfx()[:, 4]
    sim.close()
    # Same inputs, same library: the runs agree up to the order of particles
    # inside a cell (ranks come from atomics) and the differences summation
    # order makes in P2G, which the flow then amplifies.  A plumbing error (a
    # parameter or obstacle passed differently) shows up as O(h) differences.
    assert n == gp.shape[0]
    assert abs(its - st.pcg_iterations) <= 1

    # pair every facade particle with the nearest C-ABI particle
    spatial = pytest.importorskip("scipy.spatial")
    dist, idx = spatial.cKDTree(gp.astype(np.float64)).query(fp.astype(np.float64))
    assert dist.max() <= 1e-4  # h = 1/32
    assert np.unique(idx).size == n
    vs = max(np.abs(gv).max(), 1e-6)
    assert np.abs(fv - gv[idx]).max() <= 1e-2 * vs
    cs = max(np.abs(gc).max(), 1e-6)
    assert np.abs(fc - gc.reshape(-1, 9)[idx]).max() <= 5e-2 * cs
    # the manager's host-side density (getCellsAround + trilinearInterpoll over
    # the grid mirror) against the library's device gfx publish
    ds = max(np.abs(gdens).max(), 1e-6)
    assert np.abs(fdens - gdens[idx]).max() <= 1e-2 * ds
