"""2D mode and non-cubic grids against the oracle.

2D mode is the reference's `twoD` grid (macGrid.cpp:9-13): the z axis is three
cells of targetDimensions.z / 3 (not the x / y cell size), every particle sits
on the plane z = targetDimensions.z / 2 (HashedParticles' zConst), advection
keeps no radius margin on z (simulator.cpp:140), push-out puts particles back
on the plane and never pushes along z (simulator.cpp:276-290), and G2P sets
v.z = 0 and leaves the z row of C alone (simulator.cpp:382-385).  The oracle's
2D mode is pinned to the reference by the dam2d32_flip / obs2d32_apic golden
digests, its non-cubic grids by box32x24x16_flip.
"""
import numpy as np
import pytest

from fluid_simulator_gb300 import native as N
from fluid_simulator_gb300.scenes import GridSpec, dam_break, dam_break_2d
from oracle import oracle as O

from parity_util import (REL_GRID, REL_PARTICLE, REL_PRESSURE, assert_close_field, inject_grid_from_oracle, make_pair,
                         sync_oracle_particles_from_gpu)

DT = 1.0 / 120.0
DIMS2D = (1.0, 1.0, 0.3)  # 32 x 32 x 3 cells at resolution 32, cellD.z = 0.1
TO = {N.PIC: O.PIC, N.FLIP: O.FLIP, N.APIC: O.APIC}


def test_2d_scene_on_plane():
    grid = GridSpec(32, DIMS2D, True)
    assert grid.shape == (32, 32, 3)
    assert abs(grid.hz - 0.1) < 1e-15
    pos = dam_break_2d(grid, (0, 0), (0.4, 0.6), seed=0)
    assert pos.shape == (12 * 18 * 4, 3)
    assert np.all(pos[:, 2] == np.float32(0.15))
    cells = np.floor(pos[:, :2].astype(np.float64) / grid.h).astype(int)
    assert cells.min() >= 1 and cells[:, 0].max() <= 12 and cells[:, 1].max() <= 18


def moving_state_2d(transfer, seed=0, steps=3, hi=(0.5, 0.6)):
    grid = GridSpec(32, DIMS2D, True)
    pos = dam_break_2d(grid, (0, 0), hi, seed=seed)
    o = O.Oracle(O.make_params(32, transfer=TO[transfer], dims=DIMS2D, two_d=True), pos.astype(np.float64),
                 lib="port")
    for _ in range(steps):
        o.step(DT)
    p, v, c = o.particles()
    return p.astype(np.float32), v.astype(np.float32), c.astype(np.float32)


@pytest.mark.gpu
def test_2d_grid_geometry(gpu):
    s = N.Simulation(32, N.default_params(resolution=32), dims=DIMS2D, two_d=True)
    assert s.shape == (32, 32, 3)
    assert s.h == 1 / 32 and abs(s.hz - 0.1) < 1e-15
    assert s.dims[2] == 0.3
    fl = s.grid(N.F_FLAGS)
    # z = 0 and z = 2 are the container walls; the interior is the z = 1 layer
    assert np.all(fl[:, :, 0] == N.SOLID) and np.all(fl[:, :, 2] == N.SOLID)
    assert np.all(fl[1:-1, 1:-1, 1] != N.SOLID)
    s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("transfer", [N.PIC, N.FLIP, N.APIC])
def test_2d_p2g_marks_bitexact_and_velocities(gpu, port_lib, transfer):
    pos, vel, c = moving_state_2d(transfer)
    g, o = make_pair(pos, 32, transfer, vel=vel, c=c, threads=4, dims=DIMS2D, two_d=True)
    g.stage(N.STAGE_P2G, DT)
    o.stage(O.STAGE_P2G, DT)
    o.stage(O.STAGE_MARK, DT)
    assert np.array_equal(g.grid(N.F_FLAGS), o.grid(O.F_FLAGS))
    for fg, fo, name in ((N.F_VX, O.F_VX, "vx"), (N.F_VY, O.F_VY, "vy"), (N.F_VZ, O.F_VZ, "vz"),
                         (N.F_AVGPNUM, O.F_AVGPNUM, "avgPNum")):
        assert_close_field(g.grid(fg), o.grid(fo), REL_GRID, name)


@pytest.mark.gpu
@pytest.mark.parametrize("transfer", [N.PIC, N.FLIP, N.APIC])
def test_2d_g2p_zero_vz_and_c_row(gpu, port_lib, transfer):
    pos, vel, c = moving_state_2d(transfer)
    c = c.reshape(-1, 9).copy()
    c[:, 6:9] = np.linspace(-1, 1, 3 * c.shape[0], dtype=np.float32).reshape(-1, 3)  # must survive G2P
    g, o = make_pair(pos, 32, transfer, vel=vel, c=c, threads=4, dims=DIMS2D, two_d=True)
    for st in (O.STAGE_P2G, O.STAGE_MARK, O.STAGE_OBSTACLES, O.STAGE_WALLS, O.STAGE_POST_P2G, O.STAGE_SOLVE,
               O.STAGE_EXTRAPOLATE):
        o.stage(st, DT)
    g.stage(N.STAGE_P2G, DT)
    inject_grid_from_oracle(g, o, [N.F_FLAGS, N.F_VX, N.F_VY, N.F_VZ, N.F_V2X, N.F_V2Y, N.F_V2Z])
    g.stage(N.STAGE_G2P, DT)
    o.stage(O.STAGE_G2P, DT)
    gp, gv, gc = g.particles()
    op, ov, oc = o.particles()
    assert np.array_equal(gp.astype(np.float64), op)
    assert np.all(gv[:, 2] == 0.0)
    assert_close_field(gv, ov, REL_PARTICLE, "particle v")
    if transfer == N.APIC:
        gc = gc.reshape(-1, 9)
        oc = oc.reshape(-1, 9)
        assert np.array_equal(gc[:, 6:9], oc[:, 6:9].astype(np.float32))
        assert_close_field(gc[:, :6], oc[:, :6], REL_PARTICLE * 10, "APIC C")


def obstacles_2d(mod, t, dt, z):
    sx = 0.55 + 0.1 * np.sin(np.pi * t * 4)
    sxp = 0.55 + 0.1 * np.sin(np.pi * (t - dt) * 4)
    return [mod.obstacle(mod.OBS_SPHERE, (sx, 0.3, z), r=0.12, prev_pos=(sxp, 0.3, z), speed=((sx - sxp) / dt, 0, 0)),
            mod.obstacle(mod.OBS_BOX, (0.3, 0.15, z), size=(0.1, 0.2, 4 * z), speed=(0, 0.5, 0)),
            mod.obstacle(mod.OBS_SINK, (0.1, 0.1, z), r=0.08)]


@pytest.mark.gpu
@pytest.mark.parametrize("transfer,obstacles", [(N.PIC, False), (N.FLIP, False), (N.APIC, False), (N.FLIP, True),
                                                (N.APIC, True)])
def test_2d_full_steps_one_step_error(gpu, port_lib, transfer, obstacles):
    """Each step starts both sides from the same FP32 state; particles stay on the plane."""
    grid = GridSpec(32, DIMS2D, True)
    pos = dam_break_2d(grid, (0, 0), (0.5, 0.7) if obstacles else (0.4, 0.6), seed=3 if obstacles else 0)
    g, o = make_pair(pos, 32, transfer, threads=4, tol=1e-9, gpu_tol=1e-9, max_iters=1000, dims=DIMS2D,
                     two_d=True, despawning=obstacles)
    zc = np.float32(DIMS2D[2] / 2)
    for s in range(6):
        if obstacles:
            o.set_obstacles(obstacles_2d(O, s * DT, DT, DIMS2D[2] / 2))
            g.set_obstacles(obstacles_2d(N, s * DT, DT, DIMS2D[2] / 2))
        sync_oracle_particles_from_gpu(g, o)
        g.step(DT)
        o.step(DT)
        assert np.array_equal(g.grid(N.F_FLAGS), o.grid(O.F_FLAGS)), f"step {s}: marks"
        gp, gv, _ = g.particles()
        op, ov, _ = o.particles()
        assert gp.shape == op.shape, f"step {s}: particle count"
        assert np.all(gp[:, 2] == zc) and np.all(gv[:, 2] == 0.0)
        dv = np.abs(gv - ov).max() / max(1e-6, np.abs(ov).max())
        dp = np.abs(gp - op).max() / g.h
        assert dp < 1e-3, f"step {s}: position error {dp} cells"
        assert dv < 1e-3, f"step {s}: velocity error {dv}"


@pytest.mark.gpu
def test_2d_push_out_matches_oracle(gpu, port_lib):
    grid = GridSpec(32, DIMS2D, True)
    pos = dam_break_2d(grid, (0, 0), (0.6, 0.7), seed=5)
    g, o = make_pair(pos, 32, N.FLIP, threads=4, dims=DIMS2D, two_d=True)
    z = DIMS2D[2] / 2
    o.set_obstacles([O.obstacle(O.OBS_SPHERE, (0.3, 0.3, z), r=0.1), O.obstacle(O.OBS_BOX, (0.45, 0.5, z),
                                                                                  size=(0.1, 0.12, 4 * z))])
    g.set_obstacles([N.obstacle(N.OBS_SPHERE, (0.3, 0.3, z), r=0.1), N.obstacle(N.OBS_BOX, (0.45, 0.5, z),
                                                                                  size=(0.1, 0.12, 4 * z))])
    g.stage(N.STAGE_PUSH_OUT, DT)
    o.stage(O.STAGE_PUSH_OUT, DT)
    gp, _, _ = g.particles()
    op, _, _ = o.particles()
    assert np.abs(gp.astype(np.float64) - pos).max() > 0.01  # the obstacles did push
    assert np.abs(gp.astype(np.float64) - op).max() < 1e-5
    assert np.all(gp[:, 2] == np.float32(z))


@pytest.mark.gpu
def test_2d_push_apart_matches_oracle(gpu, port_lib):
    grid = GridSpec(32, DIMS2D, True)
    pos = dam_break_2d(grid, (0, 0), (0.4, 0.6), seed=2)
    g, o = make_pair(pos, 32, N.FLIP, threads=4, dims=DIMS2D, two_d=True, push_apart=True)
    g.stage(N.STAGE_PUSH_APART, DT)
    o.stage(O.STAGE_PUSH_APART, DT)
    gp, _, _ = g.particles()
    op, _, _ = o.particles()
    assert np.abs(gp.astype(np.float64) - pos).max() > 1e-4
    assert np.abs(gp.astype(np.float64) - op).max() < 1e-5
    assert np.all(gp[:, 2] == np.float32(DIMS2D[2] / 2))


@pytest.mark.gpu
@pytest.mark.parametrize("transfer", [N.FLIP, N.APIC])
def test_noncubic_grid_full_steps(gpu, port_lib, transfer):
    """A 32 x 24 x 16 grid: every padded / partial tile and multigrid level of odd size."""
    dims = (1.0, 0.75, 0.5)
    grid = GridSpec(32, dims)
    assert grid.shape == (32, 24, 16)
    pos = dam_break(grid, (0, 0, 0), (0.5, 0.5, 0.5), seed=1)
    g, o = make_pair(pos, 32, transfer, threads=4, tol=1e-9, gpu_tol=1e-9, max_iters=1000, dims=dims)
    assert g.shape == (32, 24, 16)
    for s in range(4):
        sync_oracle_particles_from_gpu(g, o)
        g.step(DT)
        o.step(DT)
        assert np.array_equal(g.grid(N.F_FLAGS), o.grid(O.F_FLAGS))
        gp, gv, _ = g.particles()
        op, ov, _ = o.particles()
        dv = np.abs(gv - ov).max() / max(1e-6, np.abs(ov).max())
        dp = np.abs(gp - op).max() / g.h
        assert dp < 1e-3 and dv < 1e-3, (s, dp, dv)


def _pressure_pair(pos, res, dims, two_d, precond):
    g, o = make_pair(pos, res, N.FLIP, threads=4, tol=1e-11, max_iters=3000, gpu_tol=1e-11,
                     gpu_tol_mode=N.TOL_ABS_MAX, precond=precond, dims=dims, two_d=two_d)
    g.stage(N.STAGE_P2G, DT)
    for st in (O.STAGE_P2G, O.STAGE_MARK, O.STAGE_OBSTACLES, O.STAGE_WALLS, O.STAGE_POST_P2G):
        o.stage(st, DT)
    inject_grid_from_oracle(g, o, [N.F_FLAGS, N.F_VX, N.F_VY, N.F_VZ, N.F_V2X, N.F_V2Y, N.F_V2Z])
    o.set_grid(O.F_FLAGS, o.grid(O.F_FLAGS))
    st = g.stage(N.STAGE_SOLVE, DT)
    its = o.stage(O.STAGE_SOLVE, DT)
    assert its < 3000 and st.converged == 1
    assert_close_field(g.grid(N.F_PRESSURE), o.grid(O.F_PRESSURE), REL_PRESSURE, "pressure")
    for fg, fo in ((N.F_V2X, O.F_V2X), (N.F_V2Y, O.F_V2Y), (N.F_V2Z, O.F_V2Z)):
        assert_close_field(g.grid(fg), o.grid(fo), REL_GRID * 10, f"v2 after projection {fg}")
    return st.pcg_iterations, its


@pytest.mark.gpu
@pytest.mark.parametrize("precond", [N.PRECOND_MG, N.PRECOND_RBIC])
def test_odd_grid_pressure_matches_oracle(gpu, port_lib, precond):
    """Resolution 20 on (2, 1.25, 1): a 40 x 25 x 20 grid (the shape of the reference GUI's 3D box)
    whose multigrid levels are 20 x 13 x 10, 10 x 7 x 5, 5 x 4 x 3."""
    dims = (2.0, 1.25, 1.0)
    grid = GridSpec(20, dims)
    assert grid.shape == (40, 25, 20)
    pos = dam_break(grid, (0, 0, 0), (0.8, 0.8, 1.0), seed=4)
    print("PCG iterations (GPU, oracle)", _pressure_pair(pos, 20, dims, False, precond))


@pytest.mark.gpu
@pytest.mark.parametrize("precond", [N.PRECOND_MG, N.PRECOND_RBIC])
def test_2d_pressure_matches_oracle(gpu, port_lib, precond):
    pos, _, _ = moving_state_2d(N.FLIP)
    print("PCG iterations (GPU, oracle)", _pressure_pair(pos, 32, DIMS2D, True, precond))
