"""Parity of the CUDA step against the oracle (the reference's algorithm in
FP64), stage by stage and over whole steps, through the C ABI.  Tolerances are
the constants of parity_util."""
import numpy as np
import pytest

from fluid_simulator_gb300 import native as N
from fluid_simulator_gb300.scenes import GridSpec, dam_break
from oracle import oracle as O

from parity_util import (REL_GRID, REL_PARTICLE, REL_PRESSURE, assert_close_field, inject_grid_from_oracle,
                         make_pair, ref_counts, sync_oracle_particles_from_gpu)

pytestmark = pytest.mark.gpu

DT32 = 1.0 / 120.0


def moving_state(res=32, transfer=N.FLIP, seed=0, steps=3, block_hi=(0.4, 0.6, 1.0)):
    """Particles after a few oracle steps, so velocities, C and positions are generic."""
    grid = GridSpec(res)
    pos = dam_break(grid, (0, 0, 0), block_hi, seed=seed)
    o = O.Oracle(O.make_params(res, transfer={N.PIC: O.PIC, N.FLIP: O.FLIP, N.APIC: O.APIC}[transfer]),
                 pos.astype(np.float64), lib="port")
    for _ in range(steps):
        o.step(1.0 / (4 * res))
    p, v, c = o.particles()
    return p.astype(np.float32), v.astype(np.float32), c.astype(np.float32)


@pytest.mark.parametrize("transfer", [N.PIC, N.FLIP, N.APIC])
def test_p2g_marks_counts_bitexact_and_velocities(gpu, port_lib, transfer):
    pos, vel, c = moving_state(32, transfer)
    g, o = make_pair(pos, 32, transfer, vel=vel, c=c, threads=4)
    g.stage(N.STAGE_P2G, DT32)
    o.stage(O.STAGE_P2G, DT32)
    o.stage(O.STAGE_MARK, DT32)
    assert np.array_equal(g.grid(N.F_FLAGS), o.grid(O.F_FLAGS))
    assert np.array_equal(g.grid(N.F_COUNT), ref_counts(pos, g.shape, g.h))
    for fg, fo, name in ((N.F_VX, O.F_VX, "vx"), (N.F_VY, O.F_VY, "vy"), (N.F_VZ, O.F_VZ, "vz"),
                         (N.F_AVGPNUM, O.F_AVGPNUM, "avgPNum")):
        assert_close_field(g.grid(fg), o.grid(fo), REL_GRID, name)


def test_first_step_stages_chained(gpu, port_lib):
    """Dam break from rest: advect is the identity, then every grid stage."""
    grid = GridSpec(32)
    pos = dam_break(grid, seed=0)
    g, o = make_pair(pos, 32, N.FLIP, threads=4)
    for st in (N.STAGE_ADVECT, N.STAGE_PUSH_OUT, N.STAGE_P2G):
        g.stage(st, DT32)
    for st in (O.STAGE_ADVECT, O.STAGE_PUSH_OUT):
        o.stage(st, DT32)
    # the clamp band h + 1.01 r is an FP32 constant on the GPU: positions agree to FP32 rounding
    gp, _, _ = g.particles()
    op, _, _ = o.particles()
    assert np.abs(gp.astype(np.float64) - op).max() <= 2e-7
    # continue from identical positions
    sync_oracle_particles_from_gpu(g, o)
    o.stage(O.STAGE_P2G, DT32)
    o.stage(O.STAGE_MARK, DT32)
    for st_g, st_o in ((N.STAGE_OBSTACLES, O.STAGE_OBSTACLES), (N.STAGE_WALLS, O.STAGE_WALLS),
                       (N.STAGE_POST_P2G, O.STAGE_POST_P2G)):
        g.stage(st_g, DT32)
        o.stage(st_o, DT32)
    assert np.array_equal(g.grid(N.F_FLAGS), o.grid(O.F_FLAGS))
    for fg, fo in ((N.F_VX, O.F_VX), (N.F_VY, O.F_VY), (N.F_VZ, O.F_VZ), (N.F_V2X, O.F_V2X),
                   (N.F_V2Y, O.F_V2Y), (N.F_V2Z, O.F_V2Z)):
        assert_close_field(g.grid(fg), o.grid(fo), REL_GRID, f"field {fg}")


@pytest.mark.parametrize("precision,precond", [(N.PREC_MIXED, N.PRECOND_MG), (N.PREC_MIXED, N.PRECOND_RBIC),
                                              (N.PREC_FP64, N.PRECOND_RBIC)])
def test_pressure_matches_oracle(gpu, port_lib, precision, precond):
    """Same flags and v2 on both sides; both solve to a tight tolerance."""
    pos, vel, c = moving_state(32, N.FLIP)
    g, o = make_pair(pos, 32, N.FLIP, vel=vel, threads=4, tol=1e-11, max_iters=2000,
                     gpu_tol=1e-11, gpu_tol_mode=N.TOL_ABS_MAX, precision=precision, precond=precond)
    g.stage(N.STAGE_P2G, DT32)
    for st in (O.STAGE_P2G, O.STAGE_MARK, O.STAGE_OBSTACLES, O.STAGE_WALLS, O.STAGE_POST_P2G):
        o.stage(st, DT32)
    inject_grid_from_oracle(g, o, [N.F_FLAGS, N.F_VX, N.F_VY, N.F_VZ, N.F_V2X, N.F_V2Y, N.F_V2Z])
    # the oracle's fluid list follows its flags; re-set to rebuild it identically
    o.set_grid(O.F_FLAGS, o.grid(O.F_FLAGS))
    st = g.stage(N.STAGE_SOLVE, DT32)
    its = o.stage(O.STAGE_SOLVE, DT32)
    assert its < 2000
    assert st.converged == 1
    assert_close_field(g.grid(N.F_PRESSURE), o.grid(O.F_PRESSURE), REL_PRESSURE, "pressure")
    for fg, fo in ((N.F_V2X, O.F_V2X), (N.F_V2Y, O.F_V2Y), (N.F_V2Z, O.F_V2Z)):
        assert_close_field(g.grid(fg), o.grid(fo), REL_GRID * 10, f"v2 after projection {fg}")


@pytest.mark.parametrize("res,band", [(64, 3), (96, 3), (64, -1)])
def test_multigrid_pressure_matches_oracle_on_slab_levels(gpu, port_lib, res, band):
    """The multigrid path whose 32^3 (64^3 grid) or 24^3 (96^3 grid) level runs
    as x slabs in the cluster's distributed shared memory (at 96^3 some CTAs
    hold no plane), against the oracle's MIC(0) PCG on identical flags and v2,
    both solved to 1e-11 absolute max-norm; with three free-surface band sweeps
    on the finest level (the default from 2^23 cells on, forced here) and
    without them (band -1, the default at these sizes)."""
    pos, vel, c = moving_state(res, N.FLIP, steps=2)
    g, o = make_pair(pos, res, N.FLIP, vel=vel, threads=8, tol=1e-11, max_iters=4000, gpu_tol=1e-11,
                     gpu_tol_mode=N.TOL_ABS_MAX, precision=N.PREC_MIXED, precond=N.PRECOND_MG,
                     mg_boundary_sweeps=band)
    dt = 1.0 / (4 * res)
    g.stage(N.STAGE_P2G, dt)
    for st in (O.STAGE_P2G, O.STAGE_MARK, O.STAGE_OBSTACLES, O.STAGE_WALLS, O.STAGE_POST_P2G):
        o.stage(st, dt)
    inject_grid_from_oracle(g, o, [N.F_FLAGS, N.F_VX, N.F_VY, N.F_VZ, N.F_V2X, N.F_V2Y, N.F_V2Z])
    o.set_grid(O.F_FLAGS, o.grid(O.F_FLAGS))
    st = g.stage(N.STAGE_SOLVE, dt)
    its = o.stage(O.STAGE_SOLVE, dt)
    assert its < 4000 and st.converged == 1
    assert_close_field(g.grid(N.F_PRESSURE), o.grid(O.F_PRESSURE), REL_PRESSURE, f"{res}^3 multigrid pressure")


@pytest.mark.parametrize("pressure_enabled", [False, True])
def test_sor_matches_oracle(gpu, port_lib, pressure_enabled):
    """BasicMacGrid's SOR (FSIM_SOLVER_SOR) from identical flags, v2 and densities."""
    pos, vel, c = moving_state(32, N.FLIP)
    g, o = make_pair(pos, 32, N.FLIP, vel=vel, threads=4, max_iters=30, grid_solver=N.SOLVER_SOR,
                     pressure_enabled=pressure_enabled)
    g.stage(N.STAGE_P2G, DT32)
    for st in (O.STAGE_P2G, O.STAGE_MARK, O.STAGE_OBSTACLES, O.STAGE_WALLS, O.STAGE_POST_P2G):
        o.stage(st, DT32)
    inject_grid_from_oracle(g, o, [N.F_FLAGS, N.F_AVGPNUM, N.F_V2X, N.F_V2Y, N.F_V2Z])
    st = g.stage(N.STAGE_SOLVE, DT32)
    assert st.pcg_iterations == 30 and o.stage(O.STAGE_SOLVE, DT32) == 30
    # FP32 against FP64 over 30 over-relaxed sweeps
    for fg, fo in ((N.F_V2X, O.F_V2X), (N.F_V2Y, O.F_V2Y), (N.F_V2Z, O.F_V2Z)):
        assert_close_field(g.grid(fg), o.grid(fo), 1e-4, f"v2 after SOR {fg}")


def test_push_apart_matches_oracle(gpu, port_lib):
    """One push-apart pass (Jacobi semantics) from identical, overlapping particles."""
    pos, vel, c = moving_state(32, N.FLIP)
    g, o = make_pair(pos, 32, N.FLIP, vel=vel, threads=4, push_apart=True)
    before = g.particles()[0]
    g.stage(N.STAGE_PUSH_APART, DT32)
    o.stage(O.STAGE_PUSH_APART, DT32)
    gp = g.particles()[0]
    op = o.particles()[0]
    moved = np.abs(gp - before).max(axis=1) > 0
    assert moved.mean() > 0.1  # the scene has overlapping pairs
    assert np.abs(gp - op).max() <= 2e-6


@pytest.mark.parametrize("transfer", [N.FLIP, N.APIC])
def test_full_step_with_push_apart(gpu, port_lib, transfer):
    """Whole steps with push-apart on both sides, one-step-error protocol."""
    pos = dam_break(GridSpec(32), seed=2)
    g, o = make_pair(pos, 32, transfer, threads=4, tol=1e-9, gpu_tol=1e-9, max_iters=1000, push_apart=True)
    for s in range(4):
        sync_oracle_particles_from_gpu(g, o)
        g.step(DT32)
        o.step(DT32)
        gp, gv, _ = g.particles()
        op, ov, _ = o.particles()
        assert gp.shape == op.shape
        dv = np.abs(gv - ov).max() / max(1e-6, np.abs(ov).max())
        dp = np.abs(gp - op).max() / g.h
        assert dp < 1e-3, f"step {s}: position error {dp} cells"
        assert dv < 1e-3, f"step {s}: velocity error {dv}"


@pytest.mark.parametrize("res", [32, 64, 96])
def test_multigrid_needs_far_fewer_iterations(gpu, port_lib, res):
    """Both preconditioners reach the same pressure; multigrid in far fewer
    iterations.  At 64^3 and 96^3 the 32^3 / 24^3 level runs as x slabs in the
    cluster's distributed shared memory (at 96^3 some CTAs hold no plane)."""
    pos, vel, c = moving_state(res, N.FLIP)
    result = {}
    for precond in (N.PRECOND_RBIC, N.PRECOND_MG):
        g, o = make_pair(pos, res, N.FLIP, vel=vel, gpu_tol=1e-8, gpu_tol_mode=N.TOL_REL_L2, gpu_max_iters=3000,
                         precond=precond)
        g.stage(N.STAGE_P2G, DT32)
        for st in (N.STAGE_OBSTACLES, N.STAGE_WALLS, N.STAGE_POST_P2G):
            g.stage(st, DT32)
        stats = g.stage(N.STAGE_SOLVE, DT32)
        assert stats.converged == 1
        result[precond] = (stats.pcg_iterations, g.grid(N.F_PRESSURE))
    assert result[N.PRECOND_MG][0] * 3 < result[N.PRECOND_RBIC][0]
    assert_close_field(result[N.PRECOND_MG][1], result[N.PRECOND_RBIC][1], 1e-5, "pressure MG vs RB-IC")


def test_extrapolation_matches_oracle(gpu, port_lib):
    pos, vel, c = moving_state(32, N.FLIP)
    g, o = make_pair(pos, 32, N.FLIP, vel=vel, threads=4)
    g.stage(N.STAGE_P2G, DT32)
    for st in (O.STAGE_P2G, O.STAGE_MARK, O.STAGE_OBSTACLES, O.STAGE_WALLS, O.STAGE_POST_P2G, O.STAGE_SOLVE):
        o.stage(st, DT32)
    inject_grid_from_oracle(g, o, [N.F_FLAGS, N.F_V2X, N.F_V2Y, N.F_V2Z])
    o.set_grid(O.F_FLAGS, o.grid(O.F_FLAGS))
    g.stage(N.STAGE_EXTRAPOLATE, DT32)
    o.stage(O.STAGE_EXTRAPOLATE, DT32)
    for fg, fo in ((N.F_V2X, O.F_V2X), (N.F_V2Y, O.F_V2Y), (N.F_V2Z, O.F_V2Z)):
        assert_close_field(g.grid(fg), o.grid(fo), REL_GRID, f"extrapolated {fg}")


@pytest.mark.parametrize("transfer", [N.PIC, N.FLIP, N.APIC])
def test_g2p_matches_oracle(gpu, port_lib, transfer):
    pos, vel, c = moving_state(32, transfer)
    g, o = make_pair(pos, 32, transfer, vel=vel, c=c, threads=4)
    for st in (O.STAGE_P2G, O.STAGE_MARK, O.STAGE_OBSTACLES, O.STAGE_WALLS, O.STAGE_POST_P2G, O.STAGE_SOLVE,
               O.STAGE_EXTRAPOLATE):
        o.stage(st, DT32)
    g.stage(N.STAGE_P2G, DT32)
    inject_grid_from_oracle(g, o, [N.F_FLAGS, N.F_VX, N.F_VY, N.F_VZ, N.F_V2X, N.F_V2Y, N.F_V2Z])
    g.stage(N.STAGE_G2P, DT32)
    o.stage(O.STAGE_G2P, DT32)
    gp, gv, gc = g.particles()
    op, ov, oc = o.particles()
    assert np.array_equal(gp.astype(np.float64), op)
    assert_close_field(gv, ov, REL_PARTICLE, "particle v")
    if transfer == N.APIC:
        assert_close_field(gc, oc, REL_PARTICLE * 10, "APIC C")


@pytest.mark.parametrize("transfer", [N.PIC, N.FLIP, N.APIC])
def test_full_steps_one_step_error(gpu, port_lib, transfer):
    """Each step starts both sides from the same FP32 state; compare after one step."""
    grid = GridSpec(32)
    pos = dam_break(grid, seed=1)
    g, o = make_pair(pos, 32, transfer, threads=4, tol=1e-9, gpu_tol=1e-9, max_iters=1000)
    worst = 0.0
    for s in range(6):
        sync_oracle_particles_from_gpu(g, o)
        g.step(DT32)
        o.step(DT32)
        assert np.array_equal(g.grid(N.F_FLAGS), o.grid(O.F_FLAGS))
        gp, gv, _ = g.particles()
        op, ov, _ = o.particles()
        assert gp.shape == op.shape
        dv = np.abs(gv - ov).max() / max(1e-6, np.abs(ov).max())
        dp = np.abs(gp - op).max() / g.h
        worst = max(worst, dv)
        assert dp < 1e-3, f"step {s}: position error {dp} cells"
        assert dv < 1e-3, f"step {s}: velocity error {dv}"
    print("worst one-step relative velocity error", worst)


def test_obstacles_sink_and_box_grid_bitexact(gpu, port_lib):
    grid = GridSpec(32)
    pos = dam_break(grid, (0, 0, 0), (0.5, 0.7, 1.0), seed=3)
    g, o = make_pair(pos, 32, N.FLIP, threads=4, despawning=True)
    obs_o = [O.obstacle(O.OBS_SPHERE, (0.55, 0.3, 0.5), r=0.12, speed=(0.7, 0, 0)),
             O.obstacle(O.OBS_BOX, (0.3, 0.15, 0.3), size=(0.1, 0.2, 0.15), speed=(0, 0, 0.5)),
             O.obstacle(O.OBS_SINK, (0.1, 0.1, 0.8), r=0.08)]
    obs_g = [N.obstacle(N.OBS_SPHERE, (0.55, 0.3, 0.5), r=0.12, speed=(0.7, 0, 0)),
             N.obstacle(N.OBS_BOX, (0.3, 0.15, 0.3), size=(0.1, 0.2, 0.15), speed=(0, 0, 0.5)),
             N.obstacle(N.OBS_SINK, (0.1, 0.1, 0.8), r=0.08)]
    o.set_obstacles(obs_o)
    g.set_obstacles(obs_g)
    # push-out and P2G from identical positions, then obstacle rasterisation
    g.stage(N.STAGE_PUSH_OUT, DT32)
    o.stage(O.STAGE_PUSH_OUT, DT32)
    gp, _, _ = g.particles()
    op, _, _ = o.particles()
    moved = np.abs(gp.astype(np.float64) - op).max()
    assert moved < 1e-5
    sync_oracle_particles_from_gpu(g, o)
    g.stage(N.STAGE_P2G, DT32)
    o.stage(O.STAGE_P2G, DT32)
    o.stage(O.STAGE_MARK, DT32)
    g.stage(N.STAGE_OBSTACLES, DT32)
    o.stage(O.STAGE_OBSTACLES, DT32)
    g.stage(N.STAGE_WALLS, DT32)
    o.stage(O.STAGE_WALLS, DT32)
    assert np.array_equal(g.grid(N.F_FLAGS), o.grid(O.F_FLAGS))
    for fg, fo in ((N.F_VX, O.F_VX), (N.F_VY, O.F_VY), (N.F_VZ, O.F_VZ)):
        assert_close_field(g.grid(fg), o.grid(fo), REL_GRID, f"obstacle faces {fg}")


def test_sink_despawn_counts(gpu, port_lib):
    grid = GridSpec(32)
    pos = dam_break(grid, (0, 0, 0), (0.5, 0.7, 1.0), seed=3)
    g, o = make_pair(pos, 32, N.FLIP, threads=4, despawning=True)
    o.set_obstacles([O.obstacle(O.OBS_SINK, (0.2, 0.2, 0.5), r=0.1)])
    g.set_obstacles([N.obstacle(N.OBS_SINK, (0.2, 0.2, 0.5), r=0.1)])
    g.stage(N.STAGE_ADVECT, DT32)
    o.stage(O.STAGE_ADVECT, DT32)
    assert g.n == o.n < pos.shape[0]
    gp, _, _ = g.particles()
    op, _, _ = o.particles()
    assert np.abs(gp.astype(np.float64) - op).max() <= 2e-7


@pytest.mark.parametrize("pinned", [False, True])
def test_gfx_publish_matches_particles_and_density(gpu, pinned):
    """ParticleGfxData (simulationManager.cpp:218-231): position, |v| and the
    trilinear interpolation of avgPNum at the particle, in device order."""
    import ctypes as C

    grid = GridSpec(32)
    pos = dam_break(grid, seed=2)
    sim = N.Simulation(32, N.default_params(transfer=N.FLIP, resolution=32))
    sim.set_particles(pos)
    sim.step(DT32)
    sim.step(DT32)
    n = sim.n
    arr = (N.ParticleGfx * n)()
    rt = None
    if pinned:
        for name in ("libcudart.so.13", "libcudart.so"):
            try:
                rt = C.CDLL(name)
                break
            except OSError:
                pass
        assert rt.cudaHostRegister(C.cast(arr, C.c_void_p), C.c_size_t(C.sizeof(arr)), 0) == 0
    got = C.c_int64()
    assert sim.lib.fsim_fill_gfx(sim.ctx, arr, n, C.byref(got), N.HOST) == 0
    if rt is not None:
        rt.cudaHostUnregister(C.cast(arr, C.c_void_p))
    gfx = np.frombuffer(arr, dtype=np.float32).reshape(n, 5)
    p, v, _ = sim.particles()
    avg = sim.grid(N.F_AVGPNUM).astype(np.float64)
    assert np.array_equal(gfx[:, :3], p)
    assert np.allclose(gfx[:, 3], np.linalg.norm(v.astype(np.float64), axis=1), rtol=1e-5, atol=1e-6)
    g = p.astype(np.float64) * 32 - 0.5
    b = np.floor(g).astype(int)
    dens = np.zeros(n)
    for ox in (0, 1):
        for oy in (0, 1):
            for oz in (0, 1):
                x, y, z = b[:, 0] + ox, b[:, 1] + oy, b[:, 2] + oz
                w = (1 - np.abs(g[:, 0] - x)) * (1 - np.abs(g[:, 1] - y)) * (1 - np.abs(g[:, 2] - z))
                dens += w * avg[x, y, z]
    assert np.allclose(gfx[:, 4], dens, rtol=1e-4, atol=1e-5)
    sim.close()


def test_async_gfx_handoff_equals_sync(gpu):
    """fsim_fill_gfx_async over consecutive steps (both staging slots reused)
    delivers exactly what fsim_fill_gfx gives for the same state."""
    import ctypes as C

    pos = dam_break(GridSpec(32), seed=4)
    sim = N.Simulation(32, N.default_params(transfer=N.APIC, resolution=32))
    sim.set_particles(pos)
    n = sim.n
    bufs = [(N.ParticleGfx * n)() for _ in range(3)]
    want = []
    for s in range(3):
        sim.step(DT32)
        want.append(sim.gfx())
        got = C.c_int64()
        assert sim.lib.fsim_fill_gfx_async(sim.ctx, bufs[s], n, C.byref(got)) == 0
        assert got.value == n
    assert sim.lib.fsim_gfx_wait(sim.ctx) == 0
    for s in range(3):
        arr = np.frombuffer(bufs[s], dtype=np.float32, count=5 * n).reshape(n, 5)
        assert np.array_equal(arr, want[s])
    sim.close()
