"""Failure detection at the C ABI: every call returns a status, errors carry a
message (fsim_last_error), and faults are injected on the host (bad arguments,
non-finite inputs, an iteration cap, calls out of order) -- never on the GPU.
The reference breaks out of PCG on a non-finite alpha / sigma and at its
iteration cap (bridsonSolverGrid.cpp:267-285); the library reports the first as
FSIM_E_NAN and the second, like the reference, as a finished step whose stats
say not converged."""
import ctypes as C

import numpy as np
import pytest

from fluid_simulator_gb300 import native as N
from fluid_simulator_gb300.scenes import GridSpec, dam_break


def _create(lib, res=32.0, two_d=0, dims=(1.0, 1.0, 1.0), **kw):
    g = N.GridDesc()
    g.dims[:] = list(dims)
    g.resolution = res
    g.two_d = two_d
    p = N.default_params(resolution=res if res > 0 else 32, **kw)
    ctx = C.c_void_p()
    return lib.fsim_create(C.byref(g), C.byref(p), C.byref(ctx)), ctx


# ---- argument validation (returns before any GPU work) ----------------------
def test_create_rejects_bad_grid_and_params():
    lib = N.load_library()
    assert _create(lib, res=0.0)[0] == -1
    assert _create(lib, dims=(1.0, -1.0, 1.0))[0] == -1
    assert _create(lib, res=2.0)[0] == -1          # fewer than 3 cells per axis
    assert _create(lib, res=1.0, dims=(2048.0, 2048.0, 1024.0))[0] == -1  # 2^32 cells
    assert _create(lib, transfer=7)[0] == -1        # no such P2G2PType
    assert _create(lib, tol_mode=9)[0] == -1
    assert _create(lib, fluid_density=0.0)[0] == -1
    assert lib.fsim_create(None, None, None) == -1


def test_null_context_calls_fail_cleanly():
    lib = N.load_library()
    st = N.StepStats()
    assert lib.fsim_step(None, 0.01, C.byref(st)) == -1
    assert lib.fsim_destroy(None) == 0
    assert lib.fsim_gfx_wait(None) == -1
    r = C.c_void_p()
    assert lib.fsim_render_create(0, 10, C.byref(r)) == -1


# ---- host-side fault injection on a running context -------------------------
def _sim(**kw):
    grid = GridSpec(32)
    pos = dam_break(grid, seed=0)
    p = N.default_params(transfer=N.FLIP, resolution=32, **kw)
    s = N.Simulation(32, p)
    s.set_particles(pos)
    return s, pos


def _code(exc):
    return str(exc.value)


@pytest.mark.gpu
def test_non_finite_grid_velocity_reports_nan_and_recovers(gpu):
    """A NaN face velocity before the pressure solve: the solver stops on the
    non-finite scalar (FSIM_E_NAN) and the context keeps working -- the next
    solve does not read the NaN Krylov vectors the failed one left behind."""
    s, pos = _sim()
    dt = 1 / 120
    for st in (N.STAGE_P2G, N.STAGE_OBSTACLES, N.STAGE_WALLS, N.STAGE_POST_P2G):
        s.stage(st, dt)
    v2 = s.grid(N.F_V2Y)
    fl = s.grid(N.F_FLAGS)
    x, y, z = np.argwhere(fl == N.WATER)[100]
    v2[x, y, z] = np.nan
    s.set_grid(N.F_V2Y, v2)
    with pytest.raises(N.FsimError) as e:
        s.stage(N.STAGE_SOLVE, dt)
    assert "NAN" in _code(e) and "non-finite" in _code(e)
    s.set_particles(pos)
    for _ in range(2):
        st = s.step(dt)
        assert st.converged == 1
    assert np.isfinite(s.particles()[1]).all()
    s.close()


@pytest.mark.gpu
def test_non_finite_particle_is_kept_out_of_the_grid(gpu):
    """A particle with a NaN velocity lands in no fluid face: its trilinear
    weights are NaN, and P2G keeps a face only where the weight sum exceeds
    1e-6 (simulator.cpp:339-350), so the grid and the other particles stay finite."""
    s, pos = _sim()
    vel = np.zeros_like(pos)
    vel[123, 1] = np.nan
    s.set_particles(pos, vel)
    st = s.step(1 / 120)
    assert st.converged == 1
    for f in (N.F_VX, N.F_VY, N.F_VZ, N.F_V2X, N.F_V2Y, N.F_V2Z):
        assert np.isfinite(s.grid(f)).all()
    v = s.particles()[1]
    assert np.isfinite(v).all(axis=1).sum() >= v.shape[0] - 1
    s.close()


@pytest.mark.gpu
def test_iteration_cap_finishes_the_step_unconverged(gpu):
    s, _ = _sim(max_iters=2, tol=1e-12, tol_mode=N.TOL_REL_L2)
    for _ in range(2):
        st = s.step(1 / 120)
    assert st.pcg_iterations == 2 and st.converged == 0
    assert np.isfinite(s.particles()[1]).all()
    s.close()


@pytest.mark.gpu
def test_calls_out_of_order_and_missing_network(gpu):
    s, _ = _sim()
    with pytest.raises(N.FsimError) as e:
        s.stage(N.STAGE_G2P, 1 / 120)         # G2P needs the cell sort of a P2G stage
    assert "STATE" in _code(e)
    p = N.default_params(transfer=N.FLIP, resolution=32, warm_start=N.WARM_LEARNED)
    s.set_params(p)
    with pytest.raises(N.FsimError) as e:
        s.step(1 / 120)                       # no network attached (fsim_set_net)
    assert "STATE" in _code(e) and "network" in _code(e)
    s.close()


@pytest.mark.gpu
def test_push_apart_radius_limit_and_gfx_capacity(gpu):
    s, _ = _sim(push_apart=True, particle_r=0.8 / 32)   # 2r > h: neighbours beyond one cell
    with pytest.raises(N.FsimError) as e:
        s.step(1 / 120)
    assert "UNSUPPORTED" in _code(e)
    s.close()
    s, _ = _sim()
    small = (N.ParticleGfx * 10)()
    got = C.c_int64()
    assert s.lib.fsim_fill_gfx(s.ctx, small, 10, C.byref(got), N.HOST) == -1
    assert s.lib.fsim_fill_gfx_async(s.ctx, small, 10, C.byref(got)) == -1
    assert got.value == s.n
    assert b"capacity" in s.lib.fsim_last_error(s.ctx)
    s.close()


@pytest.mark.gpu
def test_renderer_rejects_bad_parameters(gpu):
    r = N.Renderer(64, 48)
    cam = N.camera((0.0, 0.0, 0.0), -90.0, 0.0)
    prm = N.default_render_params(num_lights=N.RENDER_MAX_LIGHTS + 1)
    pts = np.zeros((4, 5), np.float32)
    with pytest.raises(N.FsimError):
        r.frame(pts, cam, prm)
    prm = N.default_render_params(particle_radius=0.0)
    with pytest.raises(N.FsimError):
        r.frame(pts, cam, prm)
    r.frame(pts, cam, N.default_render_params())  # still usable
    r.close()
