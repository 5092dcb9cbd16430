"""ctypes binding of the C ABI in include/fsim.h (libfsim.so, built in-tree).

``Simulation`` is the Python-side mirror of the reference's per-step
interface (Simulator + MacGrid + HashedParticles, src/Simulator/simulator):
set particles and obstacles, step, read grid fields and particles back.  The
library is the CUDA implementation; there is no CPU path here -- loading fails
loudly when libfsim.so is missing or no GPU is visible.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfsim.so")

PIC, FLIP, APIC = 0, 1, 2
WATER, AIR, SOLID = 0, 1, 2
HOST, DEVICE = 0, 1
OBS_SPHERE, OBS_BOX, OBS_SOURCE, OBS_SINK, OBS_DISC_SOURCE, OBS_BOX_SINK = range(6)
TOL_ABS_MAX, TOL_REL_L2 = 0, 1
PREC_MIXED, PREC_FP32, PREC_FP64 = 0, 1, 2
WARM_ZERO, WARM_PREVIOUS, WARM_GUESS, WARM_LEARNED, WARM_LEARNED_RESIDUAL = 0, 1, 2, 3, 4
PRECOND_RBIC, PRECOND_MG = 0, 1
SOLVER_PCG, SOLVER_SOR = 0, 1
(STAGE_SPAWN, STAGE_ADVECT, STAGE_PUSH_APART, STAGE_PUSH_OUT, STAGE_STOP, STAGE_P2G, STAGE_MARK,
 STAGE_OBSTACLES, STAGE_WALLS, STAGE_POST_P2G, STAGE_SOLVE, STAGE_EXTRAPOLATE, STAGE_G2P) = range(13)
(F_FLAGS, F_AVGPNUM, F_VX, F_VY, F_VZ, F_V2X, F_V2Y, F_V2Z, F_PRESSURE, F_COUNT,
 F_DIVERGENCE) = range(11)

ERRORS = {0: "OK", -1: "INVALID", -2: "OOM", -3: "CUDA", -4: "NOT_CONVERGED", -5: "NAN",
          -6: "TIMEOUT", -7: "UNSUPPORTED", -8: "STATE", -9: "CAPACITY"}


class GridDesc(C.Structure):
    _fields_ = [("dims", C.c_double * 3), ("resolution", C.c_double), ("two_d", C.c_int)]


class Params(C.Structure):
    _fields_ = [
        ("transfer", C.c_int), ("flip_ratio", C.c_float), ("gravity", C.c_float),
        ("gravity_enabled", C.c_int), ("push_apart_enabled", C.c_int), ("spawning_enabled", C.c_int),
        ("despawning_enabled", C.c_int), ("stop_particles", C.c_int), ("top_solid", C.c_int),
        ("pressure_enabled", C.c_int), ("pressure_k", C.c_double), ("average_pressure", C.c_double),
        ("max_iters", C.c_int), ("fluid_density", C.c_double), ("residual_tol", C.c_double),
        ("tol_mode", C.c_int), ("particle_r", C.c_double), ("precision", C.c_int),
        ("warm_start", C.c_int), ("track_ids", C.c_int), ("timing", C.c_int), ("precond", C.c_int),
        ("mg_sweeps", C.c_int), ("mg_coarse_sweeps", C.c_int), ("mg_cluster_sweeps", C.c_int),
        ("grid_solver", C.c_int), ("learned_backoff", C.c_int), ("refine_digits", C.c_int),
        ("mg_boundary_sweeps", C.c_int), ("deterministic", C.c_int),
    ]


class Obstacle(C.Structure):
    _fields_ = [
        ("type", C.c_int), ("pos", C.c_double * 3), ("prev_pos", C.c_double * 3),
        ("speed", C.c_double * 3), ("r", C.c_double), ("size", C.c_double * 3),
        ("spawn_rate", C.c_double), ("spawn_speed", C.c_double), ("last_spawn_fraction", C.c_double),
    ]


class ParticleGfx(C.Structure):
    _fields_ = [("pos", C.c_float * 3), ("v", C.c_float), ("density", C.c_float)]


class StepStats(C.Structure):
    _fields_ = [
        ("pcg_iterations", C.c_int), ("converged", C.c_int), ("num_particles", C.c_int),
        ("num_fluid_cells", C.c_int), ("residual_max", C.c_double), ("residual_rel", C.c_double),
        ("rhs_norm", C.c_double), ("guess_used", C.c_int), ("reliable_updates", C.c_int),
        ("ms_simulate_particles", C.c_float), ("ms_push_apart", C.c_float), ("ms_push_out", C.c_float),
        ("ms_p2g", C.c_float), ("ms_prep", C.c_float), ("ms_solve", C.c_float),
        ("ms_extrapolate", C.c_float), ("ms_g2p", C.c_float), ("ms_total", C.c_float),
        ("ms_p2g_kernel", C.c_float), ("ms_g2p_kernel", C.c_float), ("ms_pcg_setup", C.c_float),
        ("kernel_launches", C.c_int), ("num_active_bricks", C.c_int), ("ms_guess", C.c_float),
        ("reserved", C.c_int * 2),
    ]


# ---- renderer structures (include/fsim_render.h) ----
RENDER_MAX_LIGHTS = 8
IMG_COLOR, IMG_DEPTH, IMG_THICKNESS, IMG_NORMAL_DEPTH, IMG_RAW_DEPTH = 0, 1, 2, 3, 4


class Camera(C.Structure):
    _fields_ = [("view", C.c_float * 16), ("view_inv", C.c_float * 16), ("proj", C.c_float * 16),
                ("proj_inv", C.c_float * 16), ("position", C.c_float * 4)]


class Light(C.Structure):
    _fields_ = [("position", C.c_float * 4), ("power_density", C.c_float * 3)]


class RenderParams(C.Structure):
    _fields_ = [
        ("particle_radius", C.c_float), ("particle_color", C.c_float * 3), ("specular_color", C.c_float * 3),
        ("shininess", C.c_float), ("bilateral_filter", C.c_int), ("smoothing_size", C.c_float),
        ("blur_scale", C.c_float), ("blur_depth_falloff", C.c_float), ("spray_enabled", C.c_int),
        ("spray_density_threshold", C.c_float), ("transparency_enabled", C.c_int),
        ("transparency_blur_size", C.c_float), ("transparency", C.c_float), ("noise_enabled", C.c_int),
        ("noise_scale", C.c_float), ("noise_strength", C.c_float), ("noise_offset", C.c_float),
        ("num_lights", C.c_int), ("lights", Light * RENDER_MAX_LIGHTS), ("background", C.c_float * 4),
    ]


# exported symbols, in the order include/fsim.h and include/fsim_render.h declare them
EXPORTS = [
    "fsim_create", "fsim_destroy", "fsim_set_params", "fsim_get_params", "fsim_grid_info",
    "fsim_last_error", "fsim_stream", "fsim_synchronize", "fsim_set_particles", "fsim_add_particles",
    "fsim_get_particles", "fsim_num_particles", "fsim_set_obstacles", "fsim_get_obstacles",
    "fsim_step", "fsim_stage", "fsim_get_grid", "fsim_set_grid", "fsim_fill_gfx",
    "fsim_fill_gfx_async", "fsim_gfx_wait",
    "fsim_set_pressure_guess", "fsim_solve_pressure", "fsim_solve_current", "fsim_p2g_noalloc",
    "fsim_net_create", "fsim_net_destroy", "fsim_net_last_error", "fsim_net_num_params",
    "fsim_net_get_params", "fsim_net_set_params", "fsim_net_forward", "fsim_net_backward",
    "fsim_net_set_loss", "fsim_net_train_batch", "fsim_net_zero_grad", "fsim_net_adam", "fsim_net_train_step",
    "fsim_net_synchronize",
    "fsim_net_conv", "fsim_set_net",
    "fsim_render_default_params", "fsim_render_camera", "fsim_render_create", "fsim_render_destroy",
    "fsim_render_last_error", "fsim_render_frame", "fsim_render_ctx", "fsim_render_read", "fsim_render_stats",
]

_lib = None


def load_library(path: str = LIB_PATH) -> C.CDLL:
    """Load libfsim.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: run `python __graft_entry__.py build` first")
    lib = C.CDLL(path)
    P, fp, dp, i64 = C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_double), C.c_int64
    sig = {
        "fsim_create": (C.c_int, [C.POINTER(GridDesc), C.POINTER(Params), C.POINTER(P)]),
        "fsim_destroy": (C.c_int, [P]),
        "fsim_set_params": (C.c_int, [P, C.POINTER(Params)]),
        "fsim_get_params": (C.c_int, [P, C.POINTER(Params)]),
        "fsim_grid_info": (C.c_int, [P, C.POINTER(C.c_int), dp, dp]),
        "fsim_last_error": (C.c_char_p, [P]),
        "fsim_stream": (P, [P]),
        "fsim_synchronize": (C.c_int, [P]),
        "fsim_set_particles": (C.c_int, [P, P, P, P, i64, C.c_int]),
        "fsim_add_particles": (C.c_int, [P, P, P, P, i64, C.c_int]),
        "fsim_get_particles": (C.c_int, [P, P, P, P, i64, C.POINTER(i64), C.c_int]),
        "fsim_num_particles": (C.c_int, [P, C.POINTER(i64)]),
        "fsim_set_obstacles": (C.c_int, [P, C.POINTER(Obstacle), C.c_int]),
        "fsim_get_obstacles": (C.c_int, [P, C.POINTER(Obstacle), C.c_int, C.POINTER(C.c_int)]),
        "fsim_step": (C.c_int, [P, C.c_double, C.POINTER(StepStats)]),
        "fsim_stage": (C.c_int, [P, C.c_int, C.c_double, C.POINTER(StepStats)]),
        "fsim_get_grid": (C.c_int, [P, C.c_int, P, C.c_int]),
        "fsim_set_grid": (C.c_int, [P, C.c_int, P, C.c_int]),
        "fsim_fill_gfx": (C.c_int, [P, C.POINTER(ParticleGfx), i64, C.POINTER(i64), C.c_int]),
        "fsim_fill_gfx_async": (C.c_int, [P, C.POINTER(ParticleGfx), i64, C.POINTER(i64)]),
        "fsim_gfx_wait": (C.c_int, [P]),
        "fsim_set_pressure_guess": (C.c_int, [P, fp, C.c_int]),
        "fsim_solve_pressure": (C.c_int, [P, dp, C.c_double, C.c_int, C.c_int, C.c_double, C.c_int, dp,
                                          C.POINTER(StepStats)]),
        "fsim_solve_current": (C.c_int, [P, C.c_double, C.c_int, C.c_int, C.POINTER(StepStats)]),
        "fsim_p2g_noalloc": (C.c_int, [C.POINTER(GridDesc), C.c_int, P, P, P, i64, P, P, P, P, P, P]),
        "fsim_net_create": (C.c_int, [C.c_uint64, C.c_float, C.POINTER(P)]),
        "fsim_net_destroy": (C.c_int, [P]),
        "fsim_net_last_error": (C.c_char_p, [P]),
        "fsim_net_num_params": (i64, [P]),
        "fsim_net_get_params": (C.c_int, [P, P, C.c_int, C.c_int]),
        "fsim_net_set_params": (C.c_int, [P, P, C.c_int]),
        "fsim_net_forward": (C.c_int, [P, C.c_int, C.c_int, C.c_int, C.c_int, P, P, C.c_int, C.c_int]),
        "fsim_net_backward": (C.c_int, [P, P, P, fp, C.c_int]),
        "fsim_net_set_loss": (C.c_int, [P, C.c_float]),
        "fsim_net_train_batch": (C.c_int, [P, C.c_int, C.c_int, C.c_int, P, P, P, P, C.c_int, C.c_float, P]),
        "fsim_net_zero_grad": (C.c_int, [P]),
        "fsim_net_adam": (C.c_int, [P, C.c_float]),
        "fsim_net_train_step": (C.c_int, [P, C.c_int, C.c_int, C.c_int, C.c_int, P, P, P, C.c_float, fp,
                                          C.c_int]),
        "fsim_net_synchronize": (C.c_int, [P]),
        "fsim_net_conv": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                    P, P, P, P, C.c_int]),
        "fsim_set_net": (C.c_int, [P, P]),
        "fsim_render_default_params": (None, [C.POINTER(RenderParams)]),
        "fsim_render_camera": (None, [C.POINTER(Camera), dp, C.c_double, C.c_double, C.c_double, C.c_double,
                                      C.c_double, C.c_double]),
        "fsim_render_create": (C.c_int, [C.c_int, C.c_int, C.POINTER(P)]),
        "fsim_render_destroy": (C.c_int, [P]),
        "fsim_render_last_error": (C.c_char_p, [P]),
        "fsim_render_frame": (C.c_int, [P, P, i64, C.c_int, C.POINTER(Camera), C.POINTER(RenderParams), P, P]),
        "fsim_render_ctx": (C.c_int, [P, P, C.POINTER(Camera), C.POINTER(RenderParams), P]),
        "fsim_render_read": (C.c_int, [P, C.c_int, P, C.c_int]),
        "fsim_render_stats": (C.c_int, [P, fp, C.POINTER(C.c_int)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class FsimError(RuntimeError):
    pass


def default_params(*, transfer: int = FLIP, resolution: float = 32, flip_ratio: float = 0.95,
                   gravity: float = -9.81, max_iters: int = 200, tol: float = 1e-6,
                   tol_mode: int = TOL_ABS_MAX, precision: int = PREC_MIXED, warm_start: int = WARM_ZERO,
                   top_solid: bool = True, particle_r: float | None = None, spawning: bool = False,
                   despawning: bool = False, stop_particles: bool = False, gravity_enabled: bool = True,
                   pressure_enabled: bool = False, pressure_k: float = 2.0, average_pressure: float = 2.0,
                   fluid_density: float = 1.0, timing: bool = False, precond: int = PRECOND_MG,
                   mg_sweeps: int = 0, mg_coarse_sweeps: int = 0, mg_cluster_sweeps: int = 0,
                   grid_solver: int = SOLVER_PCG, push_apart: bool = False, learned_backoff: bool = False,
                   refine_digits: int = 0, mg_boundary_sweeps: int = 0, deterministic: bool = False) -> Params:
    """Parameters of the dam-break workloads (reference parameter names in fsim.h)."""
    p = Params()
    p.transfer = transfer
    p.flip_ratio = flip_ratio
    p.gravity = gravity
    p.gravity_enabled = int(gravity_enabled)
    p.push_apart_enabled = int(push_apart)
    p.spawning_enabled = int(spawning)
    p.despawning_enabled = int(despawning)
    p.stop_particles = int(stop_particles)
    p.top_solid = int(top_solid)
    p.pressure_enabled = int(pressure_enabled)
    p.pressure_k = pressure_k
    p.average_pressure = average_pressure
    p.max_iters = max_iters
    p.fluid_density = fluid_density
    p.residual_tol = tol
    p.tol_mode = tol_mode
    h = 1.0 / float(np.float32(resolution))
    p.particle_r = h / 4.0 if particle_r is None else particle_r
    p.precision = precision
    p.warm_start = warm_start
    p.track_ids = 0
    p.timing = int(timing)
    p.precond = precond
    p.mg_sweeps = mg_sweeps
    p.mg_coarse_sweeps = mg_coarse_sweeps
    p.mg_cluster_sweeps = mg_cluster_sweeps
    p.grid_solver = grid_solver
    p.learned_backoff = int(learned_backoff)
    p.refine_digits = refine_digits
    p.mg_boundary_sweeps = mg_boundary_sweeps
    p.deterministic = int(deterministic)
    return p


def _ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


class Simulation:
    """One simulation context on the current CUDA device."""

    def __init__(self, resolution: float, params: Params, *, dims=(1.0, 1.0, 1.0), track_ids: bool = False,
                 two_d: bool = False):
        self.lib = load_library()
        g = GridDesc()
        g.dims[:] = list(dims)
        g.resolution = resolution
        g.two_d = int(two_d)
        params.track_ids = int(track_ids)
        self.params = params
        self.ctx = C.c_void_p()
        rc = self.lib.fsim_create(C.byref(g), C.byref(params), C.byref(self.ctx))
        if rc != 0:
            raise FsimError(f"fsim_create failed: {ERRORS.get(rc, rc)}")
        n3 = (C.c_int * 3)()
        h3 = (C.c_double * 3)()
        d3 = (C.c_double * 3)()
        self.lib.fsim_grid_info(self.ctx, n3, h3, d3)
        self.shape = (n3[0], n3[1], n3[2])
        self.h = h3[0]
        self.hz = h3[2]
        self.two_d = bool(two_d)
        self.dims = (d3[0], d3[1], d3[2])

    def _check(self, rc: int, what: str):
        if rc != 0:
            msg = self.lib.fsim_last_error(self.ctx).decode()
            raise FsimError(f"{what} failed: {ERRORS.get(rc, rc)}: {msg}")

    def close(self):
        if self.ctx:
            self.lib.fsim_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, params: Params):
        params.track_ids = self.params.track_ids
        self._check(self.lib.fsim_set_params(self.ctx, C.byref(params)), "fsim_set_params")
        self.params = params

    @property
    def n(self) -> int:
        n = C.c_int64()
        self.lib.fsim_num_particles(self.ctx, C.byref(n))
        return n.value

    def set_particles(self, pos, vel=None, c=None):
        pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
        vel = None if vel is None else np.ascontiguousarray(vel, np.float32).reshape(-1, 3)
        c = None if c is None else np.ascontiguousarray(c, np.float32).reshape(-1, 9)
        self._check(self.lib.fsim_set_particles(self.ctx, _ptr(pos), _ptr(vel), _ptr(c), pos.shape[0], HOST),
                    "fsim_set_particles")

    def add_particles(self, pos, vel=None, c=None):
        pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 3)
        vel = None if vel is None else np.ascontiguousarray(vel, np.float32).reshape(-1, 3)
        c = None if c is None else np.ascontiguousarray(c, np.float32).reshape(-1, 9)
        self._check(self.lib.fsim_add_particles(self.ctx, _ptr(pos), _ptr(vel), _ptr(c), pos.shape[0], HOST),
                    "fsim_add_particles")

    def particles(self):
        n = self.n
        pos = np.empty((n, 3), np.float32)
        vel = np.empty((n, 3), np.float32)
        c = np.empty((n, 3, 3), np.float32)
        got = C.c_int64()
        self._check(self.lib.fsim_get_particles(self.ctx, _ptr(pos), _ptr(vel), _ptr(c), n, C.byref(got), HOST),
                    "fsim_get_particles")
        return pos, vel, c

    def set_obstacles(self, obstacles):
        arr = (Obstacle * max(1, len(obstacles)))()
        for i, o in enumerate(obstacles):
            arr[i] = o
        self._check(self.lib.fsim_set_obstacles(self.ctx, arr, len(obstacles)), "fsim_set_obstacles")

    def obstacles(self):
        arr = (Obstacle * 64)()
        n = C.c_int()
        self._check(self.lib.fsim_get_obstacles(self.ctx, arr, 64, C.byref(n)), "fsim_get_obstacles")
        return [arr[i] for i in range(min(n.value, 64))]

    def step(self, dt: float) -> StepStats:
        st = StepStats()
        self._check(self.lib.fsim_step(self.ctx, dt, C.byref(st)), "fsim_step")
        return st

    def stage(self, stage: int, dt: float) -> StepStats:
        st = StepStats()
        self._check(self.lib.fsim_stage(self.ctx, stage, dt, C.byref(st)), f"fsim_stage({stage})")
        return st

    def grid(self, field: int) -> np.ndarray:
        dtype = {F_FLAGS: np.uint8, F_COUNT: np.int32}.get(field, np.float32)
        out = np.empty(self.shape, dtype)
        self._check(self.lib.fsim_get_grid(self.ctx, field, _ptr(out), HOST), "fsim_get_grid")
        return out

    def set_grid(self, field: int, values):
        dtype = np.uint8 if field == F_FLAGS else np.float32
        a = np.ascontiguousarray(values, dtype).reshape(self.shape)
        self._check(self.lib.fsim_set_grid(self.ctx, field, _ptr(a), HOST), "fsim_set_grid")

    def gfx(self) -> np.ndarray:
        n = self.n
        arr = (ParticleGfx * max(1, n))()
        got = C.c_int64()
        self._check(self.lib.fsim_fill_gfx(self.ctx, arr, n, C.byref(got), HOST), "fsim_fill_gfx")
        out = np.frombuffer(arr, dtype=np.float32, count=5 * n).reshape(n, 5)
        return out.copy()

    def set_pressure_guess(self, p):
        a = np.ascontiguousarray(p, np.float32).reshape(self.shape)
        self._check(self.lib.fsim_set_pressure_guess(self.ctx, a.ctypes.data_as(C.POINTER(C.c_float)), HOST),
                    "fsim_set_pressure_guess")

    def solve_pressure(self, rhs, dt: float, *, precision: int = PREC_MIXED, tol_mode: int = TOL_REL_L2,
                       tol: float = 1e-6, max_iters: int = 2000):
        b = np.ascontiguousarray(rhs, np.float64).reshape(self.shape)
        p = np.empty(self.shape, np.float64)
        st = StepStats()
        self._check(self.lib.fsim_solve_pressure(self.ctx, b.ctypes.data_as(C.POINTER(C.c_double)), dt,
                                                 precision, tol_mode, tol, max_iters,
                                                 p.ctypes.data_as(C.POINTER(C.c_double)), C.byref(st)),
                    "fsim_solve_pressure")
        return p, st

    def solve_current(self, dt: float, warm_start: int, apply: bool = False) -> StepStats:
        """Pressure solve of the current state with an explicit warm start (fsim_solve_current)."""
        st = StepStats()
        self._check(self.lib.fsim_solve_current(self.ctx, dt, warm_start, int(apply), C.byref(st)),
                    "fsim_solve_current")
        return st

    def synchronize(self):
        self._check(self.lib.fsim_synchronize(self.ctx), "fsim_synchronize")

    def set_net(self, net: "WarmStartNet | None"):
        """Attach the warm-start network used by WARM_LEARNED (the context keeps no ownership)."""
        self._net = net
        self._check(self.lib.fsim_set_net(self.ctx, None if net is None else net.net), "fsim_set_net")


class WarmStartNet:
    """The learned pressure warm start (fsim_net_* in fsim.h).

    Inputs are [n, d, h, w, 4] float32 (rhs / rms(rhs over fluid), fluid, solid,
    air), outputs [n, d, h, w] float32 (pressure / rms(rhs)), in the solver's
    integer-stencil units.  Arrays may be numpy (host) or anything exposing a
    device pointer through ``data_ptr()`` (device).
    """

    def __init__(self, seed: int = 1, out_scale: float = 1.0):
        self.lib = load_library()
        self.net = C.c_void_p()
        self.out_scale = float(out_scale)
        rc = self.lib.fsim_net_create(seed, out_scale, C.byref(self.net))
        if rc != 0:
            raise FsimError(f"fsim_net_create failed: {ERRORS.get(rc, rc)}")
        self.num_params = int(self.lib.fsim_net_num_params(self.net))

    def _check(self, rc: int, what: str):
        if rc != 0:
            msg = self.lib.fsim_net_last_error(self.net).decode()
            raise FsimError(f"{what} failed: {ERRORS.get(rc, rc)}: {msg}")

    def close(self):
        if self.net:
            self.lib.fsim_net_destroy(self.net)
            self.net = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _arg(a):
        if hasattr(a, "data_ptr"):
            return C.c_void_p(a.data_ptr()), DEVICE
        return C.c_void_p(a.ctypes.data), HOST

    def params(self, grad: bool = False) -> np.ndarray:
        out = np.empty(self.num_params, np.float32)
        self._check(self.lib.fsim_net_get_params(self.net, _ptr(out), 1 if grad else 0, HOST), "fsim_net_get_params")
        return out

    def set_params(self, theta):
        theta = np.ascontiguousarray(theta, np.float32)
        assert theta.size == self.num_params
        self._check(self.lib.fsim_net_set_params(self.net, _ptr(theta), HOST), "fsim_net_set_params")

    def forward(self, x, train: bool = False):
        if hasattr(x, "data_ptr"):
            import torch
            out = torch.empty(tuple(x.shape[:4]), dtype=torch.float32, device=x.device)
            self._check(self.lib.fsim_net_forward(self.net, *x.shape[:4], C.c_void_p(x.data_ptr()),
                                                  C.c_void_p(out.data_ptr()), int(train), DEVICE), "fsim_net_forward")
            return out
        x = np.ascontiguousarray(x, np.float32)
        out = np.empty(x.shape[:4], np.float32)
        self._check(self.lib.fsim_net_forward(self.net, *x.shape[:4], _ptr(x), _ptr(out), int(train), HOST),
                    "fsim_net_forward")
        return out

    def backward(self, target, mask) -> float:
        loss = C.c_float()
        t, where = self._arg(target if hasattr(target, "data_ptr") else np.ascontiguousarray(target, np.float32))
        m, _ = self._arg(mask if hasattr(mask, "data_ptr") else np.ascontiguousarray(mask, np.uint8))
        self._check(self.lib.fsim_net_backward(self.net, t, m, C.byref(loss), where), "fsim_net_backward")
        return loss.value

    def set_loss(self, l2_weight: float):
        self._check(self.lib.fsim_net_set_loss(self.net, l2_weight), "fsim_net_set_loss")

    def train_batch(self, types, rhs, target, idx, lr: float, loss_out=None):
        """One Adam step on pool samples idx (CUDA tensors: types uint8, rhs and
        target float32 [samples, d, h, w], idx int32 [batch]); no host sync."""
        d, h, w = types.shape[1:4]
        self._check(self.lib.fsim_net_train_batch(self.net, d, h, w, C.c_void_p(types.data_ptr()),
                                                  C.c_void_p(rhs.data_ptr()), C.c_void_p(target.data_ptr()),
                                                  C.c_void_p(idx.data_ptr()), int(idx.shape[0]), lr,
                                                  None if loss_out is None else C.c_void_p(loss_out.data_ptr())),
                    "fsim_net_train_batch")

    def synchronize(self):
        self._check(self.lib.fsim_net_synchronize(self.net), "fsim_net_synchronize")

    def zero_grad(self):
        self._check(self.lib.fsim_net_zero_grad(self.net), "fsim_net_zero_grad")

    def adam(self, lr: float):
        self._check(self.lib.fsim_net_adam(self.net, lr), "fsim_net_adam")

    def train_step(self, x, target, mask, lr: float) -> float:
        loss = C.c_float()
        dev = hasattr(x, "data_ptr")
        if not dev:
            x = np.ascontiguousarray(x, np.float32)
            target = np.ascontiguousarray(target, np.float32)
            mask = np.ascontiguousarray(mask, np.uint8)
        xp, where = self._arg(x)
        tp, _ = self._arg(target)
        mp, _ = self._arg(mask)
        self._check(self.lib.fsim_net_train_step(self.net, *x.shape[:4], xp, tp, mp, lr, C.byref(loss), where),
                    "fsim_net_train_step")
        return loss.value


def net_conv(taps: int, mode: int, x=None, w=None, g=None, *, shape, cin: int, cout: int) -> np.ndarray:
    """One tensor-core convolution on host FP32 arrays (fsim_net_conv)."""
    lib = load_library()
    n, d, h, ww = shape
    vox = n * d * h * ww
    if mode == 0:
        out = np.empty((vox, cout), np.float32)
    elif mode == 1:
        out = np.empty((vox, cin), np.float32)
    else:
        out = np.empty((taps, cout, cin), np.float32)
    args = [None if a is None else np.ascontiguousarray(a, np.float32) for a in (x, w, g)]
    rc = lib.fsim_net_conv(taps, mode, n, d, h, ww, cin, cout, *[_ptr(a) for a in args], _ptr(out), HOST)
    if rc != 0:
        msg = lib.fsim_net_last_error(None).decode()
        raise FsimError(f"fsim_net_conv failed: {ERRORS.get(rc, rc)}: {msg}")
    return out


def obstacle(kind: int, pos, *, r: float = 0.0, size=(0, 0, 0), speed=(0, 0, 0), prev_pos=None,
             spawn_rate: float = 0.0, spawn_speed: float = 0.0, frac: float = 0.0) -> Obstacle:
    o = Obstacle()
    o.type = kind
    o.pos[:] = list(pos)
    o.prev_pos[:] = list(pos if prev_pos is None else prev_pos)
    o.speed[:] = list(speed)
    o.r = r
    o.size[:] = list(size)
    o.spawn_rate = spawn_rate
    o.spawn_speed = spawn_speed
    o.last_spawn_fraction = frac
    return o


# ---------------------------------------------------------------- renderer
def default_render_params(**kw) -> RenderParams:
    """The reference GUI's fluid-surface settings and lights (fsim_render_default_params),
    with any field overridden by keyword."""
    p = RenderParams()
    load_library().fsim_render_default_params(C.byref(p))
    for k, v in kw.items():
        f = getattr(p, k)
        if isinstance(f, C.Array):
            for i, x in enumerate(v):
                f[i] = x
        else:
            setattr(p, k, v)
    return p


def camera(eye, yaw: float, pitch: float, fov: float = 40.0, aspect: float = 1.0, near: float = 0.5,
           far: float = 300.0) -> Camera:
    """Camera3D-style camera: eye position, yaw / pitch in degrees (fsim_render_camera)."""
    c = Camera()
    e = (C.c_double * 3)(*eye)
    load_library().fsim_render_camera(C.byref(c), e, yaw, pitch, fov, aspect, near, far)
    return c


def look_at_angles(eye, target):
    """(yaw, pitch) in degrees of Camera3D's front vector from eye towards target."""
    d = np.asarray(target, np.float64) - np.asarray(eye, np.float64)
    d /= np.linalg.norm(d)
    return float(np.degrees(np.arctan2(d[2], d[0]))), float(np.degrees(np.arcsin(d[1])))


class Renderer:
    """Headless screen-space fluid renderer (include/fsim_render.h)."""

    def __init__(self, width: int, height: int):
        self.lib = load_library()
        self.width, self.height = width, height
        self.r = C.c_void_p()
        rc = self.lib.fsim_render_create(width, height, C.byref(self.r))
        if rc != 0:
            raise FsimError(f"fsim_render_create failed: {ERRORS.get(rc, rc)}")

    def _check(self, rc: int, what: str):
        if rc != 0:
            raise FsimError(f"{what} failed: {ERRORS.get(rc, rc)}: {self.lib.fsim_render_last_error(self.r).decode()}")

    def close(self):
        if self.r:
            self.lib.fsim_render_destroy(self.r)
            self.r = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def frame(self, particles, cam: Camera, params: RenderParams, scene_depth=None):
        """particles: (n, 5) float32 (pos, |v|, density) on the host, or a CUDA tensor of that shape."""
        sd = None
        if scene_depth is not None:
            sd = C.c_void_p(scene_depth.data_ptr())
        if hasattr(particles, "data_ptr"):
            n = particles.shape[0]
            self._check(self.lib.fsim_render_frame(self.r, C.c_void_p(particles.data_ptr()), n, DEVICE,
                                                   C.byref(cam), C.byref(params), sd, None), "fsim_render_frame")
        else:
            pts = np.ascontiguousarray(particles, np.float32).reshape(-1, 5)
            self._keep = pts
            self._check(self.lib.fsim_render_frame(self.r, _ptr(pts) if pts.size else None, pts.shape[0], HOST,
                                                   C.byref(cam), C.byref(params), sd, None), "fsim_render_frame")

    def frame_sim(self, sim: "Simulation", cam: Camera, params: RenderParams, scene_depth=None):
        """Render a simulation context's particles (fsim_render_ctx; no host round trip)."""
        sd = None if scene_depth is None else C.c_void_p(scene_depth.data_ptr())
        self._check(self.lib.fsim_render_ctx(self.r, sim.ctx, C.byref(cam), C.byref(params), sd), "fsim_render_ctx")

    def read(self, image: int = IMG_COLOR) -> np.ndarray:
        four = image in (IMG_COLOR, IMG_NORMAL_DEPTH)
        out = np.empty((self.height, self.width, 4) if four else (self.height, self.width), np.float32)
        self._check(self.lib.fsim_render_read(self.r, image, _ptr(out), HOST), "fsim_render_read")
        return out

    def stats(self):
        ms = C.c_float()
        n = C.c_int()
        self._check(self.lib.fsim_render_stats(self.r, C.byref(ms), C.byref(n)), "fsim_render_stats")
        return ms.value, n.value
