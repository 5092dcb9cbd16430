"""ctypes bindings of the CPU oracles (test infrastructure only).

Two libraries export the interface declared in ``oracle_api.h``:

* ``oracle/_ref/libfsim_ref.so`` -- the reference's own Simulator sources
  (dkiovics/fluid_simulator ``src/Simulator/simulator/**``) compiled against
  ``oracle/glmshim`` and driven by ``oracle/ref_harness.cpp``.  It exists only
  where the reference sources are present (``make -C oracle ref``).
* ``oracle/liboracle.so`` -- ``oracle/fsim_oracle.c``, the FP64 C restatement of
  the same algorithm, pinned against the reference library by the golden
  fixtures in ``tests/golden``.  It builds anywhere (``make -C oracle``).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this module; the product never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libfsim_ref.so")

PIC, FLIP, APIC = 0, 1, 2
WATER, AIR, SOLID = 0, 1, 2
OBS_SPHERE, OBS_BOX, OBS_SOURCE, OBS_SINK, OBS_DISC_SOURCE, OBS_BOX_SINK = 0, 1, 2, 3, 4, 5

(STAGE_SPAWN, STAGE_ADVECT, STAGE_PUSH_APART, STAGE_PUSH_OUT, STAGE_STOP, STAGE_P2G,
 STAGE_MARK, STAGE_OBSTACLES, STAGE_WALLS, STAGE_POST_P2G, STAGE_SOLVE,
 STAGE_EXTRAPOLATE, STAGE_G2P) = range(13)

F_FLAGS, F_AVGPNUM, F_VX, F_VY, F_VZ, F_V2X, F_V2Y, F_V2Z, F_PRESSURE, F_WX, F_WY, F_WZ, \
    F_FLUID_ID = range(13)


class OracleParams(C.Structure):
    _fields_ = [
        ("resolution", C.c_double),
        ("dims", C.c_double * 3),
        ("two_d", C.c_int),
        ("particle_r", C.c_double),
        ("transfer", C.c_int),
        ("flip_ratio", C.c_float),
        ("gravity", C.c_float),
        ("gravity_enabled", C.c_int),
        ("push_apart_enabled", C.c_int),
        ("spawning_enabled", C.c_int),
        ("despawning_enabled", C.c_int),
        ("stop_particles", C.c_int),
        ("top_solid", C.c_int),
        ("pressure_enabled", C.c_int),
        ("max_iters", C.c_int),
        ("pressure_k", C.c_double),
        ("average_pressure", C.c_double),
        ("fluid_density", C.c_double),
        ("residual_tol", C.c_double),
        ("grid_solver", C.c_int),
    ]


class OracleObstacle(C.Structure):
    _fields_ = [
        ("type", C.c_int),
        ("pos", C.c_double * 3),
        ("prev_pos", C.c_double * 3),
        ("speed", C.c_double * 3),
        ("r", C.c_double),
        ("size", C.c_double * 3),
        ("spawn_rate", C.c_double),
        ("spawn_speed", C.c_double),
        ("last_spawn_fraction", C.c_double),
    ]


def build_port(quiet: bool = True) -> str:
    """Compile oracle/liboracle.so (gcc; a second or two)."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True,
                   stdout=subprocess.DEVNULL if quiet else None)
    return PORT_LIB


def reference_dir() -> str | None:
    """The reference checkout (dkiovics/fluid_simulator): $FSIM_REFERENCE_DIR,
    else the directory ``reference`` beside this repository; None when neither
    holds the Simulator sources (e.g. on a machine that only runs the GPU tests)."""
    cands = [os.environ.get("FSIM_REFERENCE_DIR"), os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")]
    for d in cands:
        if d and os.path.isdir(os.path.join(d, "src", "Simulator")):
            return d
    return None


def build_ref(ref_dir: str | None = None, quiet: bool = True) -> str | None:
    """Compile oracle/_ref/libfsim_ref.so when the reference sources exist."""
    ref_dir = ref_dir or reference_dir()
    if ref_dir is None:
        return None
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_DIR={ref_dir}"], check=True,
                   stdout=subprocess.DEVNULL if quiet else None)
    return REF_LIB


def have_ref() -> bool:
    return os.path.exists(REF_LIB)


_LIBS: dict[str, C.CDLL] = {}


def _load(path: str) -> C.CDLL:
    if path in _LIBS:
        return _LIBS[path]
    lib = C.CDLL(path)
    P = C.c_void_p
    dp = C.POINTER(C.c_double)
    lib.oracle_create.restype = P
    lib.oracle_create.argtypes = [C.POINTER(OracleParams), C.c_int, dp, dp, dp]
    lib.oracle_destroy.argtypes = [P]
    lib.oracle_set_threads.argtypes = [C.c_int]
    lib.oracle_grid_size.argtypes = [P, C.POINTER(C.c_int)]
    lib.oracle_cell_size.argtypes = [P, dp]
    lib.oracle_num_particles.argtypes = [P]
    lib.oracle_num_particles.restype = C.c_int
    lib.oracle_get_particles.argtypes = [P, dp, dp, dp]
    lib.oracle_set_particles.argtypes = [P, C.c_int, dp, dp, dp]
    lib.oracle_set_params.argtypes = [P, C.POINTER(OracleParams)]
    lib.oracle_set_obstacles.argtypes = [P, C.c_int, C.POINTER(OracleObstacle)]
    lib.oracle_get_obstacles.argtypes = [P, C.c_int, C.POINTER(OracleObstacle)]
    lib.oracle_get_obstacles.restype = C.c_int
    lib.oracle_step.argtypes = [P, C.c_double]
    lib.oracle_step.restype = C.c_int
    lib.oracle_stage.argtypes = [P, C.c_int, C.c_double]
    lib.oracle_stage.restype = C.c_int
    lib.oracle_get_grid.argtypes = [P, C.c_int, C.c_void_p]
    lib.oracle_set_grid.argtypes = [P, C.c_int, C.c_void_p]
    lib.oracle_fluid_count.argtypes = [P]
    lib.oracle_fluid_count.restype = C.c_int
    lib.oracle_last_iterations.argtypes = [P]
    lib.oracle_last_iterations.restype = C.c_int
    _LIBS[path] = lib
    return lib


def make_params(resolution: float, *, transfer: int = FLIP, flip_ratio: float = 0.95,
                gravity: float = -9.81, particle_r: float | None = None, top_solid: bool = True,
                max_iters: int = 200, tol: float = 1e-6, dims=(1.0, 1.0, 1.0),
                gravity_enabled: bool = True, spawning: bool = False, despawning: bool = False,
                stop_particles: bool = False, pressure_enabled: bool = False,
                pressure_k: float = 2.0, average_pressure: float = 2.0,
                fluid_density: float = 1.0, two_d: bool = False, grid_solver: int = 0,
                push_apart: bool = False) -> OracleParams:
    p = OracleParams()
    p.resolution = resolution
    p.dims[:] = list(dims)
    p.two_d = int(two_d)
    p.particle_r = (1.0 / resolution) / 4.0 if particle_r is None else particle_r
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
    p.max_iters = max_iters
    p.pressure_k = pressure_k
    p.average_pressure = average_pressure
    p.fluid_density = fluid_density
    p.residual_tol = tol
    p.grid_solver = grid_solver
    return p


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


class Oracle:
    """One simulation instance inside an oracle library."""

    def __init__(self, params: OracleParams, pos, vel=None, c=None, *, lib: str = "port"):
        path = {"port": PORT_LIB, "ref": REF_LIB}.get(lib, lib)
        self.lib = _load(path)
        self.kind = lib
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        n = pos.shape[0]
        vel = np.zeros((n, 3)) if vel is None else np.ascontiguousarray(vel, np.float64).reshape(-1, 3)
        c = np.zeros((n, 3, 3)) if c is None else np.ascontiguousarray(c, np.float64).reshape(-1, 3, 3)
        self.params = params
        self.h = self.lib.oracle_create(C.byref(params), n, _dp(pos), _dp(vel), _dp(c))
        n3 = (C.c_int * 3)()
        self.lib.oracle_grid_size(self.h, n3)
        self.shape = (n3[0], n3[1], n3[2])
        h3 = (C.c_double * 3)()
        self.lib.oracle_cell_size(self.h, h3)
        self.cell = (h3[0], h3[1], h3[2])

    def close(self):
        if self.h:
            self.lib.oracle_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_threads(self, n: int):
        self.lib.oracle_set_threads(int(n))

    @property
    def n(self) -> int:
        return self.lib.oracle_num_particles(self.h)

    def particles(self):
        n = self.n
        pos = np.empty((n, 3)); vel = np.empty((n, 3)); c = np.empty((n, 3, 3))
        self.lib.oracle_get_particles(self.h, _dp(pos), _dp(vel), _dp(c))
        return pos, vel, c

    def set_particles(self, pos, vel=None, c=None):
        pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        n = pos.shape[0]
        vel = np.zeros((n, 3)) if vel is None else np.ascontiguousarray(vel, np.float64).reshape(-1, 3)
        c = np.zeros((n, 3, 3)) if c is None else np.ascontiguousarray(c, np.float64).reshape(-1, 3, 3)
        self.lib.oracle_set_particles(self.h, n, _dp(pos), _dp(vel), _dp(c))

    def set_params(self, params: OracleParams):
        self.params = params
        self.lib.oracle_set_params(self.h, C.byref(params))

    def set_obstacles(self, obstacles):
        arr = (OracleObstacle * max(1, len(obstacles)))()
        for i, o in enumerate(obstacles):
            arr[i] = o
        self.lib.oracle_set_obstacles(self.h, len(obstacles), arr)

    def obstacles(self):
        arr = (OracleObstacle * 64)()
        n = self.lib.oracle_get_obstacles(self.h, 64, arr)
        return [arr[i] for i in range(min(n, 64))]

    def step(self, dt: float) -> int:
        return self.lib.oracle_step(self.h, dt)

    def stage(self, stage: int, dt: float) -> int:
        return self.lib.oracle_stage(self.h, stage, dt)

    def grid(self, field: int) -> np.ndarray:
        if field == F_FLAGS:
            out = np.empty(self.shape, np.uint8)
        elif field == F_FLUID_ID:
            out = np.empty(self.shape, np.int32)
        else:
            out = np.empty(self.shape, np.float64)
        self.lib.oracle_get_grid(self.h, field, out.ctypes.data_as(C.c_void_p))
        return out

    def set_grid(self, field: int, values):
        dtype = np.uint8 if field == F_FLAGS else np.float64
        a = np.ascontiguousarray(values, dtype=dtype).reshape(self.shape)
        self.lib.oracle_set_grid(self.h, field, a.ctypes.data_as(C.c_void_p))

    def fluid_count(self) -> int:
        return self.lib.oracle_fluid_count(self.h)

    def last_iterations(self) -> int:
        return self.lib.oracle_last_iterations(self.h)


def obstacle(kind: int, pos, *, r: float = 0.0, size=(0, 0, 0), speed=(0, 0, 0), prev_pos=None,
             spawn_rate: float = 0.0, spawn_speed: float = 0.0, frac: float = 0.0) -> OracleObstacle:
    o = OracleObstacle()
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
def render_frame(particles, camera, params, width: int, height: int, scene_depth=None):
    """The CPU restatement of the reference's fluid shaders (render_oracle.c).

    particles: (n, 5) float32 records (pos xyz, |v|, density) in the layout of
    fsim_particle_gfx; camera / params: ctypes structures laid out as
    fsim_camera / fsim_render_params.  Returns a dict of images (row 0 at the
    bottom): raw_depth, depth, thickness (H, W) and normal_depth, color (H, W, 4).
    """
    lib = _load(PORT_LIB)
    fn = lib.render_oracle_frame
    fn.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    pts = np.ascontiguousarray(particles, np.float32).reshape(-1, 5)
    out = {"raw_depth": np.empty((height, width), np.float32), "depth": np.empty((height, width), np.float32),
           "thickness": np.empty((height, width), np.float32),
           "normal_depth": np.empty((height, width, 4), np.float32),
           "color": np.empty((height, width, 4), np.float32)}
    sc = None if scene_depth is None else np.ascontiguousarray(scene_depth, np.float32)
    rc = fn(pts.ctypes.data if pts.size else None, pts.shape[0], C.addressof(camera), C.addressof(params),
            None if sc is None else sc.ctypes.data, width, height, out["raw_depth"].ctypes.data,
            out["depth"].ctypes.data, out["thickness"].ctypes.data, out["normal_depth"].ctypes.data,
            out["color"].ctypes.data)
    if rc != 0:
        raise RuntimeError(f"render_oracle_frame failed: {rc}")
    return out
