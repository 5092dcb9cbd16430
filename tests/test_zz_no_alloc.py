"""fsim_p2g_noalloc: the particle-to-grid transfer for callers that may not
allocate GPU memory (see include/fsim.h).  It must give the same grid as the
context path (fsim_stage FSIM_STAGE_P2G) on the same particles, call after
call, although its scratch array keeps the previous call's contents.

Collected last on purpose (file name), so a run that stops at the first
failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

from fluid_simulator_gb300 import native as N
from fluid_simulator_gb300.scenes import GridSpec, dam_break

from parity_util import REL_GRID, assert_close_field

pytestmark = pytest.mark.gpu


def cudart():
    for name in ("libcudart.so.13", "libcudart.so"):
        try:
            return C.CDLL(name)
        except OSError:
            pass
    import glob

    return C.CDLL(sorted(glob.glob("/usr/local/cuda/lib64/libcudart.so*"))[0])


class DeviceBuffers:
    """Caller-owned device memory (the test is the caller that allocates)."""

    def __init__(self, rt):
        self.rt = rt
        self.ptrs = []

    def alloc(self, nbytes):
        p = C.c_void_p()
        assert self.rt.cudaMalloc(C.byref(p), C.c_size_t(max(1, nbytes))) == 0
        self.ptrs.append(p)
        return p

    def upload(self, arr):
        arr = np.ascontiguousarray(arr)
        p = self.alloc(arr.nbytes)
        assert self.rt.cudaMemcpy(p, arr.ctypes.data_as(C.c_void_p), C.c_size_t(arr.nbytes), 1) == 0
        return p

    def download(self, p, shape, dtype):
        out = np.empty(shape, dtype)
        assert self.rt.cudaMemcpy(out.ctypes.data_as(C.c_void_p), p, C.c_size_t(out.nbytes), 2) == 0
        return out

    def free(self):
        for p in self.ptrs:
            self.rt.cudaFree(p)
        self.ptrs = []


def particles(seed, res=32):
    pos = dam_break(GridSpec(res), (0, 0, 0), (0.5, 0.6, 1.0), seed=seed)
    rng = np.random.default_rng(seed)
    vel = rng.uniform(-1.0, 1.0, pos.shape).astype(np.float32)
    c = rng.uniform(-2.0, 2.0, (pos.shape[0], 9)).astype(np.float32)
    return pos, vel, c


def context_p2g(pos, vel, c, transfer, res=32):
    sim = N.Simulation(res, N.default_params(transfer=transfer, resolution=res))
    sim.set_particles(pos, vel, c)
    sim.stage(N.STAGE_P2G, 1.0 / 120)
    out = {f: sim.grid(f) for f in (N.F_FLAGS, N.F_AVGPNUM, N.F_VX, N.F_VY, N.F_VZ)}
    sim.close()
    return out


def noalloc_p2g(lib, rt, pos, vel, c, transfer, res=32):
    n = pos.shape[0]
    g = N.GridDesc()
    g.dims[:] = [1.0, 1.0, 1.0]
    g.resolution = res
    g.two_d = 0
    shape = (res, res, res)
    ncell = res ** 3
    buf = DeviceBuffers(rt)
    try:
        # SoA planes: component a of particle i at a*n + i
        dpos = buf.upload(pos.T.copy())
        dvel = buf.upload(vel.T.copy())
        dc = buf.upload(c.T.copy())
        outs = [buf.alloc(ncell * 4) for _ in range(3)]
        dflags = buf.alloc(ncell)
        davg = buf.alloc(ncell * 4)
        rc = lib.fsim_p2g_noalloc(C.byref(g), transfer, dpos, dvel, dc, n, outs[0], outs[1], outs[2], dflags,
                                  davg, None)
        assert rc == 0, N.ERRORS.get(rc, rc)
        assert rt.cudaDeviceSynchronize() == 0
        # the caller's particle buffers are inputs only: the call leaves them as they were
        assert np.array_equal(buf.download(dpos, (3, n), np.float32), pos.T)
        assert np.array_equal(buf.download(dvel, (3, n), np.float32), vel.T)
        assert np.array_equal(buf.download(dc, (9, n), np.float32), c.T)
        return {N.F_VX: buf.download(outs[0], shape, np.float32), N.F_VY: buf.download(outs[1], shape, np.float32),
                N.F_VZ: buf.download(outs[2], shape, np.float32), N.F_FLAGS: buf.download(dflags, shape, np.uint8),
                N.F_AVGPNUM: buf.download(davg, shape, np.float32)}
    finally:
        buf.free()


def compare(got, want):
    assert np.array_equal(got[N.F_FLAGS], want[N.F_FLAGS])
    for f, name in ((N.F_VX, "vx"), (N.F_VY, "vy"), (N.F_VZ, "vz"), (N.F_AVGPNUM, "avgPNum")):
        assert_close_field(got[f], want[f], REL_GRID, name)


def test_noalloc_p2g_matches_context_path_twice(gpu):
    lib = N.load_library()
    rt = cudart()
    # first call: APIC; second call: other particles (different count), FLIP --
    # the second result must not see the first call's scratch contents
    for seed, transfer in ((11, N.APIC), (12, N.FLIP)):
        pos, vel, c = particles(seed)
        if seed == 12:
            pos, vel, c = pos[:-777], vel[:-777], c[:-777]
        want = context_p2g(pos, vel, c, transfer)
        got = noalloc_p2g(lib, rt, pos, vel, c, transfer)
        compare(got, want)


def test_noalloc_rejects_sizes_above_capacity(gpu):
    lib = N.load_library()
    g = N.GridDesc()
    g.dims[:] = [1.0, 1.0, 1.0]
    g.two_d = 0
    g.resolution = 128  # 128^3 cells > FSIM_NOALLOC_MAX_CELLS
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = lib.fsim_p2g_noalloc(C.byref(g), N.FLIP, dummy, dummy, None, 1000, dummy, dummy, dummy, dummy, dummy, None)
    assert N.ERRORS[rc] == "CAPACITY"
    g.resolution = 32
    rc = lib.fsim_p2g_noalloc(C.byref(g), N.FLIP, dummy, dummy, None, (1 << 20) + 1, dummy, dummy, dummy, dummy,
                              dummy, None)
    assert N.ERRORS[rc] == "CAPACITY"
