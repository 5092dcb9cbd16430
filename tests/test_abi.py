"""CPU checks of the drop-in boundary: the C ABI library builds for sm_103a,
loads, and exports every function include/fsim.h declares; the ctypes
structures match the header's layout."""
import ctypes as C
import os
import re

import pytest

from fluid_simulator_gb300 import native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", h) for h in ("fsim.h", "fsim_render.h")]


def declared_functions():
    names = set()
    for h in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        names |= set(re.findall(r"\b(fsim_[a-z_0-9]+)\s*\(", text))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from fluid_simulator_gb300 import _build

    _build.build_library()
    # loading needs only the CUDA runtime, not a GPU
    return C.CDLL(native.LIB_PATH)


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n


def test_binding_covers_header():
    assert sorted(native.EXPORTS) == declared_functions()


def test_struct_sizes_match_header(tmp_path):
    """Compile a tiny C program against fsim.h and compare sizeof/offsetof."""
    src = tmp_path / "sz.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "fsim.h"\n#include "fsim_render.h"\n'
        "int main(){printf(\"%zu %zu %zu %zu %zu %zu %zu\\n\", sizeof(fsim_params), sizeof(fsim_obstacle),"
        " sizeof(fsim_step_stats), sizeof(fsim_grid_desc), sizeof(fsim_particle_gfx),"
        " offsetof(fsim_params, residual_tol), offsetof(fsim_step_stats, ms_total));"
        "printf(\"%zu %zu %zu %zu\\n\", sizeof(fsim_camera), sizeof(fsim_render_params),"
        " offsetof(fsim_render_params, lights), offsetof(fsim_render_params, background));return 0;}\n")
    exe = tmp_path / "sz"
    os.system(f"gcc -I{ROOT}/include {src} -o {exe}")
    out = os.popen(str(exe)).read().split()
    got = [int(x) for x in out]
    want = [C.sizeof(native.Params), C.sizeof(native.Obstacle), C.sizeof(native.StepStats),
            C.sizeof(native.GridDesc), C.sizeof(native.ParticleGfx),
            native.Params.residual_tol.offset, native.StepStats.ms_total.offset,
            C.sizeof(native.Camera), C.sizeof(native.RenderParams), native.RenderParams.lights.offset,
            native.RenderParams.background.offset]
    assert got == want



def test_noalloc_rejects_wrapping_grid_sizes_before_any_cuda_call(lib):
    """fsim_p2g_noalloc bounds each axis before forming the cell count: dims whose
    product of cells would wrap a 64-bit count are a capacity error, and
    non-finite dims are invalid.  Both are decided before any CUDA call, so this
    runs without a GPU."""
    f = lib.fsim_p2g_noalloc
    f.restype = C.c_int
    f.argtypes = [C.POINTER(native.GridDesc), C.c_int] + [C.c_void_p] * 3 + [C.c_int64] + [C.c_void_p] * 6
    dummy = C.c_void_p(16)  # never dereferenced
    g = native.GridDesc()
    g.two_d = 0
    g.resolution = 1.0
    g.dims[:] = [float(1 << 22), float(1 << 21), float(1 << 21)]  # 2^64 cells: wraps to 0 in 64-bit integers
    rc = f(C.byref(g), native.FLIP, dummy, dummy, None, 10, dummy, dummy, dummy, dummy, dummy, None)
    assert native.ERRORS[rc] == "CAPACITY"
    g.dims[:] = [1e300, 1.0, 1.0]
    rc = f(C.byref(g), native.FLIP, dummy, dummy, None, 10, dummy, dummy, dummy, dummy, dummy, None)
    assert native.ERRORS[rc] == "CAPACITY"
    g.dims[:] = [float("nan"), 1.0, 1.0]
    rc = f(C.byref(g), native.FLIP, dummy, dummy, None, 10, dummy, dummy, dummy, dummy, dummy, None)
    assert native.ERRORS[rc] == "INVALID"
    g.dims[:] = [1.0, 1.0, 1.0]
    g.resolution = float("inf")
    rc = f(C.byref(g), native.FLIP, dummy, dummy, None, 10, dummy, dummy, dummy, dummy, dummy, None)
    assert native.ERRORS[rc] == "INVALID"
