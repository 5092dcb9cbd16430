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

