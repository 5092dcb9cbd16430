import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built libfsim.so")
    config.addinivalue_line("markers", "slow: long-running case")


@pytest.fixture(scope="session")
def port_lib():
    """Build oracle/liboracle.so (the FP64 C restatement) once per session."""
    from oracle import oracle as O

    return O.build_port()


def _gpu_available() -> bool:
    try:
        import ctypes

        rt = ctypes.CDLL("libcudart.so")
    except OSError:
        try:
            import glob

            cands = glob.glob("/usr/local/cuda/lib64/libcudart.so*")
            rt = ctypes.CDLL(cands[0]) if cands else None
        except OSError:
            rt = None
    if rt is None:
        return False
    n = ctypes.c_int(0)
    return rt.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0


@pytest.fixture(scope="session")
def gpu():
    """The built CUDA library; GPU tests fail (not skip) when it cannot load on a machine with a GPU."""
    if not _gpu_available():
        pytest.skip("no CUDA device visible")
    from fluid_simulator_gb300 import _build, native

    _build.build_library()
    return native.load_library()
