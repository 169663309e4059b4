import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.build(O.reference_dir())
    return O


@pytest.fixture(scope="session")
def hostcheck():
    """The product's prologue/per-bin headers compiled for the host (test build)."""
    import ctypes
    src = os.path.join(ROOT, "tests", "native", "host_check.cpp")
    lib = os.path.join(ROOT, "tests", "native", "libgwgpu_hostcheck.so")
    csrc = os.path.join(ROOT, "gw_analysis_tools_gb300", "csrc")
    newest = max([os.path.getmtime(src)] + [os.path.getmtime(os.path.join(csrc, f)) for f in os.listdir(csrc)
                                            if f.endswith(".h")])
    if not os.path.exists(lib) or os.path.getmtime(lib) < newest:
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-o", lib, src])
    L = ctypes.CDLL(lib)
    dp = ctypes.POINTER(ctypes.c_double)
    for fn in (L.gwh_loglik_fp64, L.gwh_loglik_mixed):
        fn.restype = ctypes.c_double
        fn.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, dp, ctypes.c_int, ctypes.c_int,
                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    L.gwh_waveform.argtypes = [dp, ctypes.c_int, dp, dp, ctypes.c_int, ctypes.c_void_p]
    L.gwh_d_internals.argtypes = [ctypes.c_void_p, dp]
    return L


@pytest.fixture(scope="session")
def gpu_ctx():
    import gw_analysis_tools_gb300 as G
    from gw_analysis_tools_gb300 import _native
    _native.build()
    ctx = G.Context(0)
    yield ctx
    ctx.close()
