"""The C ABI library loads and exports every symbol include/gwgpu.h declares
(no compute call: runs without a GPU)."""
import ctypes
import os

from gw_analysis_tools_gb300 import _native


def test_library_builds_and_exports_declared_symbols():
    lib = _native.build()
    assert os.path.exists(lib)
    L = ctypes.CDLL(lib)
    declared = _native.exported_symbols()
    assert len(declared) >= 20
    missing = [s for s in declared if not hasattr(L, s)]
    assert not missing, missing


def test_python_layer_declares_every_symbol():
    L = _native.load()
    for s in _native.exported_symbols():
        fn = getattr(L, s)
        assert fn.argtypes is not None or fn.restype is not None, s


def test_status_strings():
    L = _native.load()
    assert L.gwgpu_status_string(0) == b"ok"
    assert b"budget" in L.gwgpu_status_string(3)
