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


def test_dropin_library_exports_reference_signatures():
    """libgwat_dropin.so loads and defines the reference-signature C++ entry
    points declared in include/gwat_dropin.h."""
    import shutil
    import subprocess
    _native.build()
    L = ctypes.CDLL(_native.DROPIN_LIB)
    assert hasattr(L, "gwat_dropin_test_loglik")
    if shutil.which("nm") is None:
        return
    out = subprocess.run(["nm", "-DC", "--defined-only", _native.DROPIN_LIB], capture_output=True, text=True).stdout
    for name in ("MCMC_likelihood_extrinsic(bool, gen_params_base<double>*", "Log_Likelihood_internal(",
                 "fourier_waveform(double*, int, std::complex<double>*", "fourier_waveform<double>(",
                 "fourier_detector_response<double>(", "fisher_numerical(double*, int",
                 "maximized_Log_Likelihood_aligned_spin_internal(std::complex<double>*",
                 "maximized_Log_Likelihood_unaligned_spin_internal(std::complex<double>*",
                 "allocate_LOSC_data(std::", "read_LOSC_data_file(std::", "read_LOSC_PSD_file(std::",
                 "populate_noise(double*", "count_lines_LOSC_data_file(std::"):
        assert name in out, name
