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


def test_orientation_transform_host_code(oracle):
    """gwgpu_transform_orientation_coords (host code, no launch) against the
    oracle's transform_orientation_coords, which is pinned bit for bit to the
    reference's (tests/test_oracle_pins.py)."""
    import numpy as np
    import gw_analysis_tools_gb300 as G
    from gw_analysis_tools_gb300 import workloads as W
    rng = np.random.Generator(np.random.PCG64(5))
    for ap, name, prec in ((0, "IMRPhenomD", False), (1, "IMRPhenomPv2", True)):
        for d in W.prior_draws(16, 6, precessing=prec):
            d = dict(d, theta_l=float(np.arccos(rng.uniform(-1, 1))), phi_l=float(rng.uniform(0, 2 * np.pi)),
                     equatorial_orientation=1)
            if prec and rng.uniform() < 0.5:
                d.update(chip=float(rng.uniform(0.1, 0.7)), phip=float(rng.uniform(0, 2 * np.pi)))
            want = oracle.transform_orientation_coords(oracle.params_from_dict(d), ap)
            got = G.transform_orientation_coords(G.gen_params(**d), name)
            assert abs(got.psi - want.psi) <= 1e-12 and abs(got.incl_angle - want.incl_angle) <= 1e-12


def test_dropin_compiles_against_reference_headers(oracle):
    """gwat_dropin.cpp compiled with the reference's own headers
    (GWAT_DROPIN_USE_REFERENCE_HEADERS) against oracle/shim: the drop-in's
    definitions match the reference declarations they replace."""
    import shutil
    import subprocess
    import pytest
    ref = oracle.reference_dir()
    if ref is None or shutil.which("g++") is None:
        pytest.skip("reference headers not present")
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    src = os.path.join(root, "gw_analysis_tools_gb300", "dropin", "gwat_dropin.cpp")
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-w", "-DGWAT_DROPIN_USE_REFERENCE_HEADERS",
           "-include", "util.h", "-include", "waveform_generator.h", "-include", "mcmc_gw.h",
           "-I", os.path.join(root, "oracle", "shim"), "-I", os.path.join(ref, "include", "gwat"), src]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
