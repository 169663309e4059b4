"""The likelihood maximised over arrival time and phase
(maximized_Log_Likelihood_aligned_spin_internal, mcmc_gw.cpp:595-658) and the
sampler's intrinsic mode (mcmc_gw.cpp:2611-2631) against the oracle (numpy's
DFT in place of FFTW's)."""
import numpy as np
import pytest

import gw_analysis_tools_gb300 as G
from gw_analysis_tools_gb300 import workloads as W

pytestmark = pytest.mark.gpu
RTOL = 1e-9


@pytest.fixture(scope="module")
def setup(oracle):
    f = W.uniform_grid(20.0, 512.0, 1.0 / 8.0)
    src = W.config1_source()
    dets = list(W.DETECTORS3)
    injp = oracle.params_from_dict(dict(src, tc=3.0))
    psd = W.analytic_psd(f)
    data = [oracle.detector_response(f, injp, d) + W.noise(f, 80 + i) for i, d in enumerate(dets)]
    return dict(f=f, src=src, dets=dets, psd=psd, data=data)


def test_maximized_internal(gpu_ctx, oracle, setup):
    s = setup
    for d in [s["src"]] + W.prior_draws(4, 81):
        r = oracle.detector_response(s["f"], oracle.params_from_dict(d), "Livingston")
        ref = oracle.maximized_loglik_internal(s["data"][1], s["psd"], s["f"], r)
        got = gpu_ctx.maximized_log_likelihood_internal(s["data"][1], s["psd"], s["f"], r)
        assert abs(got - ref) <= RTOL * max(1.0, abs(ref)), (got, ref)


def test_maximized_intrinsic_batch(gpu_ctx, oracle, setup):
    s = setup
    hs = [gpu_ctx.register_data(d, s["f"], s["data"][i], s["psd"]) for i, d in enumerate(s["dets"])]
    draws = [s["src"]] + W.prior_draws(47, 82)
    out, st = gpu_ctx.maximized_loglik_batch(G.params_array(draws), hs)
    assert np.all(st == 0)
    ref = np.array([oracle.maximized_loglik_intrinsic(d, s["f"], s["data"], [s["psd"]] * 3) for d in draws])
    assert np.all(np.abs(out - ref) <= RTOL * np.maximum(1.0, np.abs(ref))), np.max(np.abs(out - ref) / np.abs(ref))
    # the injected source is the best of the draws
    assert np.argmax(out) == 0


def test_maximized_unaligned_internal(gpu_ctx, oracle, setup):
    s = setup
    for d in W.prior_draws(5, 83, precessing=True):
        hp, hc = oracle.fourier_waveform(s["f"], oracle.params_from_dict(d), oracle.IMRPhenomPv2)
        ref = oracle.maximized_loglik_unaligned_internal(s["data"][0], s["psd"], s["f"], hp, hc)
        got = gpu_ctx.maximized_log_likelihood_unaligned_internal(s["data"][0], s["psd"], s["f"], hp, hc)
        assert abs(got - ref) <= RTOL * max(1.0, abs(ref)), (got, ref)


def test_maximized_intrinsic_batch_pv2(gpu_ctx, oracle, setup):
    s = setup
    hs = [gpu_ctx.register_data(d, s["f"], s["data"][i], s["psd"]) for i, d in enumerate(s["dets"])]
    draws = W.prior_draws(33, 84, precessing=True)
    out, st = gpu_ctx.maximized_loglik_batch(G.params_array(draws), hs, approximant=G.IMRPhenomPv2)
    assert np.all(st == 0)
    ref = np.array([oracle.maximized_loglik_intrinsic(d, s["f"], s["data"], [s["psd"]] * 3, oracle.IMRPhenomPv2)
                    for d in draws])
    assert np.all(np.abs(out - ref) <= RTOL * np.maximum(1.0, np.abs(ref))), np.max(np.abs(out - ref) / np.abs(ref))


def test_maximized_batch_bad_request(gpu_ctx, oracle, setup):
    s = setup
    hs = [gpu_ctx.register_data(d, s["f"], s["data"][i], s["psd"]) for i, d in enumerate(s["dets"])]
    draws = W.prior_draws(3, 85)
    draws[1] = dict(draws[1], mass1=float("nan"))   # outside the model domain
    out, st = gpu_ctx.maximized_loglik_batch(G.params_array(draws), hs)
    assert st[0] == 0 and st[2] == 0 and st[1] != 0
    assert np.isnan(out[1]) and np.all(np.isfinite(out[[0, 2]]))


def test_maximized_through_reference_signatures(oracle, setup):
    """maximized_Log_Likelihood_{aligned,unaligned}_spin_internal of the C++
    drop-in (the reference's argument lists; the FFTW plan argument unused)."""
    import ctypes
    from gw_analysis_tools_gb300 import _native
    _native.build()
    L = ctypes.CDLL(_native.DROPIN_LIB)
    fn = L.gwat_dropin_test_maxll
    fn.restype = ctypes.c_double
    fn.argtypes = [ctypes.c_void_p] * 5 + [ctypes.c_int]
    s = setup
    d = W.prior_draws(1, 86, precessing=True)[0]
    hp, hc = oracle.fourier_waveform(s["f"], oracle.params_from_dict(d), oracle.IMRPhenomPv2)
    hp, hc = np.ascontiguousarray(hp), np.ascontiguousarray(hc)
    data, psd, f = s["data"][2], s["psd"], s["f"]
    got_a = fn(data.ctypes.data, psd.ctypes.data, f.ctypes.data, hp.ctypes.data, None, f.size)
    got_u = fn(data.ctypes.data, psd.ctypes.data, f.ctypes.data, hp.ctypes.data, hc.ctypes.data, f.size)
    ref_a = oracle.maximized_loglik_internal(data, psd, f, hp)
    ref_u = oracle.maximized_loglik_unaligned_internal(data, psd, f, hp, hc)
    assert abs(got_a - ref_a) <= RTOL * abs(ref_a) and abs(got_u - ref_u) <= RTOL * abs(ref_u)


@pytest.mark.parametrize("nbins", [4000, 4096, 2 * 3 * 5 * 7 * 11])
def test_maximized_transform_paths(gpu_ctx, oracle, nbins):
    """Grid lengths with only factors up to 7 go through cuFFT directly, others
    (here 2310 = 2*3*5*7*11; the fixture's 3937 = 31*127) through Bluestein."""
    f = 20.0 + np.arange(nbins) / 8.0
    psd = W.analytic_psd(f)
    d = W.prior_draws(2, 87)
    data = oracle.detector_response(f, oracle.params_from_dict(d[0]), "Hanford") + W.noise(f, 88)
    r = oracle.detector_response(f, oracle.params_from_dict(d[1]), "Hanford")
    hp, hc = oracle.fourier_waveform(f, oracle.params_from_dict(d[1]), oracle.IMRPhenomD)
    ref = oracle.maximized_loglik_internal(data, psd, f, r)
    got = gpu_ctx.maximized_log_likelihood_internal(data, psd, f, r)
    assert abs(got - ref) <= RTOL * max(1.0, abs(ref)), (got, ref)
    ref = oracle.maximized_loglik_unaligned_internal(data, psd, f, hp, hc * (1 + 0.3j))
    got = gpu_ctx.maximized_log_likelihood_unaligned_internal(data, psd, f, hp, hc * (1 + 0.3j))
    assert abs(got - ref) <= RTOL * max(1.0, abs(ref)), (got, ref)


@pytest.fixture(scope="module")
def fp64_ctx():
    """A context whose maximised likelihood uses FP64 transforms only."""
    import os
    old = os.environ.get("GWGPU_MAXLL")
    os.environ["GWGPU_MAXLL"] = "fp64"
    try:
        ctx = G.Context(0)
    finally:
        if old is None:
            del os.environ["GWGPU_MAXLL"]
        else:
            os.environ["GWGPU_MAXLL"] = old
    yield ctx
    ctx.close()


@pytest.mark.parametrize("approx", [G.IMRPhenomD, G.IMRPhenomPv2])
def test_search_path_matches_fp64_transforms(gpu_ctx, fp64_ctx, setup, approx):
    """The FP32 search with FP64 refinement gives the maximum of the FP64
    transforms: same values, draws near the injection and far from it."""
    s = setup
    prec = approx == G.IMRPhenomPv2
    draws = [dict(s["src"], spin1=(0.1, 0.0, 0.2), spin2=(0.0, 0.1, 0.1)) if prec else s["src"]]
    draws += W.perturbed(draws[0], 20, 89, frac=0.002) + W.prior_draws(43, 90, precessing=prec)
    outs = []
    for ctx in (gpu_ctx, fp64_ctx):
        hs = [ctx.register_data(d, s["f"], s["data"][i], s["psd"]) for i, d in enumerate(s["dets"])]
        out, st = ctx.maximized_loglik_batch(G.params_array(draws), hs, approximant=approx)
        assert np.all(st == 0)
        outs.append(out)
    assert np.all(np.abs(outs[0] - outs[1]) <= 1e-10 * np.abs(outs[1])), np.max(np.abs(outs[0] - outs[1]) / np.abs(outs[1]))


def test_flat_spectrum_takes_the_fp64_transforms(gpu_ctx, oracle, setup):
    """Zero data: every bin scores the same, so a pair has more candidates
    than the FP32 search keeps and the batch goes to the FP64 transforms; the
    result is the oracle's (zero) all the same, for both forms."""
    s = setup
    zero = np.zeros(s["f"].size, dtype=np.complex128)
    d = W.prior_draws(1, 91, precessing=True)[0]
    hp, hc = oracle.fourier_waveform(s["f"], oracle.params_from_dict(d), oracle.IMRPhenomPv2)
    got = gpu_ctx.maximized_log_likelihood_internal(zero, s["psd"], s["f"], hp)
    assert got == oracle.maximized_loglik_internal(zero, s["psd"], s["f"], hp) == 0.0
    got_u = gpu_ctx.maximized_log_likelihood_unaligned_internal(zero, s["psd"], s["f"], hp, hc)
    ref_u = oracle.maximized_loglik_unaligned_internal(zero, s["psd"], s["f"], hp, hc)
    assert abs(got_u - ref_u) <= 1e-12 and abs(ref_u) <= 1e-12
    hs = [gpu_ctx.register_data(det, s["f"], zero, s["psd"]) for det in s["dets"]]
    out, st = gpu_ctx.maximized_loglik_batch(G.params_array(W.prior_draws(5, 92)), hs)
    assert np.all(st == 0) and np.all(out == 0.0)
