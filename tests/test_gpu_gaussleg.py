"""The GAUSSLEG integration of Log_Likelihood_internal (mcmc_gw.cpp:820-833,
843-862) against the oracle: weighted streams on a Gauss-Legendre grid in the
FP64 forms (plain, batched, the C++ drop-in), log10F, and a weighted stream on
a uniform grid in the mixed form."""
import ctypes

import numpy as np
import pytest

import gw_analysis_tools_gb300 as G
from gw_analysis_tools_gb300 import _native, workloads as W

pytestmark = pytest.mark.gpu
FP64_RTOL = 1e-9
MIXED_TOL = 1e-3


def gl_grid(n, f0, f1):
    x, w = np.polynomial.legendre.leggauss(n)
    h = 0.5 * (f1 - f0)
    return f0 + h * (x + 1.0), w * h


@pytest.fixture(scope="module")
def gl(gpu_ctx, oracle):
    f, w = gl_grid(3000, 20.0, 1024.0)
    dets = list(W.DETECTORS3)
    src = W.config1_source()
    T = 8.0
    injp = oracle.params_from_dict(dict(src, tc=T - src["tc"]))
    rng = np.random.default_rng(5)
    psd = W.analytic_psd(f)
    data = []
    for i, d in enumerate(dets):
        r = oracle.detector_response(f, injp, d)
        dt = oracle.dtoa(src["RA"], src["DEC"], src["gmst"], dets[0], d)
        sig = np.sqrt(psd) * 0.05
        data.append(r * np.exp(-2j * np.pi * dt * f) + sig * (rng.standard_normal(f.size) + 1j * rng.standard_normal(f.size)))
    out = dict(f=f, w=w, dets=dets, src=src, T=T, psd=psd, data=data)
    for log10F in (0, 1):
        out["h%d" % log10F] = [gpu_ctx.register_data(d, f, data[i], psd, weights=w, log10F=log10F)
                               for i, d in enumerate(dets)]
    return out


def test_log_likelihood_internal_gaussleg(gpu_ctx, oracle, gl):
    g = gl
    r = oracle.detector_response(g["f"], oracle.params_from_dict(g["src"]), "Hanford")
    for log10F in (0, 1):
        ref = oracle.lib().gwo_log_likelihood_internal_gl(
            oracle._dp(g["data"][0]), oracle._dp(g["psd"]), oracle._dp(g["f"]), oracle._dp(g["w"]),
            oracle._dp(r.view(np.float64).copy()), g["f"].size, log10F)
        got = gpu_ctx.log_likelihood_internal(g["data"][0], g["psd"], g["f"], r, weights=g["w"], log10F=log10F)
        assert abs(got - ref) <= FP64_RTOL * max(1.0, abs(ref)), (got, ref)


def test_plain_and_batched_fp64_gaussleg(gpu_ctx, oracle, gl):
    g = gl
    draws = [g["src"]] + W.perturbed(g["src"], 15, seed=21)
    for log10F in (0, 1):
        hs = g["h%d" % log10F]
        ref = np.array([oracle.loglik_gl(oracle.params_from_dict(d), g["f"], g["dets"], g["data"], [g["psd"]] * 3,
                                         [g["w"]] * 3, log10F=bool(log10F), T_segment=g["T"]) for d in draws])
        plain = np.array([gpu_ctx.mcmc_likelihood_extrinsic(G.gen_params(**d), "IMRPhenomD", hs, g["T"])
                          for d in draws])
        assert np.all(np.abs(plain - ref) <= FP64_RTOL * np.maximum(1.0, np.abs(ref)))
        batch, st = gpu_ctx.loglik_batch(G.params_array(draws), 0, hs, g["T"], G.PREC_FP64)
        assert np.all(st == 0)
        assert np.all(np.abs(batch - ref) <= FP64_RTOL * np.maximum(1.0, np.abs(ref)))
        # the mixed form needs a uniform grid: the requests are refused, not wrong
        _, st = gpu_ctx.loglik_batch(G.params_array(draws[:2]), 0, hs, g["T"], G.PREC_MIXED)
        assert np.all(st != 0)


def test_weighted_uniform_grid_mixed(gpu_ctx, oracle):
    f = W.uniform_grid(20.0, 512.0, 1.0 / 8.0)
    w = np.full(f.size, f[1] - f[0])
    w[0] = w[-1] = 0.5 * (f[1] - f[0])  # trapezoid rule
    dets = list(W.DETECTORS3)
    psd = W.analytic_psd(f)
    data = [W.noise(f, 60 + i) for i in range(3)]
    hs = [gpu_ctx.register_data(d, f, data[i], psd, weights=w) for i, d in enumerate(dets)]
    T = 1.0 / (f[1] - f[0])
    draws = W.prior_draws(24, 61)
    ref = np.array([oracle.loglik_gl(oracle.params_from_dict(d), f, dets, data, [psd] * 3, [w] * 3, T_segment=T)
                    for d in draws])
    got, st = gpu_ctx.loglik_batch(G.params_array(draws), 0, hs, T, G.PREC_MIXED)
    assert np.all(st == 0)
    assert np.max(np.abs(got - ref)) <= MIXED_TOL


def test_dropin_gaussleg(oracle, gl):
    g = gl
    _native.build()
    L = ctypes.CDLL(_native.DROPIN_LIB)
    fn = L.gwat_dropin_test_loglik_gl
    fn.restype = ctypes.c_double
    dp = ctypes.POINTER(ctypes.c_double)
    fn.argtypes = [dp, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                   ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, dp]
    f = np.ascontiguousarray(g["f"])
    n = 3
    dptr = (ctypes.c_void_p * n)(*[d.ctypes.data for d in g["data"]])
    psd = np.ascontiguousarray(g["psd"])
    sptr = (ctypes.c_void_p * n)(*[psd.ctypes.data] * n)
    w = np.ascontiguousarray(g["w"])
    wptr = (ctypes.c_void_p * n)(*[w.ctypes.data] * n)
    names = (ctypes.c_char_p * n)(*[d.encode() for d in g["dets"]])
    for log10F in (0, 1):
        p = G.gen_params(**g["src"])
        tc = np.zeros(2)
        ll = fn(f.ctypes.data_as(dp), f.size, dptr, sptr, wptr, log10F, names, n, ctypes.byref(p),
                tc.ctypes.data_as(dp))
        ref = oracle.loglik_gl(oracle.params_from_dict(g["src"]), f, g["dets"], g["data"], [psd] * 3, [w] * 3,
                               log10F=bool(log10F), T_segment=tc[1])
        assert abs(ll - ref) <= FP64_RTOL * max(1.0, abs(ref)), (ll, ref)
