"""The kernels' prologue and per-bin arithmetic, compiled for the host
(tests/native/host_check.cpp), against the oracle.  Runs without a GPU."""
import ctypes

import numpy as np
import pytest

from gw_analysis_tools_gb300 import workloads as W


@pytest.fixture(scope="module")
def setup3(oracle):
    f = W.config1_grid()
    src = W.config1_source()
    T = 1.0 / (f[1] - f[0])
    dets = list(W.DETECTORS3)
    injp = oracle.params_from_dict(dict(src, tc=T - src["tc"]))
    data = []
    for i, d in enumerate(dets):
        r = oracle.detector_response(f, injp, d)
        dt = oracle.dtoa(src["RA"], src["DEC"], src["gmst"], dets[0], d)
        data.append(r * np.exp(1j * (-2 * np.pi * dt) * f) + W.noise(f, 100 + i))
    psd = [W.analytic_psd(f)] * 3
    return f, T, dets, data, psd


def _call(lib_fn, oracle, p, ap, T, f, dets, data, psd):
    idx = (ctypes.c_int * len(dets))(*[oracle.detector_index(d) for d in dets])
    return lib_fn(ctypes.byref(p), ap, T, oracle._dp(f), f.size, len(dets), idx, oracle._ptr_array(data),
                  oracle._ptr_array(psd))


def test_host_waveform_matches_oracle(oracle, hostcheck):
    f = W.config1_grid()
    cases = [(0, W.config1_source()), (1, dict(W.config1_source(), spin1=(0.3, 0.2, 0.3), spin2=(-0.1, 0.4, -0.1)))]
    for ap, d in cases:
        p = oracle.params_from_dict(d)
        a = oracle.fourier_waveform(f, p, ap)
        hp = np.zeros(f.size, complex)
        hc = np.zeros(f.size, complex)
        hostcheck.gwh_waveform(oracle._dp(f), f.size, oracle._dp(hp), oracle._dp(hc), ap, ctypes.byref(p))
        for x, y in ((a[0], hp), (a[1], hc)):
            assert np.max(np.abs(x - y)) <= 1e-13 * np.abs(x).max()


def test_host_fp64_loglik_matches_oracle(oracle, hostcheck, setup3):
    f, T, dets, data, psd = setup3
    for ap, draws in ((0, W.prior_draws(16, 7)), (1, W.prior_draws(8, 11, precessing=True))):
        for d in draws:
            p = oracle.params_from_dict(d)
            ref = oracle.loglik(p, f, dets, data, psd, approximant=ap)
            got = _call(hostcheck.gwh_loglik_fp64, oracle, p, ap, T, f, dets, data, psd)
            assert abs(got - ref) <= 1e-9 * max(1.0, abs(ref))


def test_host_mixed_loglik_within_tolerance(oracle, hostcheck, setup3):
    """Mixed form: |delta log L| <= 1e-3 absolute against the FP64 oracle."""
    f, T, dets, data, psd = setup3
    worst = 0.0
    for ap, draws in ((0, [W.config1_source()] + W.prior_draws(40, 7)), (1, W.prior_draws(20, 11, precessing=True))):
        for d in draws:
            p = oracle.params_from_dict(d)
            ref = oracle.loglik(p, f, dets, data, psd, approximant=ap)
            got = _call(hostcheck.gwh_loglik_mixed, oracle, p, ap, T, f, dets, data, psd)
            worst = max(worst, abs(got - ref))
    assert worst <= 1e-3, worst


def test_host_mixed_pv2_precession_cone_through_zero(oracle, hostcheck, setup3):
    """Pv2 draws where L + S_L changes sign on the grid (high mass ratio, anti-
    aligned primary spin): cos(beta) = 1/sqrt(1 + s^2) stays positive."""
    f, T, dets, data, psd = setup3
    draws = W.prior_draws(40, 22, precessing=True)
    worst = 0.0
    for d in draws[18:24]:
        p = oracle.params_from_dict(d)
        ref = oracle.loglik(p, f, dets, data, psd, approximant=1)
        got = _call(hostcheck.gwh_loglik_mixed, oracle, p, 1, T, f, dets, data, psd)
        worst = max(worst, abs(got - ref))
    assert worst <= 1e-3, worst


def test_host_internals_match_oracle(oracle, hostcheck):
    for d in W.prior_draws(10, 5):
        p = oracle.params_from_dict(d)
        a = np.zeros(32)
        b = np.zeros(32)
        oracle.lib().gwo_d_internals(ctypes.byref(p), oracle._dp(a))
        hostcheck.gwh_d_internals(ctypes.byref(p), oracle._dp(b))
        # The kernels form integer and rational powers by products and cube
        # roots where the reference calls pow; the C1-matching coefficients
        # (deltas, alpha, beta) amplify that last-bit difference to ~1e-12.
        np.testing.assert_allclose(b[:21], a[:21], rtol=2e-11, atol=0)


def test_host_batched_fisher_algebra_matches_oracle(oracle, hostcheck):
    """Moment-form batched Fisher (amplitude/phase differences) against the
    reference algorithm (complex central differences) in the oracle."""
    dp = ctypes.POINTER(ctypes.c_double)
    hostcheck.gwh_fisher_batch.argtypes = [ctypes.c_void_p, ctypes.c_int, dp, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_int, dp, dp]
    f = W.uniform_grid(10.0, 2048.0, 1 / 16.)
    dets = list(W.DETECTORS3)
    psd = [W.analytic_psd(f)] * 3
    idx = (ctypes.c_int * 3)(*[oracle.detector_index(d) for d in dets])
    for eps, mode, tol in ((1e-6, 1, 1e-5), (1e-8, 0, 1e-3)):
        for d in W.prior_draws(3, 77):
            p = oracle.params_from_dict(d)
            ref = oracle.fisher_network(f, p, dets, psd, epsilon=eps, step_mode=mode)
            out = np.zeros(121)
            cov = np.zeros(121)
            hostcheck.gwh_fisher_batch(ctypes.byref(p), 0, oracle._dp(f), f.size, 3, idx, oracle._ptr_array(psd), eps,
                                       mode, oracle._dp(out), oracle._dp(cov))
            G = out.reshape(11, 11)
            rel = np.abs(G - ref) / np.sqrt(np.outer(np.diag(ref), np.diag(ref)))
            assert rel.max() <= tol, (eps, rel.max())


def test_host_five_point_moment_form_matches_oracle(oracle, hostcheck):
    """The moment form at order 4 on the host (the product's fisher_setup
    with the five-point coefficients kappa a + c G, kappa b, kappa G) against
    the oracle's order-4 network Fisher, which evaluates the +-2 eps responses
    with the reference's constant phase at the non-reference detectors;
    both parameterisations and both step rules."""
    dp = ctypes.POINTER(ctypes.c_double)
    fn = hostcheck.gwh_fisher_batch_order
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, dp, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                   ctypes.c_void_p, ctypes.c_double, ctypes.c_int, dp, dp]
    f = W.uniform_grid(10.0, 512.0, 1 / 8.)
    dets = list(W.DETECTORS3)
    psd = [W.analytic_psd(f)] * 3
    idx = (ctypes.c_int * 3)(*[oracle.detector_index(d) for d in dets])
    checked = 0
    for method, name in ((0, "IMRPhenomD"), (1, "MCMC_IMRPhenomD")):
        for eps, mode, tol in ((1e-6, 1, 2e-5), (1e-8, 0, 1e-3)):
            for d in W.prior_draws(3, 79):
                p = oracle.params_from_dict(d)
                out = np.zeros(121)
                st = fn(ctypes.byref(p), method, 4, oracle._dp(f), f.size, 3, idx, oracle._ptr_array(psd), eps, mode,
                        oracle._dp(out), None)
                if st == 10:  # left to the reference algorithm
                    continue
                assert st == 0
                ref = oracle.fisher_network(f, p, dets, psd, method=name, order=4, epsilon=eps, step_mode=mode)
                G = out.reshape(11, 11)
                rel = np.abs(G - ref) / np.sqrt(np.outer(np.diag(ref), np.diag(ref)))
                assert rel.max() <= tol, (name, eps, rel.max())
                checked += 1
    assert checked >= 10


def test_fisher_pair_differences_every_bin(hostcheck):
    """The batched Fisher's per-bin intrinsic differences (the
    coefficient-difference polynomials, fisher_phase_deriv / fisher_amp_deriv
    and their series in the half phase step) against the pair's two waveforms
    taken bin by bin, over every bin of the benchmark grid: across the
    inspiral / intermediate / ringdown boundaries of both waveforms, past the
    cut f = 0.2/M, one-sided pairs at eta = 1/4, both step rules."""
    import ctypes
    import numpy as np
    import gw_analysis_tools_gb300 as G
    from gw_analysis_tools_gb300 import workloads as W
    fn = hostcheck.gwh_fisher_pair_check
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                   ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    df, n0, N = 1.0 / 16, 160, 32608
    pool = W.prior_draws(10000, 13)
    draws = W.prior_draws(24, 91) + [pool[i] for i in (228, 284, 4213, 6931)]
    draws.append(dict(W.config1_source(), mass1=30.0, mass2=30.0))  # eta = 1/4: one-sided pair
    worst = {1: 0.0, 0: 0.0}
    for d in draws:
        for method in (0, 1):
            for eps, mode in ((1e-6, 1), (1e-8, 0)):
                e = (ctypes.c_double * 4)()
                assert fn(ctypes.byref(G.gen_params(**d)), method, df, n0, N, eps, mode, e) == 0
                worst[mode] = max(worst[mode], max(e))
    # relative steps: FP32 results of FP64 differences, a few ulp of the
    # pair's largest value.  The reference's 1e-8 absolute step moves M_c by
    # ~3e-10 of itself, so the two-waveform difference used as the yardstick
    # carries its own rounding, ~1e-16 |Phi| over a phase step of ~1e-6 rad.
    assert worst[1] <= 3e-6, worst
    assert worst[0] <= 2e-5, worst
