"""The C oracle against the reference itself.

* reference_waveforms.npz holds bins of the reference's own IMRPhenomD.cpp /
  IMRPhenomP.cpp output (tests/golden/make_golden.py); the oracle must agree
  bit for bit (same compiler family, same operation order) or to 1e-14 where
  the platform's libm differs.
* Where the reference sources are present (oracle/_ref built), every case is
  also compared on the full grid and on prior draws, bit for bit.
"""
import ast
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "reference_waveforms.npz")


def test_oracle_matches_reference_golden_vectors(oracle):
    g = np.load(GOLD, allow_pickle=False)
    freqs = 20.0 + np.arange(32128) / 32.0
    idx = g["idx"]
    ncase = len([k for k in g.files if k.endswith("_approx")])
    assert ncase >= 7
    for i in range(ncase):
        ap = int(g["case%d_approx" % i])
        kw = ast.literal_eval(str(g["case%d_params" % i]))
        hp, hc = oracle.fourier_waveform(freqs, oracle.make_params(**kw), ap)
        for got, want in ((hp[idx], g["case%d_hp" % i]), (hc[idx], g["case%d_hc" % i])):
            scale = np.abs(want).max()
            assert scale > 0
            np.testing.assert_allclose(got, want, rtol=0, atol=1e-13 * scale)


def _ref_or_skip(oracle):
    ref = oracle.ref_lib()
    if ref is None:
        if oracle.reference_dir():
            oracle.build(oracle.reference_dir())
            ref = oracle.ref_lib()
    if ref is None:
        pytest.skip("reference sources not present; golden vectors cover this")
    return ref


def test_oracle_bit_exact_against_reference_build(oracle):
    _ref_or_skip(oracle)
    from gw_analysis_tools_gb300 import workloads as W
    freqs = W.config1_grid()
    draws = W.prior_draws(12, 3) + W.prior_draws(12, 4, precessing=True)
    for j, d in enumerate(draws):
        ap = oracle.IMRPhenomD if j < 12 else oracle.IMRPhenomPv2
        p = oracle.params_from_dict(d)
        a = oracle.fourier_waveform(freqs, p, ap)
        b = oracle.fourier_waveform(freqs, p, ap, use_ref=True)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]), "case %d differs" % j


def test_model_internals_match_reference(oracle):
    import ctypes
    ref = _ref_or_skip(oracle)
    from gw_analysis_tools_gb300 import workloads as W
    for d in W.prior_draws(8, 5):
        p = oracle.params_from_dict(d)
        a = np.zeros(32)
        b = np.zeros(32)
        oracle.lib().gwo_d_internals(ctypes.byref(p), oracle._dp(a))
        ref.ref_d_internals(ctypes.byref(p), oracle._dp(b))
        assert np.array_equal(a[:21], b[:21])


# ---- the glue of the path: the reference's own detector, likelihood, sampler
# callback, Fisher and maximised-likelihood code (oracle/_ref/libgwatref_full.so)
GLUE = os.path.join(HERE, "golden", "reference_glue.npz")
PRIOR_DIAG_D = np.array([1 / (4 * np.pi ** 2), 0.25, 1 / (4 * np.pi ** 2), 0.25, 1 / (4 * np.pi ** 2), 100.0, 0.0, 0.0,
                         4.0, 0.25, 0.25])  # MCMC_fisher_transformations, mcmc_gw.cpp:2147-2156


def _close(got, want, rtol=1e-12):
    """Bit-exact on the machine that wrote the fixture; 1e-12 relative covers
    another libm."""
    got, want = np.asarray(got), np.asarray(want)
    scale = max(np.max(np.abs(want)), 1e-300)
    assert np.max(np.abs(got - want)) <= rtol * scale, np.max(np.abs(got - want)) / scale


def test_glue_golden_antenna_dtoa_response(oracle):
    g = np.load(GLUE, allow_pickle=False)
    names = [str(x) for x in g["antenna_dets"]]
    for row, want in zip(g["antenna_in"], g["antenna_out"]):
        _close(oracle.antenna(names[int(row[0])], *row[1:]), want, 1e-14)
    k = 0
    from gw_analysis_tools_gb300 import workloads as W
    for d in W.prior_draws(8, 31):
        for det in ("Hanford", "Livingston", "Virgo"):
            _close(oracle.dtoa(d["RA"], d["DEC"], d["gmst"], "Hanford", det), g["dtoa_out"][k], 1e-14)
            k += 1
    f = g["freqs"]
    for case, want in zip(g["response_cases"], g["response_out"]):
        ap, d, psi_after, incl_after = ast.literal_eval(str(case))
        p = oracle.params_from_dict(d)
        _close(oracle.detector_response(f, p, "Livingston", ap), want)
        if d.get("equatorial_orientation"):
            t = oracle.transform_orientation_coords(p, ap)
            _close([t.psi, t.incl_angle], [psi_after, incl_after], 1e-14)


def test_glue_golden_loglik_and_sampler_callback(oracle):
    g = np.load(GLUE, allow_pickle=False)
    f, psd, data = g["freqs"], g["psd"], list(g["data"])
    dets = ["Hanford", "Livingston", "Virgo"]
    for case, want in zip(g["loglik_cases"], g["loglik_out"]):
        d = ast.literal_eval(str(case))
        ll, T, tc_after = want[:3]
        p = oracle.params_from_dict(d)
        _close(oracle.loglik(p, f, dets, data, [psd] * 3, T_segment=T), ll)
        assert tc_after == T - d["tc"]
        r = oracle.detector_response(f, p, "Hanford")
        _close(oracle.lib().gwo_log_likelihood_internal(oracle._dp(data[0]), oracle._dp(psd), oracle._dp(f),
                                                        oracle._dp(r), f.size), want[3])
        w = np.linspace(0.5, 1.5, f.size) / f.size
        _close(oracle.lib().gwo_log_likelihood_internal_gl(oracle._dp(data[0]), oracle._dp(psd), oracle._dp(f),
                                                           oracle._dp(w), oracle._dp(r), f.size, 1), want[4])
    # MCMC_likelihood_wrapper / MCMC_fisher_wrapper: the arrays of the fixture
    # were laid out back to back, so the reference's T is 1/len(f)
    gmst = float(g["wrapper_gmst"])
    T = 1.0 / f.size
    for pos, ll, fi in zip(g["wrapper_pos_d"], g["wrapper_ll_d"], g["wrapper_fisher_d"]):
        _close(oracle.loglik(oracle.mcmc_repack(pos, oracle.IMRPhenomD, gmst), f, dets, data, [psd] * 3,
                             T_segment=T), ll)
        got = oracle.fisher_network(f, oracle.mcmc_repack(pos, oracle.IMRPhenomD, gmst), dets, [psd] * 3,
                                    method="MCMC_IMRPhenomD", order=4) + np.diag(PRIOR_DIAG_D)
        _close(got, fi)
    for pos, ll in zip(g["wrapper_pos_p"], g["wrapper_ll_p"]):
        _close(oracle.loglik(oracle.mcmc_repack(pos, oracle.IMRPhenomPv2, gmst), f, dets, data, [psd] * 3,
                             approximant=oracle.IMRPhenomPv2, T_segment=T), ll)
    for pos, ll in zip(g["wrapper_pos_i"], g["wrapper_ll_i"]):
        mc, eta = np.exp(pos[0]), pos[1]
        m1 = 0.5 * (mc / eta ** 0.6 + np.sqrt(1 - 4 * eta) * mc / eta ** 0.6)
        m2 = 0.5 * (mc / eta ** 0.6 - np.sqrt(1 - 4 * eta) * mc / eta ** 0.6)
        d = dict(mass1=m1, mass2=m2, spin1=(0, 0, pos[2]), spin2=(0, 0, pos[3]), Luminosity_Distance=100.0)
        _close(oracle.maximized_loglik_intrinsic(d, f, data, [psd] * 3, oracle.IMRPhenomD), ll, 1e-11)


def test_glue_golden_fisher_and_maxll(oracle):
    g = np.load(GLUE, allow_pickle=False)
    f, psd, data = g["freqs"], g["psd"], list(g["data"])
    for case, want in zip(g["fisher_cases"], g["fisher_out"]):
        d, method, order = ast.literal_eval(str(case))
        got = oracle.fisher_numerical(f, oracle.params_from_dict(d), "Livingston", "Hanford", psd, method=method,
                                      order=order)
        _close(got, want)
    for case, want in zip(g["maxll_cases"], g["maxll_out"]):
        d = ast.literal_eval(str(case))
        hp, _ = oracle.fourier_waveform(f, oracle.params_from_dict(d), oracle.IMRPhenomD)
        hp2, hc2 = oracle.fourier_waveform(f, oracle.params_from_dict(d), oracle.IMRPhenomPv2)
        # numpy's FFT against the reference with a direct DFT in FFTW's place
        _close(oracle.maximized_loglik_internal(data[0], psd, f, hp), want[0], 1e-11)
        _close(oracle.maximized_loglik_unaligned_internal(data[0], psd, f, hp2, hc2), want[1], 1e-11)


def _ref_full_or_skip(oracle):
    if oracle.ref_full_lib() is None and oracle.reference_dir():
        oracle.build(oracle.reference_dir())
    if oracle.ref_full_lib() is None:
        pytest.skip("reference sources not present; the glue golden vectors cover this")


def test_glue_bit_exact_against_reference_build(oracle):
    """Fresh draws, bit for bit: responses (with and without the orientation
    transform), MCMC_likelihood_extrinsic, fisher_numerical."""
    _ref_full_or_skip(oracle)
    from gw_analysis_tools_gb300 import workloads as W
    f = W.uniform_grid(20.0, 200.0, 1.0 / 8.0)
    dets = ["Hanford", "Livingston", "Virgo"]
    src = oracle.params_from_dict(W.config1_source())
    data = [oracle.detector_response(f, src, d) + W.noise(f, 40 + i) for i, d in enumerate(dets)]
    psd = W.analytic_psd(f)
    rng = np.random.Generator(np.random.PCG64(41))
    for ap, name in ((oracle.IMRPhenomD, "IMRPhenomD"), (oracle.IMRPhenomPv2, "IMRPhenomPv2")):
        for d in W.prior_draws(4, 42, precessing=ap == oracle.IMRPhenomPv2):
            d = dict(d, theta_l=float(np.arccos(rng.uniform(-1, 1))), phi_l=float(rng.uniform(0, 2 * np.pi)),
                     equatorial_orientation=int(rng.uniform() < 0.5))
            p = oracle.params_from_dict(d)
            want, _ = oracle.ref_detector_response(f, p, "Virgo", name)
            assert np.array_equal(oracle.detector_response(f, p, "Virgo", ap), want)
            ll, T, _ = oracle.ref_mcmc_likelihood_extrinsic(oracle.params_from_dict(dict(d, equatorial_orientation=0)),
                                                            f, dets, data, [psd] * 3, method=name)
            got = oracle.loglik(oracle.params_from_dict(dict(d, equatorial_orientation=0)), f, dets, data, [psd] * 3,
                                approximant=ap, T_segment=T)
            assert got == ll
    oriented = [dict(d, theta_l=0.4 + 0.3 * k, phi_l=1.0 + 1.7 * k, equatorial_orientation=1)
                for k, d in enumerate(W.prior_draws(2, 44))]
    for d in W.prior_draws(2, 43) + oriented:
        for method in ("IMRPhenomD", "MCMC_IMRPhenomD"):
            for order in (2, 4):
                p = oracle.params_from_dict(d)
                want = oracle.ref_fisher_numerical(f, p, "Hanford", "Hanford", psd, method=method, order=order)
                got = oracle.fisher_numerical(f, p, "Hanford", "Hanford", psd, method=method, order=order)
                assert np.array_equal(got, want)
