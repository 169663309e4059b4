"""Self-consistency checks of the oracle that the reference relies on."""
import ctypes

import numpy as np


def test_simpson_weights_and_inner_product(oracle):
    # <h|h> of a constant integrand: 4 * Simpson(1) = 4 * (N-1) df for odd N
    f = 20.0 + np.arange(101) / 4.0
    r = np.ones(101, dtype=complex)
    psd = np.ones(101)
    ll = oracle.lib().gwo_log_likelihood_internal(oracle._dp(np.zeros(202)), oracle._dp(psd), oracle._dp(f),
                                                  oracle._dp(r.view(np.float64).copy()), 101)
    hh = -2 * ll
    assert abs(hh - 4 * 100 * 0.25) < 1e-12


def test_cspline_reproduces_cubic_interior_and_natural_ends(oracle):
    x = np.linspace(-1, 1, 41)
    y = 3 * x ** 3 - x ** 2 + 0.5
    c = np.zeros_like(x)
    oracle.lib().gwo_cspline_coeffs(oracle._dp(x), oracle._dp(y), x.size, oracle._dp(c))
    assert c[0] == 0 and c[-1] == 0
    # a natural spline is not exact for a cubic near the ends; interior error is small
    xv = 0.013
    v = oracle.lib().gwo_cspline_eval(oracle._dp(x), oracle._dp(y), oracle._dp(c), x.size, xv, 0)
    assert abs(v - (3 * xv ** 3 - xv ** 2 + 0.5)) < 1e-4
    # linear data is reproduced exactly
    y2 = 2 * x + 1
    oracle.lib().gwo_cspline_coeffs(oracle._dp(x), oracle._dp(y2), x.size, oracle._dp(c))
    v = oracle.lib().gwo_cspline_eval(oracle._dp(x), oracle._dp(y2), oracle._dp(c), x.size, 0.377, 0)
    assert abs(v - (2 * 0.377 + 1)) < 1e-14


def test_waveform_is_continuous_across_region_joins(oracle):
    """Amplitude and phase are C1 at f1 and f3 (IMRPhenomD.cpp:1614-1702)."""
    p = oracle.make_params(mass1=36.0, mass2=29.0, spin1=(0, 0, 0.3), spin2=(0, 0, -0.1), Luminosity_Distance=410.0,
                           f_ref=20.0, shift_time=0, shift_phase=0)
    internals = np.zeros(32)
    oracle.lib().gwo_d_internals(ctypes.byref(p), oracle._dp(internals))
    f1, f3, f1p, f2p = internals[2], internals[3], internals[4], internals[5]
    for fb in (f1, f3):
        eps = 1e-6 * fb
        f = np.array([fb - eps, fb + eps])
        hp, _ = oracle.fourier_waveform(f, p)
        a = np.abs(hp)
        assert abs(a[1] / a[0] - 1) < 1e-5
    for fb in (f1p, f2p):
        eps = 1e-7 * fb
        f = np.array([fb - eps, fb + eps])
        hp, _ = oracle.fourier_waveform(f, p)
        dphi = np.angle(hp[1] / hp[0])
        assert abs(dphi) < 1e-3


def test_antenna_pattern_matches_analytic_formula(oracle):
    """F+^2 + Fx^2 is invariant under psi; psi -> psi + pi/2 flips the signs."""
    for det in ("Hanford", "Livingston", "Virgo"):
        fp, fc = oracle.antenna(det, 1.1, -0.4, 0.3, 2.0)
        gp, gc = oracle.antenna(det, 1.1, -0.4, 0.3 + np.pi / 2, 2.0)
        assert abs(fp + gp) < 1e-12 and abs(fc + gc) < 1e-12
        hp, hc = oracle.antenna(det, 1.1, -0.4, 1.7, 2.0)
        assert abs((fp * fp + fc * fc) - (hp * hp + hc * hc)) < 1e-12
        assert fp * fp + fc * fc <= 1.0 + 1e-12


def test_dtoa_antisymmetric_and_bounded(oracle):
    for ra, dec in ((0.1, 0.2), (3.0, -1.0), (5.5, 0.9)):
        a = oracle.dtoa(ra, dec, 1.0, "Hanford", "Livingston")
        b = oracle.dtoa(ra, dec, 1.0, "Livingston", "Hanford")
        assert a == -b
        assert abs(a) < 0.0101  # 10 ms light travel time between the LIGO sites
        assert oracle.dtoa(ra, dec, 1.0, "Virgo", "Virgo") == 0.0


def test_fisher_is_symmetric_and_positive(oracle):
    from gw_analysis_tools_gb300 import workloads as W
    f = 10.0 + np.arange(1000) / 4.0
    psd = W.analytic_psd(f)
    p = oracle.make_params(mass1=30.0, mass2=25.0, spin1=(0, 0, 0.2), spin2=(0, 0, 0.1), Luminosity_Distance=400.0,
                           incl_angle=0.7, phiRef=0.5, f_ref=20.0, tc=0.0, RA=1.0, DEC=0.2, psi=0.3, gmst=1.0)
    F = oracle.fisher_numerical(f, p, "Livingston", "Hanford", psd)
    assert F.shape == (11, 11)
    assert np.array_equal(F, F.T)
    assert np.all(np.diag(F) > 0)


def test_cholesky_inverse(oracle):
    rng = np.random.default_rng(3)
    a = rng.standard_normal((11, 11))
    m = a @ a.T + 11 * np.eye(11)
    st, inv = oracle.cholesky_invert(m)
    assert st == 0
    np.testing.assert_allclose(inv @ m, np.eye(11), atol=1e-12)
