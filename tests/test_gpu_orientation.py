"""equatorial_orientation (transform_orientation_coords, waveform_util.cpp:1523-1586)
through the C ABI: the detector response and both Fisher forms take the
inclination and polarisation from the equatorial direction (theta_l, phi_l) of
the orbital angular momentum, against the oracle (which is pinned to the
reference's own transform, tests/test_oracle_pins.py).  Also the five-point
(order 4) plain Fisher and the 15-dim IMRPhenomPv2 MCMC repack on the GPU."""
import numpy as np
import pytest

import gw_analysis_tools_gb300 as G
from gw_analysis_tools_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _oriented(n, seed, precessing=False):
    rng = np.random.Generator(np.random.PCG64(seed + 7))
    out = []
    for d in W.prior_draws(n, seed, precessing=precessing):
        d = dict(d, theta_l=float(np.arccos(rng.uniform(-1, 1))), phi_l=float(rng.uniform(0, 2 * np.pi)),
                 equatorial_orientation=1)
        if precessing and rng.uniform() < 0.5:
            d.update(chip=float(rng.uniform(0.1, 0.7)), phip=float(rng.uniform(0, 2 * np.pi)))
        out.append(d)
    return out


def _norm_err(A, B):
    return np.max(np.abs(A - B) / np.sqrt(np.outer(np.abs(np.diag(B)), np.abs(np.diag(B)))))


def test_response_with_equatorial_orientation(gpu_ctx, oracle):
    f = W.config1_grid()
    for ap, name, prec in ((0, "IMRPhenomD", False), (1, "IMRPhenomPv2", True)):
        for d in _oriented(4, 61, prec):
            for det in ("Hanford", "Virgo"):
                a = oracle.detector_response(f, oracle.params_from_dict(d), det, ap)
                b = gpu_ctx.fourier_detector_response(f, det, name, G.gen_params(**d))
                assert np.max(np.abs(a - b)) <= 1e-11 * np.abs(a).max()
            # the flag changes the answer: psi and iota come from theta_l, phi_l
            plain = oracle.detector_response(f, oracle.params_from_dict(dict(d, equatorial_orientation=0)), "Hanford",
                                             ap)
            assert np.max(np.abs(plain - oracle.detector_response(f, oracle.params_from_dict(d), "Hanford", ap))) > 0


@pytest.mark.parametrize("order", [2, 4])
def test_plain_fisher_orders_and_orientation(gpu_ctx, oracle, order):
    f = W.uniform_grid(10.0, 1024.0, 1 / 4.)
    psd = W.analytic_psd(f)
    draws = W.prior_draws(2, 62) + _oriented(2, 63)
    for d in draws:
        p = oracle.params_from_dict(d)
        for method in ("IMRPhenomD", "MCMC_IMRPhenomD"):
            for det, ref_det in (("Hanford", "Hanford"), ("Livingston", "Hanford")):
                ref = oracle.fisher_numerical(f, p, det, ref_det, psd, method=method, order=order)
                got = gpu_ctx.fisher_numerical(f, method, det, ref_det, G.gen_params(**d), psd, order=order)
                # the reference's step (1e-8 absolute) turns the FP64 rounding
                # differences of two implementations into derivative noise of
                # ~1e-16 |r| / eps; the five-point weights amplify it 1.5 times
                assert _norm_err(got, ref) <= (1e-4 if order == 2 else 3e-4), (method, det, order)


def test_batched_fisher_with_orientation(gpu_ctx, oracle):
    f = W.uniform_grid(10.0, 2048.0, 1 / 16.)
    dets = list(W.DETECTORS3)
    psd = W.analytic_psd(f)
    hs = [gpu_ctx.register_data(d, f, np.zeros(f.size, complex), psd) for d in dets]
    draws = _oriented(8, 64)
    fish, cov, st = gpu_ctx.fisher_batch(G.params_array(draws), 0, hs, epsilon=1e-6, step_mode=1)
    assert np.all(st == 0)
    for i in range(len(draws)):
        ref = oracle.fisher_network(f, oracle.params_from_dict(draws[i]), dets, [psd] * 3, epsilon=1e-6, step_mode=1)
        assert _norm_err(fish[i], ref) <= 1e-5
    for h in hs:
        gpu_ctx.release_data(h)


def test_mcmc_pv2_15dim_repack(gpu_ctx, oracle):
    """gwgpu_mcmc_loglik_batch with the 15-dim IMRPhenomPv2 vector (spherical
    spins, repack_parameters, fisher.cpp:2171-2227) against the oracle's repack
    and likelihood, FP64 and mixed."""
    f = W.uniform_grid(20.0, 1024.0, 1 / 8.)
    T = 1.0 / (f[1] - f[0])
    dets = list(W.DETECTORS3)
    src = dict(W.config1_source(), spin1=(0.3, 0.2, 0.3), spin2=(-0.1, 0.4, -0.1))
    injp = oracle.params_from_dict(dict(src, tc=T - src["tc"]))
    data = []
    for i, d in enumerate(dets):
        r = oracle.detector_response(f, injp, d, oracle.IMRPhenomPv2)
        dt = oracle.dtoa(src["RA"], src["DEC"], src["gmst"], dets[0], d)
        data.append(r * np.exp(-2j * np.pi * dt * f) + W.noise(f, 70 + i))
    psd = [W.analytic_psd(f)] * 3
    hs = [gpu_ctx.register_data(d, f, data[i], psd[i]) for i, d in enumerate(dets)]
    rng = np.random.Generator(np.random.PCG64(65))
    n = 24
    theta = np.array([[rng.uniform(0, 2 * np.pi), rng.uniform(-1, 1), rng.uniform(0, np.pi), rng.uniform(-1, 1),
                       rng.uniform(0, 2 * np.pi), rng.uniform(-0.05, 0.05), np.log(rng.uniform(200, 900)),
                       np.log(rng.uniform(10, 30)), rng.uniform(0.15, 0.249), rng.uniform(0, 0.8),
                       rng.uniform(0, 0.8), rng.uniform(-1, 1), rng.uniform(-1, 1), rng.uniform(0, 2 * np.pi),
                       rng.uniform(0, 2 * np.pi)] for _ in range(n)])
    gmst = W.GMST
    ref = np.array([oracle.loglik(oracle.mcmc_repack(t, oracle.IMRPhenomPv2, gmst), f, dets, data, psd,
                                  approximant=oracle.IMRPhenomPv2, T_segment=T) for t in theta])
    got64, st = gpu_ctx.mcmc_loglik_batch(theta, G.IMRPhenomPv2, gmst, hs, T, precision=G.PREC_FP64)
    assert np.all(st == 0)
    assert np.max(np.abs(got64 - ref) / np.maximum(1.0, np.abs(ref))) <= 1e-9
    gotm, st = gpu_ctx.mcmc_loglik_batch(theta, G.IMRPhenomPv2, gmst, hs, T, precision=G.PREC_MIXED)
    assert np.all(st == 0)
    assert np.max(np.abs(gotm - ref)) <= 1e-3
    for h in hs:
        gpu_ctx.release_data(h)
