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
