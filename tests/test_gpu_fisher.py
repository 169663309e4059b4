"""GPU Fisher matrices against the oracle: the plain drop-in (reference
algorithm, 1e-8 absolute step) and the batched network Fisher + inverse."""
import numpy as np
import pytest

import gw_analysis_tools_gb300 as G
from gw_analysis_tools_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _norm_err(A, B):
    return np.max(np.abs(A - B) / np.sqrt(np.outer(np.abs(np.diag(B)), np.abs(np.diag(B)))))


def test_plain_fisher_numerical(gpu_ctx, oracle):
    f = W.uniform_grid(10.0, 1024.0, 1 / 4.)
    psd = W.analytic_psd(f)
    for d in W.prior_draws(3, 81):
        p = oracle.params_from_dict(d)
        for det, ref_det in (("Hanford", "Hanford"), ("Virgo", "Hanford")):
            ref = oracle.fisher_numerical(f, p, det, ref_det, psd)
            got = gpu_ctx.fisher_numerical(f, "IMRPhenomD", det, ref_det, G.gen_params(**d), psd)
            assert _norm_err(got, ref) <= 1e-4


def test_batched_fisher_network(gpu_ctx, oracle):
    f = W.uniform_grid(10.0, 2048.0, 1 / 16.)
    dets = list(W.DETECTORS3)
    psd = W.analytic_psd(f)
    hs = [gpu_ctx.register_data(d, f, np.zeros(f.size, complex), psd) for d in dets]
    draws = W.prior_draws(16, 83)
    fish, cov, st = gpu_ctx.fisher_batch(G.params_array(draws), 0, hs, epsilon=1e-6, step_mode=1)
    assert np.all(st == 0)
    for i in range(4):
        ref = oracle.fisher_network(f, oracle.params_from_dict(draws[i]), dets, [psd] * 3, epsilon=1e-6,
                                    step_mode=1)
        assert _norm_err(fish[i], ref) <= 1e-5
        assert np.allclose(fish[i], fish[i].T)
        # the inverse is the inverse of the returned matrix
        ident = cov[i] @ fish[i]
        assert np.max(np.abs(ident - np.eye(11))) < 1e-4
    for h in hs:
        gpu_ctx.release_data(h)
