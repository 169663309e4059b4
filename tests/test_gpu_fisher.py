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


def _inv_err(C, R):
    return np.max(np.abs(C - R) / np.sqrt(np.abs(np.outer(np.diag(R), np.diag(R)))))


def test_batched_fisher_network(gpu_ctx, oracle):
    """gwgpu_fisher_batch (the moment form, FP64 sums) against the FP64 oracle
    on all 16 sources: the Fisher matrix and its inverse, each normalised by
    the oracle's diagonal."""
    f = W.uniform_grid(10.0, 2048.0, 1 / 16.)
    dets = list(W.DETECTORS3)
    psd = W.analytic_psd(f)
    hs = [gpu_ctx.register_data(d, f, np.zeros(f.size, complex), psd) for d in dets]
    draws = W.prior_draws(16, 83)
    fish, cov, st = gpu_ctx.fisher_batch(G.params_array(draws), 0, hs, epsilon=1e-6, step_mode=1)
    assert np.all(st == 0)
    for i in range(len(draws)):
        ref = oracle.fisher_network(f, oracle.params_from_dict(draws[i]), dets, [psd] * 3, epsilon=1e-6,
                                    step_mode=1)
        assert _norm_err(fish[i], ref) <= 1e-5
        assert np.allclose(fish[i], fish[i].T)
        ist, rinv = oracle.cholesky_invert(ref)
        assert ist == 0
        # the inverse's error is the matrix's error in its weakest direction
        # times the condition number of the normalised matrix (1e5-1e8 here)
        cond = np.linalg.cond(ref / np.sqrt(np.outer(np.diag(ref), np.diag(ref))))
        assert _inv_err(cov[i], rinv) <= 2e-11 * cond, (i, cond, _inv_err(cov[i], rinv))
    for h in hs:
        gpu_ctx.release_data(h)


@pytest.mark.parametrize("add_prior", [False, True])
def test_batched_fisher_fp64_sums(gpu_ctx, oracle, add_prior):
    """The moment form with FP64 per-bin differences and sums
    (gwgpu_fisher_batch_ex, FISHER_MOMENTS, PREC_FP64) on ordinary and
    near-degenerate sources: the matrix and its inverse at the FP64 reference
    algorithm's accuracy, the prior diagonal of MCMC_fisher_transformations
    added on request."""
    f = W.uniform_grid(10.0, 2048.0, 1 / 16.)
    dets = list(W.DETECTORS3)
    psd = W.analytic_psd(f)
    hs = [gpu_ctx.register_data(d, f, np.zeros(f.size, complex), psd) for d in dets]
    pool = W.prior_draws(10000, 13)
    draws = [pool[i] for i in (228, 3139, 4213, 6593)] + W.prior_draws(12, 83)
    # the sampler's parameterisation with its prior diagonal, or the plain one
    method, name = (1, "MCMC_IMRPhenomD") if add_prior else (0, "IMRPhenomD")
    fish, cov, st = gpu_ctx.fisher_batch_ex(G.params_array(draws), method, hs, order=2, epsilon=1e-6, step_mode=1,
                                            precision=G.PREC_FP64, algorithm=G.FISHER_MOMENTS, add_prior=add_prior)
    prior = np.diag(oracle.mcmc_fisher_prior_diag()) if add_prior else 0.0
    for i, d in enumerate(draws):
        ref = oracle.fisher_network(f, oracle.params_from_dict(d), dets, [psd] * 3, method=name, epsilon=1e-6,
                                    step_mode=1) + prior
        # both sides FP64: the rounding differences of two implementations
        # divided by the 1e-6 step (up to 2e-5 normalised on the four
        # near-degenerate sources, normalised smallest eigenvalue 2e-10-4e-9)
        assert _norm_err(fish[i], ref) <= (1e-4 if i < 4 else 1e-5), (i, _norm_err(fish[i], ref))
        ist, rinv = oracle.cholesky_invert(ref)
        assert st[i] == (0 if ist == 0 else 9), (i, st[i], ist)
        if ist == 0:
            # 1e-6: the floor of a well-conditioned matrix (the prior diagonal
            # brings the condition number down to ~1e4)
            cond = np.linalg.cond(ref / np.sqrt(np.outer(np.diag(ref), np.diag(ref))))
            assert _inv_err(cov[i], rinv) <= 2e-11 * cond + 1e-6, (i, cond, _inv_err(cov[i], rinv))
    # the FP32-compensated form of the same call
    fm, _, stm = gpu_ctx.fisher_batch_ex(G.params_array(draws), method, hs, order=2, epsilon=1e-6, step_mode=1,
                                         precision=G.PREC_MIXED, algorithm=G.FISHER_MOMENTS, add_prior=add_prior)
    assert np.array_equal(stm, st)
    for i in range(len(draws)):
        assert _norm_err(fm[i], fish[i]) <= 1e-4
    for h in hs:
        gpu_ctx.release_data(h)


def test_fisher_batch_ex_rejects_bad_options(gpu_ctx):
    f = W.uniform_grid(10.0, 512.0, 1 / 4.)
    h = gpu_ctx.register_data("Hanford", f, np.zeros(f.size, complex), W.analytic_psd(f))
    p = G.params_array(W.prior_draws(1, 86))
    for kw in (dict(order=3, algorithm=G.FISHER_MOMENTS), dict(precision=G.PREC_MIXED),
               dict(algorithm=7), dict(order=3)):
        with pytest.raises(G.GwGpuError):
            gpu_ctx.fisher_batch_ex(p, 0, [h], **kw)
    gpu_ctx.release_data(h)


def test_batched_fisher_refines_singular_sources(gpu_ctx, oracle):
    """Sources whose matrix the FP32-compensated sums (PREC_MIXED) leave
    indefinite (equal masses, a face-on orientation) are recomputed by the FP64
    reference algorithm: status OK and the oracle's matrix."""
    f = W.uniform_grid(10.0, 2048.0, 1 / 16.)
    dets = list(W.DETECTORS3)
    psd = W.analytic_psd(f)
    hs = [gpu_ctx.register_data(d, f, np.zeros(f.size, complex), psd) for d in dets]
    pool = W.prior_draws(10000, 13)
    draws = [pool[i] for i in (228, 3139, 4213, 6593, 8425, 4968)] + W.prior_draws(6, 84)
    fish, cov, st = gpu_ctx.fisher_batch_ex(G.params_array(draws), 0, hs, epsilon=1e-6, step_mode=1,
                                            precision=G.PREC_MIXED, algorithm=G.FISHER_MOMENTS)
    for i, d in enumerate(draws):
        ref = oracle.fisher_network(f, oracle.params_from_dict(d), dets, [psd] * 3, epsilon=1e-6, step_mode=1)
        # near-degenerate sources: the FP64 rounding of two implementations,
        # divided by steps of 1e-6 of parameters near zero
        assert _norm_err(fish[i], ref) <= 1e-4, i
        ist, _ = oracle.cholesky_invert(ref)
        dn = np.sqrt(np.abs(np.diag(ref)))
        if np.linalg.eigvalsh(ref / np.outer(dn, dn))[0] < 1e-13:
            # singular to FP64 rounding (4968: within 3 degrees of face-on,
            # normalised smallest eigenvalue 6e-15): whether a Cholesky
            # factorisation succeeds is decided by the rounding of each
            # implementation
            assert st[i] in (0, 9)
        else:
            assert st[i] == (0 if ist == 0 else 9), (i, st[i], ist)
    for h in hs:
        gpu_ctx.release_data(h)


@pytest.mark.parametrize("order", [2, 4])
def test_fisher_reference_algorithm(gpu_ctx, oracle, order):
    """gwgpu_fisher_batch_ex in FP64: the reference algorithm on the device,
    both parameterisations, orders 2 and 4 (the five-point rule keeps the
    reference's constant phase on the +-2 eps responses of a non-reference
    detector), against the oracle's network Fisher."""
    f = W.uniform_grid(10.0, 1024.0, 1 / 8.)
    dets = list(W.DETECTORS3)
    psd = W.analytic_psd(f)
    hs = [gpu_ctx.register_data(d, f, np.zeros(f.size, complex), psd) for d in dets]
    draws = W.prior_draws(12, 85)
    for method, name in ((0, "IMRPhenomD"), (1, "MCMC_IMRPhenomD")):
        # FP64 rounding differences of two implementations, divided by the step
        # (1e-6 relative: steps of parameters near zero -- sin DEC, cos iota,
        # spins -- are far below 1e-6)
        for eps, mode, tol in ((1e-6, 1, 1e-4), (1e-8, 0, 3e-4)):
            fish, cov, st = gpu_ctx.fisher_batch_ex(G.params_array(draws), method, hs, order=order, epsilon=eps,
                                                    step_mode=mode, precision=G.PREC_FP64)
            for i, d in enumerate(draws):
                ref = oracle.fisher_network(f, oracle.params_from_dict(d), dets, [psd] * 3, method=name, order=order,
                                            epsilon=eps, step_mode=mode)
                assert _norm_err(fish[i], ref) <= tol, (name, eps, i, _norm_err(fish[i], ref))
                ist, rinv = oracle.cholesky_invert(ref)
                assert st[i] == (0 if ist == 0 else 9)
                if ist == 0 and eps == 1e-6:
                    cond = np.linalg.cond(ref / np.sqrt(np.outer(np.diag(ref), np.diag(ref))))
                    assert _inv_err(cov[i], rinv) <= 2e-11 * cond * (3 if order == 4 else 1), (i, cond)
    for h in hs:
        gpu_ctx.release_data(h)


def test_mcmc_fisher_proposal_golden(gpu_ctx):
    """gwgpu_mcmc_fisher_batch against the reference's own MCMC_fisher_wrapper
    output (order 4, MCMC_IMRPhenomD, prior diagonal) stored in the golden
    fixture, on the fixture's data and positions."""
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_glue.npz"))
    f, psd = g["freqs"], g["psd"]
    dets = list(W.DETECTORS3)
    hs = [gpu_ctx.register_data(d, f, g["data"][i], psd) for i, d in enumerate(dets)]
    fish, st = gpu_ctx.mcmc_fisher_batch(g["wrapper_pos_d"], hs, float(g["wrapper_gmst"]))
    assert np.all(st == 0)
    for got, want in zip(fish, g["wrapper_fisher_d"]):
        assert _norm_err(got, want) <= 1e-4
    for h in hs:
        gpu_ctx.release_data(h)


@pytest.mark.parametrize("method,name", [(0, "IMRPhenomD"), (1, "MCMC_IMRPhenomD")])
def test_moment_form_five_point(gpu_ctx, oracle, method, name):
    """The moment form at order 4 (gwgpu_fisher_batch_ex, FISHER_MOMENTS):
    the five-point rule with the reference's constant phase on the +-2 eps
    responses of the non-reference detectors (fisher.cpp:426-458), taken
    analytically, against the oracle's network Fisher at order 4; among the
    sources, one within 1000 steps of eta = 1/4 (left to the reference
    algorithm).  Both step rules."""
    f = W.uniform_grid(10.0, 1024.0, 1 / 8.)
    dets = list(W.DETECTORS3)
    psd = W.analytic_psd(f)
    hs = [gpu_ctx.register_data(d, f, np.zeros(f.size, complex), psd) for d in dets]
    draws = W.prior_draws(10, 87) + [dict(W.prior_draws(1, 88)[0], mass1=30.0, mass2=30.0 * (1 - 1e-5))]
    for eps, mode, tol in ((1e-6, 1, 1e-4), (1e-8, 0, 3e-4)):
        fish, cov, st = gpu_ctx.fisher_batch_ex(G.params_array(draws), method, hs, order=4, epsilon=eps,
                                                step_mode=mode, precision=G.PREC_FP64, algorithm=G.FISHER_MOMENTS)
        for i, d in enumerate(draws):
            ref = oracle.fisher_network(f, oracle.params_from_dict(d), dets, [psd] * 3, method=name, order=4,
                                        epsilon=eps, step_mode=mode)
            # the FP64 rounding of the reference's own differences, divided by
            # the step, against the analytic form
            assert _norm_err(fish[i], ref) <= tol, (name, eps, i, _norm_err(fish[i], ref))
            ist, _ = oracle.cholesky_invert(ref)
            if ist != 0:
                assert st[i] in (0, 9)
            else:
                assert st[i] == 0, (i, st[i])
    for h in hs:
        gpu_ctx.release_data(h)
