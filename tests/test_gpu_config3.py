"""The uneven IMRPhenomPv2 batch at its full size, against the FP64 oracle.

Grids of T = 4, 8, 32 and 128 s over 20-2048 Hz (N = 2028 T: 8,112 to 259,584
bins), all in one launch, each request on its own grid (T_segment = 0: 1/df of
the request's grid, the t_c <- T - t_c rewrite of mcmc_gw.cpp:2466-2473).  On
the 128 s grid 2 pi f t_c reaches about 1.6e6 rad, the hardest case for the
mixed form's fixed-point phase.  The data hold a loud Pv2 injection on every
grid plus seeded noise; half of the requests are drawn close to the injection
(high SNR), half from the priors."""
import numpy as np
import pytest

import gw_analysis_tools_gb300 as G
from gw_analysis_tools_gb300 import workloads as W

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-3   # |delta log L| absolute, mixed form
FP64_RTOL = 1e-9   # relative, FP64 form
DURATIONS = (4, 8, 32, 128)
INJECTION = dict(mass1=31.0, mass2=24.0, spin1=(0.35, -0.2, 0.3), spin2=(-0.25, 0.3, -0.2), Luminosity_Distance=180.0,
                 incl_angle=0.7, phiRef=0.9, f_ref=20.0, tc=0.02, RA=2.2, DEC=-0.5, psi=0.8, gmst=W.GMST)


@pytest.fixture(scope="module")
def uneven(gpu_ctx, oracle):
    dets = list(W.DETECTORS3)
    grids, datas, psds, handles = {}, {}, {}, {}
    for T in DURATIONS:
        f = W.uniform_grid(20.0, 2048.0, 1.0 / T)
        assert f.size == 2028 * T
        injp = oracle.params_from_dict(dict(INJECTION, tc=T - INJECTION["tc"]))
        data = []
        for i, d in enumerate(dets):
            r = oracle.detector_response(f, injp, d, oracle.IMRPhenomPv2)
            dt = oracle.dtoa(INJECTION["RA"], INJECTION["DEC"], INJECTION["gmst"], dets[0], d)
            data.append(r * np.exp(-2j * np.pi * dt * f) + W.noise(f, 3000 + T + i))
        grids[T], datas[T], psds[T] = f, data, [W.analytic_psd(f)] * 3
        handles[T] = [gpu_ctx.register_data(d, f, data[i], psds[T][i]) for i, d in enumerate(dets)]
    near = W.perturbed(INJECTION, 40, 31, frac=0.002)
    far = W.prior_draws(40, 32, precessing=True)
    draws = [x for pair in zip(near, far) for x in pair]
    Ts = [DURATIONS[i % 4] for i in range(len(draws))]
    ref = np.zeros(len(draws))
    for T in DURATIONS:
        idx = [i for i in range(len(draws)) if Ts[i] == T]
        ref[idx] = oracle.loglik_batch([oracle.params_from_dict(draws[i]) for i in idx], grids[T], dets, datas[T],
                                       psds[T], approximants=[oracle.IMRPhenomPv2] * len(idx))
    yield dict(draws=draws, Ts=Ts, ref=ref, handles=np.array([handles[T] for T in Ts], dtype=np.int32))
    for T in DURATIONS:
        for h in handles[T]:
            gpu_ctx.release_data(h)


def test_config3_full_size_fp64(gpu_ctx, uneven):
    u = uneven
    out, st = gpu_ctx.loglik_batch(G.params_array(u["draws"]), 1, u["handles"], 0.0, G.PREC_FP64)
    assert np.all(st == 0)
    rel = np.abs(out - u["ref"]) / np.maximum(1.0, np.abs(u["ref"]))
    assert np.max(rel) <= FP64_RTOL, (np.max(rel), int(np.argmax(rel)))


def test_config3_full_size_mixed(gpu_ctx, uneven):
    u = uneven
    out, st = gpu_ctx.loglik_batch(G.params_array(u["draws"]), 1, u["handles"], 0.0, G.PREC_MIXED)
    assert np.all(st == 0)
    err = np.abs(out - u["ref"])
    # the near-injection draws are loud: |log L| of order SNR^2 / 2
    assert np.max(np.abs(u["ref"][0::2])) > 1e3
    for T in DURATIONS:
        sel = [i for i in range(len(err)) if u["Ts"][i] == T]
        assert np.max(err[sel]) <= MIXED_TOL, (T, float(np.max(err[sel])))
