"""The reference-signature C++ layer (libgwat_dropin.so, include/gwat_dropin.h)
against the oracle: MCMC_likelihood_extrinsic (mcmc_gw.cpp:2374) called with
the reference's own argument conventions, including T formed from the
difference of the frequency-array pointers (mcmc_gw.cpp:2466) and the
caller's tc rewritten to T - tc (mcmc_gw.cpp:2467-2473)."""
import ctypes

import numpy as np
import pytest

from gw_analysis_tools_gb300 import _native, engine, workloads

pytestmark = pytest.mark.gpu
FP64_RTOL = 1e-9
MIXED_TOL = 1e-3


def _dropin():
    _native.build()
    L = ctypes.CDLL(_native.DROPIN_LIB)
    f = L.gwat_dropin_test_loglik
    f.restype = ctypes.c_double
    dp = ctypes.POINTER(ctypes.c_double)
    f.argtypes = [dp, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                  ctypes.c_int, dp]
    return f


def _call(fn, f, data, psd, dets, p, served):
    n = len(dets)
    dptr = (ctypes.c_void_p * n)(*[d.ctypes.data for d in data])
    sptr = (ctypes.c_void_p * n)(*[s.ctypes.data for s in psd])
    names = (ctypes.c_char_p * n)(*[d.encode() for d in dets])
    tc = np.zeros(2)
    ll = fn(f.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), f.size, dptr, sptr, names, n, ctypes.byref(p),
            served, tc.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    return ll, tc


@pytest.mark.parametrize("served", [0, 1, 2])  # plain; served by the device loop; by the host scheduler
def test_mcmc_likelihood_extrinsic_dropin(oracle, served):
    fn = _dropin()
    f = np.ascontiguousarray(workloads.uniform_grid(20.0, 512.0, 1.0 / 8.0))
    dets = list(workloads.DETECTORS3)
    src = workloads.config1_source()
    injp = oracle.params_from_dict(dict(src, tc=8.0 - src["tc"]))
    psd = [np.ascontiguousarray(workloads.analytic_psd(f))] * 3
    data = [np.ascontiguousarray(oracle.detector_response(f, injp, d) + workloads.noise(f, 40 + i))
            for i, d in enumerate(dets)]
    for q in [src] + workloads.perturbed(src, 5, seed=11):
        p = engine.gen_params(**q)
        ll, tc = _call(fn, f, data, psd, dets, p, served)
        T = tc[1]
        assert T == pytest.approx(1.0 / f.size)
        assert tc[0] == T - q["tc"]
        ref = oracle.loglik(oracle.params_from_dict(q), f, dets, data, psd, T_segment=T)
        if served:
            assert abs(ll - ref) <= MIXED_TOL, (ll, ref)
        else:
            assert abs(ll - ref) <= FP64_RTOL * max(1.0, abs(ref)), (ll, ref)


def test_served_dropin_threads_two_segment_lengths(oracle):
    """Concurrent callers in served mode with two grid lengths, so two values of
    the reference's T: one server per T, none freed while another thread uses
    it (the drop-in keeps every server until the process exits)."""
    from concurrent.futures import ThreadPoolExecutor
    fn = _dropin()
    dets = list(workloads.DETECTORS3)
    src = workloads.config1_source()
    cases = []
    for hi in (300.0, 400.0):
        f = np.ascontiguousarray(workloads.uniform_grid(20.0, hi, 1.0 / 8.0))
        injp = oracle.params_from_dict(dict(src, tc=8.0 - src["tc"]))
        psd = [np.ascontiguousarray(workloads.analytic_psd(f))] * 3
        data = [np.ascontiguousarray(oracle.detector_response(f, injp, d) + workloads.noise(f, 60 + i))
                for i, d in enumerate(dets)]
        cases.append((f, data, psd))
    draws = workloads.perturbed(src, 24, seed=12)
    jobs = [(k % 2, draws[k]) for k in range(len(draws))]

    def run(job):
        g, q = job
        f, data, psd = cases[g]
        return _call(fn, f, data, psd, dets, engine.gen_params(**q), 1)

    with ThreadPoolExecutor(8) as ex:
        got = list(ex.map(run, jobs * 3))
    errs = []
    for (g, q), (ll, tc) in zip(jobs * 3, got):
        f, data, psd = cases[g]
        errs.append(abs(ll - oracle.loglik(oracle.params_from_dict(q), f, dets, data, psd, T_segment=tc[1])))
    assert max(errs) <= MIXED_TOL, max(errs)
