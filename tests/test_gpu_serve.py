"""Serving: continuous batching.  Each result is the same alone and in the mix;
requests overlap on the device; admission by HBM budget; slot exhaustion."""
import time

import numpy as np
import pytest

import gw_analysis_tools_gb300 as G
from gw_analysis_tools_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def served(gpu_ctx):
    f = W.config1_grid()
    T = 1.0 / (f[1] - f[0])
    psd = W.analytic_psd(f)
    hs = [gpu_ctx.register_data(d, f, W.noise(f, 300 + i), psd) for i, d in enumerate(W.DETECTORS3)]
    return dict(f=f, T=T, hs=hs)


def test_results_same_alone_and_in_the_mix(gpu_ctx, oracle, served):
    s = served
    dd = W.prior_draws(150, 101)
    dp = W.prior_draws(150, 102, precessing=True)
    draws = [x for pair in zip(dd, dp) for x in pair]
    aps = [0, 1] * 150
    srv = G.Server(gpu_ctx, s["T"], max_inflight=1024, max_batch=64, lanes=3)
    tickets = [srv.submit(G.gen_params(**d), aps[i], s["hs"]) for i, d in enumerate(draws)]
    mixed = np.array([srv.wait(t)[0] for t in tickets])
    st = srv.stats()
    assert st["completed"] == len(draws)
    assert st["launches"] >= 2  # arrivals were admitted into several overlapping launches
    for i in (0, 1, 77, 298, 299):
        alone, _ = gpu_ctx.loglik_batch(G.params_array([draws[i]]), aps[i], s["hs"], s["T"], G.PREC_MIXED)
        assert mixed[i] == alone[0]
    srv.close()


def test_served_results_match_oracle(gpu_ctx, oracle, served):
    s = served
    draws = W.prior_draws(40, 103)
    srv = G.Server(gpu_ctx, s["T"], max_inflight=256, max_batch=16, lanes=2)
    tickets = [srv.submit(G.gen_params(**d), 0, s["hs"]) for d in draws]
    got = np.array([srv.wait(t)[0] for t in tickets])
    srv.close()
    f = s["f"]
    data = [W.noise(f, 300 + i) for i in range(3)]
    ref = oracle.loglik_batch([oracle.params_from_dict(d) for d in draws], f, list(W.DETECTORS3), data,
                              [W.analytic_psd(f)] * 3)
    assert np.max(np.abs(got - ref)) <= 1e-3


def test_admission_by_budget_and_slot_exhaustion(gpu_ctx, served):
    s = served
    draws = W.prior_draws(24, 104)
    # a budget below one request's scratch: requests are admitted one launch at a time and still complete
    srv = G.Server(gpu_ctx, s["T"], max_inflight=8, max_batch=8, lanes=2, hbm_budget=4096)
    ts = []
    for d in draws[:8]:
        ts.append(srv.submit(G.gen_params(**d), 0, s["hs"]))
    with pytest.raises(G.GwGpuError):
        srv.submit(G.gen_params(**draws[8]), 0, s["hs"])  # every slot taken
    out = [srv.wait(t) for t in ts]
    assert all(o[1] == 0 for o in out)
    assert srv.stats()["launches"] >= 4
    # slots are reusable once collected
    t = srv.submit(G.gen_params(**draws[9]), 0, s["hs"])
    assert srv.wait(t)[1] == 0
    srv.close()


def test_poisson_driver_latency(gpu_ctx, served):
    s = served
    n = 2000
    draws = W.prior_draws(n, 105)
    rng = np.random.default_rng(5)
    arrivals = np.cumsum(rng.exponential(1.0 / 5e4, n))
    srv = G.Server(gpu_ctx, s["T"], max_inflight=4096, max_batch=512, lanes=4)
    out, st, lat, wall = srv.drive(G.params_array(draws), 0, s["hs"], arrivals)
    assert np.all(st == 0)
    assert np.all(np.isfinite(out))
    stats = srv.stats()
    assert stats["completed"] == n
    assert 0 < stats["p50_s"] <= stats["p99_s"] < 5.0
    srv.close()


def test_unknown_ticket(gpu_ctx, served):
    srv = G.Server(gpu_ctx, served["T"], max_inflight=4, max_batch=4, lanes=1)
    assert srv.lib.gwgpu_server_poll(srv.h, 12345, None, None) == 7
    srv.close()


def test_odd_batches_and_lane_errors_do_not_hang(gpu_ctx, oracle, served):
    """Odd batch sizes (max_batch 7, 3 lanes) complete with the oracle's values."""
    s = served
    draws = W.prior_draws(61, 106)
    srv = G.Server(gpu_ctx, s["T"], max_inflight=128, max_batch=7, lanes=3)
    tickets = [srv.submit(G.gen_params(**d), 0, s["hs"]) for d in draws]
    got = np.array([srv.wait(t)[0] for t in tickets])
    srv.close()
    f = s["f"]
    data = [W.noise(f, 300 + i) for i in range(3)]
    ref = oracle.loglik_batch([oracle.params_from_dict(d) for d in draws], f, list(W.DETECTORS3), data,
                              [W.analytic_psd(f)] * 3)
    assert np.max(np.abs(got - ref)) <= 1e-3
