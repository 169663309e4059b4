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


# ---------------------------------------------------------------- device loop
def _mix(n, seed):
    dd = W.prior_draws(n // 2, seed)
    dp = W.prior_draws(n - n // 2, seed + 1, precessing=True)
    draws = [x for pair in zip(dd, dp) for x in pair]
    return draws, [0, 1] * (n // 2)


def test_device_loop_matches_batch_and_oracle(gpu_ctx, oracle, served):
    """The device-resident loop gives the batched kernel's values bit for bit
    (same tile) and the oracle's within 1e-3, D and Pv2 mixed."""
    s = served
    draws, aps = _mix(120, 111)
    srv = G.Server(gpu_ctx, s["T"], max_inflight=512, device_loop=True, tile=4096)
    tickets = [srv.submit(G.gen_params(**d), aps[i], s["hs"]) for i, d in enumerate(draws)]
    got = np.array([srv.wait(t) for t in tickets])
    info = srv.loop_info()
    srv.close()
    assert np.all(got[:, 1] == 0)
    assert info["tile"] == 4096 and info["launches"] >= 1 and info["ring_slots"] == 512
    gpu_ctx.set_tile(4096)
    try:
        for ap in (0, 1):
            idx = [i for i in range(len(draws)) if aps[i] == ap]
            ref, _ = gpu_ctx.loglik_batch(G.params_array([draws[i] for i in idx]), ap, s["hs"], s["T"], G.PREC_MIXED)
            assert np.array_equal(got[idx, 0], ref)
    finally:
        gpu_ctx.set_tile(0)
    f = s["f"]
    data = [W.noise(f, 300 + i) for i in range(3)]
    ref = oracle.loglik_batch([oracle.params_from_dict(d) for d in draws], f, list(W.DETECTORS3), data,
                              [W.analytic_psd(f)] * 3, approximants=aps)
    assert np.max(np.abs(got[:, 0] - ref)) <= 1e-3


def test_device_loop_same_alone_and_in_the_mix(gpu_ctx, served):
    s = served
    draws, aps = _mix(300, 121)
    srv = G.Server(gpu_ctx, s["T"], max_inflight=1024, device_loop=True)
    tickets = [srv.submit(G.gen_params(**d), aps[i], s["hs"]) for i, d in enumerate(draws)]
    mixed = np.array([srv.wait(t)[0] for t in tickets])
    for i in (0, 1, 150, 299):
        t = srv.submit(G.gen_params(**draws[i]), aps[i], s["hs"])
        assert srv.wait(t)[0] == mixed[i]
    srv.close()


def test_device_loop_leaves_when_idle_and_relaunches(gpu_ctx, served):
    """A launch's blocks leave after idle_us without work (bounded device
    polling); the next request relaunches the loop and gets the same value."""
    s = served
    d = W.prior_draws(1, 131)[0]
    srv = G.Server(gpu_ctx, s["T"], max_inflight=16, device_loop=True, idle_us=2000)
    a = srv.wait(srv.submit(G.gen_params(**d), 0, s["hs"]))
    deadline = time.time() + 5.0
    while time.time() < deadline:
        info = srv.loop_info()
        if info["exits_idle"] >= info["blocks"]:
            break
        time.sleep(0.01)
    assert info["exits_idle"] == info["blocks"] and info["launches"] == 1
    b = srv.wait(srv.submit(G.gen_params(**d), 0, s["hs"]))
    assert b == a and srv.loop_info()["launches"] == 2
    srv.close()


def test_device_loop_relaunches_on_new_registration(gpu_ctx, served):
    """Data registered while the loop runs: the running launch is told to leave
    and the next one sees the new stream table; same data, same values."""
    s = served
    f = s["f"]
    draws = W.prior_draws(8, 141)
    srv = G.Server(gpu_ctx, s["T"], max_inflight=64, device_loop=True, idle_us=500000)
    first = [srv.wait(srv.submit(G.gen_params(**d), 0, s["hs"]))[0] for d in draws]
    h2 = [gpu_ctx.register_data(dd, f, W.noise(f, 300 + i), W.analytic_psd(f)) for i, dd in enumerate(W.DETECTORS3)]
    try:
        again = [srv.wait(srv.submit(G.gen_params(**d), 0, h2))[0] for d in draws]
        info = srv.loop_info()
        assert again == first
        # the first launch left (told to stop, or idle if the registration waited for it)
        assert info["launches"] == 2 and info["exits_stop"] + info["exits_idle"] == info["blocks"]
    finally:
        srv.close()
        for h in h2:
            gpu_ctx.release_data(h)


def test_device_loop_bad_requests_and_limits(gpu_ctx, served):
    s = served
    good = W.prior_draws(4, 151)
    srv = G.Server(gpu_ctx, s["T"], max_inflight=32, device_loop=True)
    bad = dict(good[0], mass1=-1.0)
    ts = [srv.submit(G.gen_params(**d), 0, s["hs"]) for d in (good[0], bad, good[1])]
    out = [srv.wait(t) for t in ts]
    assert out[0][1] == 0 and out[2][1] == 0
    assert out[1][1] == 4 and np.isnan(out[1][0])  # outside the model domain
    with pytest.raises(G.GwGpuError):  # one detector count per loop
        srv.submit(G.gen_params(**good[2]), 0, s["hs"][:2])
    srv.close()
    with pytest.raises(G.GwGpuError):  # the loop is mixed precision only
        G.Server(gpu_ctx, s["T"], max_inflight=32, device_loop=True, precision=G.PREC_FP64)
    with pytest.raises(G.GwGpuError):  # tile not a multiple of 256
        G.Server(gpu_ctx, s["T"], max_inflight=32, device_loop=True, tile=1000)


def test_device_loop_poisson_driver(gpu_ctx, oracle, served):
    s = served
    n = 4000
    draws, aps = _mix(n, 161)
    rng = np.random.default_rng(6)
    arrivals = np.cumsum(rng.exponential(1.0 / 1e5, n))
    srv = G.Server(gpu_ctx, s["T"], max_inflight=4096, device_loop=True)
    out, st, lat, wall = srv.drive(G.params_array(draws), aps, s["hs"], arrivals)
    stats = srv.stats()
    srv.close()
    assert np.all(st == 0) and stats["completed"] == n
    assert 0 < stats["p50_s"] <= stats["p99_s"] < 5.0
    pick = list(range(0, n, 97))
    f = s["f"]
    data = [W.noise(f, 300 + i) for i in range(3)]
    ref = oracle.loglik_batch([oracle.params_from_dict(draws[i]) for i in pick], f, list(W.DETECTORS3), data,
                              [W.analytic_psd(f)] * 3, approximants=[aps[i] for i in pick])
    assert np.max(np.abs(out[pick] - ref)) <= 1e-3


def test_device_loop_small_ring_wraps(gpu_ctx, served):
    """A ring of a few slots (the HBM budget admits four) reused many times:
    every slot, claim word and completion entry goes round ~25 laps, and the
    values stay the batched kernel's bit for bit."""
    s = served
    draws, aps = _mix(100, 171)
    per_slot = 4096  # about one slot's bytes for the 32k-bin grid (model constants, partials of 8 items)
    srv = G.Server(gpu_ctx, s["T"], max_inflight=64, device_loop=True, hbm_budget=4 * per_slot)
    try:
        slots = srv.loop_info()["ring_slots"]
        assert 1 <= slots <= 8
        out, st, lat, wall = srv.drive(G.params_array(draws), aps, s["hs"], np.zeros(len(draws)))
    finally:
        srv.close()
    assert np.all(st == 0)
    gpu_ctx.set_tile(4096)
    try:
        for ap in (0, 1):
            idx = [i for i in range(len(draws)) if aps[i] == ap]
            ref, _ = gpu_ctx.loglik_batch(G.params_array([draws[i] for i in idx]), ap, s["hs"], s["T"], G.PREC_MIXED)
            assert np.array_equal(out[idx], ref)
    finally:
        gpu_ctx.set_tile(0)


@pytest.mark.parametrize("dets", [("Hanford",), ("Hanford", "Livingston"),
                                  ("Hanford", "Livingston", "Virgo", "Kagra")])
def test_device_loop_detector_counts(gpu_ctx, served, dets):
    """The loop's kernel for 1, 2 and 4 detectors: the batched kernel's values
    bit for bit at the same tile, D and Pv2."""
    s = served
    f = s["f"]
    hs = [gpu_ctx.register_data(d, f, W.noise(f, 400 + i), W.analytic_psd(f)) for i, d in enumerate(dets)]
    draws, aps = _mix(40, 181)
    srv = G.Server(gpu_ctx, s["T"], max_inflight=128, device_loop=True)
    try:
        got = np.array([srv.wait(t)[0] for t in [srv.submit(G.gen_params(**d), aps[i], hs)
                                                 for i, d in enumerate(draws)]])
    finally:
        srv.close()
    gpu_ctx.set_tile(4096)
    try:
        for ap in (0, 1):
            idx = [i for i in range(len(draws)) if aps[i] == ap]
            ref, st = gpu_ctx.loglik_batch(G.params_array([draws[i] for i in idx]), ap, hs, s["T"], G.PREC_MIXED)
            assert np.all(st == 0)
            assert np.array_equal(got[idx], ref)
    finally:
        gpu_ctx.set_tile(0)
        for h in hs:
            gpu_ctx.release_data(h)


def test_device_loop_bursts_across_idle_exits(gpu_ctx, served):
    """Bursts separated by gaps around idle_us: requests arrive while a
    launch's blocks are leaving, and every one completes with the value it
    has alone."""
    s = served
    draws, aps = _mix(40, 191)
    srv = G.Server(gpu_ctx, s["T"], max_inflight=512, device_loop=True, idle_us=300)
    try:
        alone = [srv.wait(srv.submit(G.gen_params(**d), aps[i], s["hs"]))[0] for i, d in enumerate(draws)]
        rng = np.random.default_rng(3)
        for burst in range(30):
            time.sleep(float(rng.choice([0.0, 0.0002, 0.0003, 0.0004, 0.001])))
            pick = rng.choice(len(draws), size=int(rng.integers(1, 20)), replace=False)
            ts = [(i, srv.submit(G.gen_params(**draws[i]), aps[i], s["hs"])) for i in pick]
            for i, t in ts:
                ll, st = srv.wait(t, timeout_ms=20000)
                assert st == 0 and ll == alone[i]
        info = srv.loop_info()
        assert info["launches"] >= 2  # the loop left idle and was launched again
    finally:
        srv.close()
