"""GPU parity tests through the C ABI: waveform, detector response, the plain
FP64 form, the batched FP64 and mixed forms, against the FP64 oracle."""
import numpy as np
import pytest

import gw_analysis_tools_gb300 as G
from gw_analysis_tools_gb300 import workloads as W

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-3     # |delta log L| absolute, mixed form against the FP64 oracle
FP64_RTOL = 1e-9     # relative, FP64 forms against the FP64 oracle


@pytest.fixture(scope="module")
def network(gpu_ctx, oracle):
    f = W.config1_grid()
    T = 1.0 / (f[1] - f[0])
    src = W.config1_source()
    dets = list(W.DETECTORS3)
    injp = oracle.params_from_dict(dict(src, tc=T - src["tc"]))
    data = []
    for i, d in enumerate(dets):
        r = oracle.detector_response(f, injp, d)
        dt = oracle.dtoa(src["RA"], src["DEC"], src["gmst"], dets[0], d)
        data.append(r * np.exp(-2j * np.pi * dt * f) + W.noise(f, 100 + i))
    psd = [W.analytic_psd(f)] * 3
    handles = [gpu_ctx.register_data(d, f, data[i], psd[i]) for i, d in enumerate(dets)]
    return dict(f=f, T=T, src=src, dets=dets, data=data, psd=psd, handles=handles)


def test_waveform_parity(gpu_ctx, oracle):
    f = W.config1_grid()
    cases = [("IMRPhenomD", 0, W.config1_source()),
             ("IMRPhenomD", 0, W.prior_draws(1, 9)[0]),
             ("IMRPhenomPv2", 1, dict(W.config1_source(), spin1=(0.3, 0.2, 0.3), spin2=(-0.1, 0.4, -0.1))),
             ("IMRPhenomPv2", 1, W.prior_draws(1, 9, precessing=True)[0])]
    for name, ap, d in cases:
        a = oracle.fourier_waveform(f, oracle.params_from_dict(d), ap)
        b = gpu_ctx.fourier_waveform(f, name, G.gen_params(**d))
        for x, y in zip(a, b):
            assert np.max(np.abs(x - y)) <= 1e-11 * np.abs(x).max()


def test_detector_response_parity(gpu_ctx, oracle):
    f = W.config1_grid()
    d = dict(W.config1_source(), RA=2.0, DEC=-0.7, psi=1.3)
    for det in ("Hanford", "Livingston", "Virgo", "Kagra", "ET1"):
        a = oracle.detector_response(f, oracle.params_from_dict(d), det)
        b = gpu_ctx.fourier_detector_response(f, det, "IMRPhenomD", G.gen_params(**d))
        assert np.max(np.abs(a - b)) <= 1e-11 * np.abs(a).max()


def test_log_likelihood_internal(gpu_ctx, oracle, network):
    n = network
    r = oracle.detector_response(n["f"], oracle.params_from_dict(n["src"]), "Hanford")
    ref = oracle.lib().gwo_log_likelihood_internal(oracle._dp(n["data"][0]), oracle._dp(n["psd"][0]),
                                                   oracle._dp(n["f"]), oracle._dp(r.view(np.float64).copy()),
                                                   n["f"].size)
    got = gpu_ctx.log_likelihood_internal(n["data"][0], n["psd"][0], n["f"], r)
    assert abs(got - ref) <= FP64_RTOL * max(1, abs(ref))


def test_plain_single_detector_config1(gpu_ctx, oracle, network):
    """Config 1: single-detector IMRPhenomD, parameters perturbed by 1%."""
    n = network
    draws = W.perturbed(n["src"], 24, seed=5)
    for d in draws:
        ref = oracle.loglik(oracle.params_from_dict(d), n["f"], n["dets"][:1], n["data"][:1], n["psd"][:1])
        got = gpu_ctx.mcmc_likelihood_extrinsic(G.gen_params(**d), "IMRPhenomD", n["handles"][:1], n["T"])
        assert abs(got - ref) <= FP64_RTOL * max(1, abs(ref))


def test_plain_three_detectors_arrival_rotations(gpu_ctx, oracle, network):
    """The plain form on a uniform grid with H/L/V: the arrival-time phase of
    L and V from the per-block rotation tables, D and Pv2, within the FP64
    tolerance of the oracle's per-bin phase."""
    n = network
    cases = [("IMRPhenomD", 0, d) for d in W.perturbed(n["src"], 8, seed=6) + W.prior_draws(8, 61)]
    cases += [("IMRPhenomPv2", 1, d) for d in W.prior_draws(8, 62, precessing=True)]
    for name, ap, d in cases:
        ref = oracle.loglik(oracle.params_from_dict(d), n["f"], n["dets"], n["data"], n["psd"], approximant=ap)
        got = gpu_ctx.mcmc_likelihood_extrinsic(G.gen_params(**d), name, n["handles"], n["T"])
        assert abs(got - ref) <= FP64_RTOL * max(1, abs(ref)), (name, got, ref)


def test_batched_forms_config2(gpu_ctx, oracle, network):
    """Config 2: 512 requests, 3 detectors, prior draws."""
    n = network
    draws = [n["src"]] + W.prior_draws(511, 7)
    ref = oracle.loglik_batch([oracle.params_from_dict(d) for d in draws], n["f"], n["dets"], n["data"], n["psd"])
    fp64, st = gpu_ctx.loglik_batch(G.params_array(draws), G.IMRPhenomD, n["handles"], n["T"], G.PREC_FP64)
    assert np.all(st == 0)
    assert np.max(np.abs(fp64 - ref) / np.maximum(1, np.abs(ref))) <= FP64_RTOL
    mixed, st = gpu_ctx.loglik_batch(G.params_array(draws), G.IMRPhenomD, n["handles"], n["T"], G.PREC_MIXED)
    assert np.all(st == 0)
    assert np.max(np.abs(mixed - ref)) <= MIXED_TOL


def test_batched_pv2(gpu_ctx, oracle, network):
    n = network
    draws = W.prior_draws(96, 11, precessing=True)
    ref = oracle.loglik_batch([oracle.params_from_dict(d) for d in draws], n["f"], n["dets"], n["data"], n["psd"],
                              approximants=[1] * len(draws))
    for prec, tol in ((G.PREC_FP64, None), (G.PREC_MIXED, MIXED_TOL)):
        out, st = gpu_ctx.loglik_batch(G.params_array(draws), G.IMRPhenomPv2, n["handles"], n["T"], prec)
        assert np.all(st == 0)
        if tol is None:
            assert np.max(np.abs(out - ref) / np.maximum(1, np.abs(ref))) <= FP64_RTOL
        else:
            assert np.max(np.abs(out - ref)) <= tol


def test_mixed_approximants_in_one_batch(gpu_ctx, oracle, network):
    n = network
    dd = W.prior_draws(40, 21)
    dp = W.prior_draws(40, 22, precessing=True)
    draws = [x for pair in zip(dd, dp) for x in pair]
    aps = [0, 1] * 40
    ref = oracle.loglik_batch([oracle.params_from_dict(d) for d in draws], n["f"], n["dets"], n["data"], n["psd"],
                              approximants=aps)
    out, st = gpu_ctx.loglik_batch(G.params_array(draws), aps, n["handles"], n["T"], G.PREC_MIXED)
    assert np.all(st == 0)
    assert np.max(np.abs(out - ref)) <= MIXED_TOL


def test_determinism(gpu_ctx, network):
    n = network
    draws = W.prior_draws(300, 31)
    for prec in (G.PREC_FP64, G.PREC_MIXED):
        a, _ = gpu_ctx.loglik_batch(G.params_array(draws), 0, n["handles"], n["T"], prec)
        b, _ = gpu_ctx.loglik_batch(G.params_array(draws), 0, n["handles"], n["T"], prec)
        assert np.array_equal(a, b)


def test_same_result_alone_and_in_the_mix(gpu_ctx, network):
    n = network
    draws = W.prior_draws(200, 41)
    many, _ = gpu_ctx.loglik_batch(G.params_array(draws), 0, n["handles"], n["T"], G.PREC_MIXED)
    for i in (0, 57, 199):
        one, _ = gpu_ctx.loglik_batch(G.params_array([draws[i]]), 0, n["handles"], n["T"], G.PREC_MIXED)
        assert abs(one[0] - many[i]) <= 1e-9 * max(1, abs(many[i]))


def test_bad_requests_flagged_rest_complete(gpu_ctx, oracle, network):
    n = network
    draws = W.prior_draws(8, 51)
    bad = [dict(draws[0], mass1=float("nan")), dict(draws[1], mass2=-3.0)]
    allp = draws[2:] + bad
    ref = oracle.loglik_batch([oracle.params_from_dict(d) for d in draws[2:]], n["f"], n["dets"], n["data"], n["psd"])
    for prec in (G.PREC_FP64, G.PREC_MIXED):
        out, st = gpu_ctx.loglik_batch(G.params_array(allp), 0, n["handles"], n["T"], prec)
        assert np.all(st[:6] == 0) and np.all(st[6:] != 0)
        assert np.all(np.isnan(out[6:]))
        assert np.max(np.abs(out[:6] - ref)) <= MIXED_TOL


def test_uneven_grids_one_launch(gpu_ctx, oracle):
    """Config 3 shape on a reduced band: requests on grids of different T."""
    durations = [4, 8, 32]
    grids, hs, datas, psds = {}, {}, {}, {}
    for T in durations:
        f = W.uniform_grid(20.0, 512.0, 1.0 / T)
        grids[T] = f
        datas[T] = [W.noise(f, 200 + T + i) for i in range(3)]
        psds[T] = [W.analytic_psd(f)] * 3
        hs[T] = [gpu_ctx.register_data(d, f, datas[T][i], psds[T][i]) for i, d in enumerate(W.DETECTORS3)]
    draws = W.prior_draws(30, 61, precessing=True)
    Ts = [durations[i % 3] for i in range(30)]
    handles = np.array([hs[T] for T in Ts], dtype=np.int32)
    for prec, tol in ((G.PREC_FP64, 1e-7), (G.PREC_MIXED, MIXED_TOL)):
        # every grid in one launch; T_segment = 0 -> 1/df of each request's own grid
        out, st = gpu_ctx.loglik_batch(G.params_array(draws), 1, handles, 0.0, prec)
        assert np.all(st == 0)
        for i in range(30):
            T = Ts[i]
            ref = oracle.loglik(oracle.params_from_dict(draws[i]), grids[T], list(W.DETECTORS3), datas[T], psds[T],
                                approximant=1)
            assert abs(out[i] - ref) <= tol * (max(1, abs(ref)) if tol < 1e-6 else 1), (i, out[i], ref)
    for T in durations:
        for h in hs[T]:
            gpu_ctx.release_data(h)


@pytest.mark.parametrize("n", [1, 3, 77])
def test_odd_batch_sizes(gpu_ctx, oracle, network, n):
    """Odd request counts: the per-request outputs of the host-buffer entry
    points sit on their own aligned arrays."""
    nw = network
    draws = W.prior_draws(n, 300 + n)
    ref = oracle.loglik_batch([oracle.params_from_dict(d) for d in draws], nw["f"], nw["dets"], nw["data"],
                              nw["psd"])
    for prec, tol in ((G.PREC_MIXED, MIXED_TOL), (G.PREC_FP64, None)):
        out, st = gpu_ctx.loglik_batch(G.params_array(draws), 0, nw["handles"], nw["T"], prec)
        assert np.all(st == 0)
        err = np.abs(out - ref)
        assert np.all(err <= (tol if tol else FP64_RTOL * np.maximum(1.0, np.abs(ref))))
    # the sampler's 11-dimensional parameters (mcmc_gw.cpp:2492-2568)
    theta = []
    for d in draws:
        m1, m2 = d["mass1"], d["mass2"]
        mc = (m1 * m2) ** 0.6 / (m1 + m2) ** 0.2
        eta = m1 * m2 / (m1 + m2) ** 2
        theta.append([d["RA"], np.sin(d["DEC"]), d["psi"], np.cos(d["incl_angle"]), d["phiRef"], d["tc"],
                      np.log(d["Luminosity_Distance"]), np.log(mc), eta, d["spin1"][2], d["spin2"][2]])
    theta = np.array(theta)
    ref = np.array([oracle.loglik(oracle.mcmc_repack(t, 0, W.GMST), nw["f"], nw["dets"], nw["data"], nw["psd"])
                    for t in theta])
    for prec, tol in ((G.PREC_MIXED, MIXED_TOL), (G.PREC_FP64, None)):
        out, st = gpu_ctx.mcmc_loglik_batch(theta, 0, W.GMST, nw["handles"], nw["T"], prec)
        assert np.all(st == 0)
        err = np.abs(out - ref)
        assert np.all(err <= (tol if tol else FP64_RTOL * np.maximum(1.0, np.abs(ref))))


def test_cooperative_prologue_matches_serial(gpu_ctx, network):
    """The batched prologue spread over four warps gives the constants of the
    one-thread-per-request prologue (GWGPU_PROLOGUE=serial)."""
    import os
    n = network
    dd = W.prior_draws(48, 401)
    dp = W.prior_draws(48, 402, precessing=True)
    draws = [x for pair in zip(dd, dp) for x in pair]
    aps = [0, 1] * 48
    os.environ["GWGPU_PROLOGUE"] = "serial"
    try:
        ser = G.Context(0)
    finally:
        del os.environ["GWGPU_PROLOGUE"]
    try:
        hs = [ser.register_data(d, n["f"], n["data"][i], n["psd"][i]) for i, d in enumerate(n["dets"])]
        # FP64: the cooperative prologue also writes the IMRPhenomD grid
        # coefficients, so its batches take the table form (h within ~2e-12 of
        # the frequency form the serial prologue's batches use)
        for prec, tol in ((G.PREC_FP64, 1e-10), (G.PREC_MIXED, 1e-6)):
            a, sa = gpu_ctx.loglik_batch(G.params_array(draws), aps, n["handles"], n["T"], prec)
            b, sb = ser.loglik_batch(G.params_array(draws), aps, hs, n["T"], prec)
            assert np.array_equal(sa, sb)
            assert np.max(np.abs(a - b) / np.maximum(1.0, np.abs(b))) <= tol
    finally:
        ser.close()


def test_device_batches_rotating_buffers_and_launch_shapes(gpu_ctx, oracle, network):
    """gwgpu_loglik_batch_device over twelve buffer sets in turn (more than the
    eight captured graphs the engine keeps: the least recently used are
    dropped and captured again), before and after the autotuner has picked a
    tile and a blocks-per-SM launch shape; every result against the oracle."""
    import ctypes
    torch = pytest.importorskip("torch")
    n = network
    nsets, m = 12, 40
    draws = [W.prior_draws(m, 500 + s) for s in range(nsets)]
    refs = [oracle.loglik_batch([oracle.params_from_dict(d) for d in dr], n["f"], n["dets"], n["data"], n["psd"])
            for dr in draws]
    pb = ctypes.sizeof(G.GenParams) * m
    dev = torch.device("cuda", 0)
    params = [torch.frombuffer(bytearray(G.params_array(dr)), dtype=torch.uint8).to(dev) for dr in draws]
    approx = torch.zeros(m, dtype=torch.int32, device=dev)
    outs = [torch.zeros(m, dtype=torch.float64, device=dev) for _ in range(nsets)]
    stats = [torch.zeros(m, dtype=torch.int32, device=dev) for _ in range(nsets)]
    assert params[0].numel() == pb

    def run_all():
        for rep in range(2):
            for s in range(nsets):
                gpu_ctx.loglik_batch_device(params[s].data_ptr(), approx.data_ptr(), m, n["handles"], n["T"],
                                            G.PREC_MIXED, outs[s].data_ptr(), stats[s].data_ptr())
        torch.cuda.synchronize()
        for s in range(nsets):
            assert np.all(stats[s].cpu().numpy() == 0)
            assert np.max(np.abs(outs[s].cpu().numpy() - refs[s])) <= MIXED_TOL

    run_all()
    tile, ms = gpu_ctx.autotune(params[0].data_ptr(), approx.data_ptr(), m, n["handles"], n["T"], G.PREC_MIXED,
                                outs[0].data_ptr(), stats[0].data_ptr())
    assert tile in (1024, 2048, 4096, 8192, 16384) and ms > 0
    run_all()


def test_work_order_and_launch_shape_leave_results_unchanged(gpu_ctx, oracle, monkeypatch):
    """The mixed batch's items run in work order (most live bins first,
    written by the prologue) or in plan order (GWGPU_ITEM_ORDER=listed), with 3
    or 4 blocks per SM: each item writes its own partials and each request's
    finalize sums them in item order, so the results are the same to the last
    bit.  An uneven D/Pv2 batch with two requests outside the model domain."""
    durations = [4, 8, 16]
    grids, datas, psds = {}, {}, {}
    for T in durations:
        f = W.uniform_grid(20.0, 1024.0, 1.0 / T)
        grids[T] = f
        datas[T] = [W.noise(f, 700 + T + i) for i in range(3)]
        psds[T] = [W.analytic_psd(f)] * 3
    draws = W.prior_draws(24, 71) + W.prior_draws(24, 72, precessing=True)
    draws[5] = dict(draws[5], mass1=-1.0)
    draws[30] = dict(draws[30], mass2=0.0)
    aps = np.array([0] * 24 + [1] * 24, dtype=np.int32)
    Ts = [durations[i % 3] for i in range(len(draws))]
    monkeypatch.setenv("GWGPU_ITEM_ORDER", "listed")
    listed = G.Context(0)
    monkeypatch.delenv("GWGPU_ITEM_ORDER")
    results = []
    for ctx in (gpu_ctx, listed):
        hs = {T: [ctx.register_data(d, grids[T], datas[T][i], psds[T][i]) for i, d in enumerate(W.DETECTORS3)]
              for T in durations}
        handles = np.array([hs[T] for T in Ts], dtype=np.int32)
        ctx.set_tile(2048)
        for blocks in (3, 4):
            ctx.set_blocks_per_sm(blocks)
            out, st = ctx.loglik_batch(G.params_array(draws), aps, handles, 0.0, G.PREC_MIXED)
            assert ctx.last_launch_shape()[:2] == (2048, blocks)
            results.append((out.copy(), st.copy()))
        ctx.set_tile(0)
        ctx.set_blocks_per_sm(0)
        for T in durations:
            for h in hs[T]:
                ctx.release_data(h)
    listed.close()
    out0, st0 = results[0]
    assert st0[5] == 4 and st0[30] == 4 and np.count_nonzero(st0) == 2
    for out, st in results[1:]:
        assert np.array_equal(st, st0)
        assert np.array_equal(out, out0, equal_nan=True)
    for i in range(len(draws)):
        if st0[i]:
            continue
        T = Ts[i]
        ref = oracle.loglik(oracle.params_from_dict(draws[i]), grids[T], list(W.DETECTORS3), datas[T], psds[T],
                            approximant=int(aps[i]))
        assert abs(out0[i] - ref) <= MIXED_TOL, (i, out0[i], ref)
    with pytest.raises(G.GwGpuError):
        gpu_ctx.set_blocks_per_sm(5)
