#!/usr/bin/env python
"""Benchmark of the gw_analysis_tools likelihood path on GB300.

Headline workload: the batched parallel-tempering step -- IMRPhenomD over
Hanford/Livingston/Virgo, 64 chains x 8 temperatures = 512 log-likelihood
requests per step, parameters drawn from the priors, on the 20-1024 Hz grid at
df = 1/32 Hz (32,128 bins), analytic PSD, injected signal plus seeded noise.
A step is one pass of the hot path over one batch of 512 requests.

  value   evals/s of the batched mixed-precision form, parameters resident on
          the device, CUDA events on the engine stream; L2 flushed (256 MiB
          write) before every step, outside the events.
  e2e     the same through the C ABI entry point gwgpu_loglik_batch with host
          buffers: the parameters host -> device and log L + status device ->
          host inside the timed region (the kernels read and write the pinned
          staging buffer over the host-device link), wall clock per step, L2
          flushed before every step.

Beside them: the plain FP64 one-request-per-launch form, the batched FP64
form, the served form (the device-resident request loop under Poisson
arrivals, mixed D/Pv2, p50/p99, saturation and latency against offered load,
with the host scheduler's numbers beside it), the uneven Pv2 batch and the
batched Fisher, a roofline of the fused bin kernel, and the CPU oracle timed
on the host cores.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_REQ = 512
METRIC = "logL evals/s (batched+served vs plain FP64, |dlogL|<=1e-3); p50/p99 latency"
WORKLOAD = ("batched PT step: IMRPhenomD, H/L/V, 64 chains x 8 temperatures = 512 requests/step, "
            "20-1024 Hz at df=1/32 Hz (32128 bins), prior draws, analytic PSD, injected signal + seeded noise")


_T0 = time.time()


def log(msg):
    """Progress line on stderr (the JSON result is the only stdout line)."""
    sys.stderr.write("[bench %7.1fs] %s\n" % (time.time() - _T0, msg))
    sys.stderr.flush()


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--quick", action="store_true", help="skip the secondary forms")
    ap.add_argument("--forms", default="", help="comma-separated secondary forms to run (default: all)")
    ap.add_argument("--tile", type=int, default=0, help="fixed bin tile of the headline step (0: autotuned)")
    ap.add_argument("--blocks-per-sm", type=int, default=0,
                    help="fixed resident blocks per SM of the headline step (0: autotuned)")
    return ap.parse_args()


def dist_setup(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1 and args.impl == "ours":
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group(backend="nccl")
        pg = dist
    return rank, world, local, pg


# ----------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# --------------------------------------------------------------- workload
def make_network(ctx, G, W, O=None):
    """Grid, injected data (signal from the engine's FP64 detector response)."""
    f = W.config1_grid()
    T = 1.0 / (f[1] - f[0])
    src = W.config1_source()
    inj = G.gen_params(**dict(src, tc=T - src["tc"]))
    data = []
    for i, d in enumerate(W.DETECTORS3):
        r = ctx.fourier_detector_response(f, d, "IMRPhenomD", inj)
        # time-of-arrival shift relative to Hanford, as the likelihood applies it
        dt = _dtoa(src, W.DETECTORS3[0], d)
        data.append(r * np.exp(-2j * np.pi * dt * f) + W.noise(f, 100 + i))
    psd = W.analytic_psd(f)
    handles = [ctx.register_data(d, f, data[i], psd) for i, d in enumerate(W.DETECTORS3)]
    return f, T, data, psd, handles


_LOC = {"Hanford": (-2.16141492636e+06, -3.83469517889e+06, 4.60035022664e+06),
        "Livingston": (-7.42760447238e+04, -5.49628371971e+06, 3.22425701744e+06),
        "Virgo": (4.54637409900e+06, 8.42989697626e+05, 4.37857696241e+06)}


def _dtoa(src, d1, d2):  # DTOA_earth_centered_coord (detector_util.cpp:760-780)
    a, b = np.array(_LOC[d1]), np.array(_LOC[d2])
    ha = src["gmst"] - src["RA"]
    e = np.array([np.cos(src["DEC"]) * np.cos(ha), np.cos(src["DEC"]) * -np.sin(ha), np.sin(src["DEC"])])
    return float((a - b) @ e / 299792458.0)


def flush_l2(buf):
    buf.add_(1.0)  # 256 MiB read+write > 126 MiB L2


# ------------------------------------------------------------- our arm
def run_ours(args, rank, world, local, pg):
    import torch
    import gw_analysis_tools_gb300 as G
    from gw_analysis_tools_gb300 import _native, workloads as W

    log("build")
    _native.build()
    torch.cuda.set_device(local)
    ctx = G.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))
    flush = torch.zeros(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    f, T, data, psd, handles = make_network(ctx, G, W)

    nbatch = 8
    draws = [W.prior_draws(N_REQ, 1000 + 97 * rank + b) for b in range(nbatch)]
    draws[0][0] = W.config1_source()
    host_params = [G.params_array(d) for d in draws]
    pbytes = ctypes_sizeof(G.GenParams) * N_REQ
    d_params = torch.empty((nbatch, pbytes), dtype=torch.uint8, device="cuda")
    for b in range(nbatch):
        d_params[b].copy_(torch.frombuffer(bytearray(host_params[b]), dtype=torch.uint8))
    d_approx = torch.zeros(N_REQ, dtype=torch.int32, device="cuda")
    d_out = torch.zeros((nbatch, N_REQ), dtype=torch.float64, device="cuda")
    d_stat = torch.zeros((nbatch, N_REQ), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()

    def step(b, prec=G.PREC_MIXED):
        ctx.loglik_batch_device(d_params[b].data_ptr(), d_approx.data_ptr(), N_REQ, handles, T, prec,
                                d_out[b].data_ptr(), d_stat[b].data_ptr())

    if args.tile or args.blocks_per_sm:
        # a fixed launch shape (profiling a given shape)
        ctx.set_tile(args.tile)
        ctx.set_blocks_per_sm(args.blocks_per_sm)
    else:
        log("autotune")
        # autotune the launch shape once on this workload, then warm up (graph capture)
        ctx.autotune(d_params[0].data_ptr(), d_approx.data_ptr(), N_REQ, handles, T, G.PREC_MIXED,
                     d_out[0].data_ptr(), d_stat[0].data_ptr())
    for i in range(args.warmup):
        step(i % nbatch)
    torch.cuda.synchronize()
    tile, blocks_per_sm, grid = ctx.last_launch_shape()

    log("timed steps")
    # ---------------- value: device-resident, CUDA events on the engine stream
    e0 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    e1 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for i in range(args.steps):
            with torch.cuda.stream(stream):
                flush_l2(flush)
                e0[i].record(stream)
            step(i % nbatch)
            with torch.cuda.stream(stream):
                e1[i].record(stream)
        torch.cuda.synchronize()
    step_ms = [a.elapsed_time(b) for a, b in zip(e0, e1)]
    tot_ms, units, value = replica_aggregate(float(np.sum(step_ms)), N_REQ * args.steps, pg, "cuda")
    # prologue (which also writes the work order) and fused bin kernel per step
    # (the memset node is not ours)
    gpu_launches = 2 * args.steps

    # status and a parity sample for |dlogL| against the oracle (cpu_baseline leg below)
    out_mixed = d_out[0].cpu().numpy().copy()
    stat0 = d_stat[0].cpu().numpy().copy()

    # ---------------- per-kernel timing (roofline): events around prologue and bin kernel
    ctx.lib.gwgpu_batch_timing(ctx.h, 1)
    import ctypes
    pro, ker = [], []
    for i in range(max(5, args.steps // 2)):
        with torch.cuda.stream(stream):
            flush_l2(flush)
        step(i % nbatch)
        a, b = ctypes.c_float(), ctypes.c_float()
        ctx.lib.gwgpu_batch_last_timing(ctx.h, ctypes.byref(a), ctypes.byref(b))
        pro.append(a.value)
        ker.append(b.value)
    ctx.lib.gwgpu_batch_timing(ctx.h, 0)
    kernel_ms = float(np.mean(ker))
    prologue_ms = float(np.mean(pro))

    log("e2e")
    # ---------------- e2e: C ABI with host buffers
    e2e_t = []
    for i in range(args.warmup + args.steps):
        with torch.cuda.stream(stream):
            flush_l2(flush)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ll, st = ctx.loglik_batch(host_params[i % nbatch], 0, handles, T, G.PREC_MIXED)
        t1 = time.perf_counter()
        if i >= args.warmup:
            e2e_t.append(t1 - t0)
    _, _, e2e_value = replica_aggregate(max(float(np.sum(e2e_t)), 1e-12) * 1e3, N_REQ * len(e2e_t), pg, "cuda")
    h2d = N_REQ * (ctypes_sizeof(G.GenParams) + 4)
    d2h = N_REQ * (8 + 4)

    res = {}
    res.update(dict(value=value, tot_ms=tot_ms, step_ms=step_ms, kernel_ms=kernel_ms, prologue_ms=prologue_ms,
                    e2e_value=e2e_value, h2d=h2d, d2h=d2h, clocks=clk.summary(), tile=tile,
                    launch_shape={"tile": tile, "blocks_per_sm": blocks_per_sm, "grid": grid,
                                  "chosen_by": "fixed" if (args.tile or args.blocks_per_sm) else "autotuner"},
                    gpu_launches=gpu_launches, stat_ok=int((stat0 == 0).sum())))

    if not args.quick and rank == 0:
        res["extras"] = secondary_forms(ctx, G, W, torch, stream, flush, f, T, handles, host_params, d_params,
                                        d_approx, d_out, d_stat, args)
    log("device work done")
    res["out_mixed"] = out_mixed
    res["draws0"] = draws[0]
    res["f"], res["data"], res["psd"], res["T"] = f, data, psd, T
    return res


def replica_aggregate(local_ms, local_units, pg, device="cpu"):
    """Replicas: the job's time is the slowest rank's, its work the sum of
    all ranks' units.  Returns (max ms, total units, units/s)."""
    if pg is None:
        return local_ms, local_units, local_units / (local_ms / 1e3)
    import torch
    t = torch.tensor([local_ms], dtype=torch.float64, device=device)
    u = torch.tensor([float(local_units)], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    pg.all_reduce(u, op=pg.ReduceOp.SUM)
    ms, units = float(t.item()), float(u.item())
    return ms, units, units / (ms / 1e3)


def ctypes_sizeof(t):
    import ctypes
    return ctypes.sizeof(t)


def secondary_forms(ctx, G, W, torch, stream, flush, f, T, handles, host_params, d_params, d_approx, d_out, d_stat,
                    args):
    """The other forms, each timed on its own; an error in one is recorded in
    the result and the others still run."""
    ex = {}

    def plain():
        # plain FP64, one request per launch (host params, synchronous drop-in call)
        plist = host_params[1]
        nplain = 128
        times = []
        for i in range(nplain + 8):
            with torch.cuda.stream(stream):
                flush_l2(flush)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ctx.mcmc_likelihood_extrinsic(plist[i % N_REQ], "IMRPhenomD", handles, T)
            if i >= 8:
                times.append(time.perf_counter() - t0)
        ex["plain_fp64_evals_per_s"] = len(times) / float(np.sum(times))
        ex["plain_fp64_p50_ms"] = float(np.median(times) * 1e3)
        # the plain workload itself: Hanford only, 1000 calls at the injection
        # scaled by 1 + 0.01 N(0,1) per parameter, FP64, L2 flushed before each
        h1 = handles[:1]
        c1 = W.perturbed(W.config1_source(), 1000, 21, frac=0.01)
        c1p = [G.gen_params(**d) for d in c1]
        t1, o1 = [], np.zeros(len(c1p))
        for i in range(-8, len(c1p)):  # 8 warm-up calls, then each request once
            with torch.cuda.stream(stream):
                flush_l2(flush)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            v = ctx.mcmc_likelihood_extrinsic(c1p[i % len(c1p)], "IMRPhenomD", h1, T)
            if i >= 0:
                t1.append(time.perf_counter() - t0)
                o1[i] = v
        ex["plain_config1"] = {"evals_per_s": len(t1) / float(np.sum(t1)), "p50_ms": float(np.median(t1) * 1e3),
                               "p99_ms": float(np.percentile(t1, 99) * 1e3), "calls": len(t1),
                               "workload": "IMRPhenomD, Hanford only, 32128 bins, the injection scaled by "
                                           "1 + 0.01 N(0,1) per parameter, FP64, one call per request"}
        ex["_parity_plain1"] = (c1[:200], o1[:200].copy())

    def batched_fp64():
        # batched FP64 (device resident)
        ctx.loglik_batch_device(d_params[1].data_ptr(), d_approx.data_ptr(), N_REQ, handles, T, G.PREC_FP64,
                                d_out[1].data_ptr(), d_stat[1].data_ptr())
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        tot = 0.0
        for i in range(3):
            with torch.cuda.stream(stream):
                flush_l2(flush)
                ev[0].record(stream)
            ctx.loglik_batch_device(d_params[1].data_ptr(), d_approx.data_ptr(), N_REQ, handles, T, G.PREC_FP64,
                                    d_out[1].data_ptr(), d_stat[1].data_ptr())
            with torch.cuda.stream(stream):
                ev[1].record(stream)
            torch.cuda.synchronize()
            tot += ev[0].elapsed_time(ev[1])
        ex["batched_fp64_evals_per_s"] = 3 * N_REQ / (tot / 1e3)

    def served():
        # 16 ensembles (chains 8-256, temperatures 4-16), Poisson 2e5/s, D/Pv2 50/50
        rng = np.random.default_rng(7)
        ens = [(int(rng.integers(8, 257)), int(rng.integers(4, 17))) for _ in range(16)]
        nserve = 60000
        dd = W.prior_draws(nserve // 2, 501)
        dp = W.prior_draws(nserve - nserve // 2, 502, precessing=True)
        sp, sa = [], []
        for i in range(nserve):
            if i % 2 == 0:
                sp.append(dd[i // 2])
                sa.append(0)
            else:
                sp.append(dp[i // 2])
                sa.append(1)
        arrivals = np.cumsum(rng.exponential(1.0 / 2e5, nserve))
        pick = np.arange(0, nserve, 29)  # a parity sample, both approximants
        # the same mix offered faster than the engine serves it: its capacity
        nsat = 200000
        ds = W.prior_draws(nsat // 2, 503)
        dq = W.prior_draws(nsat - nsat // 2, 504, precessing=True)
        sp2 = [ds[i // 2] if i % 2 == 0 else dq[i // 2] for i in range(nsat)]
        sa2 = [i % 2 for i in range(nsat)]
        arr2 = np.cumsum(rng.exponential(1.0 / 5e6, nsat))

        def run(srv, info=None):
            """2e5/s, saturation (5e6/s offered) and latency against offered load;
            info(): the device loop's counters after the first two."""
            srv.drive(G.params_array(sp[:2000]), sa[:2000], handles, arrivals[:2000] - arrivals[0])  # warm-up
            srv.reset_stats()
            out, st, lat, wall = srv.drive(G.params_array(sp), sa, handles, arrivals - arrivals[0])
            s = srv.stats()
            r = {"evals_per_s": nserve / wall, "p50_ms": s["p50_s"] * 1e3, "p99_ms": s["p99_s"] * 1e3,
                 "offered_rate": 2e5, "requests": nserve, "launches": s["launches"], "ok": int((st == 0).sum())}
            got = out[pick].copy()
            if info:
                r["loop"] = info()
            srv.reset_stats()
            _, st2, _, wall2 = srv.drive(G.params_array(sp2), sa2, handles, arr2 - arr2[0])
            s2 = srv.stats()
            r["saturated"] = {"evals_per_s": nsat / wall2, "p50_ms": s2["p50_s"] * 1e3, "p99_ms": s2["p99_s"] * 1e3,
                              "offered_rate": 5e6, "requests": nsat, "launches": s2["launches"],
                              "ok": int((st2 == 0).sum())}
            if info:
                r["saturated"]["loop"] = info()
            curve = []
            for rate in (5e5, 1e6, 2e6, 3e6):
                nr = int(min(100000, max(20000, rate * 0.05)))
                arr3 = np.cumsum(np.random.default_rng(int(rate)).exponential(1.0 / rate, nr))
                srv.reset_stats()
                _, st3, _, wall3 = srv.drive(G.params_array(sp2[:nr]), sa2[:nr], handles, arr3 - arr3[0])
                s3 = srv.stats()
                curve.append({"offered_rate": rate, "evals_per_s": nr / wall3, "p50_ms": s3["p50_s"] * 1e3,
                              "p99_ms": s3["p99_s"] * 1e3, "requests": nr, "launches": s3["launches"],
                              "ok": int((st3 == 0).sum())})
            r["load_curve"] = curve
            return r, got

        # the device-resident request loop (the served form)
        srv = G.Server(ctx, T, max_inflight=65536, device_loop=True, hbm_budget=120 * 1024 ** 3)
        try:
            r, got = run(srv, srv.loop_info)
        finally:
            srv.close()
        r.update({"form": "device-resident request loop", "ensembles": ens})
        ex["served"] = r
        ex["_parity_served"] = ([sp[i] for i in pick], [sa[i] for i in pick], got)
        # the host scheduler: fused batches on 4 stream lanes
        srv = G.Server(ctx, T, max_inflight=65536, max_batch=2048, lanes=4, hbm_budget=120 * 1024 ** 3)
        try:
            r2, got2 = run(srv)
        finally:
            srv.close()
        r2.update({"form": "host scheduler, batches up to 2048 on 4 lanes"})
        ex["served"]["host_scheduler"] = r2
        ex["_parity_served_host"] = got2

    def uneven():
        # uneven Pv2 batch: T in {4, 8, 32, 128}, 20-2048 Hz, 1024 requests, one launch
        Ts = W.uneven_durations(1024, 9)
        hmap, udata = {}, {}
        for Tu in (4, 8, 32, 128):
            fu = W.uniform_grid(20.0, 2048.0, 1.0 / Tu)
            psd_u = W.analytic_psd(fu)
            udata[Tu] = [uneven_injection(ctx, G, fu, Tu, d) + W.noise(fu, 900 + Tu + i)
                         for i, d in enumerate(W.DETECTORS3)]
            hmap[Tu] = [ctx.register_data(d, fu, udata[Tu][i], psd_u) for i, d in enumerate(W.DETECTORS3)]
        # T_segment = 0: each request uses 1/df of its own grid
        pu = W.prior_draws(1024, 11, precessing=True)
        hs = np.array([hmap[int(t)] for t in Ts], dtype=np.int32)
        bins = int(sum(int(2028 * t) for t in Ts))
        parr = G.params_array(pu)
        # the launch shape tuned on this batch (device copies of its inputs)
        dp = torch.frombuffer(bytearray(parr), dtype=torch.uint8).cuda()
        da = torch.ones(len(pu), dtype=torch.int32, device="cuda")
        do = torch.zeros(len(pu), dtype=torch.float64, device="cuda")
        ds = torch.zeros(len(pu), dtype=torch.int32, device="cuda")
        utile, _ = ctx.autotune(dp.data_ptr(), da.data_ptr(), len(pu), hs, 0.0, G.PREC_MIXED, do.data_ptr(),
                                ds.data_ptr())
        ctx.loglik_batch(parr, 1, hs, 0.0, G.PREC_MIXED)
        t0 = time.perf_counter()
        reps = 3
        for _ in range(reps):
            _, st = ctx.loglik_batch(parr, 1, hs, 0.0, G.PREC_MIXED)
        dt = (time.perf_counter() - t0) / reps
        ex["uneven_pv2"] = {"evals_per_s": 1024 / dt, "ms_per_launch": dt * 1e3, "bins_per_launch": bins,
                            "tile": utile,
                            "grid_bins": sorted(set(int(2028 * t) for t in Ts)), "ok": int((st == 0).sum()),
                            "data": "Pv2 injection (SNR ~ 50 on the 128 s grid) + seeded noise per grid"}
        out_u, _ = ctx.loglik_batch(parr, 1, hs, 0.0, G.PREC_MIXED)
        ex["_parity_uneven"] = (pu, [int(t) for t in Ts], udata, out_u.copy())

    def fisher():
        # batched Fisher: IMRPhenomD 3 detectors, 10-2048 Hz at df=1/16, step 1e-6 relative
        ff = W.uniform_grid(10.0, 2048.0, 1.0 / 16.0)
        psd_f = W.analytic_psd(ff)
        hf = [ctx.register_data(d, ff, np.zeros(ff.size, complex), psd_f) for d in W.DETECTORS3]
        nf = 10000
        pf = G.params_array(W.prior_draws(nf, 13))
        ctx.fisher_batch(G.params_array(W.prior_draws(64, 14)), 0, hf, epsilon=1e-6, step_mode=1)
        t0 = time.perf_counter()
        fish, cov, fst = ctx.fisher_batch(pf, 0, hf, epsilon=1e-6, step_mode=1)
        dt = time.perf_counter() - t0
        codes, counts = np.unique(fst, return_counts=True)
        ex["fisher"] = {"fishers_per_s": nf / dt, "sources": nf, "bins": int(ff.size), "seconds": dt,
                        "ok": int((fst == 0).sum()),
                        "status_counts": {str(int(c)): int(k) for c, k in zip(codes, counts)},
                        "form": "moment sums (FP64 waveform differences, weights and sums), order 2; "
                                "sources it cannot invert redone by the FP64 reference algorithm",
                        "oracle_singular": "4 of these 10,000 (664, 1017, 4710, 6707: within 3 degrees of face-on) "
                                           "are not positive definite in the FP64 oracle either"}
        # the moment form with FP32 values in compensated FP32 sums
        ctx.fisher_batch_ex(G.params_array(W.prior_draws(64, 14)), 0, hf, epsilon=1e-6, step_mode=1,
                            precision=G.PREC_MIXED, algorithm=G.FISHER_MOMENTS)
        t0 = time.perf_counter()
        f32, c32, st32 = ctx.fisher_batch_ex(pf, 0, hf, epsilon=1e-6, step_mode=1, precision=G.PREC_MIXED,
                                             algorithm=G.FISHER_MOMENTS)
        dt32 = time.perf_counter() - t0
        codes, counts = np.unique(st32, return_counts=True)
        ex["fisher"]["fp32_sums"] = {"fishers_per_s": nf / dt32, "seconds": dt32, "ok": int((st32 == 0).sum()),
                                     "status_counts": {str(int(c)): int(k) for c, k in zip(codes, counts)}}
        # the reference algorithm in FP64 (orders 2 and 4) and the sampler's proposal
        nr = 2048
        pr = G.params_array(W.prior_draws(nr, 13))
        for order in (2, 4):
            ctx.fisher_batch_ex(G.params_array(W.prior_draws(64, 14)), 0, hf, order=order, epsilon=1e-6, step_mode=1)
            t0 = time.perf_counter()
            ctx.fisher_batch_ex(pr, 0, hf, order=order, epsilon=1e-6, step_mode=1)
            ex["fisher"]["reference_algorithm_order%d_per_s" % order] = nr / (time.perf_counter() - t0)
        theta = mcmc_theta(W.prior_draws(nr, 15))
        ctx.mcmc_fisher_batch(theta[:64], hf, W.GMST)
        t0 = time.perf_counter()
        ctx.mcmc_fisher_batch(theta, hf, W.GMST)
        ex["fisher"]["mcmc_proposal_per_s"] = nr / (time.perf_counter() - t0)
        ex["fisher"]["mcmc_proposal_form"] = ("moment form at order 4 (five-point rule with the reference's constant "
                                              "phase), epsilon 1e-8 absolute, prior diagonal")
        ns = 64  # parity sample: the moment form and the reference algorithm against the oracle
        fr, cr, _ = ctx.fisher_batch_ex(G.params_array(W.prior_draws(ns, 13)), 0, hf, order=2, epsilon=1e-6,
                                        step_mode=1)
        ex["_fisher_sample"] = (pf, fish[:ns].copy(), cov[:ns].copy(), fr, cr, ff, psd_f, f32[:ns].copy(),
                                c32[:ns].copy())
        # the five-point rule in the moment form, on 16 of them
        f4, _, _ = ctx.fisher_batch_ex(G.params_array(W.prior_draws(16, 13)), 0, hf, order=4, epsilon=1e-6,
                                       step_mode=1, algorithm=G.FISHER_MOMENTS)
        ex["_fisher_sample4"] = (W.prior_draws(16, 13), f4, ff, psd_f)

    def maximized():
        # the sampler's intrinsic mode: likelihood maximised over t_c and phi_c
        # (one batched FFT per step), IMRPhenomD and IMRPhenomPv2, same network
        out = {}
        for name, ap, draws in (("D", G.IMRPhenomD, host_params[1][:N_REQ]),
                                ("Pv2", G.IMRPhenomPv2, W.prior_draws(N_REQ, 15, precessing=True))):
            parr = G.params_array(draws)
            ctx.maximized_loglik_batch(parr, handles, approximant=ap)
            reps = 3
            t0 = time.perf_counter()
            for _ in range(reps):
                _, st = ctx.maximized_loglik_batch(parr, handles, approximant=ap)
            dt = (time.perf_counter() - t0) / reps
            res_mx, _ = ctx.maximized_loglik_batch(parr, handles, approximant=ap)
            out[name] = {"evals_per_s": N_REQ / dt, "ms_per_step": dt * 1e3, "ok": int((st == 0).sum())}
            ex.setdefault("_parity_maximized", {})[name] = (draws[:64], ap, res_mx[:64].copy())
        ex["maximized"] = dict(out, requests=N_REQ, bins=int(f.size), transforms_per_step=N_REQ * len(handles))

    def ingest():
        # strain text files (GWOSC layout, 3 detectors x 128 s x 4096 Hz) and a
        # PSD table (T_obs 32 s) -> windowed, transformed, band-limited spectra
        import tempfile
        fs_i, dur_i, t0_i, nd_i = 4096, 128, 1126259446, 3
        rng = np.random.default_rng(17)
        tmp = tempfile.mkdtemp(prefix="gwgpu_ingest_")
        files, nbytes = [], 0
        series = rng.normal(0, 1e-21, (nd_i, fs_i * dur_i))
        for d in range(nd_i):
            p = os.path.join(tmp, "strain%d.txt" % d)
            with open(p, "w") as fh:
                fh.write("# synthetic strain\n# This file has %d samples per second\n# starting GPS %d duration %d\n"
                         % (fs_i, t0_i, dur_i))
                fh.write("\n".join(map(repr, series[d].tolist())) + "\n")
            nbytes += os.path.getsize(p)
            files.append(p)
        fpsd = np.arange(20.0, 2048.0, 1.0 / 32)
        psd_path = os.path.join(tmp, "psd.txt")
        with open(psd_path, "w") as fh:
            fh.write("# freq H1 L1 V1\n")
            fh.write("".join("%r %r %r %r\n" % (x, 1e-46, 1e-46, 2e-46) for x in fpsd.tolist()))
        npsd = G.count_lines_losc_psd_file(psd_path)
        ndata = G.count_lines_losc_data_file(files[0])
        ctx.allocate_losc_data(files, psd_path, npsd, ndata, t0_i + 64.0, 2.0)  # warm-up (plans)
        t0 = time.perf_counter()
        ctx.allocate_losc_data(files, psd_path, npsd, ndata, t0_i + 64.0, 2.0)
        t_files = time.perf_counter() - t0
        tab = np.column_stack([fpsd] + [np.full(fpsd.size, 1e-46)] * nd_i)
        t0 = time.perf_counter()
        reps = 5
        for _ in range(reps):
            ctx.losc_prepare(series, float(t0_i), float(dur_i), float(fs_i), tab, t0_i + 64.0, 2.0)
        t_mem = (time.perf_counter() - t0) / reps
        ex["ingest"] = {"detectors": nd_i, "samples_per_detector": fs_i * dur_i, "text_bytes": nbytes,
                        "files_to_spectra_s": t_files, "text_mb_per_s": nbytes / t_files / 1e6,
                        "transform_from_memory_ms": t_mem * 1e3, "bins": int(npsd), "host_threads": os.cpu_count()}
        for p in files + [psd_path]:
            os.remove(p)
        os.rmdir(tmp)

    def gaussleg():
        # GAUSSLEG integration: a 3000-node Gauss-Legendre grid over 20-1024 Hz,
        # weighted streams, batched FP64 (the mixed form needs uniform grids)
        x, wq = np.polynomial.legendre.leggauss(3000)
        h = 0.5 * (1024.0 - 20.0)
        fg, wg = 20.0 + h * (x + 1.0), wq * h
        psd_g = W.analytic_psd(fg)
        dg = [W.noise(fg, 700 + i) for i in range(3)]
        hg = [ctx.register_data(d, fg, dg[i], psd_g, weights=wg) for i, d in enumerate(W.DETECTORS3)]
        parr = host_params[1]
        ctx.loglik_batch(parr, 0, hg, 8.0, G.PREC_FP64)
        reps = 5
        t0 = time.perf_counter()
        for _ in range(reps):
            _, st = ctx.loglik_batch(parr, 0, hg, 8.0, G.PREC_FP64)
        dt = (time.perf_counter() - t0) / reps
        out_g, _ = ctx.loglik_batch(parr, 0, hg, 8.0, G.PREC_FP64)
        ex["gaussleg_fp64"] = {"evals_per_s": N_REQ / dt, "ms_per_call": dt * 1e3, "nodes": int(fg.size),
                               "ok": int((st == 0).sum())}
        ex["_parity_gaussleg"] = (host_params[1], fg, wg, dg, psd_g, out_g.copy())

    for name, fn in (("plain", plain), ("batched_fp64", batched_fp64), ("served", served), ("uneven", uneven),
                     ("fisher", fisher), ("maximized", maximized), ("ingest", ingest), ("gaussleg", gaussleg)):
        if args.forms and name not in args.forms.split(","):
            continue
        log(name)
        try:
            fn()
        except Exception as e:  # recorded in the result line; the remaining forms still run
            ex.setdefault("errors", {})[name] = repr(e)
            log("%s failed: %r" % (name, e))
    return ex


# --------------------------------------------------------- CPU baseline
def cpu_baseline(res, seconds=10.0):
    """The C oracle (FP64 restatement of the reference path, OpenMP over
    requests) on the host cores: a bounded sample of the same workload."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from gw_analysis_tools_gb300 import workloads as W
    O.build()
    f, data, psd = res["f"], res["data"], res["psd"]
    dets = list(W.DETECTORS3)
    draws = res["draws0"]
    plist = [O.params_from_dict(d) for d in draws]
    ref = O.loglik_batch(plist, f, dets, data, [psd] * 3)
    t0 = time.perf_counter()
    n = 0
    while time.perf_counter() - t0 < seconds:
        O.loglik_batch(plist, f, dets, data, [psd] * 3)
        n += len(plist)
    dt = time.perf_counter() - t0
    cores = os.cpu_count()
    err = np.abs(res["out_mixed"] - ref)
    m, t1 = 0, time.perf_counter()  # the same port on one thread
    while time.perf_counter() - t1 < 4.0:
        O.loglik_batch(plist[:16], f, dets, data, [psd] * 3, nthreads=1)
        m += 16
    one = m / (time.perf_counter() - t1)
    return {"value": n / dt, "unit": "evals/s", "cores": cores, "kind": "port",
            "sample": "%d requests of the 512-request step (prior draws), %.1f s on %d threads" % (n, dt, cores),
            "value_1_core": one, "reference_code": reference_code_rate(O, f, dets, data, psd, plist)}, \
        {"max_abs_dlogL": float(err.max()), "p99_abs_dlogL": float(np.percentile(err, 99)),
         "median_abs_dlogL": float(np.median(err)), "requests": int(err.size)}


def reference_code_rate(O, f, dets, data, psd, plist, seconds=6.0):
    """The reference's own MCMC_likelihood_extrinsic (mcmc_gw.cpp:2374-2487,
    compiled unmodified from its sources by oracle/Makefile target "full") on
    one host thread, beside the C port on one thread over the same requests:
    how the port's timing relates to the reference's code on the same cores.
    Where the reference library was not built (its sources absent on this
    host) it says so."""
    if O.ref_full_lib() is None:
        return {"unavailable": "oracle/_ref/libgwatref_full.so is not built on this host (the reference's sources "
                               "are absent)"}
    n, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        # the call rewrites t_c in place (mcmc_gw.cpp:2466-2473): a fresh copy each time
        O.ref_mcmc_likelihood_extrinsic(O.GenParams.from_buffer_copy(plist[n % len(plist)]), f, dets, data, psd)
        n += 1
    ref_rate = n / (time.perf_counter() - t0)
    m, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        O.loglik_batch(plist[:16], f, dets, data, psd, nthreads=1)
        m += 16
    port_rate = m / (time.perf_counter() - t0)
    return {"value": ref_rate, "unit": "evals/s", "cores": 1, "kind": "reference", "port_value_1_core": port_rate,
            "port_over_reference": port_rate / ref_rate,
            "sample": "%d calls of MCMC_likelihood_extrinsic, 3 detectors x %d bins, %.0f s per arm" %
                      (n, len(f), seconds)}


def fisher_err(sample):
    """The Fisher parity sample against the FP64 oracle: max normalised error
    |dGamma_ij| / sqrt(Gamma_ii Gamma_jj) of the moment form (FP64 sums, and
    FP32-compensated sums) and of the reference algorithm, and of their
    inverses (normalised by the oracle's inverse diagonal), with the condition
    numbers of the normalised matrices."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from gw_analysis_tools_gb300 import workloads as W
    pf, fish, cov, fr, cr, ff, psd, f32, c32 = sample
    plist = []
    for i in range(len(fish)):
        op = O.GenParams()
        for k, _ in O.GenParams._fields_:
            setattr(op, k, getattr(pf[i], k))
        plist.append(op)
    ref = O.fisher_batch(plist, ff, list(W.DETECTORS3), [psd] * 3, epsilon=1e-6, step_mode=1)

    def nerr(a, b):
        return float(np.max(np.abs(a - b) / np.sqrt(np.abs(np.outer(np.diag(b), np.diag(b))))))
    e_m, e_r, e_6, c_m, c_r, c_6, conds = [], [], [], [], [], [], []
    for i in range(len(fish)):
        e_m.append(nerr(fish[i], ref[i]))
        e_r.append(nerr(fr[i], ref[i]))
        e_6.append(nerr(f32[i], ref[i]))
        st, rinv = O.cholesky_invert(ref[i])
        if st == 0:
            c_m.append(nerr(cov[i], rinv))
            c_r.append(nerr(cr[i], rinv))
            c_6.append(nerr(c32[i], rinv))
            conds.append(float(np.linalg.cond(ref[i] / np.sqrt(np.outer(np.diag(ref[i]), np.diag(ref[i]))))))
    return {"sources": len(fish), "step": "1e-6 relative",
            "max_normalized_err": max(e_m), "median_normalized_err": float(np.median(e_m)),
            "max_normalized_err_inverse": max(c_m), "median_normalized_err_inverse": float(np.median(c_m)),
            "reference_algorithm_max_normalized_err": max(e_r),
            "reference_algorithm_max_normalized_err_inverse": max(c_r),
            "fp32_sums_max_normalized_err": max(e_6), "fp32_sums_max_normalized_err_inverse": max(c_6),
            "median_condition_number": float(np.median(conds)), "max_condition_number": max(conds)}


def fisher_err4(sample):
    """The moment form at order 4 against the oracle's five-point network
    Fisher (with the reference's constant phase on the +-2 eps responses)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from gw_analysis_tools_gb300 import workloads as W
    draws, f4, ff, psd = sample
    errs = []
    for i, d in enumerate(draws):
        ref = O.fisher_network(ff, O.params_from_dict(d), list(W.DETECTORS3), [psd] * 3, order=4, epsilon=1e-6,
                               step_mode=1)
        errs.append(float(np.max(np.abs(f4[i] - ref) / np.sqrt(np.abs(np.outer(np.diag(ref), np.diag(ref)))))))
    return {"sources": len(draws), "max_normalized_err": max(errs), "median_normalized_err": float(np.median(errs))}


def parity_stats(got, ref, tol, rel=False):
    err = np.abs(np.asarray(got) - np.asarray(ref))
    if rel:
        err = err / np.maximum(1.0, np.abs(np.asarray(ref)))
    return {"max_abs_dlogL" if not rel else "max_rel_dlogL": float(err.max()),
            "p99": float(np.percentile(err, 99)), "median": float(np.median(err)), "requests": int(err.size),
            "tolerance": tol, "within": bool(err.max() <= tol)}


def secondary_parity(ex, res):
    """|dlogL| against the FP64 oracle for the secondary forms' samples."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from gw_analysis_tools_gb300 import workloads as W
    dets = list(W.DETECTORS3)
    out = {}
    if "_parity_plain1" in ex:
        pp, got = ex.pop("_parity_plain1")
        # one detector: the plain call's T is 1/df of the grid, as the oracle's
        ref = O.loglik_batch([O.params_from_dict(d) for d in pp], res["f"], dets[:1], res["data"][:1], [res["psd"]])
        out["plain_config1"] = parity_stats(got, ref, 1e-9, rel=True)
    if "_parity_served" in ex:
        sp, sa, got = ex.pop("_parity_served")
        ref = O.loglik_batch([O.params_from_dict(d) for d in sp], res["f"], dets, res["data"], [res["psd"]] * 3,
                             approximants=list(sa), T_segment=res["T"])
        out["served"] = parity_stats(got, ref, 1e-3)
        if "_parity_served_host" in ex:  # the same sample through the host scheduler
            out["served_host_scheduler"] = parity_stats(ex.pop("_parity_served_host"), ref, 1e-3)
    if "_parity_uneven" in ex:
        pu, Ts, udata, got = ex.pop("_parity_uneven")
        ref = np.zeros(len(pu))
        for T in sorted(set(Ts)):
            idx = [i for i in range(len(pu)) if Ts[i] == T]
            fu = W.uniform_grid(20.0, 2048.0, 1.0 / T)
            ref[idx] = O.loglik_batch([O.params_from_dict(pu[i]) for i in idx], fu, dets, udata[T],
                                      [W.analytic_psd(fu)] * 3, approximants=[O.IMRPhenomPv2] * len(idx))
        st = parity_stats(got, ref, 1e-3)
        if 128 in Ts:
            st["max_abs_dlogL_T128"] = float(np.max(np.abs(got - ref)[np.array(Ts) == 128]))
        st["max_abs_logL"] = float(np.max(np.abs(ref)))
        out["uneven_pv2"] = st
    if "_parity_maximized" in ex:
        for name, (draws, ap, got) in ex.pop("_parity_maximized").items():
            ref = [O.maximized_loglik_intrinsic(params_dict(d), res["f"], res["data"], [res["psd"]] * 3, ap)
                   for d in draws]
            out["maximized_" + name] = parity_stats(got, ref, 1e-9, rel=True)
    if "_parity_gaussleg" in ex:
        parr, fg, wg, dg, psd_g, got = ex.pop("_parity_gaussleg")
        ref = []
        for i in range(len(got)):
            op = O.GenParams()
            for k, _ in O.GenParams._fields_:
                setattr(op, k, getattr(parr[i], k))
            ref.append(O.loglik_gl(op, fg, dets, dg, [psd_g] * 3, [wg] * 3, T_segment=8.0))
        out["gaussleg_fp64"] = parity_stats(got, ref, 1e-9, rel=True)
    return out


def params_dict(p):
    """A parameter dict of a gen-params structure (or the dict itself)."""
    if isinstance(p, dict):
        return p
    out = {}
    for k, _ in p._fields_:
        v = getattr(p, k)
        out[k] = tuple(v) if k in ("spin1", "spin2") else v
    return out


def mcmc_theta(draws):
    """The sampler's 11-dim IMRPhenomD vectors of parameter dicts
    (MCMC_prep_params order, mcmc_gw.cpp:2492-2568)."""
    th = []
    for d in draws:
        m1, m2 = d["mass1"], d["mass2"]
        th.append([d["RA"], np.sin(d["DEC"]), d["psi"], np.cos(d["incl_angle"]), d["phiRef"], d["tc"],
                   np.log(d["Luminosity_Distance"]), np.log((m1 * m2) ** 0.6 / (m1 + m2) ** 0.2),
                   m1 * m2 / (m1 + m2) ** 2, d["spin1"][2], d["spin2"][2]])
    return np.array(th)


def uneven_injection(ctx, G, f, T, det):
    """The IMRPhenomPv2 injection of the uneven-grid workload on one detector's
    grid of duration T (t_c <- T - t_c as the likelihood sees it), shifted by
    the arrival time from Hanford; the engine's FP64 detector response, as for
    the main workload."""
    src = UNEVEN_INJECTION
    r = ctx.fourier_detector_response(f, det, "IMRPhenomPv2", G.gen_params(**dict(src, tc=T - src["tc"])))
    return r * np.exp(-2j * np.pi * _dtoa(src, "Hanford", det) * f)


UNEVEN_INJECTION = dict(mass1=31.0, mass2=24.0, spin1=(0.35, -0.2, 0.3), spin2=(-0.25, 0.3, -0.2),
                        Luminosity_Distance=900.0, incl_angle=0.7, phiRef=0.9, f_ref=20.0, tc=0.02, RA=2.2, DEC=-0.5,
                        psi=0.8, gmst=1.2345)


# ------------------------------------------------------------ reference arm
def run_reference(args, rank, world):
    """The reference's CPU path on the host cores: the FP64 oracle port (the
    reference needs GSL/ADOL-C/FFTW that are absent), all threads, one step =
    the 512-request batch."""
    if rank != 0:
        return None
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from gw_analysis_tools_gb300 import workloads as W
    O.build()
    f = W.config1_grid()
    T = 1.0 / (f[1] - f[0])
    src = W.config1_source()
    dets = list(W.DETECTORS3)
    injp = O.params_from_dict(dict(src, tc=T - src["tc"]))
    data = []
    for i, d in enumerate(dets):
        r = O.detector_response(f, injp, d)
        dt = O.dtoa(src["RA"], src["DEC"], src["gmst"], dets[0], d)
        data.append(r * np.exp(-2j * np.pi * dt * f) + W.noise(f, 100 + i))
    psd = [W.analytic_psd(f)] * 3
    plist = [O.params_from_dict(d) for d in W.prior_draws(N_REQ, 1000)]
    # each step is a bounded sample of the 512-request step, sized so that the
    # whole run stays near two minutes of host time
    t0 = time.perf_counter()
    O.loglik_batch(plist[:64], f, dets, data, psd)
    rate = 64 / (time.perf_counter() - t0)
    per_step_s = 120.0 / max(1, args.steps + args.warmup)
    nsample = int(max(16, min(N_REQ, rate * per_step_s)))
    sample = plist[:nsample]
    for _ in range(args.warmup):
        O.loglik_batch(sample, f, dets, data, psd)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        O.loglik_batch(sample, f, dets, data, psd)
    dt = time.perf_counter() - t0
    v = nsample * args.steps / dt
    cores = os.cpu_count()
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "evals/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": WORKLOAD, "global_batch": N_REQ},
            "cpu_baseline": {"value": v, "unit": "evals/s", "cores": cores, "kind": "port",
                             "sample": "%d steps of %d of the 512 requests (prior draws), OpenMP over requests on "
                                       "%d threads" % (args.steps, nsample, cores),
                             "reference_code": reference_code_rate(O, f, dets, data, psd, plist)},
            "e2e": {"value": v, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    return line


def main():
    args = parse()
    rank, world, local, pg = dist_setup(args)
    if args.impl == "reference":
        line = run_reference(args, rank, world)
        if line is not None:
            print(json.dumps(line))
        return
    res = run_ours(args, rank, world, local, pg)
    if rank != 0:
        return
    log("cpu baseline")
    base, parity = cpu_baseline(res)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    # roofline of the fused bin kernel: the reference algorithm's work of one
    # step (flops counted on the reference's model code) per kernel time,
    # against the FP32 peak -- the pipe that carries most of the mixed form
    units_wave = N_REQ * 32128
    algo_flops = units_wave * REF_FLOPS_PER_WAVE_BIN + 3 * units_wave * REF_FLOPS_PER_DET_BIN
    kernel_s = res["kernel_ms"] / 1e3
    achieved = algo_flops / kernel_s / 1e12
    log("fp32/fp64 peaks")
    fp32_peak = measure_peak("float32")
    fp64_peak = measure_peak("float64")
    ex = res.get("extras", {})
    fisher_parity = fisher_err(ex.pop("_fisher_sample")) if "_fisher_sample" in ex else None
    if fisher_parity is not None and "_fisher_sample4" in ex:
        fisher_parity["moment_order4"] = fisher_err4(ex.pop("_fisher_sample4"))
    log("secondary parity")
    sec_parity = secondary_parity(ex, res)
    line = {
        "metric": METRIC, "value": res["value"], "unit": "evals/s", "n_gpus": world, "steps": len(res["step_ms"]),
        "warmup": parse_warmup(), "ms_per_step": res["tot_ms"] / len(res["step_ms"]), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64 (FP64 phase)", "data": "synthetic",
        "config": {"workload": WORKLOAD, "global_batch": N_REQ * world, "precision": "mixed",
                   "l2": "flushed before every step (256 MiB write)", "tile": res["tile"],
                   "launch_shape": res["launch_shape"],
                   "parallelism": "replicas" if world > 1 else "single"},
        "e2e": {"value": res["e2e_value"], "unit": "evals/s", "h2d_bytes_per_step": res["h2d"],
                "d2h_bytes_per_step": res["d2h"]},
        "gpu_launches": res["gpu_launches"],
        "clocks": res["clocks"],
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved / fp32_peak if fp32_peak else None, "traffic": TRAFFIC_PER_LAUNCH,
                     "kernel": "k_batch<3,1,%d> (fused mixed bin kernel)" % res["launch_shape"]["blocks_per_sm"],
                     "kernel_ms": res["kernel_ms"],
                     "prologue_ms": res["prologue_ms"], "algorithmic_flops_per_launch": algo_flops,
                     "algorithm": "reference flops per waveform-bin %.2f and per detector-bin %.1f "
                                  "(oracle/op_counts.json)" % (REF_FLOPS_PER_WAVE_BIN, REF_FLOPS_PER_DET_BIN),
                     "peak_source": "measured in this run: FP32 GEMM 8192^3 without TF32 (FMA pipe)",
                     "note": "achieved counts add/mul/div of the reference algorithm; its elementary functions "
                             "(3.9 per waveform-bin, 3 per detector-bin) are not in it",
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch of this "
                                       "kernel on this workload, " + PROFILE_SOURCE,
                     "fp64": {"achieved_tflops": FP64_FLOP_PER_LAUNCH / kernel_s / 1e12, "peak_tflops": fp64_peak,
                              "frac": FP64_FLOP_PER_LAUNCH / kernel_s / 1e12 / fp64_peak if fp64_peak else None,
                              "flop_per_launch": FP64_FLOP_PER_LAUNCH,
                              "flop_source": "ncu DFMA x 2 + DMUL + DADD of one launch, " + PROFILE_SOURCE,
                              "peak_source": "measured in this run: FP64 GEMM 4096^3"},
                     "hbm": {"achieved_gbs": TRAFFIC_PER_LAUNCH / kernel_s / 1e9, "peak_gbs": peaks.get("hbm_gbs"),
                             "frac": TRAFFIC_PER_LAUNCH / kernel_s / 1e9 / peaks["hbm_gbs"]
                             if peaks.get("hbm_gbs") else None, "peak_source": "MEASURED_PEAKS.json"},
                     "issue": issue_roofline(kernel_s, res["clocks"])},
        "cpu_baseline": base,
        "parity": dict(parity, tolerance=1e-3, status_ok=res["stat_ok"]),
    }
    if ex:
        plain = ex.get("plain_fp64_evals_per_s")
        for k in ("plain_fp64_evals_per_s", "plain_fp64_p50_ms", "plain_config1", "batched_fp64_evals_per_s", "served",
                  "uneven_pv2", "maximized", "ingest", "gaussleg_fp64", "errors"):
            if k in ex:
                line[k] = ex[k]
        if plain:
            line["speedup_vs_plain_fp64"] = res["value"] / plain
            if "served" in ex:  # the server's capacity; at 2e5/s offered it serves the offered rate
                line["served"]["speedup_vs_plain_fp64"] = ex["served"]["saturated"]["evals_per_s"] / plain
                line["served"]["speedup_basis"] = "saturated rate (5e6/s offered) over the plain FP64 form"
        if "fisher" in ex:
            line["fisher"] = dict(ex["fisher"], parity=fisher_parity)
        if "served_host_scheduler" in sec_parity and "served" in line:
            line["served"]["host_scheduler"]["parity"] = sec_parity.pop("served_host_scheduler")
        for k, v in sec_parity.items():
            key = k if k in line else ("maximized" if k.startswith("maximized") else k)
            if k.startswith("maximized") and "maximized" in line:
                line["maximized"].setdefault("parity", {})[k.split("_", 1)[1]] = v
            elif key in line:
                line[key]["parity"] = v
    print(json.dumps(line))


# Work of the 512-request IMRPhenomD step: reference flops per unit, counted
# by oracle/count_ops.py on the reference's own model code (oracle/op_counts.json);
# and, from one ncu capture of k_batch<3,1> on this workload
# (profiles/k_batch_mixed_ptstep512.md), its DRAM bytes, FP64 flops and warp
# instructions per launch.
PROFILE_SOURCE = "profiles/k_batch_mixed_ptstep512.md"
REF_FLOPS_PER_WAVE_BIN = 66.56
REF_FLOPS_PER_DET_BIN = 33.0
TRAFFIC_PER_LAUNCH = 2.39e6
FP64_FLOP_PER_LAUNCH = 1.98e7
INST_PER_LAUNCH = 8.17e7


def issue_roofline(kernel_s, clocks):
    """The bin kernel against the instruction-issue limit (it is issue-bound:
    no pipe saturates): warp instructions per launch (ncu) / event-timed
    duration, against 4 issue slots per SM per cycle at the SM clock seen
    under load."""
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    mhz = (clocks or {}).get("sm_mhz") or (clocks or {}).get("sm_max_mhz")
    if not mhz:
        return None
    peak = sms * 4 * mhz * 1e6
    achieved = INST_PER_LAUNCH / kernel_s
    return {"achieved_warp_inst_per_s": achieved, "peak_warp_inst_per_s": peak, "frac": achieved / peak,
            "inst_per_launch": INST_PER_LAUNCH, "inst_source": "ncu smsp__inst_executed.sum of one launch, " +
            PROFILE_SOURCE, "peak_source": "%d SMs x 4 schedulers x %.0f MHz (clocks under load)" % (sms, mhz)}


def measure_peak(dtype):
    """Dense GEMM throughput (TFLOP/s) on this GPU: FP32 without TF32 (8192^3),
    FP64 (4096^3); best of 5."""
    import torch
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    n = 8192 if dtype == "float32" else 4096
    dt = getattr(torch, dtype)
    a = torch.randn(n, n, dtype=dt, device="cuda")
    b = torch.randn(n, n, dtype=dt, device="cuda")
    for _ in range(2):
        a @ b
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = 0.0
    for _ in range(5):
        e0.record()
        a @ b
        e1.record()
        torch.cuda.synchronize()
        best = max(best, 2 * n ** 3 / (e0.elapsed_time(e1) / 1e3) / 1e12)
    torch.backends.cuda.matmul.allow_tf32 = prev
    del a, b
    return best


def parse_warmup():
    return parse().warmup


if __name__ == "__main__":
    main()
