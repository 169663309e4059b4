"""Generate tests/golden/reference_glue.npz from the reference itself.

Runs the reference's own translation units of the likelihood and Fisher path
(oracle/Makefile target "full" -> oracle/_ref/libgwatref_full.so: the
reference sources compiled unmodified against oracle/shim/, entered through
oracle/ref_glue.cpp) on seeded inputs, and stores inputs and outputs:

* detector_response_functions_equatorial and DTOA_DETECTOR,
* fourier_detector_response with and without equatorial_orientation
  (transform_orientation_coords),
* Log_Likelihood_internal (Simpson and Gauss-Legendre) and
  MCMC_likelihood_extrinsic,
* MCMC_likelihood_wrapper and MCMC_fisher_wrapper through the reference's
  sampler set-up (11-dim IMRPhenomD, 15-dim IMRPhenomPv2, 4-dim intrinsic),
* fisher_numerical (IMRPhenomD and MCMC_IMRPhenomD, orders 2 and 4),
* the maximised likelihoods (aligned and unaligned).

The committed fixture lets tests/test_oracle_pins.py check the C oracle where
the reference sources are absent.

    GWAT_REFERENCE_DIR=<reference checkout> python tests/golden/make_golden_glue.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)
import oracle as O  # noqa: E402
from gw_analysis_tools_gb300 import workloads as W  # noqa: E402

DETS = ["Hanford", "Livingston", "Virgo"]
GPS = 1126259462.4


def grid():
    """20-120 Hz at df = 1/8 Hz (800 bins): T = 8 s, short enough for the
    direct DFT standing in for FFTW in the maximised likelihoods."""
    return W.uniform_grid(20.0, 120.0, 1.0 / 8.0)


def mcmc_positions_d(n, seed):
    pos = []
    for d in W.prior_draws(n, seed):
        mc = (d["mass1"] * d["mass2"]) ** 0.6 / (d["mass1"] + d["mass2"]) ** 0.2
        eta = d["mass1"] * d["mass2"] / (d["mass1"] + d["mass2"]) ** 2
        pos.append([d["RA"], np.sin(d["DEC"]), d["psi"], np.cos(d["incl_angle"]), d["phiRef"], d["tc"],
                    np.log(d["Luminosity_Distance"]), np.log(mc), eta, d["spin1"][2], d["spin2"][2]])
    return np.array(pos)


def mcmc_positions_pv2(n, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    pos = []
    for _ in range(n):
        pos.append([rng.uniform(0, 2 * np.pi), rng.uniform(-1, 1), rng.uniform(0, np.pi), rng.uniform(-1, 1),
                    rng.uniform(0, 2 * np.pi), rng.uniform(-0.05, 0.05), np.log(rng.uniform(200, 900)),
                    np.log(rng.uniform(10, 30)), rng.uniform(0.15, 0.249), rng.uniform(0, 0.8), rng.uniform(0, 0.8),
                    rng.uniform(-1, 1), rng.uniform(-1, 1), rng.uniform(0, 2 * np.pi), rng.uniform(0, 2 * np.pi)])
    return np.array(pos)


def intrinsic_positions(n, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    return np.array([[np.log(rng.uniform(10, 30)), rng.uniform(0.15, 0.249), rng.uniform(-0.8, 0.8),
                      rng.uniform(-0.8, 0.8)] for _ in range(n)])


def plain(d):
    """The parameter dict with plain Python numbers, so that its repr reads
    back with ast.literal_eval."""
    return {k: (tuple(float(x) for x in v) if isinstance(v, (tuple, list)) else
                (int(v) if isinstance(v, (int, np.integer)) else float(v))) for k, v in d.items()}


def oriented_draws(n, seed, precessing):
    rng = np.random.Generator(np.random.PCG64(seed + 1000))
    out = []
    for d in W.prior_draws(n, seed, precessing=precessing):
        d = dict(d, theta_l=float(np.arccos(rng.uniform(-1, 1))), phi_l=float(rng.uniform(0, 2 * np.pi)),
                 equatorial_orientation=1)
        if precessing and rng.uniform() < 0.5:
            d.update(chip=float(rng.uniform(0.1, 0.7)), phip=float(rng.uniform(0, 2 * np.pi)))
        out.append(d)
    return out


def main():
    ref_dir = O.reference_dir()
    if ref_dir is None:
        raise SystemExit("set GWAT_REFERENCE_DIR to the reference checkout")
    O.build(ref_dir)
    if O.ref_full_lib() is None:
        raise SystemExit("reference pin library was not built")
    f = grid()
    src = W.config1_source()
    p_inj = O.params_from_dict(src)
    data = [O.ref_detector_response(f, p_inj, det)[0] + W.noise(f, 3 + i) for i, det in enumerate(DETS)]
    psd = W.analytic_psd(f)
    out = {"freqs": f, "psd": psd, "data": np.array(data), "gps": np.array(GPS)}

    # antenna patterns and arrival times
    ant_in, ant_out, dt_out = [], [], []
    names = DETS + ["Kagra", "Indigo", "CE", "ET1", "ET2", "ET3"]
    for d in W.prior_draws(8, 31):
        for k, det in enumerate(names):
            ant_in.append([k, d["RA"], d["DEC"], d["psi"], d["gmst"]])
            ant_out.append(O.ref_antenna(det, d["RA"], d["DEC"], d["psi"], d["gmst"]))
        for det in DETS:
            dt_out.append(O.ref_dtoa(d["RA"], d["DEC"], d["gmst"], "Hanford", det))
    out["antenna_dets"] = np.array(names)
    out["antenna_in"] = np.array(ant_in)
    out["antenna_out"] = np.array(ant_out)
    out["dtoa_out"] = np.array(dt_out)

    # responses, plain and with the orientation transform
    cases, resp = [], []
    for ap, name, prec in ((O.IMRPhenomD, "IMRPhenomD", False), (O.IMRPhenomPv2, "IMRPhenomPv2", True)):
        for d in W.prior_draws(2, 32, precessing=prec) + oriented_draws(3, 33, prec):
            r, after = O.ref_detector_response(f, O.params_from_dict(d), "Livingston", name)
            cases.append(repr((ap, plain(d), after.psi, after.incl_angle)))
            resp.append(r)
    out["response_cases"] = np.array(cases)
    out["response_out"] = np.array(resp)

    # Log_Likelihood_internal and MCMC_likelihood_extrinsic
    ll_cases, ll_out = [], []
    for d in W.prior_draws(6, 34):
        q = O.params_from_dict(d)
        ll, T, tc = O.ref_mcmc_likelihood_extrinsic(q, f, DETS, data, [psd] * 3)
        r = O.ref_detector_response(f, q, "Hanford")[0]
        lli = O.ref_log_likelihood_internal(data[0], psd, f, r)
        w = np.linspace(0.5, 1.5, f.size) / f.size
        llg = O.ref_log_likelihood_internal(data[0], psd, f, r, weights=w, log10F=True)
        ll_cases.append(repr(plain(d)))
        ll_out.append([ll, T, tc, lli, llg])
    out["loglik_cases"] = np.array(ll_cases)
    out["loglik_out"] = np.array(ll_out)

    # the sampler callbacks through the reference's own set-up
    pos_d = mcmc_positions_d(6, 35)
    ll_d, fi_d, _ = O.ref_sampler_eval("IMRPhenomD", pos_d, f, DETS, data, [psd] * 3, GPS, fisher=True)
    pos_p = mcmc_positions_pv2(4, 36)
    ll_p, _, _ = O.ref_sampler_eval("IMRPhenomPv2", pos_p, f, DETS, data, [psd] * 3, GPS)
    pos_i = intrinsic_positions(3, 37)
    ll_i, _, _ = O.ref_sampler_eval("IMRPhenomD", pos_i, f, DETS, data, [psd] * 3, GPS)
    out.update(wrapper_pos_d=pos_d, wrapper_ll_d=ll_d, wrapper_fisher_d=fi_d, wrapper_pos_p=pos_p,
               wrapper_ll_p=ll_p, wrapper_pos_i=pos_i, wrapper_ll_i=ll_i,
               wrapper_gmst=np.array(O.ref_gps_to_gmst(GPS)))

    # fisher_numerical
    fi_cases, fi_out = [], []
    for d in W.prior_draws(2, 38):
        for method in ("IMRPhenomD", "MCMC_IMRPhenomD"):
            for order in (2, 4):
                fi_cases.append(repr((plain(d), method, order)))
                fi_out.append(O.ref_fisher_numerical(f, O.params_from_dict(d), "Livingston", "Hanford", psd,
                                                     method=method, order=order))
    out["fisher_cases"] = np.array(fi_cases)
    out["fisher_out"] = np.array(fi_out)

    # maximised likelihoods
    mx_cases, mx_out = [], []
    for d in W.prior_draws(3, 39):
        hp, _ = O.ref_fourier_waveform(f, O.params_from_dict(d), "IMRPhenomD")
        hp2, hc2 = O.ref_fourier_waveform(f, O.params_from_dict(d), "IMRPhenomPv2")
        mx_cases.append(repr(plain(d)))
        mx_out.append([O.ref_maximized_loglik(data[0], psd, f, hp), O.ref_maximized_loglik(data[0], psd, f, hp2, hc2)])
    out["maxll_cases"] = np.array(mx_cases)
    out["maxll_out"] = np.array(mx_out)

    np.savez_compressed(os.path.join(HERE, "reference_glue.npz"), **out)
    print("wrote reference_glue.npz")


if __name__ == "__main__":
    main()
