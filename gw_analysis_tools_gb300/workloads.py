"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No public dataset is used: every workload is generated here from fixed seeds.

* PSD: S(f) = 1e-49 [x^-4.14 - 5 x^-2 + 111 (1 - x^2 + x^4/2) / (1 + x^2/2)],
  x = f / 215 Hz, the same curve for every detector.
* Noise: n_k = sqrt(S_k / (4 df)) (g1 + i g2), g ~ N(0, 1), so that
  E|n_k|^2 = S_k / (2 df), matching the one-sided 4 Re <.|.> inner product of
  Log_Likelihood_internal (mcmc_gw.cpp:801-873).
* Priors (batched PT step, uneven batch, Fisher): masses U(5, 80) Msun sorted
  m1 >= m2, aligned spins U(-0.9, 0.9), D_L uniform in volume on [100, 2000] Mpc,
  RA U(0, 2 pi), sin DEC U(-1, 1), psi U(0, pi), cos iota U(-1, 1),
  phi_ref U(0, 2 pi), t_c U(-0.1, 0.1) s; Pv2 in-plane spins |chi| <= 0.8 with
  isotropic directions.
"""
import numpy as np

DETECTORS3 = ("Hanford", "Livingston", "Virgo")
GMST = 1.2345  # fixed sidereal time (rad) of every workload


def analytic_psd(f):
    x = np.asarray(f, dtype=np.float64) / 215.0
    return 1e-49 * (x ** -4.14 - 5.0 * x ** -2.0 + 111.0 * (1.0 - x * x + 0.5 * x ** 4) / (1.0 + 0.5 * x * x))


def uniform_grid(f0, f1, df, endpoint=False):
    """f_k = f0 + k df for f0 <= f_k < f1 (or <= f1 with endpoint)."""
    n = int(np.floor((f1 - f0) / df + 1e-9)) + (1 if endpoint else 0)
    return f0 + np.arange(n, dtype=np.float64) * df


def config1_grid():
    return uniform_grid(20.0, 1024.0, 1.0 / 32.0, endpoint=True)[:32128]


def noise(freqs, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    df = freqs[1] - freqs[0]
    s = np.sqrt(analytic_psd(freqs) / (4.0 * df))
    return s * (rng.standard_normal(freqs.size) + 1j * rng.standard_normal(freqs.size))


def config1_source():
    """Config 1 injection: m1=36, m2=29, chi1z=0.3, chi2z=-0.1, D_L=410 Mpc, iota=0.5."""
    return dict(mass1=36.0, mass2=29.0, spin1=(0.0, 0.0, 0.3), spin2=(0.0, 0.0, -0.1), Luminosity_Distance=410.0,
                incl_angle=0.5, phiRef=0.0, f_ref=20.0, tc=0.0, RA=1.0, DEC=0.3, psi=0.4, gmst=GMST)


def perturbed(src, n, seed, frac=0.01):
    """n copies of src with every continuous parameter scaled by 1 + frac N(0,1)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    keys = ("mass1", "mass2", "Luminosity_Distance", "incl_angle", "phiRef", "tc", "RA", "DEC", "psi")
    for _ in range(n):
        d = dict(src)
        for k in keys:
            d[k] = src[k] * (1.0 + frac * rng.standard_normal()) if src[k] != 0 else frac * rng.standard_normal()
        if d["mass2"] > d["mass1"]:
            d["mass1"], d["mass2"] = d["mass2"], d["mass1"]
        s1 = list(src["spin1"])
        s2 = list(src["spin2"])
        s1[2] *= 1.0 + frac * rng.standard_normal()
        s2[2] *= 1.0 + frac * rng.standard_normal()
        d["spin1"], d["spin2"] = tuple(s1), tuple(s2)
        out.append(d)
    return out


def prior_draws(n, seed, precessing=False, tc_range=0.1):
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for _ in range(n):
        m = np.sort(rng.uniform(5.0, 80.0, 2))[::-1]
        dl = (rng.uniform(100.0 ** 3, 2000.0 ** 3)) ** (1.0 / 3.0)
        d = dict(mass1=float(m[0]), mass2=float(m[1]), Luminosity_Distance=float(dl),
                 RA=float(rng.uniform(0, 2 * np.pi)), DEC=float(np.arcsin(rng.uniform(-1, 1))),
                 psi=float(rng.uniform(0, np.pi)), incl_angle=float(np.arccos(rng.uniform(-1, 1))),
                 phiRef=float(rng.uniform(0, 2 * np.pi)), tc=float(rng.uniform(-tc_range, tc_range)), f_ref=20.0,
                 gmst=GMST)
        if precessing:
            sp = []
            for _k in range(2):
                mag = rng.uniform(0.0, 0.8)
                ct = rng.uniform(-1, 1)
                ph = rng.uniform(0, 2 * np.pi)
                st = np.sqrt(1 - ct * ct)
                sp.append((mag * st * np.cos(ph), mag * st * np.sin(ph), mag * ct))
            d["spin1"], d["spin2"] = sp
        else:
            d["spin1"] = (0.0, 0.0, float(rng.uniform(-0.9, 0.9)))
            d["spin2"] = (0.0, 0.0, float(rng.uniform(-0.9, 0.9)))
        out.append(d)
    return out


def uneven_durations(n, seed):
    """Segment durations T in {4, 8, 32, 128} s, uniform choice."""
    rng = np.random.Generator(np.random.PCG64(seed))
    return rng.choice(np.array([4, 8, 32, 128]), size=n)
