"""Algorithmic work per unit of the likelihood path, counted on the reference's
own model code (test infrastructure; needs the reference sources).

    python oracle/count_ops.py /path/to/gw_analysis_tools > oracle/op_counts.json

Builds oracle/_ref/libgwatref_count.so (make -C oracle count), then counts the
operations the reference algorithm performs:
  * per waveform-bin of IMRPhenomD and IMRPhenomPv2, averaged over the
    1024-Hz / df=1/32 grid of 32,128 bins and over seeded prior draws (the
    aligned-spin and precessing priors of the batched and uneven workloads);
  * per detector-bin (projection, arrival-time shift, two integrands and two
    Simpson sums).
"flops" = additions + multiplications + divisions (a*b+c counts 2); the
elementary functions are listed by kind.  The per-bin figure is
(count(N bins) - prologue) / N with the prologue = count(1) - (count(2) -
count(1)), both with the grid's first bins.
"""
import ctypes
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(HERE))

import oracle as O  # noqa: E402
from gw_analysis_tools_gb300 import workloads as W  # noqa: E402

KINDS = ["add", "mul", "div", "sqrt", "exp", "log", "pow", "sin", "cos", "atan", "cbrt", "other"]


def _lib(ref):
    subprocess.check_call(["make", "-s", "-C", HERE, "count", "REF=" + ref])
    L = ctypes.CDLL(os.path.join(HERE, "_ref", "libgwatref_count.so"))
    L.count_waveform.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    L.count_detector_bins.argtypes = [ctypes.c_int, ctypes.c_void_p]
    return L


def _count(L, p, approx, f):
    out = np.zeros(len(KINDS), dtype=np.int64)
    L.count_waveform(ctypes.byref(p), approx, f.ctypes.data, f.size, out.ctypes.data)
    return out


def per_bin(L, d, approx, f):
    p = O.params_from_dict(d)
    c1 = _count(L, p, approx, f[:1])
    c2 = _count(L, p, approx, f[:2])
    cn = _count(L, p, approx, f)
    prologue = c1 - (c2 - c1)
    return (cn - prologue) / f.size, prologue


def summarise(v):
    d = {k: float(x) for k, x in zip(KINDS, v)}
    d["flops"] = float(v[0] + v[1] + v[2])
    d["transcendentals"] = float(v[3:].sum())
    return d


def main(ref):
    L = _lib(ref)
    f = np.ascontiguousarray(W.config1_grid())
    out = {"grid": "20-1024 Hz, df=1/32 Hz, 32128 bins"}
    for name, approx, draws in (("IMRPhenomD", O.IMRPhenomD, [W.config1_source()] + W.prior_draws(63, 7)),
                                ("IMRPhenomPv2", O.IMRPhenomPv2, W.prior_draws(64, 9, precessing=True))):
        bins = np.zeros(len(KINDS))
        pro = np.zeros(len(KINDS))
        for d in draws:
            b, p = per_bin(L, d, approx, f)
            bins += b
            pro += p
        out[name] = {"per_waveform_bin": summarise(bins / len(draws)), "prologue": summarise(pro / len(draws)),
                     "draws": len(draws)}
    c = np.zeros(len(KINDS), dtype=np.int64)
    n = 4096
    L.count_detector_bins(n, c.ctypes.data)
    out["per_detector_bin"] = summarise(c / n)
    json.dump(out, sys.stdout, indent=1)
    sys.stdout.write("\n")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GWAT_REFERENCE_DIR", ""))
