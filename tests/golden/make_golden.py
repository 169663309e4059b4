"""Generate tests/golden/reference_waveforms.npz from the reference itself.

Runs the reference's own IMRPhenomD.cpp / IMRPhenomP.cpp, compiled here from
the reference sources against test-only shim headers (oracle/Makefile target
"ref" -> oracle/_ref/libgwatref.so), on a fixed set of source parameters and
stores a subsample of the bins.  The committed fixture lets the oracle be
checked where the reference sources are absent.

    GWAT_REFERENCE_DIR=<reference checkout> python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402

CASES = [
    # (approximant, params)
    (O.IMRPhenomD, dict(mass1=36.0, mass2=29.0, spin1=(0, 0, 0.3), spin2=(0, 0, -0.1), Luminosity_Distance=410.0,
                        incl_angle=0.5, phiRef=0.0, f_ref=20.0, tc=0.0)),
    (O.IMRPhenomD, dict(mass1=80.0, mass2=5.0, spin1=(0, 0, 0.9), spin2=(0, 0, -0.9), Luminosity_Distance=100.0,
                        incl_angle=2.5, phiRef=1.0, f_ref=20.0, tc=31.9)),
    (O.IMRPhenomD, dict(mass1=5.5, mass2=5.0, spin1=(0, 0, -0.5), spin2=(0, 0, 0.2), Luminosity_Distance=2000.0,
                        incl_angle=0.1, phiRef=4.0, f_ref=20.0, tc=-0.05, shift_time=0, shift_phase=0)),
    (O.IMRPhenomD, dict(mass1=45.0, mass2=44.0, spin1=(0, 0, 0.0), spin2=(0, 0, 0.0), Luminosity_Distance=800.0,
                        incl_angle=1.2, phiRef=2.0, f_ref=30.0, tc=10.0, dep_postmerger=1)),
    (O.IMRPhenomPv2, dict(mass1=36.0, mass2=29.0, spin1=(0.3, 0.2, 0.3), spin2=(-0.1, 0.4, -0.1),
                          Luminosity_Distance=410.0, incl_angle=0.5, phiRef=0.3, f_ref=20.0, tc=0.0)),
    (O.IMRPhenomPv2, dict(mass1=60.0, mass2=12.0, spin1=(0.5, -0.4, 0.1), spin2=(0.0, 0.7, 0.2),
                          Luminosity_Distance=300.0, incl_angle=2.0, phiRef=5.0, f_ref=20.0, tc=3.0)),
    (O.IMRPhenomPv2, dict(mass1=20.0, mass2=18.0, spin1=(0, 0, 0.4), spin2=(0, 0, 0.1), Luminosity_Distance=500.0,
                          incl_angle=0.9, phiRef=0.7, f_ref=25.0, tc=1.0, chip=0.45, phip=1.1)),
]


def main(ref_dir):
    O.build(ref_dir)
    if O.ref_lib() is None:
        raise SystemExit("reference pin library was not built")
    freqs = 20.0 + np.arange(32128) / 32.0
    idx = np.arange(0, 32128, 97)
    out = {"freqs": freqs[idx], "idx": idx}
    for i, (ap, kw) in enumerate(CASES):
        p = O.make_params(**kw)
        hp, hc = O.fourier_waveform(freqs, p, ap, use_ref=True)
        out["case%d_approx" % i] = np.array(ap)
        out["case%d_params" % i] = np.array(repr(kw))
        out["case%d_hp" % i] = hp[idx]
        out["case%d_hc" % i] = hc[idx]
    np.savez_compressed(os.path.join(HERE, "reference_waveforms.npz"), **out)
    print("wrote %d cases" % len(CASES))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ["GWAT_REFERENCE_DIR"])
