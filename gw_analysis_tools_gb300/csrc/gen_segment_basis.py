"""Generate segment_basis.h: the interpolation basis of the segment phase
polynomials of the mixed form.

A segment is 256 consecutive bins, m = n - n_c in [-128, 127] with n_c the
segment start + 128, u = m / 128.  The FP64 phase is evaluated at nine integer
nodes near the Chebyshev-Lobatto points of [-128, 127] (centre included) and
at two check points between the outermost node pairs; the degree-8
interpolating polynomial in u has coefficients c = VINV (v - v(0)).

    python gw_analysis_tools_gb300/csrc/gen_segment_basis.py
"""
import os

import numpy as np

NODES = [-128, -118, -90, -49, 0, 49, 90, 118, 127]
CHECKS = [-123, 122]
SCALE = 128.0


def main():
    u = np.array(NODES, dtype=np.float64) / SCALE
    V = np.vander(u, len(NODES), increasing=True)  # V[i, j] = u_i^j
    vinv = np.linalg.inv(V)
    assert np.allclose(vinv @ V, np.eye(len(NODES)), atol=1e-12)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "segment_basis.h")
    with open(out, "w") as f:
        f.write("/* Generated by gen_segment_basis.py -- do not edit. */\n")
        f.write("/* Segment phase polynomials of the mixed form: node offsets m (u = m / 128)\n")
        f.write("   and the inverse Vandermonde matrix of the nodes (coefficients of u^j). */\n")
        f.write("#ifndef GWT_SEGMENT_BASIS_H\n#define GWT_SEGMENT_BASIS_H\n")
        f.write("#define GWT_SEG_NODES %d\n#define GWT_SEG_CHECKS %d\n" % (len(NODES), len(CHECKS)))
        offs = ", ".join(str(x) for x in NODES + CHECKS)
        rows = ",\n  ".join("{" + ", ".join(repr(float(x)) for x in r) + "}" for r in vinv)
        f.write("#define GWT_SEG_OFFSETS_INIT {%s}\n" % offs)
        f.write("#define GWT_SEG_VINV_INIT {%s}\n" % rows.replace("\n", " \\\n"))
        f.write("#if defined(__CUDACC__)\n")
        f.write("static __constant__ int gwt_seg_offsets_d[%d] = GWT_SEG_OFFSETS_INIT;\n" % (len(NODES) + len(CHECKS)))
        f.write("static __constant__ double gwt_seg_vinv_d[%d][%d] = GWT_SEG_VINV_INIT;\n" % (len(NODES), len(NODES)))
        f.write("#endif\n")
        f.write("static const int gwt_seg_offsets_h[%d] = GWT_SEG_OFFSETS_INIT;\n" % (len(NODES) + len(CHECKS)))
        f.write("static const double gwt_seg_vinv_h[%d][%d] = GWT_SEG_VINV_INIT;\n" % (len(NODES), len(NODES)))
        f.write("#endif\n")
    print("wrote", out, "cond", np.linalg.cond(V))


if __name__ == "__main__":
    main()
