"""Regenerates the constant-data headers shared by the oracle and the CUDA path.

The IMRPhenomD calibration fits (19 x 11 coefficients, Khan et al. 2016,
arXiv:1508.07253), the quasi-normal-mode ringdown/damping table (1003 points
of final spin a, 2*pi*M*f_RD and 2*pi*M*f_damp, as tabulated by LALSuite) and
the ground-detector geometry (ECEF locations in metres, 3x3 response tensors,
geometric factors) are published numbers that must be bit-identical to the
ones the reference evaluates.  This script reads them once from the reference
headers (include/gwat/IMRPhenomD.h:190-270, include/gwat/QNM_data.h:11-455,
include/gwat/detector_util.h:30-161) and writes them out in this project's own
layout:

    oracle/gwo_tables.h                         (used by the C oracle)
    gw_analysis_tools_gb300/csrc/phenom_tables.h (used by the CUDA path)

Run it only where the reference sources are present:
    GWAT_REFERENCE_DIR=<reference checkout> python oracle/gen_tables.py
The generated headers are committed; nothing at build or run time reads the
reference.
"""
import os
import re
import sys


def _floats(text):
    text = re.sub(r"([-+])\s+(?=[\d.])", r"\1", text)  # "- 0.12" is one number
    return [float(x) for x in re.findall(r"[-+]?\d*\.?\d+(?:[eE][-+]?\d+)?", text)]


def _block(src, start_pat, end_pat):
    i = src.index(start_pat)
    j = src.index(end_pat, i)
    return src[i + len(start_pat):j]


def _strip_comments(s):
    s = re.sub(r"/\*.*?\*/", "", s, flags=re.S)
    return re.sub(r"//[^\n]*", "", s)


def main(ref):
    inc = os.path.join(ref, "include", "gwat")
    with open(os.path.join(inc, "IMRPhenomD.h")) as f:
        d_src = f.read()
    lam_txt = _strip_comments(_block(d_src, "const double lambda_num_params[19][11]=", "}};"))
    lam = _floats(lam_txt)
    assert len(lam) == 19 * 11, len(lam)

    with open(os.path.join(inc, "QNM_data.h")) as f:
        q_src = _strip_comments(f.read())
    qa = _floats(_block(q_src, "QNMData_a[] =", "};"))
    qr = _floats(_block(q_src, "QNMData_fring[] =", "};"))
    qd = _floats(_block(q_src, "QNMData_fdamp[] =", "};"))
    assert len(qa) == len(qr) == len(qd) == 1003, (len(qa), len(qr), len(qd))

    with open(os.path.join(inc, "detector_util.h")) as f:
        det_src = _strip_comments(f.read())
    dets = [("H", "Hanford"), ("L", "Livingston"), ("V", "Virgo"), ("K", "Kagra"),
            ("I", "Indigo"), ("CE", "CE"), ("ET1", "ET1"), ("ET2", "ET2"), ("ET3", "ET3")]
    loc, tens, geo = {}, {}, {}
    for short, tname in dets:
        loc[short] = _floats(_block(det_src, "const double %s_location[3] =" % short, ";"))
        geo[short] = _floats(_block(det_src, "const double %s_geometric_factor =" % short, ";"))[0]
        tens[short] = _floats(_block(det_src, "const double %s_D[3][3]" % tname, ";"))
        assert len(loc[short]) == 3 and len(tens[short]) == 9

    def fmt(v):
        return repr(float(v))

    def emit(path, prefix, dual):
        """dual=False: plain static const arrays (C oracle).
        dual=True: each table twice, a host copy NAME_h and, under nvcc, a
        __constant__ device copy NAME_d; GWT_T(NAME) picks the right one."""
        P = prefix.upper()
        tabs = []
        rows = []
        for r in range(19):
            rows.append("{" + ", ".join(fmt(x) for x in lam[r * 11:(r + 1) * 11]) + "}")
        tabs.append(("lambda_fit", "[19][11]", "{" + ",\\\n  ".join(rows) + "}", True))
        for name, arr in (("qnm_a", qa), ("qnm_fring", qr), ("qnm_fdamp", qd)):
            body = ",\\\n  ".join(", ".join(fmt(x) for x in arr[i:i + 6]) for i in range(0, 1003, 6))
            tabs.append((name, "[1003]", "{" + body + "}", False))
        tabs.append(("det_location", "[9][3]", "{" + ", ".join("{" + ", ".join(fmt(x) for x in loc[s_]) + "}" for s_, _ in dets) + "}", True))
        tabs.append(("det_tensor", "[9][9]", "{" + ", ".join("{" + ", ".join(fmt(x) for x in tens[s_]) + "}" for s_, _ in dets) + "}", True))
        tabs.append(("det_geometric", "[9]", "{" + ", ".join(fmt(geo[s_]) for s_, _ in dets) + "}", True))
        lines = []
        lines.append("/* Generated by oracle/gen_tables.py -- constant data only, do not edit. */")
        lines.append("/* IMRPhenomD calibration fits (rows: rho1..3, v2, gamma1..3, sigma1..4, beta1..3,")
        lines.append("   alpha1..5; columns: polynomial in eta and chi_PN - 1); quasi-normal-mode table")
        lines.append("   (final spin, ringdown and damping frequency times M); ground detectors in the")
        lines.append("   order Hanford, Livingston, Virgo, Kagra, Indigo, CE, ET1, ET2, ET3 (ECEF")
        lines.append("   location in m, response tensor row major, geometric factor). */")
        lines.append("#ifndef %sTABLES_H" % P)
        lines.append("#define %sTABLES_H" % P)
        lines.append("#define %sQNM_LEN 1003" % P)
        lines.append("#define %sNDET_KNOWN 9" % P)
        if dual:
            lines.append("#if defined(__CUDA_ARCH__)")
            lines.append("#define GWT_T(name) name##_d")
            lines.append("#else")
            lines.append("#define GWT_T(name) name##_h")
            lines.append("#endif")
        for name, dims, init, devcopy in tabs:
            if dual:
                lines.append("#define %s%s_INIT %s" % (P, name.upper(), init))
                lines.append("static const double %s%s_h%s = %s%s_INIT;" % (prefix, name, dims, P, name.upper()))
                if devcopy:
                    lines.append("#if defined(__CUDACC__)")
                    lines.append("static __constant__ double %s%s_d%s = %s%s_INIT;" % (prefix, name, dims, P, name.upper()))
                    lines.append("#endif")
            else:
                lines.append("static const double %s%s%s = %s;" % (prefix, name, dims, init.replace("\\\n", "\n")))
        lines.append("#endif")
        with open(path, "w") as f:
            f.write("\n".join(lines) + "\n")

    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    emit(os.path.join(here, "gwo_tables.h"), "gwo_", False)
    emit(os.path.join(root, "gw_analysis_tools_gb300", "csrc", "phenom_tables.h"), "gwt_", True)
    print("wrote tables: lambda %d, qnm %d, detectors %d" % (len(lam), len(qa), len(dets)))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ["GWAT_REFERENCE_DIR"])
