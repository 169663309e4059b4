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
    python oracle/gen_tables.py /root/reference
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

    def emit(path, prefix, qualifier):
        lines = []
        lines.append("/* Generated by oracle/gen_tables.py -- constant data only, do not edit. */")
        lines.append("#ifndef %sTABLES_H" % prefix.upper())
        lines.append("#define %sTABLES_H" % prefix.upper())
        lines.append("#define %sQNM_LEN 1003" % prefix.upper())
        lines.append("#define %sNDET_KNOWN 9" % prefix.upper())
        lines.append("/* IMRPhenomD calibration fits: row = lambda index (rho1..3, v2, gamma1..3,")
        lines.append("   sigma1..4, beta1..3, alpha1..5), columns = polynomial in (eta, chi_PN - 1). */")
        lines.append("%s double %slambda_fit[19][11] = {" % (qualifier, prefix))
        for r in range(19):
            row = lam[r * 11:(r + 1) * 11]
            lines.append("  {" + ", ".join(fmt(x) for x in row) + "},")
        lines.append("};")
        for name, arr in (("qnm_a", qa), ("qnm_fring", qr), ("qnm_fdamp", qd)):
            lines.append("%s double %s%s[1003] = {" % (qualifier, prefix, name))
            for i in range(0, 1003, 6):
                lines.append("  " + ", ".join(fmt(x) for x in arr[i:i + 6]) + ",")
            lines.append("};")
        lines.append("/* Ground detectors, in this order: Hanford, Livingston, Virgo, Kagra, Indigo,")
        lines.append("   Cosmic Explorer, Einstein Telescope 1/2/3.  ECEF location (m), response")
        lines.append("   tensor (row major), geometric factor. */")
        lines.append("%s double %sdet_location[9][3] = {" % (qualifier, prefix))
        for short, _ in dets:
            lines.append("  {" + ", ".join(fmt(x) for x in loc[short]) + "},")
        lines.append("};")
        lines.append("%s double %sdet_tensor[9][9] = {" % (qualifier, prefix))
        for short, _ in dets:
            lines.append("  {" + ", ".join(fmt(x) for x in tens[short]) + "},")
        lines.append("};")
        lines.append("%s double %sdet_geometric[9] = {" % (qualifier, prefix))
        lines.append("  " + ", ".join(fmt(geo[s]) for s, _ in dets))
        lines.append("};")
        lines.append("#endif")
        with open(path, "w") as f:
            f.write("\n".join(lines) + "\n")

    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    emit(os.path.join(here, "gwo_tables.h"), "gwo_", "static const")
    emit(os.path.join(root, "gw_analysis_tools_gb300", "csrc", "phenom_tables.h"), "gwt_", "static const")
    print("wrote tables: lambda %d, qnm %d, detectors %d" % (len(lam), len(qa), len(dets)))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
