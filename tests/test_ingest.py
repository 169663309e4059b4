"""Data and noise ingestion readers (host code of the C ABI) against the
oracle's restatement of read_LOSC_data_file / read_LOSC_PSD_file /
count_lines_* (io_util.cpp:403-500, 682-714) and populate_noise
(detector_util.cpp:86-283).  No GPU."""
import os

import numpy as np
import pytest

import gw_analysis_tools_gb300 as G

def _reference_noise_dir():
    """The reference's tabulated noise curves, where its checkout is known
    (GWAT_REFERENCE_DIR, or the checkout the oracle's pin libraries were built
    from)."""
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.join(os.path.dirname(here), "oracle"))
    import oracle
    d = oracle.reference_dir()
    return os.path.join(d, "data", "noise_data", "currently_supported") if d else ""


REFERENCE_NOISE_DIR = _reference_noise_dir()


@pytest.fixture(scope="module")
def io_oracle():
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.join(os.path.dirname(here), "oracle"))
    import ingest_oracle
    return ingest_oracle


def _losc_text(samples, fs=4096, start=1126256640, duration=None, per_line=1, newline="\n", final_newline=True):
    duration = len(samples) / fs if duration is None else duration
    head = ["# Gravitational wave strain (synthetic) for H1",
            "# This file has %d samples per second" % fs,
            "# starting GPS %d duration %d" % (start, duration)]
    body = []
    for i in range(0, len(samples), per_line):
        body.append(",".join(repr(float(x)) for x in samples[i:i + per_line]))
    text = newline.join(head + body)
    return text + newline if final_newline else text


def _write(tmp_path, name, text):
    p = tmp_path / name
    p.write_bytes(text.encode())
    return str(p)


def test_losc_data_file_matches_oracle(tmp_path, io_oracle):
    rng = np.random.default_rng(1)
    x = rng.normal(0, 1e-19, 4096 * 4)
    p = _write(tmp_path, "H.txt", _losc_text(x))
    got, start, dur, fs = G.read_losc_data_file(p)
    ref, rstart, rdur, rfs = io_oracle.read_losc_data_file(p)
    assert np.array_equal(got, ref) and np.array_equal(got, x)
    assert (start, dur, fs) == (rstart, rdur, rfs) == (1126256640.0, 4.0, 4096.0)
    assert G.count_lines_losc_data_file(p) == x.size
    assert G.count_lines_data_file(p) == io_oracle.count_lines_data_file(p) == x.size + 3


@pytest.mark.parametrize("variant", ["crlf", "no_final_newline", "three_per_line", "trailing_comma", "blank_lines"])
def test_losc_data_file_layouts(tmp_path, io_oracle, variant):
    rng = np.random.default_rng(2)
    x = rng.normal(0, 1e-19, 999)
    if variant == "crlf":
        text = _losc_text(x, newline="\r\n")
    elif variant == "no_final_newline":
        text = _losc_text(x, final_newline=False)
    elif variant == "three_per_line":
        text = _losc_text(x, per_line=3)
    elif variant == "trailing_comma":
        text = _losc_text(x).replace("\n", ",\n")
        text = text.replace("duration 0,", "duration 0")  # header lines keep their own text
    else:
        text = _losc_text(x) + "\n\n"
    p = _write(tmp_path, "v.txt", text)
    got = G.read_losc_data_file(p)
    ref = io_oracle.read_losc_data_file(p)
    assert np.array_equal(got[0], ref[0]) and np.array_equal(got[0], x)
    assert got[1:] == ref[1:]
    assert G.count_lines_data_file(p) == io_oracle.count_lines_data_file(p)


def test_losc_data_file_errors(tmp_path):
    p = _write(tmp_path, "bad.txt", _losc_text([1.0, 2.0]) + "abc\n")
    with pytest.raises(G.GwGpuError, match="invalid"):
        G.read_losc_data_file(p)
    p = _write(tmp_path, "empty_item.txt", _losc_text([1.0]) + ",2.0\n")
    with pytest.raises(G.GwGpuError, match="invalid"):
        G.read_losc_data_file(p)
    p = _write(tmp_path, "ok.txt", _losc_text(np.arange(10.0)))
    with pytest.raises(G.GwGpuError, match="too large"):
        G.read_losc_data_file(p, capacity=5)
    with pytest.raises(G.GwGpuError, match="not found"):
        G.read_losc_data_file(str(tmp_path / "missing.txt"))


def test_losc_psd_file_matches_oracle(tmp_path, io_oracle):
    f = np.arange(20.0, 30.0, 0.125)
    rows = np.column_stack([f, 1e-46 * (1 + f), 2e-46 * (1 + f)])
    text = "# freq H1 L1\n" + "".join("%r\t%r  %r\n" % tuple(map(float, r)) for r in rows)
    p = _write(tmp_path, "psd.txt", text)
    n = G.count_lines_losc_psd_file(p)
    assert n == f.size
    got = G.read_losc_psd_file(p, n, 3)
    assert np.array_equal(got, io_oracle.read_losc_psd_file(p, n, 3)) and np.array_equal(got, rows)
    # more rows asked than the file holds: zeros (unset in the reference)
    got2 = G.read_losc_psd_file(p, n + 2, 3)
    assert np.array_equal(got2[:n], rows) and not got2[n:].any()
    with pytest.raises(G.GwGpuError, match="too large"):
        G.read_losc_psd_file(p, n - 1, 3)


def test_noise_analytic_matches_oracle(io_oracle):
    # Hanford_O1_fitted sums terms of size ~500 to an exponent near -45, so a
    # last-bit difference in any term (the C library's log or the order of
    # rounding) moves the result by ~1e-13 relative: hence its looser bound
    f = np.geomspace(10.0, 4096.0, 777)
    for name, fn, rtol in (("aLIGO_analytic", io_oracle.aligo_analytic, 1e-14),
                           ("Hanford_O1_fitted", io_oracle.hanford_o1_fitted, 1e-11)):
        got = G.populate_noise(f, name)
        ref = np.array([fn(x) for x in f])
        assert np.allclose(got, ref, rtol=rtol, atol=0), name


def test_noise_table_matches_oracle(tmp_path, io_oracle):
    rng = np.random.default_rng(3)
    x = np.cumsum(rng.uniform(0.1, 3.0, 500)) + 5.0
    y = np.exp(rng.normal(-50, 1, 500))
    (tmp_path / "aligo_O4high.csv").write_text("".join("%r,%r\n" % (float(a), float(b)) for a, b in zip(x, y)))
    f = np.concatenate([x[:5], rng.uniform(x[0], x[-1], 2000), x[-3:]])
    got = G.populate_noise(f, "AdLIGODesign", noise_dir=str(tmp_path))
    ref = io_oracle.populate_noise_table(f, str(tmp_path / "aligo_O4high.csv"))
    assert np.array_equal(got, ref)
    assert np.allclose(got, np.interp(f, x, y), rtol=1e-13, atol=0)
    # outside the table: the reference's GSL domain error
    with pytest.raises(G.GwGpuError, match="domain"):
        G.populate_noise([x[0] - 1.0], "AdLIGODesign", noise_dir=str(tmp_path))
    # listed by the reference without a file, and unknown names
    for name in ("KAGRA_opt_smoothed", "NoSuchCurve"):
        with pytest.raises(G.GwGpuError, match="not found"):
            G.populate_noise(f, name, noise_dir=str(tmp_path))


@pytest.mark.skipif(not os.path.isdir(REFERENCE_NOISE_DIR), reason="the reference's noise curves are not here")
def test_noise_reference_curves(io_oracle):
    """The reference's own tabulated curves, where its data directory is present."""
    f = np.linspace(10.0, 2000.0, 3001)
    for name, fname in (("AdLIGODesign", "aligo_O4high.csv"), ("CE2", "CE2_strain.csv"),
                        ("AdVIRGOPlus1", "avirgo_O4high_NEW.csv")):
        ref = io_oracle.populate_noise_table(f, os.path.join(REFERENCE_NOISE_DIR, fname))
        ok = np.isfinite(ref)
        try:
            got = G.populate_noise(f, name, noise_dir=REFERENCE_NOISE_DIR)
        except G.GwGpuError:
            got = G.populate_noise(f[ok], name, noise_dir=REFERENCE_NOISE_DIR)
            assert np.array_equal(got, ref[ok]), name
            continue
        assert np.array_equal(got, ref), name
