"""The strain transform of allocate_LOSC_data (io_util.cpp:523-664: trim around
the trigger, Tukey window, forward DFT times dt, the PSD's band) on the device
against the oracle's numpy restatement, from memory and from files, and
through the reference signature of the C++ drop-in."""
import ctypes
import os
import sys

import numpy as np
import pytest

import gw_analysis_tools_gb300 as G

pytestmark = pytest.mark.gpu
RTOL = 1e-12   # of the largest bin: FFTW and cuFFT round differently


@pytest.fixture(scope="module")
def io_oracle():
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.join(os.path.dirname(here), "oracle"))
    import ingest_oracle
    return ingest_oracle


def _strain(nd, fs, duration, seed):
    rng = np.random.default_rng(seed)
    n = int(fs * duration)
    t = np.arange(n) / fs
    x = rng.normal(0, 1e-21, (nd, n))
    # a chirp-like tone to give the band structure
    x += 1e-21 * np.sin(2 * np.pi * (30 + 8 * t) * t)[None, :]
    return x


def _psd_table(nd, f0, f1, T):
    f = np.arange(f0, f1 + 0.5 / T, 1.0 / T)
    cols = [f] + [1e-46 * (1 + (f / 100.0) ** 2) * (1 + 0.1 * d) for d in range(nd)]
    return np.column_stack(cols)


def _compare(got, ref):
    gd, gp, gf, gb = got
    rd, rp, rf, rb = ref
    assert gb == rb
    assert np.array_equal(gp, rp) and np.array_equal(gf, rf)
    scale = np.max(np.abs(rd))
    assert np.max(np.abs(gd - rd)) <= RTOL * scale, np.max(np.abs(gd - rd)) / scale


@pytest.mark.parametrize("fs,duration,T,band,trigger,post", [
    (4096.0, 64.0, 8.0, (20.0, 1024.0), 40.3, 2.0),
    (4096.0, 128.0, 32.0, (10.0, 2048.0), 100.0, 2.0),     # band up to fs/2
    (1024.0, 32.0, 4.0, (16.0, 700.0), 17.77, 1.0),        # band above fs/2: mirrored bins
    (2048.0, 16.0, 8.0, (20.0, 512.0), 7.5, 0.5),          # window starting near the file's start
])
def test_losc_prepare_matches_oracle(gpu_ctx, io_oracle, fs, duration, T, band, trigger, post):
    nd = 3
    start = 1126256640.0
    x = _strain(nd, fs, duration, 7)
    tab = _psd_table(nd, band[0], band[1], T)
    got = gpu_ctx.losc_prepare(x, start, duration, fs, tab, start + trigger, post)
    ref = io_oracle.losc_prepare(x, start, duration, fs, tab, start + trigger, post)
    _compare(got, ref)


def test_losc_prepare_trigger_outside(gpu_ctx):
    x = _strain(2, 1024.0, 16.0, 8)
    tab = _psd_table(2, 20.0, 400.0, 8.0)
    with pytest.raises(G.GwGpuError, match="domain"):
        gpu_ctx.losc_prepare(x, 0.0, 16.0, 1024.0, tab, 3.0, 1.0)   # window starts before the file


def _write_losc(path, x, fs, start, duration):
    with open(path, "w") as f:
        f.write("# Gravitational wave strain (synthetic)\n# This file has %d samples per second\n"
                "# starting GPS %d duration %d\n" % (fs, start, duration))
        f.write("\n".join(repr(float(v)) for v in x))
        f.write("\n")


def test_allocate_losc_data_from_files(gpu_ctx, io_oracle, tmp_path):
    nd, fs, duration, start = 3, 4096, 32, 1126259446
    x = _strain(nd, float(fs), float(duration), 9)
    files = []
    for d in range(nd):
        p = str(tmp_path / ("strain%d.txt" % d))
        _write_losc(p, x[d], fs, start, duration)
        files.append(p)
    tab = _psd_table(nd, 20.0, 1000.0, 4.0)
    psd_path = str(tmp_path / "psd.txt")
    with open(psd_path, "w") as f:
        f.write("# freq H1 L1 V1\n")
        for r in tab:
            f.write(" ".join(repr(float(v)) for v in r) + "\n")
    psd_length = G.count_lines_losc_psd_file(psd_path)
    data_len = G.count_lines_losc_data_file(files[0])
    trig, post = start + 20.25, 2.0
    got = gpu_ctx.allocate_losc_data(files, psd_path, psd_length, data_len, trig, post)
    # the oracle from its own parse of the same files
    series = np.array([io_oracle.read_losc_data_file(p)[0] for p in files])
    ptab = io_oracle.read_losc_psd_file(psd_path, psd_length, nd + 1)
    ref = io_oracle.losc_prepare(series, float(start), float(duration), float(fs), ptab, trig, post)
    _compare(got + (ref[3],), ref)

    # the reference signature in the C++ drop-in
    from gw_analysis_tools_gb300 import _native
    _native.build()
    L = ctypes.CDLL(_native.DROPIN_LIB)
    fn = L.gwat_dropin_test_losc
    fn.restype = None
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                   ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    names = (ctypes.c_char_p * nd)(*[p.encode() for p in files])
    dd = np.zeros((nd, psd_length), dtype=np.complex128)
    pp = np.zeros((nd, psd_length))
    ff = np.zeros((nd, psd_length))
    fn(names, nd, psd_path.encode(), psd_length, data_len, trig, post, dd.ctypes.data, pp.ctypes.data, ff.ctypes.data)
    _compare((dd, pp, ff, ref[3]), ref)
