"""Plain-Python / numpy restatement of the reference's data and noise
ingestion (TEST INFRASTRUCTURE ONLY: only tests/ and the CPU-baseline leg of
bench.py use it, as the checker of the library's readers and strain
transform).

Each function follows the cited reference lines statement by statement where
the order matters (which header token wins, which samples and bins are kept);
the DFT is numpy's (the reference's is FFTW's forward transform, the same
definition).
"""
import math

import numpy as np


def _stod(item):
    """std::stod: leading white space skipped, the longest numeric prefix
    converted; ValueError where stod throws."""
    s = item.lstrip(" \t\n\v\f\r")
    best = None
    for end in range(len(s), 0, -1):
        if "_" in s[:end]:  # Python's float takes digit separators, strtod does not
            continue
        try:
            best = float(s[:end])
            break
        except ValueError:
            continue
    if best is None:
        raise ValueError("no conversion: %r" % item)
    return best


def _getline_items(line, delim=","):
    """Items of getline(lineStream, item, delim): an empty last item is not
    produced."""
    if line == "":
        return []
    parts = line.split(delim)
    if parts[-1] == "":
        parts = parts[:-1]
    return parts


def _lines(text):
    """Lines as std::getline yields them."""
    if text == "":
        return []
    lines = text.split("\n")
    if text.endswith("\n"):
        lines = lines[:-1]
    return lines


def count_lines_data_file(path):
    """count_lines_data_file (io_util.cpp:682-699)."""
    with open(path, "r", newline="") as f:
        return len(_lines(f.read()))


def read_losc_data_file(path):
    """read_LOSC_data_file (io_util.cpp:403-464) -> (samples, start, duration, fs)."""
    with open(path, "r", newline="") as f:
        text = f.read()
    out = []
    start = duration = fs = None
    j = 0
    for line in _lines(text):
        if j > 2:
            for item in _getline_items(line):
                out.append(_stod(item))
        else:
            if j == 1:
                for s in line.split():
                    if s[0].isdigit():
                        fs = _stod(s)
            elif j == 2:
                k = 0
                for s in line.split():
                    if s[0].isdigit():
                        if k == 0:
                            start = _stod(s)
                            k += 1
                        else:
                            duration = _stod(s)
            j += 1
    return np.array(out), start, duration, fs


def read_losc_psd_file(path, rows, cols):
    """read_LOSC_PSD_file (io_util.cpp:466-500): first line skipped; rows the
    file does not fill are zero here (unset in the reference)."""
    with open(path, "r", newline="") as f:
        lines = _lines(f.read())
    vals = []
    for line in lines[1:]:
        vals.extend(_stod(s) for s in line.split())
    out = np.zeros(rows * cols)
    out[:len(vals)] = vals[:rows * cols]
    return out.reshape(rows, cols)


def tukey_window(length, alpha):
    """tukey_window (util.cpp:1736-1757)."""
    imin = float(int(alpha * (length - 1) / 2.0))
    imax = float(int((length - 1) * (1. - alpha / 2.)))
    w = np.empty(length)
    for i in range(length):
        if i < imin:
            w[i] = 0.5 * (1 + math.cos(math.pi * (i / imin - 1)))
        elif i < imax:
            w[i] = 1
        else:
            w[i] = 0.5 * (1 + math.cos(math.pi * (i / imin - 2. / alpha + 1.)))
    return w


def losc_prepare(series, file_start, duration, fs, psd_table, trigger_time, post_merger_duration):
    """The transform part of allocate_LOSC_data (io_util.cpp:550-651).
    series: [ndet][n]; psd_table: [psd_length][ndet+1].  Returns (data, psds,
    freqs, bins) with data [ndet][psd_length] complex (unfilled bins zero), or
    None when the trigger window does not fit in the file."""
    series = np.asarray(series, dtype=np.float64)
    tab = np.asarray(psd_table, dtype=np.float64)
    nd = series.shape[0]
    psd_length = tab.shape[0]
    Tobs = 1. / (tab[1, 0] - tab[0, 0])
    df = 1. / Tobs
    dt = 1. / fs
    n_trim = int(Tobs * fs)
    psds = np.ascontiguousarray(tab[:, 1:].T)
    freqs = np.ascontiguousarray(np.broadcast_to(tab[:, 0], (nd, psd_length)))
    N = int(fs * duration)
    times = file_start + np.arange(N) * dt
    time_start = trigger_time - (Tobs - post_merger_duration)
    time_end = trigger_time + post_merger_duration
    if time_start < file_start or time_end > file_start + duration:
        return None, psds, freqs, 0
    alpha = 2 * .4 / Tobs
    window = tukey_window(n_trim, alpha)
    sel = np.nonzero((times > time_start) & (times <= time_end))[0][:n_trim]
    trimmed = np.zeros((nd, n_trim))
    trimmed[:, :sel.size] = series[:, sel] * window[:sel.size]
    fft = np.fft.fft(trimmed, axis=1)
    fu = np.arange(n_trim) * df
    fmin, fmax = tab[0, 0], tab[-1, 0]
    keep = np.nonzero((fu >= fmin) & (fu <= fmax))[0][:psd_length]
    data = np.zeros((nd, psd_length), dtype=np.complex128)
    data[:, :keep.size] = fft[:, keep] * dt
    return data, psds, freqs, int(keep.size)


def aligo_analytic(f):
    """aLIGO_analytic (detector_util.cpp:286-293)."""
    S = 3e-48
    fknee = 70.
    x = fknee / f
    x4 = x * x * x * x
    return math.sqrt(S * (x4 + 2 + 2 * x * x) / 5)


def hanford_o1_fitted(f):
    """Hanford_O1_fitted (detector_util.cpp:404-414)."""
    a = [47.8466, -92.1896, 35.9273, -7.61447, 0.916742, -0.0588089, 0.00156345]
    S0 = .8464
    x = math.log(f)
    return math.sqrt(S0) * math.exp(a[0] + a[1] * x + a[2] * x * x + a[3] * x * x * x + a[4] * x * x * x * x
                                    + a[5] * x * x * x * x * x + a[6] * x * x * x * x * x * x)


def interp_linear(x, y, f):
    """gsl_interp_linear evaluation: interval with x_i <= f < x_{i+1} (the
    last one at f = x_{n-1}); NaN outside the table."""
    n = len(x)
    if not (x[0] <= f <= x[n - 1]):
        return float("nan")
    lo, hi = 0, n - 1
    while hi > lo + 1:
        mid = (lo + hi) // 2
        if x[mid] > f:
            hi = mid
        else:
            lo = mid
    dx = x[lo + 1] - x[lo]
    return y[lo] + (f - x[lo]) / dx * (y[lo + 1] - y[lo])


def populate_noise_table(freqs, table_path):
    """The tabulated branch of populate_noise (detector_util.cpp:242-270):
    two comma-separated columns, linear interpolation."""
    with open(table_path, "r", newline="") as f:
        vals = []
        for line in _lines(f.read()):
            vals.extend(_stod(i) for i in _getline_items(line))
    rows = len(vals) // 2
    x = [vals[2 * i] for i in range(rows)]
    y = [vals[2 * i + 1] for i in range(rows)]
    return np.array([interp_linear(x, y, float(fi)) for fi in freqs])
