"""Python front end of the C ABI (include/gwgpu.h).

A Context owns one device, its stream, an HBM budget and the device-resident
data registry.  Functions mirror the reference's entry points:

  fourier_waveform            waveform_generator.cpp:104 (fourier_waveform)
  fourier_detector_response   waveform_util.cpp:1070
  log_likelihood_internal     mcmc_gw.cpp:801 (Log_Likelihood_internal, SIMPSONS)
  mcmc_likelihood_extrinsic   mcmc_gw.cpp:2374 (MCMC_likelihood_extrinsic), plain FP64 form
  loglik_batch                many MCMC_likelihood_extrinsic requests in one fused launch
  mcmc_loglik_batch           MCMC_likelihood_wrapper (mcmc_gw.cpp:2569) on parameter vectors
  fisher_numerical            fisher.cpp:81
  fisher_batch                batched network Fisher + FP64 inverse

Every call goes to the CUDA library; there is no CPU fallback.
"""
import ctypes
import os

import numpy as np

from . import _native

IMRPhenomD = 0
IMRPhenomPv2 = 1
PREC_FP64 = 0
PREC_MIXED = 1
FISHER_REFERENCE = 0   # gwgpu_fisher_options.algorithm
FISHER_MOMENTS = 1
METHODS = {"IMRPhenomD": IMRPhenomD, "IMRPhenomPv2": IMRPhenomPv2}
STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "HBM budget exceeded", 4: "outside model domain",
          5: "timed out", 6: "busy", 7: "not found", 8: "too large", 9: "Fisher matrix not positive definite"}


class GenParams(ctypes.Structure):
    """gwgpu_gen_params: the gen_params_base<double> fields on the path."""

    _fields_ = [
        ("mass1", ctypes.c_double), ("mass2", ctypes.c_double),
        ("spin1", ctypes.c_double * 3), ("spin2", ctypes.c_double * 3),
        ("Luminosity_Distance", ctypes.c_double),
        ("incl_angle", ctypes.c_double), ("phiRef", ctypes.c_double),
        ("f_ref", ctypes.c_double), ("tc", ctypes.c_double),
        ("RA", ctypes.c_double), ("DEC", ctypes.c_double),
        ("psi", ctypes.c_double), ("gmst", ctypes.c_double),
        ("chip", ctypes.c_double), ("phip", ctypes.c_double),
        ("shift_time", ctypes.c_int32), ("shift_phase", ctypes.c_int32),
        ("sky_average", ctypes.c_int32), ("dep_postmerger", ctypes.c_int32),
        ("theta_l", ctypes.c_double), ("phi_l", ctypes.c_double),
        ("equatorial_orientation", ctypes.c_int32), ("reserved", ctypes.c_int32),
    ]


def gen_params(**kw):
    """gen_params_py-style constructor (gwatpy/util.py): keyword fields, reference defaults."""
    p = GenParams()
    p.chip = -1.0
    p.phip = -1.0
    p.shift_time = 1
    p.shift_phase = 1
    for k, v in kw.items():
        if k in ("spin1", "spin2"):
            getattr(p, k)[:] = [float(x) for x in v]
        elif k in ("shift_time", "shift_phase", "sky_average", "dep_postmerger", "equatorial_orientation"):
            setattr(p, k, int(bool(v)))
        else:
            setattr(p, k, float(v))
    return p


def transform_orientation_coords(params, generation_method="IMRPhenomD"):
    """transform_orientation_coords (waveform_util.cpp:1523-1586), ground
    detectors: a copy of params with incl_angle and psi from theta_l, phi_l."""
    out = GenParams()
    ctypes.pointer(out)[0] = params if isinstance(params, GenParams) else gen_params(**params)
    _io_check(_native.load().gwgpu_transform_orientation_coords(ctypes.byref(out), generation_method.encode()),
              "transform_orientation_coords")
    return out


def params_array(plist):
    arr = (GenParams * len(plist))()
    for i, p in enumerate(plist):
        arr[i] = p if isinstance(p, GenParams) else gen_params(**p)
    return arr


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


class GwGpuError(_native.GwGpuError):
    pass


def _io_check(st, what):
    if st != 0:
        raise GwGpuError("%s: %s" % (what, STATUS.get(st, st)))


def count_lines_data_file(path):
    """count_lines_data_file (io_util.cpp:682-699)."""
    n = ctypes.c_int()
    _io_check(_native.load().gwgpu_count_lines_data_file(os.fsencode(path), ctypes.byref(n)), path)
    return n.value


def count_lines_losc_data_file(path):
    """count_lines_LOSC_data_file (io_util.cpp:709-714): lines less the 3 header lines."""
    n = ctypes.c_int()
    _io_check(_native.load().gwgpu_count_lines_losc_data_file(os.fsencode(path), ctypes.byref(n)), path)
    return n.value


def count_lines_losc_psd_file(path):
    """count_lines_LOSC_PSD_file (io_util.cpp:701-707): lines less the header line."""
    n = ctypes.c_int()
    _io_check(_native.load().gwgpu_count_lines_losc_psd_file(os.fsencode(path), ctypes.byref(n)), path)
    return n.value


def read_losc_data_file(path, capacity=None):
    """read_LOSC_data_file (io_util.cpp:403-464) -> (samples, start, duration, fs)."""
    L = _native.load()
    n = ctypes.c_longlong()
    start, duration, fs = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    cap = capacity if capacity is not None else max(count_lines_losc_data_file(path), 1)
    for _ in range(2):
        out = np.zeros(cap)
        st = L.gwgpu_read_losc_data_file(os.fsencode(path), _dp(out), cap, ctypes.byref(n), ctypes.byref(start),
                                         ctypes.byref(duration), ctypes.byref(fs))
        if st != 8 or capacity is not None:
            break
        cap = n.value  # more than one value on some lines
    _io_check(st, path)
    return out[:n.value].copy(), start.value, duration.value, fs.value


def read_losc_psd_file(path, rows, cols):
    """read_LOSC_PSD_file (io_util.cpp:466-500) -> array [rows][cols]."""
    out = np.zeros((rows, cols))
    _io_check(_native.load().gwgpu_read_losc_psd_file(os.fsencode(path), _dp(out), rows, cols), path)
    return out


def populate_noise(frequencies, detector, noise_dir=None, integration_time=48.0):
    """populate_noise (detector_util.cpp:86-283) for the ground-detector
    curves: the amplitude spectral density at each frequency."""
    f = np.ascontiguousarray(frequencies, dtype=np.float64)
    out = np.zeros(f.size)
    st = _native.load().gwgpu_populate_noise(_dp(f), detector.encode(), _dp(out), f.size, float(integration_time),
                                             os.fsencode(noise_dir) if noise_dir else None)
    _io_check(st, "populate_noise(%s)" % detector)
    return out


class Context:
    """One device, one stream, one HBM budget (bytes, 0 = unlimited)."""

    def __init__(self, device=0, hbm_budget=0):
        self.lib = _native.load()
        h = ctypes.c_void_p()
        st = self.lib.gwgpu_context_create(device, hbm_budget, ctypes.byref(h))
        if st != 0:
            raise GwGpuError("gwgpu_context_create failed: %s" % STATUS.get(st, st))
        self.h = h
        self._data = {}

    def close(self):
        if getattr(self, "h", None):
            self.lib.gwgpu_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st, what):
        if st != 0:
            msg = self.lib.gwgpu_last_error_string(self.h)
            raise GwGpuError("%s: %s (%s)" % (what, STATUS.get(st, st), msg.decode() if msg else ""))

    @property
    def stream(self):
        return self.lib.gwgpu_context_stream(self.h)

    def bytes_in_use(self):
        return self.lib.gwgpu_context_bytes_in_use(self.h)

    # ------------------------------------------------------------ waveform
    def fourier_waveform(self, freqs, method, params):
        f = np.ascontiguousarray(freqs, dtype=np.float64)
        hp = np.zeros(f.size, dtype=np.complex128)
        hc = np.zeros(f.size, dtype=np.complex128)
        ok = self.lib.gwgpu_fourier_waveform(self.h, _dp(f), f.size, _dp(hp), _dp(hc), method.encode(),
                                             ctypes.byref(params))
        if ok != 1:
            raise GwGpuError("fourier_waveform failed: %s" % self.lib.gwgpu_last_error_string(self.h))
        return hp, hc

    def fourier_detector_response(self, freqs, detector, method, params):
        f = np.ascontiguousarray(freqs, dtype=np.float64)
        r = np.zeros(f.size, dtype=np.complex128)
        ok = self.lib.gwgpu_fourier_detector_response(self.h, _dp(f), f.size, _dp(r), detector.encode(),
                                                      method.encode(), ctypes.byref(params))
        if ok != 1:
            raise GwGpuError("fourier_detector_response failed")
        return r

    # ---------------------------------------------------------------- data
    def register_data(self, detector, freqs, data, psd, weights=None, log10F=False):
        """One detector's grid, data and PSD on the device.  With weights, the
        stream integrates by the GAUSSLEG rule (mcmc_gw.cpp:820-862) instead of
        Simpson's."""
        f = np.ascontiguousarray(freqs, dtype=np.float64)
        d = np.ascontiguousarray(data, dtype=np.complex128)
        s = np.ascontiguousarray(psd, dtype=np.float64)
        h = ctypes.c_int()
        if weights is None:
            st = self.lib.gwgpu_data_register(self.h, detector.encode(), _dp(f), f.size, _dp(d), _dp(s),
                                              ctypes.byref(h))
        else:
            w = np.ascontiguousarray(weights, dtype=np.float64)
            st = self.lib.gwgpu_data_register_weighted(self.h, detector.encode(), _dp(f), f.size, _dp(d), _dp(s),
                                                       _dp(w), int(bool(log10F)), ctypes.byref(h))
        self._check(st, "data_register")
        self._data[h.value] = (detector, f.size)
        return h.value

    def release_data(self, handle):
        self._check(self.lib.gwgpu_data_release(self.h, handle), "data_release")
        self._data.pop(handle, None)

    # ---------------------------------------------------------- likelihood
    def log_likelihood_internal(self, data, psd, freqs, response, weights=None, log10F=False):
        d = np.ascontiguousarray(data, dtype=np.complex128)
        s = np.ascontiguousarray(psd, dtype=np.float64)
        f = np.ascontiguousarray(freqs, dtype=np.float64)
        r = np.ascontiguousarray(response, dtype=np.complex128)
        out = ctypes.c_double()
        if weights is None:
            st = self.lib.gwgpu_log_likelihood_internal(self.h, _dp(d), _dp(s), _dp(f), _dp(r), f.size,
                                                        ctypes.byref(out))
        else:
            w = np.ascontiguousarray(weights, dtype=np.float64)
            st = self.lib.gwgpu_log_likelihood_internal_weighted(self.h, _dp(d), _dp(s), _dp(f), _dp(w), _dp(r),
                                                                 f.size, int(bool(log10F)), ctypes.byref(out))
        self._check(st, "log_likelihood_internal")
        return out.value

    def losc_prepare(self, series, file_start, duration, fs, psd_table, trigger_time, post_merger_duration):
        """The transform step of allocate_LOSC_data (io_util.cpp:550-651) on the
        device.  Returns (data [ndet][psd_length] complex, psds, freqs, bins)."""
        x = np.ascontiguousarray(series, dtype=np.float64)
        if x.ndim == 1:
            x = x[None, :]
        tab = np.ascontiguousarray(psd_table, dtype=np.float64)
        nd, n = x.shape
        pl = tab.shape[0]
        data = np.zeros((nd, pl), dtype=np.complex128)
        psds = np.zeros((nd, pl))
        freqs = np.zeros((nd, pl))
        bins = ctypes.c_int(0)
        st = self.lib.gwgpu_losc_prepare(self.h, _dp(x), nd, n, float(file_start), float(duration), float(fs),
                                         _dp(tab), pl, float(trigger_time), float(post_merger_duration), _dp(data),
                                         _dp(psds), _dp(freqs), ctypes.byref(bins))
        self._check(st, "losc_prepare")
        return data, psds, freqs, bins.value

    def allocate_losc_data(self, data_files, psd_file, psd_length, data_file_length, trigger_time,
                           post_merger_duration):
        """allocate_LOSC_data (io_util.cpp:523-664): files in, (data, psds, freqs) out."""
        nd = len(data_files)
        names = (ctypes.c_char_p * nd)(*[os.fsencode(f) for f in data_files])
        data = np.zeros((nd, psd_length), dtype=np.complex128)
        psds = np.zeros((nd, psd_length))
        freqs = np.zeros((nd, psd_length))
        st = self.lib.gwgpu_allocate_losc_data(self.h, names, os.fsencode(psd_file), nd, psd_length,
                                               data_file_length, float(trigger_time), float(post_merger_duration),
                                               _dp(data), _dp(psds), _dp(freqs))
        self._check(st, "allocate_losc_data")
        return data, psds, freqs

    def maximized_log_likelihood_internal(self, data, psd, freqs, response):
        """maximized_Log_Likelihood_aligned_spin_internal (mcmc_gw.cpp:595-658)."""
        d = np.ascontiguousarray(data, dtype=np.complex128)
        s = np.ascontiguousarray(psd, dtype=np.float64)
        f = np.ascontiguousarray(freqs, dtype=np.float64)
        r = np.ascontiguousarray(response, dtype=np.complex128)
        out = ctypes.c_double()
        st = self.lib.gwgpu_maximized_log_likelihood_internal(self.h, _dp(d), _dp(s), _dp(f), _dp(r), f.size,
                                                              ctypes.byref(out))
        self._check(st, "maximized_log_likelihood_internal")
        return out.value

    def maximized_log_likelihood_unaligned_internal(self, data, psd, freqs, hplus, hcross):
        """maximized_Log_Likelihood_unaligned_spin_internal (mcmc_gw.cpp:660-800)."""
        d = np.ascontiguousarray(data, dtype=np.complex128)
        s = np.ascontiguousarray(psd, dtype=np.float64)
        f = np.ascontiguousarray(freqs, dtype=np.float64)
        hp = np.ascontiguousarray(hplus, dtype=np.complex128)
        hc = np.ascontiguousarray(hcross, dtype=np.complex128)
        out = ctypes.c_double()
        st = self.lib.gwgpu_maximized_log_likelihood_unaligned_internal(self.h, _dp(d), _dp(s), _dp(f), _dp(hp),
                                                                        _dp(hc), f.size, ctypes.byref(out))
        self._check(st, "maximized_log_likelihood_unaligned_internal")
        return out.value

    def maximized_loglik_batch(self, params, handles, approximant=IMRPhenomD):
        """The sampler's intrinsic mode over registered data (mcmc_gw.cpp:2611-2720)."""
        parr = params if isinstance(params, ctypes.Array) else params_array(params)
        n = len(parr)
        hs = np.asarray(handles, dtype=np.int32)
        if hs.ndim == 1:
            hs = np.broadcast_to(hs, (n, hs.size))
        hs = np.ascontiguousarray(hs, dtype=np.int32)
        out = np.zeros(n)
        status = np.zeros(n, dtype=np.int32)
        st = self.lib.gwgpu_maximized_loglik_batch(self.h, parr, n, approximant, _ip(hs), hs.shape[1], _dp(out),
                                                   _ip(status))
        self._check(st, "maximized_loglik_batch")
        return out, status

    def mcmc_likelihood_extrinsic(self, params, method, handles, T_segment):
        # the handle array, the method's bytes and the result cell are kept
        # between calls with the same handles and method (a few microseconds
        # of argument conversion per call otherwise)
        key = (tuple(int(h) for h in handles), method)
        c = self.__dict__.get("_plain_args")
        if c is None or c[0] != key:
            hs = np.ascontiguousarray(handles, dtype=np.int32)
            c = (key, hs, _ip(hs), hs.size, method.encode(), ctypes.c_double())
            self._plain_args = c
        _, _, hp, nh, mb, out = c
        st = self.lib.gwgpu_mcmc_likelihood_extrinsic(self.h, ctypes.byref(params), mb, hp, nh, float(T_segment),
                                                      ctypes.byref(out))
        if st not in (0, 4):
            self._check(st, "mcmc_likelihood_extrinsic")
        return out.value

    def _call_arrays(self, approximants, handles, n):
        """The approximant and handle arrays of a call; the common shapes (one
        approximant, handles shared by every request) are kept between calls."""
        cache = self.__dict__.setdefault("_arrays", {})
        akey = ("a", int(approximants), n) if isinstance(approximants, (int, np.integer)) else None
        hkey = (("h", tuple(int(h) for h in handles), n)
                if isinstance(handles, (list, tuple)) or (isinstance(handles, np.ndarray) and handles.ndim == 1)
                else None)
        ap = cache.get(akey) if akey else None
        if ap is None:
            ap = np.ascontiguousarray(np.broadcast_to(np.asarray(approximants, dtype=np.int32), (n,)))
            if akey:
                cache[akey] = ap
        hs = cache.get(hkey) if hkey else None
        if hs is None:
            hs = np.asarray(handles, dtype=np.int32)
            if hs.ndim == 1:
                hs = np.broadcast_to(hs, (n, hs.size))
            hs = np.ascontiguousarray(hs, dtype=np.int32)
            if hkey:
                if len(cache) > 64:
                    cache.clear()
                cache[hkey] = hs
        return ap, hs

    def _call_ptrs(self, approximants, handles, n):
        """(approximants address, handles address, detectors) of a call: the
        arrays of _call_arrays, their addresses kept beside them for the
        common shapes (the address lookup costs a microsecond each)."""
        key = None
        if isinstance(approximants, (int, np.integer)) and isinstance(handles, (list, tuple)):
            key = (int(approximants), tuple(handles), n)
            hit = self.__dict__.get("_ptrs", {}).get(key)
            if hit is not None:
                return hit
        ap, hs = self._call_arrays(approximants, handles, n)
        res = (ap.ctypes.data, hs.ctypes.data, hs.shape[1], ap, hs)
        if key is not None:
            ptrs = self.__dict__.setdefault("_ptrs", {})
            if len(ptrs) > 64:
                ptrs.clear()
            ptrs[key] = res
        return res

    def loglik_batch(self, params, approximants, handles, T_segment, precision=PREC_MIXED):
        """params: GenParams array or list; handles: (ndet,) shared or (n, ndet) per request."""
        parr = params if isinstance(params, ctypes.Array) else params_array(params)
        n = len(parr)
        ap_ptr, hs_ptr, ndet, _, _ = self._call_ptrs(approximants, handles, n)
        # log L (n doubles) then status (n int32) in one allocation: one address lookup
        buf = np.empty(12 * n, dtype=np.uint8)
        base = buf.ctypes.data
        out = buf[:8 * n].view(np.float64)
        status = buf[8 * n:].view(np.int32)
        fn = self.__dict__.get("_lb_raw")
        if fn is None:  # the same entry point with address arguments (no pointer objects per call)
            v = ctypes.c_void_p
            fn = ctypes.CFUNCTYPE(ctypes.c_int, v, v, v, ctypes.c_int, v, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                  v, v)(("gwgpu_loglik_batch", self.lib))
            self._lb_raw = fn
        st = fn(self.h, ctypes.addressof(parr), ap_ptr, n, hs_ptr, ndet, float(T_segment), precision, base,
                base + 8 * n)
        if st:
            self._check(st, "loglik_batch")
        return out, status

    def mcmc_loglik_batch(self, theta, approximant, gmst, handles, T_segment, precision=PREC_MIXED):
        th = np.ascontiguousarray(theta, dtype=np.float64)
        n, dim = th.shape
        hs = np.asarray(handles, dtype=np.int32)
        if hs.ndim == 1:
            hs = np.broadcast_to(hs, (n, hs.size))
        hs = np.ascontiguousarray(hs, dtype=np.int32)
        out = np.zeros(n)
        status = np.zeros(n, dtype=np.int32)
        st = self.lib.gwgpu_mcmc_loglik_batch(self.h, _dp(th), dim, n, approximant, float(gmst), _ip(hs), hs.shape[1],
                                              float(T_segment), precision, _dp(out), _ip(status))
        self._check(st, "mcmc_loglik_batch")
        return out, status

    def set_tile(self, tile):
        self._check(self.lib.gwgpu_batch_set_tile(self.h, int(tile)), "batch_set_tile")

    def set_blocks_per_sm(self, blocks):
        """Launch shape of the mixed fused kernel: 3 or 4 resident blocks per
        SM, 0 for the autotuned or default choice."""
        self._check(self.lib.gwgpu_batch_set_blocks_per_sm(self.h, int(blocks)), "batch_set_blocks_per_sm")

    def last_launch_shape(self):
        """(tile, blocks per SM, grid) of the last batch on the context stream."""
        t, b, g = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self._check(self.lib.gwgpu_batch_last_launch_shape(self.h, ctypes.byref(t), ctypes.byref(b), ctypes.byref(g)),
                    "batch_last_launch_shape")
        return t.value, b.value, g.value

    # --------------------------------------------------------------- Fisher
    def fisher_numerical(self, freqs, method, detector, reference_detector, params, noise, order=2, dimension=11):
        f = np.ascontiguousarray(freqs, dtype=np.float64)
        s = np.ascontiguousarray(noise, dtype=np.float64)
        out = np.zeros(dimension * dimension)
        st = self.lib.gwgpu_fisher_numerical(self.h, _dp(f), f.size, method.encode(), detector.encode(),
                                             reference_detector.encode(), _dp(out), dimension, ctypes.byref(params),
                                             order, _dp(s))
        self._check(st, "fisher_numerical")
        return out.reshape(dimension, dimension)

    def fisher_batch(self, params, method, handles, epsilon=1e-8, step_mode=0, covariance=True):
        parr = params if isinstance(params, ctypes.Array) else params_array(params)
        n = len(parr)
        hs = np.ascontiguousarray(handles, dtype=np.int32)
        dim = 11
        fish = np.zeros((n, dim, dim))
        cov = np.zeros((n, dim, dim)) if covariance else None
        status = np.zeros(n, dtype=np.int32)
        st = self.lib.gwgpu_fisher_batch(self.h, parr, n, method, _ip(hs), hs.size, float(epsilon), int(step_mode),
                                         _dp(fish), _dp(cov) if cov is not None else None, _ip(status))
        self._check(st, "fisher_batch")
        return fish, cov, status

    def fisher_batch_ex(self, params, method, handles, order=2, epsilon=1e-8, step_mode=0, precision=PREC_FP64,
                        add_prior=False, covariance=True, algorithm=FISHER_REFERENCE):
        """fisher_numerical for many sources summed over the detectors of
        handles (the first is the reference detector): FISHER_REFERENCE runs
        the reference algorithm in FP64 (orders 2 and 4), FISHER_MOMENTS the
        moment form (orders 2 and 4) with FP64 (PREC_FP64) or compensated FP32
        (PREC_MIXED) sums."""
        parr = params if isinstance(params, ctypes.Array) else params_array(params)
        n = len(parr)
        hs = np.ascontiguousarray(handles, dtype=np.int32)
        fish = np.zeros((n, 11, 11))
        cov = np.zeros((n, 11, 11)) if covariance else None
        status = np.zeros(n, dtype=np.int32)
        opt = FisherOptions(int(method), int(order), float(epsilon), int(step_mode), int(precision), int(add_prior),
                            int(algorithm))
        st = self.lib.gwgpu_fisher_batch_ex(self.h, parr, n, _ip(hs), hs.size, ctypes.byref(opt), _dp(fish),
                                            _dp(cov) if cov is not None else None, _ip(status))
        self._check(st, "fisher_batch_ex")
        return fish, cov, status

    def mcmc_fisher_batch(self, theta, handles, gmst, approximant=IMRPhenomD):
        """MCMC_fisher_wrapper (mcmc_gw.cpp:2230-2340) at each row of theta (the
        11-dim MCMC_IMRPhenomD vector): the order-4 network Fisher plus the prior
        diagonal."""
        th = np.ascontiguousarray(theta, dtype=np.float64)
        n, dim = th.shape
        hs = np.ascontiguousarray(handles, dtype=np.int32)
        fish = np.zeros((n, dim, dim))
        status = np.zeros(n, dtype=np.int32)
        st = self.lib.gwgpu_mcmc_fisher_batch(self.h, _dp(th), dim, n, int(approximant), float(gmst), _ip(hs), hs.size,
                                              _dp(fish), _ip(status))
        self._check(st, "mcmc_fisher_batch")
        return fish, status


class FisherOptions(ctypes.Structure):
    """gwgpu_fisher_options."""

    _fields_ = [("method", ctypes.c_int), ("order", ctypes.c_int), ("epsilon", ctypes.c_double),
                ("step_mode", ctypes.c_int), ("precision", ctypes.c_int), ("add_prior", ctypes.c_int),
                ("algorithm", ctypes.c_int)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("max_inflight", ctypes.c_int), ("max_batch", ctypes.c_int), ("lanes", ctypes.c_int),
                ("precision", ctypes.c_int), ("T_segment", ctypes.c_double), ("hbm_budget_bytes", ctypes.c_size_t),
                ("device_loop", ctypes.c_int), ("tile", ctypes.c_int), ("idle_us", ctypes.c_int),
                ("blocks_per_sm", ctypes.c_int)]


class Server:
    """Continuous-batching log-likelihood server on a Context (serve.cu).

    device_loop=True: the device-resident request loop (one persistent kernel
    consuming a mapped ring; mixed precision), with `tile` bins per item, its
    blocks leaving after `idle_us` without work, and `blocks_per_sm` of them
    on each SM (0: as many as fit)."""

    def __init__(self, ctx, T_segment, max_inflight=8192, max_batch=1024, lanes=4, precision=PREC_MIXED,
                 hbm_budget=0, device_loop=False, tile=0, idle_us=0, blocks_per_sm=0):
        self.ctx = ctx
        self.lib = ctx.lib
        cfg = ServerConfig(max_inflight, max_batch, lanes, precision, float(T_segment), hbm_budget,
                           1 if device_loop else 0, tile, idle_us, blocks_per_sm)
        h = ctypes.c_void_p()
        ctx._check(self.lib.gwgpu_server_create(ctx.h, ctypes.byref(cfg), ctypes.byref(h)), "server_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.gwgpu_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, params, approximant, handles):
        hs = np.ascontiguousarray(handles, dtype=np.int32)
        t = ctypes.c_uint64()
        st = self.lib.gwgpu_server_submit(self.h, ctypes.byref(params), approximant, _ip(hs), hs.size, ctypes.byref(t))
        if st != 0:
            raise GwGpuError("server_submit: %s" % STATUS.get(st, st))
        return t.value

    def poll(self, ticket):
        ll = ctypes.c_double()
        s = ctypes.c_int()
        st = self.lib.gwgpu_server_poll(self.h, ticket, ctypes.byref(ll), ctypes.byref(s))
        if st == 6:
            return None
        if st != 0:
            raise GwGpuError("server_poll: %s" % STATUS.get(st, st))
        return ll.value, s.value

    def wait(self, ticket, timeout_ms=10000):
        ll = ctypes.c_double()
        s = ctypes.c_int()
        st = self.lib.gwgpu_server_wait(self.h, ticket, timeout_ms, ctypes.byref(ll), ctypes.byref(s))
        if st != 0:
            raise GwGpuError("server_wait: %s" % STATUS.get(st, st))
        return ll.value, s.value

    def stats(self):
        p50 = ctypes.c_double()
        p99 = ctypes.c_double()
        done = ctypes.c_uint64()
        launches = ctypes.c_uint64()
        self.lib.gwgpu_server_stats(self.h, ctypes.byref(p50), ctypes.byref(p99), ctypes.byref(done),
                                    ctypes.byref(launches))
        return dict(p50_s=p50.value, p99_s=p99.value, completed=done.value, launches=launches.value)

    def reset_stats(self):
        self.lib.gwgpu_server_reset_stats(self.h)

    def loop_info(self):
        """Device loop: ring slots, tile, items per request, blocks, launches, the
        blocks of finished launches that left idle / on stop / at end of life,
        and the device service time percentiles (claim -> result, ns)."""
        info = (ctypes.c_longlong * 15)()
        st = self.lib.gwgpu_server_loop_info(self.h, info)
        if st != 0:
            raise GwGpuError("server_loop_info: %s" % STATUS.get(st, st))
        keys = ("ring_slots", "tile", "max_items", "blocks", "launches", "exits_idle", "exits_stop", "exits_life",
                "service_p50_ns", "service_p99_ns", "busy_item_ns", "busy_prologue_ns", "items", "prologue_claims",
                "requests_claimed")
        return dict(zip(keys, list(info)))

    def drive(self, params, approximants, handles, arrival_s):
        """Open-loop load: request i submitted at t0 + arrival_s[i] (native thread)."""
        parr = params if isinstance(params, ctypes.Array) else params_array(params)
        n = len(parr)
        ap = np.ascontiguousarray(np.broadcast_to(np.asarray(approximants, dtype=np.int32), (n,)))
        hs = np.asarray(handles, dtype=np.int32)
        if hs.ndim == 1:
            hs = np.broadcast_to(hs, (n, hs.size))
        hs = np.ascontiguousarray(hs, dtype=np.int32)
        arr = np.ascontiguousarray(arrival_s, dtype=np.float64)
        out = np.zeros(n)
        status = np.zeros(n, dtype=np.int32)
        lat = np.zeros(n)
        wall = ctypes.c_double()
        st = self.lib.gwgpu_server_drive(self.h, parr, _ip(ap), _ip(hs), hs.shape[1], _dp(arr), n, _dp(out),
                                         _ip(status), _dp(lat), ctypes.byref(wall))
        if st != 0:
            raise GwGpuError("server_drive: %s" % STATUS.get(st, st))
        return out, status, lat, wall.value


def _ctx_batch_device(self, d_params_ptr, d_approx_ptr, n, handles, T_segment, precision, d_out_ptr, d_status_ptr,
                      stream=None):
    """gwgpu_loglik_batch_device on raw device pointers (e.g. torch tensors' data_ptr())."""
    _, hs_ptr, ndet, _, _ = self._call_ptrs(0, handles, n)
    fn = self.__dict__.get("_lbd_raw")
    if fn is None:  # the entry point with address arguments
        v = ctypes.c_void_p
        fn = ctypes.CFUNCTYPE(ctypes.c_int, v, v, v, ctypes.c_int, v, ctypes.c_int, ctypes.c_double, ctypes.c_int, v, v,
                              v)(("gwgpu_loglik_batch_device", self.lib))
        self._lbd_raw = fn
    st = fn(self.h, d_params_ptr, d_approx_ptr, n, hs_ptr, ndet, float(T_segment), precision, d_out_ptr, d_status_ptr,
            stream)
    if st:
        self._check(st, "loglik_batch_device")


def _ctx_autotune(self, d_params_ptr, d_approx_ptr, n, handles, T_segment, precision, d_out_ptr, d_status_ptr):
    hs = np.ascontiguousarray(handles, dtype=np.int32)
    ndet = hs.size if hs.ndim == 1 else hs.shape[1]
    if hs.ndim == 1:
        hs = np.ascontiguousarray(np.broadcast_to(hs, (n, ndet)))
    tile = ctypes.c_int()
    ms = ctypes.c_float()
    st = self.lib.gwgpu_batch_autotune(self.h, d_params_ptr, d_approx_ptr, n, _ip(hs), ndet, float(T_segment),
                                       precision, d_out_ptr, d_status_ptr, ctypes.byref(tile), ctypes.byref(ms))
    self._check(st, "batch_autotune")
    return tile.value, ms.value


def _ctx_use_graphs(self, on):
    self._check(self.lib.gwgpu_batch_use_graphs(self.h, int(bool(on))), "batch_use_graphs")


Context.loglik_batch_device = _ctx_batch_device
Context.autotune = _ctx_autotune
Context.use_graphs = _ctx_use_graphs
