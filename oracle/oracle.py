"""ctypes front end of the FP64 C oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, the smoke check in __graft_entry__.py and the CPU-baseline leg of
bench.py import this module.  It exposes the C restatement of the reference's
likelihood path (oracle/gwat_oracle.c) and, where it was built, the reference
pin library oracle/_ref/libgwatref.so (the reference's own IMRPhenomD.cpp /
IMRPhenomP.cpp compiled against shim headers).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
IMRPhenomD = 0
IMRPhenomPv2 = 1

DETECTORS = ["Hanford", "Livingston", "Virgo", "Kagra", "Indigo", "CE", "ET1", "ET2", "ET3"]


class GenParams(ctypes.Structure):
    """Mirror of gwo_gen_params (oracle/gwat_oracle.h)."""

    _fields_ = [
        ("mass1", ctypes.c_double), ("mass2", ctypes.c_double),
        ("spin1", ctypes.c_double * 3), ("spin2", ctypes.c_double * 3),
        ("Luminosity_Distance", ctypes.c_double),
        ("incl_angle", ctypes.c_double), ("phiRef", ctypes.c_double),
        ("f_ref", ctypes.c_double), ("tc", ctypes.c_double),
        ("RA", ctypes.c_double), ("DEC", ctypes.c_double),
        ("psi", ctypes.c_double), ("gmst", ctypes.c_double),
        ("chip", ctypes.c_double), ("phip", ctypes.c_double),
        ("shift_time", ctypes.c_int), ("shift_phase", ctypes.c_int),
        ("sky_average", ctypes.c_int), ("dep_postmerger", ctypes.c_int),
        ("theta_l", ctypes.c_double), ("phi_l", ctypes.c_double),
        ("equatorial_orientation", ctypes.c_int), ("reserved", ctypes.c_int),
    ]


def make_params(**kw):
    p = GenParams()
    p.chip = -1.0
    p.phip = -1.0
    p.shift_time = 1
    p.shift_phase = 1
    for k, v in kw.items():
        if k in ("spin1", "spin2"):
            getattr(p, k)[:] = list(v)
        else:
            setattr(p, k, v)
    return p


def params_from_dict(d):
    return make_params(**d)


_lib = None
_ref = None


def reference_dir():
    """The reference checkout: GWAT_REFERENCE_DIR, else the one the pin
    libraries were last built from (oracle/_ref/source_dir.txt); None where
    neither exists on this machine."""
    d = os.environ.get("GWAT_REFERENCE_DIR")
    if not d:
        rec = os.path.join(HERE, "_ref", "source_dir.txt")
        d = open(rec).read().strip() if os.path.exists(rec) else None
    return d if d and os.path.isdir(os.path.join(d, "src")) else None


def build(ref_dir=None):
    """Compile liboracle.so (and the reference pin libraries if ref_dir exists)."""
    subprocess.check_call(["make", "-s", "-C", HERE, "liboracle.so"])
    if ref_dir and os.path.isdir(os.path.join(ref_dir, "src")):
        jobs = "-j%d" % max(1, min(16, os.cpu_count() or 1))
        subprocess.check_call(["make", "-s", "-C", HERE, jobs, "ref", "full", "REF=" + ref_dir])
        with open(os.path.join(HERE, "_ref", "source_dir.txt"), "w") as fh:
            fh.write(os.path.abspath(ref_dir) + "\n")


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        gp = ctypes.POINTER(GenParams)
        L.gwo_fourier_waveform.argtypes = [dp, ctypes.c_int, dp, dp, ctypes.c_int, gp]
        L.gwo_fourier_detector_response.argtypes = [dp, ctypes.c_int, dp, ctypes.c_int, ctypes.c_int, gp]
        L.gwo_antenna.argtypes = [ctypes.c_int] + [ctypes.c_double] * 4 + [dp, dp]
        L.gwo_dtoa.argtypes = [ctypes.c_double] * 3 + [ctypes.c_int] * 2
        L.gwo_dtoa.restype = ctypes.c_double
        L.gwo_log_likelihood_internal.argtypes = [dp, dp, dp, dp, ctypes.c_int]
        L.gwo_log_likelihood_internal.restype = ctypes.c_double
        L.gwo_loglik_extrinsic.argtypes = [gp, ctypes.c_int, ctypes.c_double, dp, ctypes.c_int, ctypes.c_int, ip,
                                           ctypes.POINTER(dp), ctypes.POINTER(dp)]
        L.gwo_loglik_extrinsic.restype = ctypes.c_double
        L.gwo_log_likelihood_internal_gl.argtypes = [dp, dp, dp, dp, dp, ctypes.c_int, ctypes.c_int]
        L.gwo_log_likelihood_internal_gl.restype = ctypes.c_double
        L.gwo_loglik_extrinsic_gl.argtypes = [gp, ctypes.c_int, ctypes.c_double, dp, ctypes.c_int, ctypes.c_int, ip,
                                              ctypes.POINTER(dp), ctypes.POINTER(dp), ctypes.POINTER(dp),
                                              ctypes.c_int]
        L.gwo_loglik_extrinsic_gl.restype = ctypes.c_double
        L.gwo_loglik_batch.argtypes = [gp, ctypes.c_int, ip, ctypes.c_double, dp, ctypes.c_int, ctypes.c_int, ip,
                                       ctypes.POINTER(dp), ctypes.POINTER(dp), dp, ctypes.c_int]
        L.gwo_mcmc_repack.argtypes = [dp, ctypes.c_int, ctypes.c_int, ctypes.c_double, gp]
        L.gwo_fisher_numerical.argtypes = [dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, gp,
                                           ctypes.c_int, dp, ctypes.c_double, ctypes.c_int]
        L.gwo_fisher_numerical.restype = ctypes.c_int
        L.gwo_fisher_network.argtypes = [dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ip, dp, gp, ctypes.c_int,
                                         ctypes.POINTER(dp), ctypes.c_double, ctypes.c_int]
        L.gwo_fisher_batch.argtypes = [gp, ctypes.c_int, dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ip,
                                       ctypes.POINTER(dp), ctypes.c_double, ctypes.c_int, dp, ctypes.c_int]
        L.gwo_cholesky_invert.argtypes = [dp, dp, ctypes.c_int]
        L.gwo_cholesky_invert.restype = ctypes.c_int
        L.gwo_transform_orientation_coords.argtypes = [gp, ctypes.c_int]
        L.gwo_analytic_psd.argtypes = [ctypes.c_double]
        L.gwo_analytic_psd.restype = ctypes.c_double
        L.gwo_cspline_coeffs.argtypes = [dp, dp, ctypes.c_int, dp]
        L.gwo_cspline_eval.argtypes = [dp, dp, dp, ctypes.c_int, ctypes.c_double, ctypes.c_int]
        L.gwo_cspline_eval.restype = ctypes.c_double
        _lib = L
    return _lib


def ref_lib():
    """The reference pin library, or None where it was not built."""
    global _ref
    if _ref is None:
        path = os.path.join(HERE, "_ref", "libgwatref.so")
        if not os.path.exists(path):
            return None
        L = ctypes.CDLL(path)
        dp = ctypes.POINTER(ctypes.c_double)
        L.ref_fourier_waveform.argtypes = [dp, ctypes.c_int, dp, dp, ctypes.c_int, ctypes.POINTER(GenParams)]
        _ref = L
    return _ref


_ref_full = None


def ref_full_lib():
    """The reference's own glue (oracle/_ref/libgwatref_full.so), or None where
    it was not built."""
    global _ref_full
    if _ref_full is None:
        path = os.path.join(HERE, "_ref", "libgwatref_full.so")
        if not os.path.exists(path):
            return None
        L = ctypes.CDLL(path)
        dp = ctypes.POINTER(ctypes.c_double)
        pdp = ctypes.POINTER(dp)
        ip = ctypes.POINTER(ctypes.c_int)
        gp = ctypes.POINTER(GenParams)
        cpp = ctypes.POINTER(ctypes.c_char_p)
        c, d, i = ctypes.c_char_p, ctypes.c_double, ctypes.c_int
        L.gwr_fourier_waveform.argtypes = [dp, i, dp, dp, c, gp]
        L.gwr_fourier_detector_response.argtypes = [dp, i, dp, c, c, gp, gp]
        L.gwr_transform_orientation_coords.argtypes = [gp, c, c, gp]
        L.gwr_antenna.argtypes = [c, d, d, d, d, dp, dp]
        L.gwr_dtoa.argtypes = [d, d, d, c, c]
        L.gwr_dtoa.restype = d
        L.gwr_log_likelihood_internal.argtypes = [dp, dp, dp, dp, dp, i, i, c]
        L.gwr_log_likelihood_internal.restype = d
        L.gwr_mcmc_likelihood_extrinsic.argtypes = [gp, c, ip, pdp, pdp, pdp, pdp, c, i, cpp, i, dp, dp]
        L.gwr_mcmc_likelihood_extrinsic.restype = d
        L.gwr_fisher_numerical.argtypes = [dp, i, c, c, c, dp, i, gp, i, dp]
        L.gwr_maximized_aligned.argtypes = [dp, dp, dp, dp, i]
        L.gwr_maximized_aligned.restype = d
        L.gwr_maximized_unaligned.argtypes = [dp, dp, dp, dp, dp, i]
        L.gwr_maximized_unaligned.restype = d
        L.gwr_gps_to_gmst_radian.argtypes = [d]
        L.gwr_gps_to_gmst_radian.restype = d
        L.gwr_sampler_eval.argtypes = [c, i, i, cpp, pdp, pdp, pdp, ip, d, i, dp, dp, dp, i]
        L.gwr_sampler_eval.restype = d
        _ref_full = L
    return _ref_full


APPROX_NAMES = {IMRPhenomD: "IMRPhenomD", IMRPhenomPv2: "IMRPhenomPv2"}


def _cstrs(names):
    return (ctypes.c_char_p * len(names))(*[n.encode() for n in names])


def ref_fourier_waveform(freqs, params, method="IMRPhenomD"):
    """The reference's fourier_waveform (waveform_generator.cpp:104)."""
    freqs = np.ascontiguousarray(freqs, dtype=np.float64)
    hp = np.zeros(freqs.size, dtype=np.complex128)
    hc = np.zeros(freqs.size, dtype=np.complex128)
    ref_full_lib().gwr_fourier_waveform(_dp(freqs), freqs.size, _dp(hp), _dp(hc), method.encode(),
                                        ctypes.byref(params))
    return hp, hc


def ref_detector_response(freqs, params, detector, method="IMRPhenomD"):
    """The reference's fourier_detector_response (waveform_util.cpp:1070);
    returns the response and the parameters as the call left them."""
    freqs = np.ascontiguousarray(freqs, dtype=np.float64)
    r = np.zeros(freqs.size, dtype=np.complex128)
    after = GenParams()
    ref_full_lib().gwr_fourier_detector_response(_dp(freqs), freqs.size, _dp(r), detector.encode(), method.encode(),
                                                 ctypes.byref(params), ctypes.byref(after))
    return r, after


def ref_transform_orientation_coords(params, method="IMRPhenomD", detector="Hanford"):
    out = GenParams()
    ref_full_lib().gwr_transform_orientation_coords(ctypes.byref(params), method.encode(), detector.encode(),
                                                    ctypes.byref(out))
    return out


def ref_antenna(detector, ra, dec, psi, gmst):
    fp, fc = ctypes.c_double(), ctypes.c_double()
    ref_full_lib().gwr_antenna(detector.encode(), ra, dec, psi, gmst, ctypes.byref(fp), ctypes.byref(fc))
    return fp.value, fc.value


def ref_dtoa(ra, dec, gmst, det1, det2):
    return ref_full_lib().gwr_dtoa(ra, dec, gmst, det1.encode(), det2.encode())


def ref_log_likelihood_internal(data, psd, freqs, response, weights=None, log10F=False):
    data = np.ascontiguousarray(data, dtype=np.complex128)
    psd = np.ascontiguousarray(psd, dtype=np.float64)
    freqs = np.ascontiguousarray(freqs, dtype=np.float64)
    response = np.ascontiguousarray(response, dtype=np.complex128)
    w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float64)
    return ref_full_lib().gwr_log_likelihood_internal(_dp(data), _dp(psd), _dp(freqs),
                                                      None if w is None else _dp(w), _dp(response), freqs.size,
                                                      int(log10F), b"SIMPSONS" if w is None else b"GAUSSLEG")


def ref_mcmc_likelihood_extrinsic(params, freqs, detectors, data, psd, method="IMRPhenomD", weights=None,
                                  log10F=False):
    """The reference's MCMC_likelihood_extrinsic (mcmc_gw.cpp:2374) with every
    detector on the grid freqs.  The detectors' frequency arrays are copies laid
    out back to back, so the T the reference forms from frequencies[1] -
    frequencies[0] (a pointer difference, mcmc_gw.cpp:2466) is 1/len(freqs).
    Returns (log L, T used, t_c as the call left it)."""
    freqs = np.ascontiguousarray(freqs, dtype=np.float64)
    n, nd = freqs.size, len(detectors)
    block = np.ascontiguousarray(np.tile(freqs, nd))
    fptrs = (ctypes.POINTER(ctypes.c_double) * nd)(
        *[ctypes.cast(block.ctypes.data + 8 * n * k, ctypes.POINTER(ctypes.c_double)) for k in range(nd)])
    data = [np.ascontiguousarray(x, dtype=np.complex128) for x in data]
    psd = [np.ascontiguousarray(x, dtype=np.float64) for x in psd]
    ws = [None] * nd if weights is None else [np.ascontiguousarray(x, dtype=np.float64) for x in weights]
    wptr = (ctypes.POINTER(ctypes.c_double) * nd)(*[None if w is None else _dp(w) for w in ws])
    lengths = (ctypes.c_int * nd)(*([n] * nd))
    T, tc = ctypes.c_double(), ctypes.c_double()
    ll = ref_full_lib().gwr_mcmc_likelihood_extrinsic(
        ctypes.byref(params), method.encode(), lengths, fptrs, _ptr_array(data), _ptr_array(psd), wptr,
        b"SIMPSONS" if weights is None else b"GAUSSLEG", int(log10F), _cstrs(detectors), nd, ctypes.byref(T),
        ctypes.byref(tc))
    return ll, T.value, tc.value


def ref_fisher_numerical(freqs, params, detector, ref_detector, psd, method="IMRPhenomD", order=2, dim=11):
    freqs = np.ascontiguousarray(freqs, dtype=np.float64)
    psd = np.ascontiguousarray(psd, dtype=np.float64)
    out = np.zeros(dim * dim)
    ref_full_lib().gwr_fisher_numerical(_dp(freqs), freqs.size, method.encode(), detector.encode(),
                                        ref_detector.encode(), _dp(out), dim, ctypes.byref(params), order, _dp(psd))
    return out.reshape(dim, dim)


def ref_maximized_loglik(data, psd, freqs, hplus, hcross=None):
    """The reference's maximised likelihoods (mcmc_gw.cpp:595-800), its FFTW
    calls answered by a direct DFT (oracle/ref_fftw.cpp)."""
    data = np.ascontiguousarray(data, dtype=np.complex128)
    psd = np.ascontiguousarray(psd, dtype=np.float64)
    freqs = np.ascontiguousarray(freqs, dtype=np.float64)
    hp = np.ascontiguousarray(hplus, dtype=np.complex128)
    L = ref_full_lib()
    if hcross is None:
        return L.gwr_maximized_aligned(_dp(data), _dp(psd), _dp(freqs), _dp(hp), freqs.size)
    hc = np.ascontiguousarray(hcross, dtype=np.complex128)
    return L.gwr_maximized_unaligned(_dp(data), _dp(psd), _dp(freqs), _dp(hp), _dp(hc), freqs.size)


def ref_gps_to_gmst(gps):
    return ref_full_lib().gwr_gps_to_gmst_radian(gps)


def ref_sampler_eval(method, positions, freqs, detectors, data, psd, gps_time, fisher=False, nthreads=1):
    """MCMC_likelihood_wrapper (and MCMC_fisher_wrapper) of the reference at
    each row of positions, after the reference's own sampler set-up
    (PTMCMC_MH_dynamic_PT_alloc_uncorrelated_GW, mcmc_gw.cpp:1422) with the
    detectors' frequency arrays laid out back to back (so the T of
    mcmc_gw.cpp:2466 is 1/len(freqs)).  Returns (log L, Fisher or None,
    seconds)."""
    positions = np.ascontiguousarray(positions, dtype=np.float64)
    npos, dim = positions.shape
    freqs = np.ascontiguousarray(freqs, dtype=np.float64)
    n, nd = freqs.size, len(detectors)
    block = np.ascontiguousarray(np.tile(freqs, nd))
    fptrs = (ctypes.POINTER(ctypes.c_double) * nd)(
        *[ctypes.cast(block.ctypes.data + 8 * n * k, ctypes.POINTER(ctypes.c_double)) for k in range(nd)])
    data = [np.ascontiguousarray(x, dtype=np.complex128) for x in data]
    psd = [np.ascontiguousarray(x, dtype=np.float64) for x in psd]
    lengths = (ctypes.c_int * nd)(*([n] * nd))
    ll = np.zeros(npos)
    fo = np.zeros(npos * dim * dim) if fisher else None
    secs = ref_full_lib().gwr_sampler_eval(method.encode(), dim, nd, _cstrs(detectors), fptrs, _ptr_array(data),
                                           _ptr_array(psd), lengths, gps_time, npos, _dp(positions), _dp(ll),
                                           None if fo is None else _dp(fo), nthreads)
    return ll, (None if fo is None else fo.reshape(npos, dim, dim)), secs


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def fourier_waveform(freqs, params, approximant=IMRPhenomD, use_ref=False):
    freqs = np.ascontiguousarray(freqs, dtype=np.float64)
    n = freqs.size
    hp = np.zeros(n, dtype=np.complex128)
    hc = np.zeros(n, dtype=np.complex128)
    L = ref_lib() if use_ref else lib()
    fn = L.ref_fourier_waveform if use_ref else L.gwo_fourier_waveform
    fn(_dp(freqs), n, _dp(hp), _dp(hc), approximant, ctypes.byref(params))
    return hp, hc


def detector_index(name):
    return DETECTORS.index(name)


def detector_response(freqs, params, detector, approximant=IMRPhenomD):
    freqs = np.ascontiguousarray(freqs, dtype=np.float64)
    r = np.zeros(freqs.size, dtype=np.complex128)
    lib().gwo_fourier_detector_response(_dp(freqs), freqs.size, _dp(r), detector_index(detector), approximant,
                                        ctypes.byref(params))
    return r


def transform_orientation_coords(params, approximant=IMRPhenomD):
    """A copy of params with incl_angle and psi from theta_l, phi_l
    (transform_orientation_coords, waveform_util.cpp:1523-1586)."""
    out = GenParams()
    ctypes.pointer(out)[0] = params
    lib().gwo_transform_orientation_coords(ctypes.byref(out), approximant)
    return out


def antenna(detector, ra, dec, psi, gmst):
    fp = ctypes.c_double()
    fc = ctypes.c_double()
    lib().gwo_antenna(detector_index(detector), ra, dec, psi, gmst, ctypes.byref(fp), ctypes.byref(fc))
    return fp.value, fc.value


def dtoa(ra, dec, gmst, det1, det2):
    return lib().gwo_dtoa(ra, dec, gmst, detector_index(det1), detector_index(det2))


def analytic_psd(freqs):
    return np.array([lib().gwo_analytic_psd(float(f)) for f in np.atleast_1d(freqs)])


def _ptr_array(arrs):
    arr_t = ctypes.POINTER(ctypes.c_double) * len(arrs)
    return arr_t(*[_dp(a) for a in arrs])


def loglik(params, freqs, detectors, data, psd, approximant=IMRPhenomD, T_segment=None):
    """MCMC_likelihood_extrinsic for one request (all detectors on one grid)."""
    freqs = np.ascontiguousarray(freqs, dtype=np.float64)
    if T_segment is None:
        T_segment = 1.0 / (freqs[1] - freqs[0])
    dets = (ctypes.c_int * len(detectors))(*[detector_index(d) for d in detectors])
    data = [np.ascontiguousarray(d, dtype=np.complex128) for d in data]
    psd = [np.ascontiguousarray(s, dtype=np.float64) for s in psd]
    return lib().gwo_loglik_extrinsic(ctypes.byref(params), approximant, T_segment, _dp(freqs), freqs.size,
                                      len(detectors), dets, _ptr_array(data), _ptr_array(psd))


def loglik_gl(params, freqs, detectors, data, psd, weights, log10F=False, approximant=IMRPhenomD, T_segment=1.0):
    """MCMC_likelihood_extrinsic with GAUSSLEG integration (weights per detector)."""
    freqs = np.ascontiguousarray(freqs, dtype=np.float64)
    dets = (ctypes.c_int * len(detectors))(*[detector_index(d) for d in detectors])
    data = [np.ascontiguousarray(d, dtype=np.complex128) for d in data]
    psd = [np.ascontiguousarray(s, dtype=np.float64) for s in psd]
    weights = [np.ascontiguousarray(w, dtype=np.float64) for w in weights]
    return lib().gwo_loglik_extrinsic_gl(ctypes.byref(params), approximant, T_segment, _dp(freqs), freqs.size,
                                         len(detectors), dets, _ptr_array(data), _ptr_array(psd),
                                         _ptr_array(weights), int(log10F))


def simpsons_sum(delta_x, x):
    """util.h:844-856: (dx/3)[x0 + 4x1 + 2x2 + ... + x_{N-1}], the odd/even
    pattern applied for any N."""
    x = np.asarray(x, dtype=np.float64)
    w = np.where(np.arange(x.size) % 2 == 0, 2.0, 4.0)
    w[0] = w[-1] = 1.0
    return float(np.sum(w * x) * delta_x / 3)


def maximized_loglik_internal(data, psd, freqs, response):
    """maximized_Log_Likelihood_aligned_spin_internal (mcmc_gw.cpp:595-658),
    with numpy's DFT in place of FFTW's."""
    freqs = np.asarray(freqs, dtype=np.float64)
    n = freqs.size
    delta_f = freqs[1] - freqs[0]
    hh = 4.0 * simpsons_sum(delta_f, (response * np.conj(response)).real / psd)
    g = 4.0 * np.conj(data) * response / psd
    G = np.fft.fft(g)
    return 0.5 * np.max(G.real ** 2 + G.imag ** 2) * delta_f * delta_f / hh


def maximized_loglik_unaligned_internal(data, psd, freqs, hplus, hcross):
    """maximized_Log_Likelihood_unaligned_spin_internal (mcmc_gw.cpp:660-800),
    with numpy's DFT in place of FFTW's."""
    freqs = np.asarray(freqs, dtype=np.float64)
    delta_f = freqs[1] - freqs[0]
    hp_root = np.sqrt(4.0 * simpsons_sum(delta_f, (hplus * np.conj(hplus)).real / psd))
    hc_root = np.sqrt(4.0 * simpsons_sum(delta_f, (hcross * np.conj(hcross)).real / psd))
    hpn = hplus / hp_root
    hcn = hcross / hc_root
    rho_p = delta_f * np.fft.fft(4.0 * np.conj(data) * hpn / psd)
    rho_c = delta_f * np.fft.fft(4.0 * np.conj(data) * hcn / psd)
    rp2 = rho_p.real ** 2 + rho_p.imag ** 2
    rc2 = rho_c.real ** 2 + rho_c.imag ** 2
    gam = (rho_p * np.conj(rho_c)).real
    ipc = 4.0 * simpsons_sum(delta_f, (hpn * np.conj(hcn)).real / psd)
    lam = (rp2 + rc2 - 2 * gam * ipc + np.sqrt((rp2 - rc2) ** 2 + 4.0 * (ipc * rp2 - gam) * (ipc * rc2 - gam))) \
        / (1.0 - ipc * ipc)
    return 0.25 * np.max(lam)


def maximized_loglik_intrinsic(params_dict, freqs, data_list, psd_list, approximant=IMRPhenomD):
    """The sampler's intrinsic mode (mcmc_gw.cpp:2611-2720): the waveform with
    the extrinsic parameters fixed (horizon frame theta = phi = psi = 0,
    inclination 0: F+ = 1, Fx = 0; f_ref 10 for IMRPhenomD, 20 for
    IMRPhenomPv2), summed over detectors; IMRPhenomD uses the aligned form with
    r = h+, IMRPhenomPv2 the unaligned form with h+ and hx."""
    d = dict(params_dict, RA=0.0, DEC=0.0, psi=0.0, phiRef=1.0, incl_angle=0.0, tc=1.0,
             f_ref=20.0 if approximant == IMRPhenomPv2 else 10.0)
    hp, hc = fourier_waveform(freqs, params_from_dict(d), approximant)
    if approximant == IMRPhenomPv2:
        return sum(maximized_loglik_unaligned_internal(dd, s, freqs, hp, hc) for dd, s in zip(data_list, psd_list))
    return sum(maximized_loglik_internal(dd, s, freqs, hp) for dd, s in zip(data_list, psd_list))


def loglik_batch(params_list, freqs, detectors, data, psd, approximants=None, T_segment=None, nthreads=0):
    freqs = np.ascontiguousarray(freqs, dtype=np.float64)
    if T_segment is None:
        T_segment = 1.0 / (freqs[1] - freqs[0])
    n = len(params_list)
    parr = (GenParams * n)(*params_list)
    if approximants is None:
        approximants = [IMRPhenomD] * n
    aarr = (ctypes.c_int * n)(*approximants)
    dets = (ctypes.c_int * len(detectors))(*[detector_index(d) for d in detectors])
    data = [np.ascontiguousarray(d, dtype=np.complex128) for d in data]
    psd = [np.ascontiguousarray(s, dtype=np.float64) for s in psd]
    out = np.zeros(n)
    lib().gwo_loglik_batch(parr, n, aarr, T_segment, _dp(freqs), freqs.size, len(detectors), dets,
                           _ptr_array(data), _ptr_array(psd), _dp(out), nthreads)
    return out


def mcmc_repack(theta, approximant=IMRPhenomD, gmst=0.0):
    theta = np.ascontiguousarray(theta, dtype=np.float64)
    p = GenParams()
    lib().gwo_mcmc_repack(_dp(theta), theta.size, approximant, gmst, ctypes.byref(p))
    return p


FISHER_METHODS = {"IMRPhenomD": 0, "MCMC_IMRPhenomD": 1, "IMRPhenomPv2": 2, "MCMC_IMRPhenomPv2": 3}


def fisher_numerical(freqs, params, detector, ref_detector, psd, method="IMRPhenomD", order=2,
                     epsilon=1e-8, step_mode=0):
    freqs = np.ascontiguousarray(freqs, dtype=np.float64)
    psd = np.ascontiguousarray(psd, dtype=np.float64)
    out = np.zeros(15 * 15)
    dim = lib().gwo_fisher_numerical(_dp(freqs), freqs.size, FISHER_METHODS[method], detector_index(detector),
                                     detector_index(ref_detector), _dp(out), ctypes.byref(params), order, _dp(psd),
                                     epsilon, step_mode)
    return out[:dim * dim].reshape(dim, dim)


def fisher_network(freqs, params, detectors, psds, method="IMRPhenomD", order=2, epsilon=1e-8, step_mode=0):
    freqs = np.ascontiguousarray(freqs, dtype=np.float64)
    psds = [np.ascontiguousarray(s, dtype=np.float64) for s in psds]
    dets = (ctypes.c_int * len(detectors))(*[detector_index(d) for d in detectors])
    out = np.zeros(15 * 15)
    lib().gwo_fisher_network(_dp(freqs), freqs.size, FISHER_METHODS[method], len(detectors), dets, _dp(out),
                             ctypes.byref(params), order, _ptr_array(psds), epsilon, step_mode)
    dim = 11 if method in ("IMRPhenomD", "MCMC_IMRPhenomD") else (13 if method == "IMRPhenomPv2" else 15)
    return out[:dim * dim].reshape(dim, dim)


def fisher_batch(params_list, freqs, detectors, psds, method="IMRPhenomD", epsilon=1e-8, step_mode=0,
                 nthreads=0):
    freqs = np.ascontiguousarray(freqs, dtype=np.float64)
    psds = [np.ascontiguousarray(s, dtype=np.float64) for s in psds]
    n = len(params_list)
    parr = (GenParams * n)(*params_list)
    dets = (ctypes.c_int * len(detectors))(*[detector_index(d) for d in detectors])
    dim = 11 if method in ("IMRPhenomD", "MCMC_IMRPhenomD") else (13 if method == "IMRPhenomPv2" else 15)
    out = np.zeros(n * dim * dim)
    lib().gwo_fisher_batch(parr, n, _dp(freqs), freqs.size, FISHER_METHODS[method], len(detectors), dets,
                           _ptr_array(psds), epsilon, step_mode, _dp(out), nthreads)
    return out.reshape(n, dim, dim)


def mcmc_fisher_prior_diag(dim=11):
    """The diagonal MCMC_fisher_transformations adds to a non-intrinsic
    sampler's Fisher matrix (mcmc_gw.cpp:2136-2160): RA, sin DEC, psi,
    cos iota, phiRef, tc, eta, the two aligned spins, and for the 15-dim
    precessing vector cos theta1, cos theta2, phi1, phi2; nothing on
    ln D_L and ln Mc."""
    tp = 1.0 / (4 * np.pi * np.pi)
    d = [tp, 1 / 4., tp, 1 / 4., tp, 1 / .01, 0.0, 0.0, 1 / .25, 1 / 4., 1 / 4.]
    if dim == 15:
        d += [1 / 4., 1 / 4., tp, tp]
    return np.array(d[:dim])


def cholesky_invert(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    inv = np.zeros_like(a)
    st = lib().gwo_cholesky_invert(_dp(a), _dp(inv), a.shape[0])
    return st, inv
