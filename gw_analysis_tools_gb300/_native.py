"""Build and load the CUDA library libgwgpu.so (sm_103a) in-tree.

The library is the product: there is no CPU fallback.  load() raises when the
library is missing or no CUDA device is usable.
"""
import ctypes
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
BUILDDIR = os.path.join(HERE, "_build")
LIB = os.path.join(LIBDIR, "libgwgpu.so")
DROPIN_SRC = os.path.join(HERE, "dropin", "gwat_dropin.cpp")
DROPIN_LIB = os.path.join(LIBDIR, "libgwat_dropin.so")
SOURCES = ["kernels.cu", "capi.cu", "batch.cu", "fisher.cu", "fisher_ref.cu", "serve.cu", "noalloc.cu", "maxll.cu", "cufft_rt.cu", "ingest.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no multiply-add contraction, so that it rounds the same on x86 and Arm hosts
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off", "--expt-relaxed-constexpr"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(os.path.dirname(HERE), "include", "gwgpu.h"))
    return hs


def build(force=False, verbose=False):
    """Compile every CUDA translation unit for sm_103a and link libgwgpu.so."""
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(BUILDDIR, exist_ok=True)
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    hdr_mtime = max(os.path.getmtime(h) for h in _headers())
    nvcc = _nvcc()

    def compile_one(src):
        obj = os.path.join(BUILDDIR, src.replace(".cu", ".o"))
        srcp = os.path.join(CSRC, src)
        if (not force and os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(srcp), hdr_mtime)):
            return obj
        cmd = [nvcc] + ARCH + NVCC_FLAGS + ["-c", srcp, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
        if verbose:
            print(r.stdout + r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(compile_one, srcs))
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart", "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    build_dropin(force)
    return LIB


def build_dropin(force=False):
    """Compile the reference-signature C++ layer (libgwat_dropin.so) over libgwgpu.so."""
    hdr = os.path.join(os.path.dirname(HERE), "include", "gwat_dropin.h")
    newest = max(os.path.getmtime(x) for x in (DROPIN_SRC, hdr, LIB))
    if not force and os.path.exists(DROPIN_LIB) and os.path.getmtime(DROPIN_LIB) >= newest:
        return DROPIN_LIB
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-ffp-contract=off", "-std=c++17", "-fPIC", "-shared", DROPIN_SRC,
           "-o", DROPIN_LIB,
           "-L" + LIBDIR, "-lgwgpu", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("drop-in build failed:\n%s\n%s" % (r.stdout, r.stderr))
    return DROPIN_LIB


_lib = None


class GwGpuError(RuntimeError):
    pass


def _declare(L):
    c_int, c_double, c_void_p, c_char_p, c_size_t = ctypes.c_int, ctypes.c_double, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t
    P = ctypes.POINTER
    dp = P(c_double)
    ip = P(c_int)
    c_longlong = ctypes.c_longlong
    llp = P(c_longlong)
    sig = {
        "gwgpu_default_params": (None, [c_void_p]),
        "gwgpu_status_string": (c_char_p, [c_int]),
        "gwgpu_context_create": (c_int, [c_int, c_size_t, P(c_void_p)]),
        "gwgpu_context_destroy": (c_int, [c_void_p]),
        "gwgpu_last_error_string": (c_char_p, [c_void_p]),
        "gwgpu_context_stream": (c_void_p, [c_void_p]),
        "gwgpu_context_bytes_in_use": (c_size_t, [c_void_p]),
        "gwgpu_fourier_waveform": (c_int, [c_void_p, dp, c_int, dp, dp, c_char_p, c_void_p]),
        "gwgpu_fourier_detector_response": (c_int, [c_void_p, dp, c_int, dp, c_char_p, c_char_p, c_void_p]),
        "gwgpu_data_register": (c_int, [c_void_p, c_char_p, dp, c_int, dp, dp, ip]),
        "gwgpu_data_release": (c_int, [c_void_p, c_int]),
        "gwgpu_data_register_weighted": (c_int, [c_void_p, c_char_p, dp, c_int, dp, dp, dp, c_int, ip]),
        "gwgpu_log_likelihood_internal_weighted": (c_int, [c_void_p, dp, dp, dp, dp, dp, c_int, c_int, dp]),
        "gwgpu_log_likelihood_internal": (c_int, [c_void_p, dp, dp, dp, dp, c_int, dp]),
        "gwgpu_mcmc_likelihood_extrinsic": (c_int, [c_void_p, c_void_p, c_char_p, ip, c_int, c_double, dp]),
        "gwgpu_loglik_batch": (c_int, [c_void_p, c_void_p, ip, c_int, ip, c_int, c_double, c_int, dp, ip]),
        "gwgpu_loglik_batch_device": (c_int, [c_void_p, c_void_p, c_void_p, c_int, ip, c_int, c_double, c_int,
                                              c_void_p, c_void_p, c_void_p]),
        "gwgpu_mcmc_loglik_batch": (c_int, [c_void_p, dp, c_int, c_int, c_int, c_double, ip, c_int, c_double, c_int,
                                            dp, ip]),
    }
    optional = {
        "gwgpu_transform_orientation_coords": (c_int, [c_void_p, c_char_p]),
        "gwgpu_fisher_numerical": (c_int, [c_void_p, dp, c_int, c_char_p, c_char_p, c_char_p, dp, c_int, c_void_p,
                                           c_int, dp]),
        "gwgpu_fisher_batch": (c_int, [c_void_p, c_void_p, c_int, c_int, ip, c_int, c_double, c_int, dp, dp, ip]),
        "gwgpu_fisher_batch_ex": (c_int, [c_void_p, c_void_p, c_int, ip, c_int, c_void_p, dp, dp, ip]),
        "gwgpu_mcmc_fisher_batch": (c_int, [c_void_p, dp, c_int, c_int, c_int, c_double, ip, c_int, dp, ip]),
        "gwgpu_server_create": (c_int, [c_void_p, c_void_p, P(c_void_p)]),
        "gwgpu_server_destroy": (c_int, [c_void_p]),
        "gwgpu_server_submit": (c_int, [c_void_p, c_void_p, c_int, ip, c_int, P(ctypes.c_uint64)]),
        "gwgpu_server_poll": (c_int, [c_void_p, ctypes.c_uint64, dp, ip]),
        "gwgpu_server_wait": (c_int, [c_void_p, ctypes.c_uint64, c_int, dp, ip]),
        "gwgpu_server_stats": (c_int, [c_void_p, dp, dp, P(ctypes.c_uint64), P(ctypes.c_uint64)]),
        "gwgpu_server_reset_stats": (c_int, [c_void_p]),
        "gwgpu_server_loop_info": (c_int, [c_void_p, P(ctypes.c_longlong)]),
        "gwgpu_server_drive": (c_int, [c_void_p, c_void_p, ip, ip, c_int, dp, c_int, dp, ip, dp, dp]),
        "gwgpu_batch_set_tile": (c_int, [c_void_p, c_int]),
        "gwgpu_batch_set_blocks_per_sm": (c_int, [c_void_p, c_int]),
        "gwgpu_batch_last_launch_shape": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
        "gwgpu_batch_use_graphs": (c_int, [c_void_p, c_int]),
        "gwgpu_batch_timing": (c_int, [c_void_p, c_int]),
        "gwgpu_batch_last_timing": (c_int, [c_void_p, P(ctypes.c_float), P(ctypes.c_float)]),
        "gwgpu_batch_autotune": (c_int, [c_void_p, c_void_p, c_void_p, c_int, ip, c_int, c_double, c_int, c_void_p,
                                         c_void_p, ip, P(ctypes.c_float)]),
        "gwgpu_mcmc_likelihood_extrinsic_noalloc": (c_int, [c_void_p, c_void_p, c_char_p, ip, c_int, c_double,
                                                            c_void_p, c_void_p]),
        "gwgpu_maximized_log_likelihood_internal": (c_int, [c_void_p, dp, dp, dp, dp, c_int, dp]),
        "gwgpu_count_lines_data_file": (c_int, [c_char_p, ip]),
        "gwgpu_count_lines_losc_data_file": (c_int, [c_char_p, ip]),
        "gwgpu_count_lines_losc_psd_file": (c_int, [c_char_p, ip]),
        "gwgpu_read_losc_data_file": (c_int, [c_char_p, dp, c_longlong, llp, dp, dp, dp]),
        "gwgpu_read_losc_psd_file": (c_int, [c_char_p, dp, c_int, c_int]),
        "gwgpu_populate_noise": (c_int, [dp, c_char_p, dp, c_int, c_double, c_char_p]),
        "gwgpu_losc_prepare": (c_int, [c_void_p, dp, c_int, c_longlong, c_double, c_double, c_double, dp, c_int,
                                       c_double, c_double, dp, dp, dp, ip]),
        "gwgpu_allocate_losc_data": (c_int, [c_void_p, c_void_p, c_char_p, c_int, c_int, c_int, c_double, c_double,
                                             dp, dp, dp]),
        "gwgpu_maximized_log_likelihood_unaligned_internal": (c_int, [c_void_p, dp, dp, dp, dp, dp, c_int, dp]),
        "gwgpu_maximized_loglik_batch": (c_int, [c_void_p, c_void_p, c_int, c_int, ip, c_int, dp, ip]),
    }
    for name, (res, args) in list(sig.items()) + list(optional.items()):
        fn = getattr(L, name, None)
        if fn is None:
            if name in sig:
                raise GwGpuError("libgwgpu.so lacks %s" % name)
            continue
        fn.restype = res
        fn.argtypes = args


def load(build_if_missing=True):
    """Load libgwgpu.so (building it first if absent).  Raises on failure."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB):
        if not build_if_missing:
            raise GwGpuError("libgwgpu.so is not built (run __graft_entry__.build())")
        build()
    L = ctypes.CDLL(LIB)
    _declare(L)
    _lib = L
    return L


def exported_symbols():
    """Names declared in include/gwgpu.h (for the ABI check)."""
    import re
    hdr = os.path.join(os.path.dirname(HERE), "include", "gwgpu.h")
    txt = open(hdr).read()
    return sorted(set(re.findall(r"\b(gwgpu_[a-z0-9_]+)\s*\(", txt)))
