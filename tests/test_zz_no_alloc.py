"""gwgpu_mcmc_likelihood_extrinsic_noalloc through the C ABI: the same log L as
gwgpu_mcmc_likelihood_extrinsic, on two calls in a row (the scratch counter is
back at zero after each launch), in this process after the other tests and in
a fresh process whose first call does the set-up."""
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FP64_RTOL = 1e-12  # same kernel and prologue as the allocating entry point

CHECK = textwrap.dedent(r'''
    import ctypes, sys
    import numpy as np
    import torch
    sys.path.insert(0, ROOT)
    import gw_analysis_tools_gb300 as G
    from gw_analysis_tools_gb300 import workloads as W

    def run(rtol):
        ctx = G.Context(0)
        f = W.config1_grid()
        T = 1.0 / (f[1] - f[0])
        psd = W.analytic_psd(f)
        hs = [ctx.register_data(d, f, W.noise(f, 700 + i), psd) for i, d in enumerate(W.DETECTORS3)]
        harr = (ctypes.c_int * 3)(*hs)
        out = torch.zeros(4, dtype=torch.float64, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        worst = 0.0
        for d in W.prior_draws(6, 17):
            p = G.gen_params(**d)
            ref = ctx.mcmc_likelihood_extrinsic(p, "IMRPhenomD", hs, T)
            for call in range(2):
                st = ctx.lib.gwgpu_mcmc_likelihood_extrinsic_noalloc(ctx.h, ctypes.byref(p), b"IMRPhenomD", harr, 3, T,
                                                                     ctypes.c_void_p(out.data_ptr() + 8 * call),
                                                                     ctypes.c_void_p(stream))
                assert st == 0, st
            torch.cuda.synchronize()
            got = out[:2].cpu().numpy()
            for g in got:
                worst = max(worst, abs(g - ref) / max(1.0, abs(ref)))
                assert abs(g - ref) <= rtol * max(1.0, abs(ref)), (g, ref)
        # a grid beyond the scratch is refused, nothing is launched
        fl = W.uniform_grid(20.0, 20.0 + 600000 / 32.0, 1.0 / 32.0)
        hl = [ctx.register_data("Hanford", fl, np.zeros(fl.size, complex), W.analytic_psd(fl))]
        st = ctx.lib.gwgpu_mcmc_likelihood_extrinsic_noalloc(ctx.h, ctypes.byref(G.gen_params(**W.config1_source())),
                                                             b"IMRPhenomD", (ctypes.c_int * 1)(*hl), 1, T,
                                                             ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream))
        assert st == 8, st
        ctx.close()
        return worst
''')


def test_noalloc_matches_plain_after_other_tests():
    ns = {"ROOT": ROOT}
    exec(CHECK, ns)
    ns["run"](FP64_RTOL)


def test_noalloc_matches_plain_in_fresh_process():
    code = CHECK + "\nprint('worst', run(%r))\n" % FP64_RTOL
    r = subprocess.run([sys.executable, "-c", "ROOT = %r\n" % ROOT + code], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
