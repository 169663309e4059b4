"""GB300-native likelihood engine for gw_analysis_tools.

IMRPhenomD / IMRPhenomPv2 waveform, detector projection and the
PSD-weighted inner product that gives each parallel-tempered chain its
log-likelihood, plus the numerical Fisher matrix, as sm_103a CUDA kernels
behind a C ABI (include/gwgpu.h).  See engine.Context.
"""
from .engine import (FISHER_MOMENTS, FISHER_REFERENCE, IMRPhenomD, IMRPhenomPv2, PREC_FP64, PREC_MIXED, Context, GenParams, GwGpuError, Server,
                     count_lines_data_file, count_lines_losc_data_file, count_lines_losc_psd_file, gen_params,
                     params_array, populate_noise, read_losc_data_file, read_losc_psd_file,
                     transform_orientation_coords)

__all__ = ["Context", "Server", "GenParams", "gen_params", "params_array", "GwGpuError", "IMRPhenomD",
           "IMRPhenomPv2", "PREC_FP64", "PREC_MIXED", "count_lines_data_file", "count_lines_losc_data_file",
           "count_lines_losc_psd_file", "read_losc_data_file", "read_losc_psd_file", "populate_noise",
           "transform_orientation_coords", "FISHER_MOMENTS", "FISHER_REFERENCE"]
