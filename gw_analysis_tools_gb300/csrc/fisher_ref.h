// fisher_ref.h -- the reference's Fisher algorithm on the device for many
// sources (fisher_ref.cu), shared with the batched moment form (fisher.cu),
// which hands it the sources whose matrices it cannot invert.
#pragma once

#include "../../include/gwgpu.h"
#include "phenom_model.h"

// Fisher matrices (and, if cov != NULL, inverses) of n sources with host
// parameters over the registered streams `handles` (reference detector =
// handles[0]); fisher/cov are host arrays n x 11 x 11; kstatus[i] is 0, 4
// (outside the model domain) or 9 (not invertible).  The caller holds the
// context lock.
int gwf_ref_run(gwgpu_context *c, const gwt::GenParams *params, int n, int method, int order, const int *handles,
                int ndet, double epsilon, int step_mode, int add_prior, double *fisher, double *cov, int *kstatus);

// The moment form (fisher.cu) for n sources, order 2 or 4 (the five-point
// rule, with the reference's constant phase on the +-2 eps responses of a
// non-reference detector); acc64: FP64 per-bin differences, weights and sums
// instead of FP32 values in compensated FP32 sums.  Takes the context lock.
// Sources it cannot invert, and five-point sources with a pair taken bin by
// bin, are redone by gwf_ref_run.
int gwf_moment_run(gwgpu_context *c, const gwgpu_gen_params *params, int n, int method, int order, const int *handles,
                   int ndet, double epsilon, int step_mode, double *fisher, double *covariance, int *status,
                   bool acc64);
