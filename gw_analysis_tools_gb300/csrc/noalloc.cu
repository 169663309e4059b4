// noalloc.cu -- gwgpu_mcmc_likelihood_extrinsic_noalloc: the plain FP64
// likelihood (one request, one launch of the plain kernel) for callers that
// may not allocate memory while it runs (a fixed memory budget, or code that
// must not call an allocator on this path).  It allocates nothing: the plain kernel's
// scratch (block partial sums and the block-arrival counter) lives in one
// file-scope device array, the log-likelihood goes to a device pointer the
// caller owns, and the call only enqueues on the caller's stream.
//
// Scratch: kNoAllocMaxBlocks blocks of the plain kernel (128 bins each), so
// grids of up to kNoAllocMaxBins bins; longer grids are rejected with
// GWGPU_ETOOLARGE.  The counter word must start at zero: the array is
// zero-initialised when the module loads and the last block of every launch
// sets it back to zero.  Calls share this one scratch array, so overlapping
// calls (two host threads, or two streams with work in flight at once) race
// on it: issue them one after the other on one stream.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>

#include "../../include/gwgpu.h"
#include "capi_internal.h"
#include "kernels.h"

namespace {

constexpr int kNoAllocMaxBlocks = 4096;
constexpr int kNoAllocMaxBins = kNoAllocMaxBlocks * 128;
constexpr int kNoAllocPartials = kNoAllocMaxBlocks * 2 * gwt::kMaxDet;  // doubles
// partial sums, then 32 doubles whose first word is the block-arrival counter
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocPartials + 32];

constexpr int kMaxDevices = 64;
bool g_loaded[kMaxDevices] = {false};
std::mutex g_setup_mu;

// The scratch address, looked up on every call with the device current
// (cudaGetSymbolAddress allocates nothing and is cheap), so that it stays
// right after a device reset.  On the first call per device, also the plain
// kernels' module (a function-attribute query, which may load the module):
// that first call must come before any stream capture that later calls are
// part of.
int setup(int device, double **out) {
  if (device < 0 || device >= kMaxDevices) return GWGPU_EINVAL;
  std::lock_guard<std::mutex> lk(g_setup_mu);
  void *p = nullptr;
  if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return GWGPU_ECUDA;
  if (!g_loaded[device]) {
    if (gwk::plain_preload() != cudaSuccess) return GWGPU_ECUDA;
    g_loaded[device] = true;
  }
  *out = (double *)p;
  return GWGPU_OK;
}

int approximant_of(const char *m) {
  if (!m) return -1;
  if (!std::strcmp(m, "IMRPhenomD") || !std::strcmp(m, "MCMC_IMRPhenomD")) return gwt::kPhenomD;
  if (!std::strcmp(m, "IMRPhenomPv2") || !std::strcmp(m, "MCMC_IMRPhenomPv2")) return gwt::kPhenomPv2;
  return -1;
}

}  // namespace

extern "C" {

int gwgpu_mcmc_likelihood_extrinsic_noalloc(gwgpu_context *c, const gwgpu_gen_params *p, const char *method,
                                            const int *handles, int ndet, double T_segment, double *d_loglik,
                                            void *stream) {
  const int ap = approximant_of(method);
  if (!c || !p || !handles || ndet < 1 || ndet > gwt::kMaxDet || !d_loglik || ap < 0) return GWGPU_EINVAL;
  std::lock_guard<std::mutex> lk(c->mu);
  if (cudaSetDevice(c->device) != cudaSuccess) return GWGPU_ECUDA;
  double *scratch;
  int st = setup(c->device, &scratch);
  if (st) return st;
  gwk::StreamDev sd[gwt::kMaxDet];
  int dets[gwt::kMaxDet];
  for (int d = 0; d < ndet; d++) {
    const gwgpu_context::Stream *s = c->get_stream(handles[d]);
    if (!s) return GWGPU_ENOTFOUND;
    sd[d] = s->dev;
    dets[d] = s->dev.det;
    if (sd[d].N != sd[0].N) return GWGPU_EINVAL;
  }
  if (sd[0].N > kNoAllocMaxBins) return GWGPU_ETOOLARGE;
  gwt::GenParams gp;
  std::memcpy(&gp, p, sizeof(gp));
  gp.tc = T_segment - gp.tc;  // mcmc_gw.cpp:2466-2473
  gwt::Request r;
  gwt::request_prologue(r, gp, ap, dets, ndet, c->qnm_host.data());
  if (r.m.status) return GWGPU_EDOMAIN;  // nothing is launched; d_loglik is left as it was
  cudaError_t e = gwk::launch_plain(r, sd, ndet, scratch, (unsigned *)(scratch + kNoAllocPartials), d_loglik,
                                    nullptr, (cudaStream_t)stream);
  return e == cudaSuccess ? GWGPU_OK : GWGPU_ECUDA;
}

}  // extern "C"
