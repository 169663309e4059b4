// batch.cu -- batched log-likelihood entry points: many requests (chains x
// temperatures x ensembles, possibly on different grids) in one prologue
// launch plus one persistent fused bin kernel.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gwgpu.h"
#include "batch_internal.h"
#include "capi_internal.h"

namespace gwb {

int default_tile(int mixed) { return mixed ? 4096 : 1024; }

int persistent_grid(int device, int mixed, int ndet) {
  static int cache[2][gwt::kMaxDet + 1] = {{0}};
  int &g = cache[mixed ? 1 : 0][ndet];
  if (g) return g;
  cudaDeviceProp p;
  cudaGetDeviceProperties(&p, device);
  int per_sm = gwk::batch_occupancy(mixed, ndet);
  if (per_sm < 1) per_sm = 1;
  g = p.multiProcessorCount * per_sm;
  return g;
}

// Plan = item list for one (n, handles, tile) shape, uploaded once.
int plan_batch(gwgpu_context *c, int n, const int *handles, int ndet, int tile, Plan &pl) {
  pl.n = n;
  pl.ndet = ndet;
  pl.tile = tile;
  std::vector<gwk::Item> items;
  std::vector<int> start(n), count(n);
  for (int r = 0; r < n; r++) {
    const gwgpu_context::Stream *s0 = c->get_stream(handles[r * ndet]);
    if (!s0) return GWGPU_ENOTFOUND;
    for (int d = 1; d < ndet; d++) {
      const gwgpu_context::Stream *s = c->get_stream(handles[r * ndet + d]);
      if (!s) return GWGPU_ENOTFOUND;
      if (s->dev.N != s0->dev.N) return GWGPU_EINVAL;
    }
    int N = s0->dev.N, nt = (N + tile - 1) / tile;
    start[r] = (int)items.size();
    count[r] = nt;
    for (int t = 0; t < nt; t++) items.push_back(gwk::Item{r, t * tile});
  }
  // longest requests first so the persistent grid drains evenly
  pl.nitems = (int)items.size();
  size_t need = sizeof(gwk::Item) * items.size() + sizeof(int) * (size_t)n * (2 + ndet);
  void *dev;
  int st = c->workspace(gwgpu_context::kWsBatchItems, need, &dev);
  if (st) return st;
  pl.items = (gwk::Item *)dev;
  pl.item_start = (int *)(pl.items + items.size());
  pl.item_count = pl.item_start + n;
  pl.handles = pl.item_count + n;
  cudaMemcpyAsync(pl.items, items.data(), sizeof(gwk::Item) * items.size(), cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(pl.item_start, start.data(), sizeof(int) * n, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(pl.item_count, count.data(), sizeof(int) * n, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(pl.handles, handles, sizeof(int) * (size_t)n * ndet, cudaMemcpyHostToDevice, c->stream);
  pl.key.assign((const char *)handles, (const char *)(handles + (size_t)n * ndet));
  pl.key += "|" + std::to_string(n) + "|" + std::to_string(tile) + "|" + std::to_string(ndet);
  return GWGPU_OK;
}

// Enqueue prologue + fused kernel on c->stream.  Device arrays in, device out.
int enqueue_batch(gwgpu_context *c, const gwgpu_gen_params *d_params, const int *d_approx, int n,
                  const int *h_handles, int ndet, double T_segment, int tc_from_segment, int precision,
                  double *d_out, int *d_status, int tile) {
  const int mixed = precision == GWGPU_PREC_MIXED;
  if (tile <= 0) tile = default_tile(mixed);
  std::string key((const char *)h_handles, (const char *)(h_handles + (size_t)n * ndet));
  key += "|" + std::to_string(n) + "|" + std::to_string(tile) + "|" + std::to_string(ndet);
  Plan &pl = c->plan;
  if (pl.key != key) {
    int st = plan_batch(c, n, h_handles, ndet, tile, pl);
    if (st) {
      pl.key.clear();
      return st;
    }
  }
  // per-request scratch: Request/MixedReq, partials, counters
  size_t rq = mixed ? sizeof(gwt::MixedReq) : sizeof(gwt::Request);
  size_t bytes = rq * n + sizeof(double) * (size_t)pl.nitems * gwk::kAcc + sizeof(unsigned) * (size_t)(n + 32);
  void *dev;
  int st = c->workspace(gwgpu_context::kWsBatch, bytes, &dev);
  if (st) return st;
  char *p = (char *)dev;
  void *reqs = p;
  p += rq * n;
  double *partials = (double *)p;
  p += sizeof(double) * (size_t)pl.nitems * gwk::kAcc;
  unsigned *cnt = (unsigned *)p;
  cudaError_t e = cudaMemsetAsync(cnt, 0, sizeof(unsigned) * (size_t)(n + 32), c->stream);
  if (e != cudaSuccess) return c->fail(e, "batch counters");
  e = gwk::launch_prologue((const gwt::GenParams *)d_params, d_approx, n, pl.handles, ndet, T_segment,
                           tc_from_segment, c->streams_dev, c->qnm_dev, mixed ? nullptr : (gwt::Request *)reqs,
                           mixed ? (gwt::MixedReq *)reqs : nullptr, mixed, d_status, c->stream);
  if (e != cudaSuccess) return c->fail(e, "prologue launch");
  gwk::BatchArgs a;
  a.req = mixed ? nullptr : (const gwt::Request *)reqs;
  a.mreq = mixed ? (const gwt::MixedReq *)reqs : nullptr;
  a.handles = pl.handles;
  a.ndet = ndet;
  a.streams = c->streams_dev;
  a.items = pl.items;
  a.nitems = pl.nitems;
  a.item_start = pl.item_start;
  a.item_count = pl.item_count;
  a.tile = tile;
  a.item_counter = cnt + n;
  a.req_done = cnt;
  a.partials = partials;
  a.out = d_out;
  a.status = d_status;
  a.tables = c->tables;
  int grid = std::min(pl.nitems, persistent_grid(c->device, mixed, ndet));
  if (grid < 1) grid = 1;
  e = gwk::launch_batch(a, mixed, grid, 0, c->stream);
  if (e != cudaSuccess) return c->fail(e, "batch launch");
  return GWGPU_OK;
}

}  // namespace gwb

extern "C" {

int gwgpu_loglik_batch_device(gwgpu_context *c, const gwgpu_gen_params *d_params, const int *d_approx, int n,
                              const int *h_handles, int ndet, double T_segment, int precision, double *d_out,
                              int *d_status, void *stream) {
  if (!c || !d_params || !d_approx || !h_handles || !d_out || !d_status || n < 1 || ndet < 1 || ndet > gwt::kMaxDet)
    return GWGPU_EINVAL;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  cudaStream_t user = (cudaStream_t)stream;
  if (user && user != c->stream) {  // order after the caller's stream, then let it wait for us
    cudaEvent_t ev;
    cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    cudaEventRecord(ev, user);
    cudaStreamWaitEvent(c->stream, ev, 0);
    cudaEventDestroy(ev);
  }
  int st = gwb::enqueue_batch(c, d_params, d_approx, n, h_handles, ndet, T_segment, 1, precision, d_out, d_status,
                              c->tile_override);
  if (!st && user && user != c->stream) {
    cudaEvent_t ev;
    cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    cudaEventRecord(ev, c->stream);
    cudaStreamWaitEvent(user, ev, 0);
    cudaEventDestroy(ev);
  }
  return st;
}

int gwgpu_loglik_batch(gwgpu_context *c, const gwgpu_gen_params *params, const int *approx, int n, const int *handles,
                       int ndet, double T_segment, int precision, double *loglik, int *status) {
  if (!c || !params || !approx || !handles || !loglik || n < 1 || ndet < 1 || ndet > gwt::kMaxDet)
    return GWGPU_EINVAL;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  size_t pb = sizeof(gwgpu_gen_params) * n, ab = sizeof(int) * n, ob = sizeof(double) * n, sb = sizeof(int) * n;
  void *h, *d;
  int st = c->pinned(gwgpu_context::kHwsBatch, pb + ab + ob + sb + 64, &h);
  if (st) return st;
  st = c->workspace(gwgpu_context::kWsServe + 1, pb + ab + ob + sb + 64, &d);
  if (st) return st;
  char *hp = (char *)h, *dp = (char *)d;
  std::memcpy(hp, params, pb);
  std::memcpy(hp + pb, approx, ab);
  cudaMemcpyAsync(dp, hp, pb + ab, cudaMemcpyHostToDevice, c->stream);
  st = gwb::enqueue_batch(c, (const gwgpu_gen_params *)dp, (const int *)(dp + pb), n, handles, ndet, T_segment, 1,
                          precision, (double *)(dp + pb + ab), (int *)(dp + pb + ab + ob), c->tile_override);
  if (st) return st;
  cudaMemcpyAsync(hp + pb + ab, dp + pb + ab, ob + sb, cudaMemcpyDeviceToHost, c->stream);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return c->fail(e, "batch");
  std::memcpy(loglik, hp + pb + ab, ob);
  const int *hs = (const int *)(hp + pb + ab + ob);
  int any = 0;
  for (int i = 0; i < n; i++) {
    int s = hs[i] ? (hs[i] == 1 ? GWGPU_EINVAL : GWGPU_EDOMAIN) : GWGPU_OK;
    if (status) status[i] = s;
    any |= s;
  }
  (void)any;
  return GWGPU_OK;
}

int gwgpu_mcmc_loglik_batch(gwgpu_context *c, const double *theta, int dim, int n, int approximant, double gmst,
                            const int *handles, int ndet, double T_segment, int precision, double *loglik,
                            int *status) {
  if (!c || !theta || !handles || !loglik || n < 1 || (dim != 11 && dim != 15) || ndet < 1 || ndet > gwt::kMaxDet)
    return GWGPU_EINVAL;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  size_t tb = sizeof(double) * (size_t)n * dim, pb = sizeof(gwgpu_gen_params) * n, ab = sizeof(int) * n,
         ob = sizeof(double) * n, sb = sizeof(int) * n;
  void *h, *d;
  int st = c->pinned(gwgpu_context::kHwsBatch, tb + ob + sb + 64, &h);
  if (st) return st;
  st = c->workspace(gwgpu_context::kWsServe + 2, tb + pb + ab + ob + sb + 64, &d);
  if (st) return st;
  char *hp = (char *)h, *dp = (char *)d;
  std::memcpy(hp, theta, tb);
  cudaMemcpyAsync(dp, hp, tb, cudaMemcpyHostToDevice, c->stream);
  gwgpu_gen_params *dparams = (gwgpu_gen_params *)(dp + tb);
  int *dapprox = (int *)(dp + tb + pb);
  cudaError_t e = gwk::launch_mcmc_repack((const double *)dp, dim, n, approximant, gmst, (gwt::GenParams *)dparams,
                                          dapprox, c->stream);
  if (e != cudaSuccess) return c->fail(e, "repack launch");
  double *dout = (double *)(dp + tb + pb + ab);
  int *dstat = (int *)(dp + tb + pb + ab + ob);
  st = gwb::enqueue_batch(c, dparams, dapprox, n, handles, ndet, T_segment, 1, precision, dout, dstat,
                          c->tile_override);
  if (st) return st;
  cudaMemcpyAsync(hp + tb, dout, ob + sb, cudaMemcpyDeviceToHost, c->stream);
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return c->fail(e, "mcmc batch");
  std::memcpy(loglik, hp + tb, ob);
  const int *hs = (const int *)(hp + tb + ob);
  for (int i = 0; i < n; i++)
    if (status) status[i] = hs[i] ? (hs[i] == 1 ? GWGPU_EINVAL : GWGPU_EDOMAIN) : GWGPU_OK;
  return GWGPU_OK;
}

}  // extern "C"
