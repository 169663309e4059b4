// batch.cu -- batched log-likelihood entry points: many requests (chains x
// temperatures x ensembles, possibly on different grids and approximants) in
// one prologue launch plus one persistent fused bin kernel, replayed through
// captured CUDA graphs, with the bin tile picked by an autotuner.
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

static int length_class(int N) {  // grid-length bucket of the tuning table
  int c = 0;
  while ((1 << (c + 11)) < N && c < 12) c++;
  return c;
}

// The tuning class of a batch: precision, detectors, the length class of its
// longest grid, and whether its requests' grids differ (an uneven batch
// spreads its items differently from a uniform one of the same longest grid).
std::string tune_key(gwgpu_context *c, int mixed, int ndet, const int *h_handles, int n) {
  int nmax = 0, nmin = 1 << 30;
  for (int i = 0; i < n; i++) {
    const gwgpu_context::Stream *s = c->get_stream(h_handles[(size_t)i * ndet]);
    if (!s) continue;
    nmax = std::max(nmax, s->dev.N);
    nmin = std::min(nmin, s->dev.N);
  }
  return std::to_string(mixed) + ":" + std::to_string(ndet) + ":" + std::to_string(length_class(nmax)) +
         (nmin < nmax ? ":u" : "");
}

int choose_tile(gwgpu_context *c, int mixed, const std::string &key) {
  if (c->tile_override > 0) return c->tile_override;
  auto it = c->tuned.find(key);
  if (it != c->tuned.end()) return it->second;
  return default_tile(mixed);
}

// Resident blocks per SM of the fused kernel's launch shape: the autotuner's
// candidate while it runs, else its choice for this batch class, else the
// default.
static int choose_occ(gwgpu_context *c, int mixed, const std::string &key) {
  if (!mixed) return gwk::batch_default_occ(0);
  if (c->occ_override > 0) return c->occ_override;
  if (c->occ_user > 0) return c->occ_user;
  auto it = c->tuned_occ.find(key);
  if (it != c->tuned_occ.end()) return it->second;
  return gwk::batch_default_occ(1);
}

static int persistent_grid(int device, int mixed, int ndet, int occ) {
  static int cache[2][gwt::kMaxDet + 1][5] = {{{0}}};
  int &g = cache[mixed ? 1 : 0][ndet][occ & 3];
  if (g) return g;
  cudaDeviceProp p;
  cudaGetDeviceProperties(&p, device);
  int per_sm = gwk::batch_occupancy(mixed, ndet, occ);
  if (per_sm < 1) per_sm = 1;
  g = p.multiProcessorCount * per_sm;
  return g;
}

static char *align256(char *p) { return (char *)(((uintptr_t)p + 255) & ~(uintptr_t)255); }

static int lane_alloc(gwgpu_context *c, Lane &L, void **p, size_t *cap, size_t bytes, const char *what) {
  if (*cap >= bytes) return GWGPU_OK;
  if (*p) {
    cudaStreamSynchronize(L.stream);
    c->dfree(*p);
    L.bytes -= *cap;
    *p = nullptr;
    *cap = 0;
  }
  size_t nb = std::max(bytes + bytes / 4, (size_t)65536);
  int st = c->dalloc(p, nb, what);
  if (st) return st;
  *cap = nb;
  L.bytes += nb;
  return GWGPU_OK;
}

void lane_release(gwgpu_context *c, Lane &L) {
  if (L.stream) cudaStreamSynchronize(L.stream);
  for (auto &g : L.graphs) cudaGraphExecDestroy(g.second.exec);
  L.graphs.clear();
  c->dfree(L.plan.mem);
  c->dfree(L.work);
  c->dfree(L.dio);
  if (L.hio) cudaFreeHost(L.hio);
  L.plan = Plan();
  L.work = L.dio = L.hio = nullptr;
  L.work_cap = L.io_cap = 0;
  L.bytes = 0;
  if (L.own_stream && L.stream) cudaStreamDestroy(L.stream);
  L.stream = nullptr;
}

// Item list of one (n, handles, tile) shape: contiguous bin tiles per request.
int plan_batch(gwgpu_context *c, Lane &L, int n, const int *handles, int ndet, int tile) {
  Plan &pl = L.plan;
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
  // Longest requests' items first: the persistent grid then drains evenly.
  std::vector<int> order(n);
  for (int r = 0; r < n; r++) order[r] = r;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return count[a] > count[b]; });
  std::vector<gwk::Item> sorted;
  sorted.reserve(items.size());
  for (int r : order)
    for (int q = 0; q < count[r]; q++) sorted.push_back(items[start[r] + q]);
  // partial sums are indexed by item: keep item ids contiguous per request
  std::vector<int> nstart(n);
  int pos = 0;
  for (int r : order) {
    nstart[r] = pos;
    pos += count[r];
  }
  pl.nitems = (int)sorted.size();
  size_t need = sizeof(gwk::Item) * sorted.size() + 256 + sizeof(int) * (size_t)n * (2 + ndet) + 256 +
                sizeof(int) * sorted.size() * gwk::kOrderBuckets + 256;
  int st = lane_alloc(c, L, &pl.mem, &pl.cap, need, "batch plan");
  if (st) return st;
  char *p = (char *)pl.mem;
  pl.items = (gwk::Item *)p;
  p = align256(p + sizeof(gwk::Item) * sorted.size());
  pl.item_start = (int *)p;
  pl.item_count = pl.item_start + n;
  pl.handles = pl.item_count + n;
  pl.order = (int *)align256((char *)(pl.handles + (size_t)n * ndet));
  cudaMemcpyAsync(pl.items, sorted.data(), sizeof(gwk::Item) * sorted.size(), cudaMemcpyHostToDevice, L.stream);
  cudaMemcpyAsync(pl.item_start, nstart.data(), sizeof(int) * n, cudaMemcpyHostToDevice, L.stream);
  cudaMemcpyAsync(pl.item_count, count.data(), sizeof(int) * n, cudaMemcpyHostToDevice, L.stream);
  cudaMemcpyAsync(pl.handles, handles, sizeof(int) * (size_t)n * ndet, cudaMemcpyHostToDevice, L.stream);
  pl.n = n;
  pl.ndet = ndet;
  pl.tile = tile;
  return GWGPU_OK;
}

static int launch_sequence(gwgpu_context *c, Lane &L, const gwgpu_gen_params *d_params, const int *d_approx, int n,
                           int ndet, double T_segment, int mixed, int occ, double *d_out, int *d_status,
                           int *status_out, void *reqs, double *partials, unsigned *cnt) {
  const Plan &pl = L.plan;
  const bool timing = c->timing && &L == &c->lane;
  if (timing) cudaEventRecord(c->t_ev[0], L.stream);
  cudaError_t e = cudaMemsetAsync(cnt, 0, sizeof(unsigned) * (size_t)(n + 32 + gwk::kOrderBuckets), L.stream);
  if (e != cudaSuccess) return c->fail(e, "batch counters");
  // mixed form: the prologue writes the work order (most live bins first)
  const bool ordered = mixed && c->order_items && !c->prologue_serial;
  // FP64 form: the cooperative prologue writes each IMRPhenomD request's
  // coefficients on the grid after the Request records, for the bin
  // kernel's table form (with the FP64 n^(-7/6) table)
  gwt::WaveF64 *w64 = nullptr;
  if (!mixed && !c->prologue_serial && c->tm76d && c->tm76d_n > 0)
    w64 = (gwt::WaveF64 *)((char *)reqs + sizeof(gwt::Request) * (size_t)n);
  gwk::OrderArgs ord;
  if (ordered) {
    ord.fill = (int *)(cnt + n + 32);
    ord.items = pl.order;
    ord.item_start = pl.item_start;
    ord.item_count = pl.item_count;
    ord.nitems = pl.nitems;
    ord.tile = pl.tile;
  }
  if (c->prologue_serial)
    e = gwk::launch_prologue_serial((const gwt::GenParams *)d_params, d_approx, n, pl.handles, ndet, T_segment, 1,
                                    c->streams_dev, c->qnm_dev, mixed ? nullptr : (gwt::Request *)reqs,
                                    mixed ? (gwt::MixedReq *)reqs : nullptr, mixed, d_status, L.stream);
  else
    e = gwk::launch_prologue((const gwt::GenParams *)d_params, d_approx, n, pl.handles, ndet, T_segment, 1,
                             c->streams_dev, c->qnm_dev, mixed ? nullptr : (gwt::Request *)reqs,
                             mixed ? (gwt::MixedReq *)reqs : nullptr, mixed, d_status, L.stream, ord, w64);
  if (e != cudaSuccess) return c->fail(e, "prologue launch");
  if (timing) cudaEventRecord(c->t_ev[1], L.stream);
  gwk::BatchArgs a;
  a.req = mixed ? nullptr : (const gwt::Request *)reqs;
  a.mreq = mixed ? (const gwt::MixedReq *)reqs : nullptr;
  a.handles = pl.handles;
  a.ndet = ndet;
  a.streams = c->streams_dev;
  a.items = pl.items;
  a.bucket_fill = ordered ? ord.fill : nullptr;
  a.bucket_items = ordered ? ord.items : nullptr;
  a.nitems = pl.nitems;
  a.item_start = pl.item_start;
  a.item_count = pl.item_count;
  a.tile = pl.tile;
  a.item_counter = cnt + n;
  a.req_done = cnt;
  a.partials = partials;
  a.out = d_out;
  a.status = d_status;
  a.status_out = status_out ? status_out : d_status;
  a.tables = c->tables;
  a.w64 = w64;
  a.tm76d = w64 ? c->tm76d : nullptr;
  a.tm76d_n = w64 ? c->tm76d_n : 0;
  int grid = std::min(pl.nitems, persistent_grid(c->device, mixed, ndet, occ));
  if (grid < 1) grid = 1;
  e = gwk::launch_batch(a, mixed, grid, occ, L.stream, c->pdl);
  if (&L == &c->lane) {
    c->last_shape[0] = pl.tile;
    c->last_shape[1] = occ;
    c->last_shape[2] = grid;
  }
  if (e != cudaSuccess) return c->fail(e, "batch launch");
  if (timing) cudaEventRecord(c->t_ev[2], L.stream);
  return GWGPU_OK;
}

int enqueue_batch(gwgpu_context *c, Lane &L, const gwgpu_gen_params *d_params, const int *d_approx, int n,
                  const int *h_handles, int ndet, double T_segment, int precision, double *d_out, int *d_status,
                  int tile, bool use_graph, const BatchCopies *io, int *status_out) {
  const int mixed = precision == GWGPU_PREC_MIXED;
  const gwgpu_context::Stream *s0 = c->get_stream(h_handles[0]);
  if (!s0) return GWGPU_ENOTFOUND;
  // the batch shape (handles, sizes, registrations, precision) of the last
  // call on this lane: the tuning class and the plan follow from it and are
  // recomputed only when it changes (one comparison of the handle array)
  const size_t nh = (size_t)n * ndet;
  const bool same = L.shape.n == n && L.shape.ndet == ndet && L.shape.epoch == c->streams_epoch &&
                    L.shape.mixed == mixed && L.shape.handles.size() == nh &&
                    std::memcmp(L.shape.handles.data(), h_handles, sizeof(int) * nh) == 0;
  if (!same) {
    L.tk = tune_key(c, mixed, ndet, h_handles, n);
    L.shape.handles.assign(h_handles, h_handles + nh);
    L.shape.n = n;
    L.shape.ndet = ndet;
    L.shape.epoch = c->streams_epoch;
    L.shape.mixed = mixed;
  }
  if (tile <= 0) tile = choose_tile(c, mixed, L.tk);
  const int occ = choose_occ(c, mixed, L.tk);
  // FP64 batches: the n^(-7/6) table of the table form, built before any
  // capture (a failure leaves the frequency form)
  if (!mixed && c->ensure_tm76d(c->tables.nmax) != GWGPU_OK) c->last_error.clear();
  bool replanned = false;
  if (!same || !L.plan.valid || L.plan.tile != tile) {
    int st = plan_batch(c, L, n, h_handles, ndet, tile);
    if (st) {
      L.plan.valid = false;
      return st;
    }
    L.plan.valid = true;
    replanned = true;
  }
  size_t rq = mixed ? sizeof(gwt::MixedReq) : sizeof(gwt::Request) + sizeof(gwt::WaveF64);
  size_t bytes = rq * n + 512 + sizeof(double) * (size_t)L.plan.nitems * gwk::kAcc + 256 +
                 sizeof(unsigned) * (size_t)(n + 32 + gwk::kOrderBuckets);
  void *old = L.work;
  int st = lane_alloc(c, L, &L.work, &L.work_cap, bytes, "batch scratch");
  if (st) return st;
  if (L.work != old || replanned) {  // captured graphs hold the old addresses
    for (auto &g : L.graphs) cudaGraphExecDestroy(g.second.exec);
    L.graphs.clear();
  }
  char *p = (char *)L.work;
  void *reqs = p;
  p = align256(p + rq * n);  // FP64: Request[n], then WaveF64[n] (below)
  double *partials = (double *)p;
  p = align256(p + sizeof(double) * (size_t)L.plan.nitems * gwk::kAcc);
  unsigned *cnt = (unsigned *)p;
  auto sequence = [&]() {
    if (io) cudaMemcpyAsync(io->h2d_dst, io->h2d_src, io->h2d_bytes, cudaMemcpyHostToDevice, L.stream);
    int r = launch_sequence(c, L, d_params, d_approx, n, ndet, T_segment, mixed, occ, d_out, d_status, status_out,
                            reqs, partials, cnt);
    if (!r && io) cudaMemcpyAsync(io->d2h_dst, io->d2h_src, io->d2h_bytes, cudaMemcpyDeviceToHost, L.stream);
    return r;
  };
  if (!use_graph || c->timing) return sequence();
  char gk[320];
  snprintf(gk, sizeof(gk), "%p|%p|%p|%p|%p|%d|%d|%.17g|%d|%p|%p|%zu|%p|%p|%zu", (const void *)d_params,
           (const void *)d_approx, (const void *)d_out, (const void *)d_status, (const void *)status_out, mixed, occ,
           T_segment, n,
           io ? io->h2d_src : nullptr, io ? io->h2d_dst : nullptr, io ? io->h2d_bytes : 0,
           io ? io->d2h_dst : nullptr, io ? (const void *)io->d2h_src : nullptr, io ? io->d2h_bytes : 0);
  auto it = L.graphs.find(gk);
  if (it == L.graphs.end()) {
    if (L.graphs.size() >= kMaxGraphs) {  // drop the least recently used one, after the work queued on it
      auto lru = L.graphs.begin();
      for (auto j = L.graphs.begin(); j != L.graphs.end(); ++j)
        if (j->second.used < lru->second.used) lru = j;
      cudaError_t e = cudaStreamSynchronize(L.stream);
      if (e != cudaSuccess) return c->fail(e, "graph cache");
      cudaGraphExecDestroy(lru->second.exec);
      L.graphs.erase(lru);
    }
    cudaGraph_t g;
    cudaError_t e = cudaStreamBeginCapture(L.stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return c->fail(e, "graph capture");
    st = sequence();
    e = cudaStreamEndCapture(L.stream, &g);
    if (st) return st;
    if (e != cudaSuccess) return c->fail(e, "graph capture end");
    cudaGraphExec_t ge;
    e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return c->fail(e, "graph instantiate");
    it = L.graphs.emplace(gk, Lane::Graph{ge, 0}).first;
  }
  it->second.used = ++L.graph_tick;
  cudaError_t e = cudaGraphLaunch(it->second.exec, L.stream);
  if (e != cudaSuccess) return c->fail(e, "graph launch");
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
  gwb::Lane &L = c->lane0();
  if (user && user != L.stream) {  // order after the caller's stream, then make it wait for us
    cudaEventRecord(c->ev_in, user);
    cudaStreamWaitEvent(L.stream, c->ev_in, 0);
  }
  int st = gwb::enqueue_batch(c, L, d_params, d_approx, n, h_handles, ndet, T_segment, precision, d_out, d_status, 0,
                              c->use_graphs);
  if (!st && user && user != L.stream) {
    cudaEventRecord(c->ev_out, L.stream);
    cudaStreamWaitEvent(user, c->ev_out, 0);
  }
  return st;
}

static int stage_io(gwgpu_context *c, gwb::Lane &L, size_t bytes) {
  if (L.io_cap >= bytes) return GWGPU_OK;
  if (L.hio) cudaFreeHost(L.hio);
  L.hio = nullptr;
  size_t nb = std::max(bytes + bytes / 4, (size_t)65536);
  if (cudaMallocHost(&L.hio, nb) != cudaSuccess) return GWGPU_ECUDA;
  c->dfree(L.dio);
  L.dio = nullptr;
  L.bytes -= L.io_cap;
  L.io_cap = 0;
  int st = c->dalloc(&L.dio, nb, "batch io");
  if (st) return st;
  L.io_cap = nb;
  L.bytes += nb;
  for (auto &g : L.graphs) cudaGraphExecDestroy(g.second.exec);
  L.graphs.clear();
  return GWGPU_OK;
}

static size_t up256(size_t x) { return (x + 255) & ~(size_t)255; }

static void statuses(const int *hs, int n, int *status) {
  if (!status) return;
  for (int i = 0; i < n; i++) status[i] = gwk::status_code(hs[i]);
}

int gwgpu_loglik_batch(gwgpu_context *c, const gwgpu_gen_params *params, const int *approx, int n, const int *handles,
                       int ndet, double T_segment, int precision, double *loglik, int *status) {
  if (!c || !params || !approx || !handles || !loglik || n < 1 || ndet < 1 || ndet > gwt::kMaxDet)
    return GWGPU_EINVAL;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  gwb::Lane &L = c->lane0();
  // params | approximants | log L | status, each on a 256-byte boundary
  const size_t pb = sizeof(gwgpu_gen_params) * n, ab = sizeof(int) * n, ob = sizeof(double) * n,
               sb = sizeof(int) * n;
  const size_t o_ap = up256(pb), o_out = o_ap + up256(ab), o_st = o_out + up256(ob), total = o_st + up256(sb);
  int st = stage_io(c, L, total);
  if (st) return st;
  char *hp = (char *)L.hio, *dp = (char *)L.dio, *hm = nullptr;
  std::memcpy(hp, params, pb);
  std::memcpy(hp + o_ap, approx, ab);
  // The kernels read the parameters from, and write log L and the status
  // into, the pinned staging buffer (mapped: the transfers cross the
  // host-device link inside the kernels, with no copy nodes); the working
  // status, which items flag atomically, stays in device memory.
  cudaError_t e = cudaHostGetDevicePointer((void **)&hm, hp, 0);
  if (e != cudaSuccess) return c->fail(e, "batch staging mapping");
  st = gwb::enqueue_batch(c, L, (const gwgpu_gen_params *)hm, (const int *)(hm + o_ap), n, handles, ndet, T_segment,
                          precision, (double *)(hm + o_out), (int *)(dp + o_st), 0, c->use_graphs, nullptr,
                          (int *)(hm + o_st));
  if (st) return st;
  e = cudaStreamSynchronize(L.stream);
  if (e != cudaSuccess) return c->fail(e, "batch");
  std::memcpy(loglik, hp + o_out, ob);
  statuses((const int *)(hp + o_st), n, status);
  return GWGPU_OK;
}

int gwgpu_mcmc_loglik_batch(gwgpu_context *c, const double *theta, int dim, int n, int approximant, double gmst,
                            const int *handles, int ndet, double T_segment, int precision, double *loglik,
                            int *status) {
  if (!c || !theta || !handles || !loglik || n < 1 || (dim != 11 && dim != 15) || ndet < 1 || ndet > gwt::kMaxDet)
    return GWGPU_EINVAL;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  gwb::Lane &L = c->lane0();
  // theta | params | approximants | log L | status, each on a 256-byte boundary
  const size_t tb = sizeof(double) * (size_t)n * dim, pb = sizeof(gwgpu_gen_params) * n, ab = sizeof(int) * n,
               ob = sizeof(double) * n, sb = sizeof(int) * n;
  const size_t o_p = up256(tb), o_ap = o_p + up256(pb), o_out = o_ap + up256(ab), o_st = o_out + up256(ob),
               total = o_st + up256(sb);
  int st = stage_io(c, L, total);
  if (st) return st;
  char *hp = (char *)L.hio, *dp = (char *)L.dio, *hm = nullptr;
  std::memcpy(hp, theta, tb);
  // the repack reads theta from the mapped staging buffer and the finalize
  // writes log L and the status back into it (no copy nodes)
  cudaError_t e = cudaHostGetDevicePointer((void **)&hm, hp, 0);
  if (e != cudaSuccess) return c->fail(e, "batch staging mapping");
  gwgpu_gen_params *dparams = (gwgpu_gen_params *)(dp + o_p);
  int *dapprox = (int *)(dp + o_ap);
  e = gwk::launch_mcmc_repack((const double *)hm, dim, n, approximant, gmst, (gwt::GenParams *)dparams, dapprox,
                              L.stream);
  if (e != cudaSuccess) return c->fail(e, "repack launch");
  st = gwb::enqueue_batch(c, L, dparams, dapprox, n, handles, ndet, T_segment, precision, (double *)(hm + o_out),
                          (int *)(dp + o_st), 0, c->use_graphs, nullptr, (int *)(hm + o_st));
  if (st) return st;
  e = cudaStreamSynchronize(L.stream);
  if (e != cudaSuccess) return c->fail(e, "mcmc batch");
  std::memcpy(loglik, hp + o_out, ob);
  statuses((const int *)(hp + o_st), n, status);
  return GWGPU_OK;
}

int gwgpu_batch_set_tile(gwgpu_context *c, int tile) {
  if (!c || tile < 0 || (tile > 0 && (tile % 256) != 0)) return GWGPU_EINVAL;
  std::lock_guard<std::mutex> lk(c->mu);
  c->tile_override = tile;
  return GWGPU_OK;
}

int gwgpu_batch_set_blocks_per_sm(gwgpu_context *c, int blocks) {
  if (!c || (blocks != 0 && blocks != 3 && blocks != 4)) return GWGPU_EINVAL;
  std::lock_guard<std::mutex> lk(c->mu);
  c->occ_user = blocks;
  return GWGPU_OK;
}

int gwgpu_batch_last_launch_shape(gwgpu_context *c, int *tile, int *blocks_per_sm, int *grid) {
  if (!c) return GWGPU_EINVAL;
  std::lock_guard<std::mutex> lk(c->mu);
  if (tile) *tile = c->last_shape[0];
  if (blocks_per_sm) *blocks_per_sm = c->last_shape[1];
  if (grid) *grid = c->last_shape[2];
  return GWGPU_OK;
}

int gwgpu_batch_timing(gwgpu_context *c, int on) {
  if (!c) return GWGPU_EINVAL;
  std::lock_guard<std::mutex> lk(c->mu);
  if (on && !c->t_ev[0])
    for (int i = 0; i < 3; i++) cudaEventCreate(&c->t_ev[i]);
  c->timing = on != 0;
  return GWGPU_OK;
}

int gwgpu_batch_last_timing(gwgpu_context *c, float *prologue_ms, float *kernel_ms) {
  if (!c || !c->t_ev[0]) return GWGPU_EINVAL;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaError_t e = cudaEventSynchronize(c->t_ev[2]);
  if (e != cudaSuccess) return c->fail(e, "timing");
  float a = 0, b = 0;
  cudaEventElapsedTime(&a, c->t_ev[0], c->t_ev[1]);
  cudaEventElapsedTime(&b, c->t_ev[1], c->t_ev[2]);
  if (prologue_ms) *prologue_ms = a;
  if (kernel_ms) *kernel_ms = b;
  return GWGPU_OK;
}

int gwgpu_batch_use_graphs(gwgpu_context *c, int on) {
  if (!c) return GWGPU_EINVAL;
  std::lock_guard<std::mutex> lk(c->mu);
  c->use_graphs = on != 0;
  return GWGPU_OK;
}

// Time each candidate tile on this batch (device arrays, results discarded)
// and remember the fastest for its (precision, detectors, grid length) class.
int gwgpu_batch_autotune(gwgpu_context *c, const gwgpu_gen_params *d_params, const int *d_approx, int n,
                         const int *h_handles, int ndet, double T_segment, int precision, double *d_out, int *d_status,
                         int *best_tile, float *best_ms) {
  if (!c || !d_params || !d_approx || !h_handles || !d_out || !d_status || n < 1 || ndet < 1 || ndet > gwt::kMaxDet)
    return GWGPU_EINVAL;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaSetDevice(c->device);
  gwb::Lane &L = c->lane0();
  const int mixed = precision == GWGPU_PREC_MIXED;
  const gwgpu_context::Stream *s0 = c->get_stream(h_handles[0]);
  if (!s0) return GWGPU_ENOTFOUND;
  static const int cand_mixed[] = {1024, 2048, 4096, 8192, 16384}, cand_fp64[] = {256, 512, 1024, 2048, 4096};
  const int *cand = mixed ? cand_mixed : cand_fp64;
  // launch shapes: bin tile x resident blocks per SM of the fused kernel
  // (the mixed form's register bound for 3 or 4 blocks of 256 threads)
  const int occs_mixed[] = {3, 4}, occs_fp64[] = {0};
  const int *occs = mixed ? occs_mixed : occs_fp64;
  const int nocc = mixed ? 2 : 1;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int best = 0, best_occ = 0;
  float bms = 1e30f;
  for (int ci = 0; ci < 5 * nocc; ci++) {
    int tile = cand[ci / nocc];
    c->occ_override = occs[ci % nocc];
    int st = gwb::enqueue_batch(c, L, d_params, d_approx, n, h_handles, ndet, T_segment, precision, d_out, d_status,
                                tile, false);  // warm-up and plan
    if (st) {
      c->occ_override = 0;
      return st;
    }
    // the fastest of three timings of two launches each (a shared GPU's
    // clocks and neighbours make single timings noisy)
    float ms = 1e30f;
    for (int rep = 0; rep < 3; rep++) {
      cudaEventRecord(e0, L.stream);
      for (int r = 0; r < 2; r++)
        gwb::enqueue_batch(c, L, d_params, d_approx, n, h_handles, ndet, T_segment, precision, d_out, d_status, tile,
                           false);
      cudaEventRecord(e1, L.stream);
      cudaError_t e = cudaEventSynchronize(e1);
      if (e != cudaSuccess) {
        c->occ_override = 0;
        return c->fail(e, "autotune");
      }
      float t = 0;
      cudaEventElapsedTime(&t, e0, e1);
      ms = std::min(ms, t / 2);
    }
    if (ms < bms) {
      bms = ms;
      best = tile;
      best_occ = c->occ_override;
    }
  }
  c->occ_override = 0;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const std::string tk = gwb::tune_key(c, mixed, ndet, h_handles, n);
  c->tuned[tk] = best;
  if (mixed) c->tuned_occ[tk] = best_occ;
  if (best_tile) *best_tile = best;
  if (best_ms) *best_ms = bms;
  return GWGPU_OK;
}

}  // extern "C"
