// serve.cu -- continuous batching of log-likelihood requests.
//
// Requests from many chains, temperatures and independent ensembles are
// submitted one at a time (or in bursts) into request slots.  A scheduler
// thread keeps up to `lanes` batches in flight on separate CUDA streams: as
// soon as a lane is free it takes every queued request that fits (up to
// max_batch, and within the HBM admission budget) and launches the fused
// prologue + bin kernels on device-resident data, PSDs, tables and detector
// geometry; requests that arrive while others run are admitted into the next
// launch, so their work overlaps on the device.  A finished lane's results
// are copied to pinned memory and each slot is completed with its
// submit -> result-visible latency.  Every device wait is an event query; the
// host never blocks the device.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/gwgpu.h"
#include "batch_internal.h"
#include "capi_internal.h"

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

enum { kFree = 0, kQueued = 1, kInflight = 2, kDone = 3 };

struct Slot {
  gwgpu_gen_params p;
  int approx = 0, ndet = 0;
  int handles[gwt::kMaxDet] = {0};
  uint64_t ticket = 0;
  double t_submit = 0, t_done = 0;
  int state = kFree;
  double ll = 0;
  int status = 0;
};

struct ServeLane {
  gwb::Lane L;
  cudaEvent_t ev = nullptr;
  std::vector<int> ids;
  bool busy = false;
  size_t reserved = 0;
  char *h = nullptr;  // pinned: params | approx | handles | out | status
  char *d = nullptr;
  size_t cap = 0;
};

}  // namespace

struct gwgpu_server {
  gwgpu_context *ctx = nullptr;
  gwgpu_server_config cfg;
  std::vector<Slot> slots;
  std::deque<int> queue;
  std::vector<int> free_list;
  uint64_t generation = 1;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::thread worker;
  std::atomic<bool> stop{false};
  std::vector<ServeLane> lanes;
  std::vector<double> latency;
  uint64_t completed = 0, launches = 0;
  size_t inflight_bytes = 0, budget = 0;
  int worker_error = 0;
};

namespace {

size_t request_bytes(int precision, int N, int tile) {  // device scratch held by one in-flight request
  size_t items = (size_t)(N + tile - 1) / tile;
  return (precision == GWGPU_PREC_MIXED ? sizeof(gwt::MixedReq) : sizeof(gwt::Request)) +
         items * (sizeof(double) * gwk::kAcc + sizeof(gwk::Item)) + sizeof(gwgpu_gen_params) + 64;
}

// Layout of a lane's pinned and device I/O buffers for n requests: every
// array starts on a 256-byte boundary (the log L array is read and written as
// doubles by the kernels).
struct IoLayout {
  size_t params, approx, handles, out, status, total;
};
IoLayout io_layout(int n) {
  auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
  IoLayout o;
  o.params = 0;
  o.approx = up(sizeof(gwgpu_gen_params) * (size_t)n);
  o.handles = o.approx + up(sizeof(int) * (size_t)n);
  o.out = o.handles + up(sizeof(int) * (size_t)n * gwt::kMaxDet);
  o.status = o.out + up(sizeof(double) * (size_t)n);
  o.total = o.status + up(sizeof(int) * (size_t)n);
  return o;
}

int lane_io(gwgpu_context *c, ServeLane &l, size_t bytes) {
  if (l.cap >= bytes) return GWGPU_OK;
  if (l.h) cudaFreeHost(l.h);
  c->dfree(l.d);
  l.h = l.d = nullptr;
  size_t nb = std::max(bytes, (size_t)1 << 20);
  if (cudaMallocHost((void **)&l.h, nb) != cudaSuccess) return GWGPU_ECUDA;
  int st = c->dalloc((void **)&l.d, nb, "serve io");
  if (st) return st;
  l.cap = nb;
  return GWGPU_OK;
}

// Complete the lane's requests: with its results when cuda_error is 0, else
// every request fails with GWGPU_ECUDA.
void retire(gwgpu_server *s, ServeLane &l, int cuda_error) {
  const int n = (int)l.ids.size();
  const IoLayout io = io_layout(n);
  const double *out = (const double *)(l.h + io.out);
  const int *st = (const int *)(l.h + io.status);
  double t = now_s();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    for (int j = 0; j < n; j++) {
      Slot &sl = s->slots[l.ids[j]];
      if (cuda_error) {
        sl.ll = NAN;
        sl.status = GWGPU_ECUDA;
      } else {
        sl.ll = out[j];
        sl.status = gwk::status_code(st[j]);
      }
      sl.t_done = t;
      sl.state = kDone;
      s->latency.push_back(t - sl.t_submit);
      s->completed++;
    }
    s->inflight_bytes -= l.reserved;
    if (cuda_error) s->worker_error = GWGPU_ECUDA;
  }
  l.reserved = 0;
  l.ids.clear();
  l.busy = false;
  s->cv_done.notify_all();
}

int launch(gwgpu_server *s, ServeLane &l) {
  gwgpu_context *c = s->ctx;
  const int n = (int)l.ids.size();
  const int ndet = s->slots[l.ids[0]].ndet;
  const IoLayout io = io_layout(n);
  std::lock_guard<std::mutex> ck(c->mu);
  int st = lane_io(c, l, io.total);
  if (st) return st;
  gwgpu_gen_params *hp = (gwgpu_gen_params *)(l.h + io.params);
  int *ha = (int *)(l.h + io.approx);
  int *hh = (int *)(l.h + io.handles);
  for (int j = 0; j < n; j++) {
    const Slot &sl = s->slots[l.ids[j]];
    hp[j] = sl.p;
    ha[j] = sl.approx;
    for (int d = 0; d < ndet; d++) hh[j * ndet + d] = sl.handles[d];
  }
  // the kernels read the parameters from, and write log L and the status
  // into, the lane's mapped pinned buffer; the working status stays on the device
  char *hm = nullptr;
  cudaError_t e = cudaHostGetDevicePointer((void **)&hm, l.h, 0);
  if (e != cudaSuccess) return c->fail(e, "serve staging mapping");
  st = gwb::enqueue_batch(c, l.L, (const gwgpu_gen_params *)(hm + io.params), (const int *)(hm + io.approx), n, hh,
                          ndet, s->cfg.T_segment, s->cfg.precision, (double *)(hm + io.out),
                          (int *)(l.d + io.status), 0, false, nullptr, (int *)(hm + io.status));
  if (st) return st;
  e = cudaEventRecord(l.ev, l.L.stream);
  if (e != cudaSuccess) return c->fail(e, "serve launch");
  l.busy = true;
  s->launches++;
  return GWGPU_OK;
}

void worker_loop(gwgpu_server *s) {
  cudaSetDevice(s->ctx->device);
  while (!s->stop.load()) {
    bool did = false;
    for (auto &l : s->lanes) {
      if (!l.busy) continue;
      cudaError_t q = cudaEventQuery(l.ev);
      if (q == cudaSuccess) {
        retire(s, l, 0);
        did = true;
      } else if (q != cudaErrorNotReady) {  // fail this lane's requests instead of waiting on it forever
        retire(s, l, 1);
        did = true;
      }
    }
    for (auto &l : s->lanes) {
      if (l.busy) continue;
      {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->queue.empty()) break;
        int ndet = s->slots[s->queue.front()].ndet;
        size_t take_bytes = 0;
        while (!s->queue.empty() && (int)l.ids.size() < s->cfg.max_batch) {
          int id = s->queue.front();
          const Slot &sl = s->slots[id];
          if (sl.ndet != ndet) break;
          const gwgpu_context::Stream *st0 = s->ctx->get_stream(sl.handles[0]);
          size_t rb = request_bytes(s->cfg.precision, st0 ? st0->dev.N : 0, s->cfg.precision ? 4096 : 1024);
          if (s->budget && s->inflight_bytes + take_bytes + rb > s->budget && !l.ids.empty()) break;
          if (s->budget && s->inflight_bytes + take_bytes + rb > s->budget && s->inflight_bytes > 0) break;
          take_bytes += rb;
          s->queue.pop_front();
          s->slots[id].state = kInflight;
          l.ids.push_back(id);
        }
        s->inflight_bytes += take_bytes;
        l.reserved = take_bytes;
      }
      if (l.ids.empty()) break;
      int st = launch(s, l);
      if (st) {  // fail the batch, keep serving
        std::lock_guard<std::mutex> lk(s->mu);
        for (int id : l.ids) {
          s->slots[id].status = st;
          s->slots[id].ll = NAN;
          s->slots[id].state = kDone;
          s->slots[id].t_done = now_s();
        }
        s->inflight_bytes -= l.reserved;
        l.ids.clear();
        l.reserved = 0;
        s->worker_error = st;
        s->cv_done.notify_all();
      }
      did = true;
    }
    if (!did) {
      std::unique_lock<std::mutex> lk(s->mu);
      bool any_busy = false;
      for (auto &l : s->lanes) any_busy |= l.busy;
      if (s->queue.empty() && !any_busy)
        s->cv_work.wait_for(lk, std::chrono::microseconds(500));
      else if (s->queue.empty())
        lk.unlock(), std::this_thread::yield();
    }
  }
}

}  // namespace

extern "C" {

int gwgpu_server_create(gwgpu_context *c, const gwgpu_server_config *cfg, gwgpu_server **out) {
  if (!c || !cfg || !out || cfg->max_inflight < 1 || cfg->max_batch < 1 || cfg->lanes < 1 || cfg->lanes > 16)
    return GWGPU_EINVAL;
  cudaSetDevice(c->device);
  gwgpu_server *s = new gwgpu_server();
  s->ctx = c;
  s->cfg = *cfg;
  s->budget = cfg->hbm_budget_bytes ? cfg->hbm_budget_bytes : c->budget;
  s->slots.resize(cfg->max_inflight);
  for (int i = cfg->max_inflight - 1; i >= 0; i--) s->free_list.push_back(i);
  s->lanes.resize(cfg->lanes);
  for (auto &l : s->lanes) {
    cudaStreamCreateWithFlags(&l.L.stream, cudaStreamNonBlocking);
    l.L.own_stream = true;
    cudaEventCreateWithFlags(&l.ev, cudaEventDisableTiming);
  }
  s->worker = std::thread(worker_loop, s);
  *out = s;
  return GWGPU_OK;
}

int gwgpu_server_destroy(gwgpu_server *s) {
  if (!s) return GWGPU_EINVAL;
  s->stop.store(true);
  s->cv_work.notify_all();
  if (s->worker.joinable()) s->worker.join();
  std::lock_guard<std::mutex> ck(s->ctx->mu);
  for (auto &l : s->lanes) {
    gwb::lane_release(s->ctx, l.L);
    if (l.ev) cudaEventDestroy(l.ev);
    if (l.h) cudaFreeHost(l.h);
    s->ctx->dfree(l.d);
  }
  delete s;
  return GWGPU_OK;
}

static int submit_at(gwgpu_server *s, const gwgpu_gen_params *p, int approx, const int *handles, int ndet, double t,
                     uint64_t *ticket) {
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->free_list.empty()) return GWGPU_EBUSY;
  int id = s->free_list.back();
  s->free_list.pop_back();
  Slot &sl = s->slots[id];
  sl.p = *p;
  sl.approx = approx;
  sl.ndet = ndet;
  for (int d = 0; d < ndet; d++) sl.handles[d] = handles[d];
  sl.ticket = (s->generation++ << 24) | (uint64_t)id;
  sl.t_submit = t;
  sl.state = kQueued;
  s->queue.push_back(id);
  *ticket = sl.ticket;
  s->cv_work.notify_one();
  return GWGPU_OK;
}

int gwgpu_server_submit(gwgpu_server *s, const gwgpu_gen_params *p, int approx, const int *handles, int ndet,
                        uint64_t *ticket) {
  if (!s || !p || !handles || !ticket || ndet < 1 || ndet > gwt::kMaxDet || (approx != 0 && approx != 1))
    return GWGPU_EINVAL;
  for (int d = 0; d < ndet; d++)
    if (!s->ctx->get_stream(handles[d])) return GWGPU_ENOTFOUND;
  return submit_at(s, p, approx, handles, ndet, now_s(), ticket);
}

static int collect(gwgpu_server *s, uint64_t ticket, double *ll, int *status) {  // s->mu held
  int id = (int)(ticket & 0xffffff);
  if (id < 0 || id >= (int)s->slots.size()) return GWGPU_ENOTFOUND;
  Slot &sl = s->slots[id];
  if (sl.ticket != ticket || sl.state == kFree) return GWGPU_ENOTFOUND;
  if (sl.state != kDone) return GWGPU_EBUSY;
  if (ll) *ll = sl.ll;
  if (status) *status = sl.status;
  sl.state = kFree;
  s->free_list.push_back(id);
  return GWGPU_OK;
}

int gwgpu_server_poll(gwgpu_server *s, uint64_t ticket, double *ll, int *status) {
  if (!s) return GWGPU_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  return collect(s, ticket, ll, status);
}

int gwgpu_server_wait(gwgpu_server *s, uint64_t ticket, int timeout_ms, double *ll, int *status) {
  if (!s) return GWGPU_EINVAL;
  std::unique_lock<std::mutex> lk(s->mu);
  auto deadline = std::chrono::steady_clock::now() + std::chrono::milliseconds(timeout_ms);
  for (;;) {
    int st = collect(s, ticket, ll, status);
    if (st != GWGPU_EBUSY) return st;
    if (s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout) {
      st = collect(s, ticket, ll, status);
      return st == GWGPU_EBUSY ? GWGPU_ETIMEDOUT : st;
    }
  }
}

int gwgpu_server_stats(gwgpu_server *s, double *p50, double *p99, uint64_t *completed, uint64_t *launches) {
  if (!s) return GWGPU_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  std::vector<double> v = s->latency;
  double a = 0, b = 0;
  if (!v.empty()) {
    size_t i50 = (size_t)(0.50 * (v.size() - 1)), i99 = (size_t)(0.99 * (v.size() - 1));
    std::nth_element(v.begin(), v.begin() + i50, v.end());
    a = v[i50];
    std::nth_element(v.begin(), v.begin() + i99, v.end());
    b = v[i99];
  }
  if (p50) *p50 = a;
  if (p99) *p99 = b;
  if (completed) *completed = s->completed;
  if (launches) *launches = s->launches;
  return GWGPU_OK;
}

int gwgpu_server_reset_stats(gwgpu_server *s) {
  if (!s) return GWGPU_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  s->latency.clear();
  s->completed = 0;
  s->launches = 0;
  return GWGPU_OK;
}

int gwgpu_server_drive(gwgpu_server *s, const gwgpu_gen_params *params, const int *approx, const int *handles,
                       int ndet, const double *arrival_s, int n, double *loglik, int *status, double *latency_s,
                       double *wall_s) {
  if (!s || !params || !approx || !handles || !arrival_s || n < 1 || !loglik) return GWGPU_EINVAL;
  for (int i = 0; i < n * ndet; i++)
    if (!s->ctx->get_stream(handles[i])) return GWGPU_ENOTFOUND;
  std::vector<uint64_t> tickets(n, 0);
  double t0 = now_s();
  // no completion for this long means the device or the worker stopped: give up
  const double stall_limit_s = 120.0;
  double last_progress = t0;
  int next_collect = 0;
  auto drain = [&](bool block) {
    while (next_collect < n && tickets[next_collect] != 0) {
      int st;
      double ll;
      int rc = block ? gwgpu_server_wait(s, tickets[next_collect], 1000, &ll, &st)
                     : gwgpu_server_poll(s, tickets[next_collect], &ll, &st);
      if (rc == GWGPU_EBUSY || (block && rc == GWGPU_ETIMEDOUT)) return false;
      loglik[next_collect] = rc == GWGPU_OK ? ll : NAN;
      if (status) status[next_collect] = rc == GWGPU_OK ? st : rc;
      next_collect++;
      last_progress = now_s();
    }
    return true;
  };
  for (int i = 0; i < n; i++) {
    double ta = t0 + arrival_s[i];
    while (now_s() < ta) {
      if (ta - now_s() > 2e-4) std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    for (;;) {
      int rc = submit_at(s, params + i, approx[i], handles + (size_t)i * ndet, ndet, ta, &tickets[i]);
      if (rc == GWGPU_OK) break;
      if (rc != GWGPU_EBUSY) return rc;
      drain(false);  // free slots
      if (now_s() - last_progress > stall_limit_s) return GWGPU_ETIMEDOUT;
      std::this_thread::yield();
    }
    if ((i & 63) == 0) drain(false);
  }
  while (!drain(true))
    if (now_s() - last_progress > stall_limit_s) return GWGPU_ETIMEDOUT;
  if (wall_s) *wall_s = now_s() - t0;
  if (latency_s) {
    std::lock_guard<std::mutex> lk(s->mu);
    size_t m = s->latency.size();
    for (int i = 0; i < n && (size_t)i < m; i++) latency_s[i] = s->latency[m - n + i];
  }
  return s->worker_error;
}

}  // extern "C"
