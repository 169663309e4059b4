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
//
// With device_loop set, the requests go instead into a ring in mapped pinned
// memory that a persistent kernel (gwk::launch_serve_loop) consumes as they
// are published: the submitting thread publishes, the host thread here reads
// the completion queue the kernel appends to, completes the slots, and
// relaunches the kernel while requests are outstanding (a launch's blocks
// leave when idle and after at most kLoopLife).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <climits>
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

// State of the device-resident loop: the mapped ring, the device arrays of
// its slots, and what the host knows of the kernel.
struct DeviceLoop {
  int R = 0, tile = 0, max_items = 0, ndet = 0, grid = 0;
  char *hbase = nullptr;  // pinned: ring | completions | tail | stop
  gwk::LoopReq *ring = nullptr;
  gwk::LoopDone *comp = nullptr;
  unsigned long long *tail = nullptr;
  unsigned *stop = nullptr;  // the launch id asked to leave
  void *dbase = nullptr;     // device: every per-slot array
  gwk::LoopArgs args;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev = nullptr;
  bool running = false;
  uint64_t epoch = 0;                   // stream table the running launch was given
  uint64_t published = 0, retired = 0;  // next sequence number; every one below retired is complete
  uint64_t cursor = 0;                  // next completion to read
  uint64_t tail_pub = 0;                // published, as stored for the device (atomic)
  bool spinning = false;                // the host thread polls (it also stores the tail)
  std::vector<int> slot_of;             // ring position -> server slot
  std::vector<char> complete;           // ring position's request finished
  std::vector<int> service_ns;          // device claim -> result, per completed request
  uint64_t launches = 0;
};

constexpr long long kLoopLife = 1000000000ll;  // ns: the longest a launch keeps claiming requests

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
  DeviceLoop *dl = nullptr;  // device-resident loop (cfg.device_loop)
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

// ------------------------------------------------------------ device loop
void loop_free(gwgpu_context *c, DeviceLoop *L) {
  {
    std::lock_guard<std::mutex> ck(c->mu);
    c->dfree(L->dbase);
  }
  if (L->hbase) cudaFreeHost(L->hbase);
  if (L->ev) cudaEventDestroy(L->ev);
  if (L->stream) cudaStreamDestroy(L->stream);
  delete L;
}

// Sizes the ring by the HBM budget and allocates every slot's device state.
int loop_create(gwgpu_server *s) {
  gwgpu_context *c = s->ctx;
  const gwgpu_server_config &cfg = s->cfg;
  if (cfg.precision != GWGPU_PREC_MIXED) return GWGPU_EINVAL;
  const int tile = cfg.tile > 0 ? cfg.tile : 4096;
  if (tile % 256 || tile > (1 << 20) || cfg.blocks_per_sm < 0) return GWGPU_EINVAL;
  int nmax = 0;
  {
    std::lock_guard<std::mutex> ck(c->mu);
    for (const auto &st : c->streams)
      if (st.live) nmax = std::max(nmax, st.dev.N);
  }
  if (nmax < 1) return GWGPU_EINVAL;  // register the data first
  const int max_items = (nmax + tile - 1) / tile;
  if (max_items > gwk::kLoopMaxItems) return GWGPU_ETOOLARGE;  // the claim word's item fields
  auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t per_slot = sizeof(gwt::MixedReq) + sizeof(gwt::GenParams) + sizeof(int) * (gwt::kMaxDet + 5) + 24 +
                          (size_t)max_items * sizeof(double) * gwk::kAcc;
  size_t R = (size_t)cfg.max_inflight;
  if (s->budget) R = std::min(R, s->budget / per_slot);
  if (R < 1) return GWGPU_ENOMEM;
  R = std::min(R, (size_t)(INT_MAX / max_items));  // item indices slot * max_items + t are ints
  DeviceLoop *L = new DeviceLoop();
  L->R = (int)R;
  L->tile = tile;
  L->max_items = max_items;
  L->slot_of.assign(R, -1);
  L->complete.assign(R, 0);
  // device layout
  size_t o = 0;
  const size_t o_ctl = o;
  o += up(sizeof(gwk::LoopCtl));
  const size_t o_part = o;
  o += up(sizeof(double) * gwk::kAcc * R * (size_t)max_items);
  const size_t o_mreq = o;
  o += up(sizeof(gwt::MixedReq) * R);
  const size_t o_par = o;
  o += up(sizeof(gwt::GenParams) * R);
  const size_t o_w64 = o;  // claim words, sequence numbers, claim times
  o += up(8 * 3 * R);
  const size_t o_hand = o;
  o += up(sizeof(int) * gwt::kMaxDet * R);
  const size_t o_int = o;  // approx, status, start, count, done
  o += up(sizeof(int) * 5 * R);
  int st;
  {
    std::lock_guard<std::mutex> ck(c->mu);
    st = c->dalloc(&L->dbase, o, "serve loop");
  }
  if (st) {
    delete L;
    return st;
  }
  char *d = (char *)L->dbase;
  cudaError_t e = cudaMemset(d, 0, o);
  std::vector<int> start(R);
  for (size_t i = 0; i < R; i++) start[i] = (int)(i * max_items);
  int *ints = (int *)(d + o_int);
  if (e == cudaSuccess) e = cudaMemcpy(ints + 2 * R, start.data(), sizeof(int) * R, cudaMemcpyHostToDevice);
  // mapped pinned ring, completions, tail and stop flag
  const size_t h_ring = 0, h_comp = up(sizeof(gwk::LoopReq) * R), h_tail = h_comp + up(sizeof(gwk::LoopDone) * R),
               h_total = h_tail + 256;
  if (e == cudaSuccess) e = cudaHostAlloc((void **)&L->hbase, h_total, cudaHostAllocMapped);
  if (e == cudaSuccess) memset(L->hbase, 0, h_total);
  char *hm = nullptr;
  if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **)&hm, L->hbase, 0);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&L->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&L->ev, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    int r = c->fail(e, "serve loop setup");
    loop_free(c, L);
    return r;
  }
  L->ring = (gwk::LoopReq *)(L->hbase + h_ring);
  L->comp = (gwk::LoopDone *)(L->hbase + h_comp);
  L->tail = (unsigned long long *)(L->hbase + h_tail);
  L->stop = (unsigned *)(L->hbase + h_tail + 64);
  gwk::LoopArgs &A = L->args;
  A = gwk::LoopArgs{};
  A.a.req = nullptr;
  A.a.mreq = (const gwt::MixedReq *)(d + o_mreq);
  A.a.handles = (const int *)(d + o_hand);
  A.a.items = nullptr;
  A.a.bucket_fill = nullptr;
  A.a.bucket_items = nullptr;
  A.a.nitems = 0;
  A.a.item_start = ints + 2 * R;
  A.a.item_count = ints + 3 * R;
  A.a.tile = tile;
  A.a.item_counter = nullptr;
  A.a.req_done = (unsigned *)(ints + 4 * R);
  A.a.partials = (double *)(d + o_part);
  A.a.out = nullptr;
  A.a.status = ints + 1 * R;
  A.a.status_out = nullptr;
  A.ring = (const gwk::LoopReq *)(hm + h_ring);
  A.comp = (gwk::LoopDone *)(hm + h_comp);
  A.tail = (const unsigned long long *)(hm + h_tail);
  A.stop = (const unsigned *)(hm + h_tail + 64);
  A.ctl = (gwk::LoopCtl *)(d + o_ctl);
  A.dparams = (gwt::GenParams *)(d + o_par);
  A.dapprox = ints;
  A.dhandles = (int *)(d + o_hand);
  A.dcount = ints + 3 * R;
  A.dwork = (unsigned long long *)(d + o_w64);
  A.dseq = A.dwork + R;
  A.dclaim = (long long *)(A.dwork + 2 * R);
  A.R = (int)R;
  A.max_items = max_items;
  A.T_segment = cfg.T_segment;
  A.idle_ns = 1000ll * (cfg.idle_us > 0 ? cfg.idle_us : 20000);
  A.life_ns = kLoopLife;
  s->dl = L;
  return GWGPU_OK;
}

// Launches the loop on the current stream table (s->mu held).
int loop_launch(gwgpu_server *s) {
  DeviceLoop &L = *s->dl;
  gwgpu_context *c = s->ctx;
  std::lock_guard<std::mutex> ck(c->mu);
  if (!L.grid) {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    int nb = std::max(1, gwk::serve_loop_blocks_per_sm(L.ndet));
    if (s->cfg.blocks_per_sm > 0) nb = std::min(nb, s->cfg.blocks_per_sm);
    L.grid = nb * std::max(1, sms);
  }
  L.args.a.ndet = L.ndet;
  L.args.a.streams = c->streams_dev;
  L.args.a.tables = c->tables;
  L.args.qnm = c->qnm_dev;
  L.epoch = c->streams_epoch;
  L.args.launch_id = (unsigned)(L.launches + 1);
  cudaError_t e = gwk::launch_serve_loop(L.args, L.grid, L.stream);
  if (e == cudaSuccess) e = cudaEventRecord(L.ev, L.stream);
  if (e != cudaSuccess) return c->fail(e, "serve loop launch");
  L.running = true;
  L.launches++;
  s->launches++;
  return GWGPU_OK;
}

// Completes every outstanding request with status st (the loop failed).
void loop_fail_outstanding(gwgpu_server *s, int st) {
  DeviceLoop &L = *s->dl;
  const double t = now_s();
  for (uint64_t q = L.retired; q < L.published; q++) {
    const int pos = (int)(q % L.R);
    if (L.complete[pos]) continue;
    Slot &sl = s->slots[L.slot_of[pos]];
    sl.ll = NAN;
    sl.status = st;
    sl.t_done = t;
    sl.state = kDone;
    s->completed++;
    L.complete[pos] = 1;
  }
  L.retired = L.published;
  s->worker_error = st;
  s->cv_done.notify_all();
}

// Raises the device-visible tail to p (any thread; the largest value wins).
void loop_store_tail(DeviceLoop &L, uint64_t p) {
  unsigned long long cur = __atomic_load_n(L.tail, __ATOMIC_RELAXED);
  while (cur < p && !__atomic_compare_exchange_n(L.tail, &cur, (unsigned long long)p, false, __ATOMIC_RELEASE,
                                                 __ATOMIC_RELAXED)) {
  }
}

// Publishes queued requests into free ring positions (s->mu held).  While
// the running launch has an older stream table the requests wait for the
// next launch and the running one is told to leave once idle.
void loop_publish(gwgpu_server *s) {
  DeviceLoop &L = *s->dl;
  const bool stale = __atomic_load_n(&s->ctx->streams_epoch, __ATOMIC_RELAXED) != L.epoch;
  if (L.running && stale) {
    __atomic_store_n(L.stop, L.args.launch_id, __ATOMIC_RELEASE);
    return;
  }
  uint64_t p = L.published;
  while (!s->queue.empty() && p - L.retired < (uint64_t)L.R) {
    const int id = s->queue.front();
    s->queue.pop_front();
    Slot &sl = s->slots[id];
    const int pos = (int)(p % (uint64_t)L.R);
    gwk::LoopReq &e = L.ring[pos];
    memcpy(&e.p, &sl.p, sizeof(e.p));
    e.approx = sl.approx;
    for (int d = 0; d < gwt::kMaxDet; d++) e.handles[d] = d < sl.ndet ? sl.handles[d] : 0;
    L.slot_of[pos] = id;
    L.complete[pos] = 0;
    sl.state = kInflight;
    p++;
  }
  if (p != L.published) {
    __atomic_store_n(&L.published, p, __ATOMIC_RELEASE);
    // while the host thread polls it stores the tail (one store for many
    // requests: the device reads that line); otherwise store it here
    if (!__atomic_load_n(&L.spinning, __ATOMIC_ACQUIRE)) loop_store_tail(L, p);
  }
}

// Keeps a launch running while requests are outstanding (s->mu held);
// check_done: first find out whether the running launch has finished.
int loop_keepalive(gwgpu_server *s, bool check_done) {
  DeviceLoop &L = *s->dl;
  if (L.running && check_done) {
    const cudaError_t q = cudaEventQuery(L.ev);
    if (q == cudaSuccess) {
      L.running = false;
    } else if (q != cudaErrorNotReady) {
      L.running = false;
      s->ctx->fail(q, "serve loop");
      loop_fail_outstanding(s, GWGPU_ECUDA);
      return GWGPU_ECUDA;
    }
  }
  if (!L.running && L.published > L.retired) {
    const int st = loop_launch(s);
    if (st) {
      loop_fail_outstanding(s, st);
      return st;
    }
  }
  return GWGPU_OK;
}

// Reads the completions the device has appended, in order (s->mu held).
int loop_collect(gwgpu_server *s) {
  DeviceLoop &L = *s->dl;
  int n = 0;
  double t = -1;
  for (;;) {
    const gwk::LoopDone &e = L.comp[L.cursor % (uint64_t)L.R];
    if (__atomic_load_n(&e.tag, __ATOMIC_ACQUIRE) != L.cursor + 1) break;
    if (t < 0) t = now_s();
    const int pos = (int)(e.seq % (uint64_t)L.R);
    if (e.seq < L.retired || e.seq >= L.published || L.complete[pos] || L.slot_of[pos] < 0) {
      // not a request outstanding in the ring: the completion is dropped
      s->worker_error = GWGPU_ECUDA;
      L.cursor++;
      continue;
    }
    Slot &sl = s->slots[L.slot_of[pos]];
    sl.ll = e.ll;
    sl.status = gwk::status_code(e.status);
    sl.t_done = t;
    sl.state = kDone;
    s->latency.push_back(t - sl.t_submit);
    L.service_ns.push_back(e.service_ns);
    s->completed++;
    L.complete[pos] = 1;
    L.cursor++;
    n++;
  }
  while (L.retired < L.published && L.complete[L.retired % (uint64_t)L.R]) L.retired++;
  if (n) s->cv_done.notify_all();
  return n;
}

// The host side of the loop: the completion queue is peeked without the
// lock (only this thread advances its cursor), the lock is taken to consume
// completions and publish what the ring has room for, and whether the
// launch has finished is asked at most every kLoopTick seconds, so that
// submitting threads are not kept from the lock.
constexpr double kLoopTick = 50e-6;
constexpr double kLoopGather = 2e-6;  // a completion waits at most this long for others to be read with it
constexpr int kLoopGatherN = 32;
bool loop_ready(const DeviceLoop &L, uint64_t c) {
  return __atomic_load_n(&L.comp[c % (uint64_t)L.R].tag, __ATOMIC_ACQUIRE) == c + 1;
}
void loop_worker(gwgpu_server *s) {
  cudaSetDevice(s->ctx->device);
  DeviceLoop &L = *s->dl;
  double next_tick = 0, first_seen = -1;
  uint64_t stored = 0;
  while (!s->stop.load()) {
    // the tail for what the submitting threads published since the last store
    const uint64_t pub = __atomic_load_n(&L.published, __ATOMIC_ACQUIRE);
    if (pub != stored) {
      loop_store_tail(L, pub);
      stored = pub;
    }
    const bool have = loop_ready(L, L.cursor);
    const double t = now_s();
    if (have && first_seen < 0) first_seen = t;
    const bool take = have && (t - first_seen >= kLoopGather || loop_ready(L, L.cursor + kLoopGatherN - 1));
    const bool tick = t >= next_tick;
    if (!take && !tick) {
      std::this_thread::yield();
      continue;
    }
    std::unique_lock<std::mutex> lk(s->mu);
    if (take) {
      loop_collect(s);
      first_seen = -1;
    }
    loop_publish(s);
    if (tick) next_tick = t + kLoopTick;
    loop_keepalive(s, tick);
    const bool busy = L.published > L.retired || !s->queue.empty();
    if (!busy) {
      __atomic_store_n(&L.spinning, false, __ATOMIC_RELEASE);
      loop_store_tail(L, L.published);  // nothing left for this thread to store
      s->cv_work.wait_for(lk, std::chrono::microseconds(500));
      __atomic_store_n(&L.spinning, true, __ATOMIC_RELEASE);
    }
  }
  __atomic_store_n(&L.spinning, false, __ATOMIC_RELEASE);
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
  if (cfg->device_loop) {
    int st = loop_create(s);
    if (st) {
      delete s;
      return st;
    }
    s->worker = std::thread(loop_worker, s);
    *out = s;
    return GWGPU_OK;
  }
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
  if (s->dl) {
    // the loop's blocks leave once they find no work; its memory is freed
    // after the launch has finished (kept, if it has not within 30 s)
    DeviceLoop *L = s->dl;
    __atomic_store_n(L->stop, L->args.launch_id, __ATOMIC_RELEASE);
    bool done = !L->running;
    for (int i = 0; i < 30000 && !done; i++) {
      if (cudaEventQuery(L->ev) != cudaErrorNotReady) done = true;
      else std::this_thread::sleep_for(std::chrono::milliseconds(1));
    }
    int rc = GWGPU_OK;
    if (done) loop_free(s->ctx, L);
    else rc = GWGPU_ETIMEDOUT;
    delete s;
    return rc;
  }
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

// One request into a free slot and the queue (s->mu held).
static int submit_locked(gwgpu_server *s, const gwgpu_gen_params *p, int approx, const int *handles, int ndet,
                         double t, uint64_t *ticket) {
  if (s->dl) {  // one detector count per loop, grids within its item count
    DeviceLoop &L = *s->dl;
    if (L.ndet && ndet != L.ndet) return GWGPU_EINVAL;
    const gwgpu_context::Stream *st0 = s->ctx->get_stream(handles[0]);
    if (!st0 || st0->dev.N > L.max_items * L.tile) return GWGPU_ETOOLARGE;
    if (!L.ndet) L.ndet = ndet;
  }
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
  return GWGPU_OK;
}

// After submissions (s->mu held): the device loop publishes them now and is
// launched if none is running; the host scheduler's thread is woken.
static void submitted(gwgpu_server *s) {
  if (s->dl) {
    loop_publish(s);
    const int st = loop_keepalive(s, false);
    if (st) s->worker_error = st;
  }
  s->cv_work.notify_one();
}

static int submit_at(gwgpu_server *s, const gwgpu_gen_params *p, int approx, const int *handles, int ndet, double t,
                     uint64_t *ticket) {
  std::lock_guard<std::mutex> lk(s->mu);
  const int st = submit_locked(s, p, approx, handles, ndet, t, ticket);
  if (st == GWGPU_OK) submitted(s);
  return st;
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
  if (s->dl) s->dl->service_ns.clear();
  return GWGPU_OK;
}

int gwgpu_server_loop_info(gwgpu_server *s, long long info[15]) {
  if (!s || !info || !s->dl) return GWGPU_EINVAL;
  std::lock_guard<std::mutex> lk(s->mu);
  const DeviceLoop &L = *s->dl;
  unsigned ex[4] = {0, 0, 0, 0};
  unsigned long long busy[5] = {0, 0, 0, 0, 0};
  cudaMemcpy(ex, L.args.ctl->exits, sizeof(ex), cudaMemcpyDeviceToHost);
  cudaMemcpy(busy, &L.args.ctl->busy_item_ns, sizeof(busy), cudaMemcpyDeviceToHost);
  info[0] = L.R;
  info[1] = L.tile;
  info[2] = L.max_items;
  info[3] = L.grid;
  info[4] = (long long)L.launches;
  info[5] = ex[0];
  info[6] = ex[1];
  info[7] = ex[2];
  std::vector<int> v = L.service_ns;
  info[8] = info[9] = 0;
  if (!v.empty()) {
    const size_t i50 = (size_t)(0.50 * (v.size() - 1)), i99 = (size_t)(0.99 * (v.size() - 1));
    std::nth_element(v.begin(), v.begin() + i50, v.end());
    info[8] = v[i50];
    std::nth_element(v.begin(), v.begin() + i99, v.end());
    info[9] = v[i99];
  }
  for (int j = 0; j < 5; j++) info[10 + j] = (long long)busy[j];
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
  // results of the submitted requests, in request order, as far as they are
  // complete: one lock for the lot (blocking: one ticket waited for first)
  auto drain = [&](bool block) {
    if (block && next_collect < n && tickets[next_collect] != 0) {
      int st;
      double ll;
      const int rc = gwgpu_server_wait(s, tickets[next_collect], 1000, &ll, &st);
      if (rc == GWGPU_EBUSY || rc == GWGPU_ETIMEDOUT) return false;
      loglik[next_collect] = rc == GWGPU_OK ? ll : NAN;
      if (status) status[next_collect] = rc == GWGPU_OK ? st : rc;
      next_collect++;
      last_progress = now_s();
    }
    std::lock_guard<std::mutex> lk(s->mu);
    while (next_collect < n && tickets[next_collect] != 0) {
      int st;
      double ll;
      const int rc = collect(s, tickets[next_collect], &ll, &st);
      if (rc == GWGPU_EBUSY) return false;
      loglik[next_collect] = rc == GWGPU_OK ? ll : NAN;
      if (status) status[next_collect] = rc == GWGPU_OK ? st : rc;
      next_collect++;
      last_progress = now_s();
    }
    return true;
  };
  int i = 0, drained_at = 0;
  while (i < n) {
    const double ta = t0 + arrival_s[i];
    while (now_s() < ta) {
      if (ta - now_s() > 2e-4) std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    // every request due by now, under one lock (each keeps its own arrival time)
    int busy = 0;
    {
      std::lock_guard<std::mutex> lk(s->mu);
      const double now = now_s();
      int k = 0;
      for (; i < n && k < 512 && t0 + arrival_s[i] <= now; i++, k++) {
        const int rc = submit_locked(s, params + i, approx[i], handles + (size_t)i * ndet, ndet, t0 + arrival_s[i],
                                     &tickets[i]);
        if (rc == GWGPU_EBUSY) {
          busy = 1;
          break;
        }
        if (rc != GWGPU_OK) return rc;
      }
      if (k) submitted(s);
    }
    if (busy) {
      drain(false);  // free slots
      if (now_s() - last_progress > stall_limit_s) return GWGPU_ETIMEDOUT;
      std::this_thread::yield();
    }
    if (i - drained_at >= 64) {
      drain(false);
      drained_at = i;
    }
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
