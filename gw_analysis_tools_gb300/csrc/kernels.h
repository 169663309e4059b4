// kernels.h -- launch interface of the GB300 kernels (host side, no CUDA types
// beyond cudaStream_t in the launchers).
#pragma once

#include <cuda_runtime.h>

#include "../../include/gwgpu.h"
#include "phenom_mixed.h"

namespace gwk {

using gwt::GenParams;
using gwt::MixedReq;
using gwt::Request;

// One registered detector stream, as the kernels see it.
struct StreamDev {
  int det;            // detector index into the constant tables
  int N;              // bins
  int n0;             // f_k = (n0 + k) df when uniform_int
  int uniform_int;    // 1 when the grid is uniform with f0 an integer multiple of df
  double df;          // f[1] - f[0]
  double simpson_df;  // f[N/2] - f[N/2-1] (mcmc_gw.cpp:811)
  const double *freqs, *data, *psd;  // FP64 originals (data interleaved complex)
  const double *ipsd;                // 1 / psd (null: divide per bin)
  const float *dhat, *what;          // mixed-form streams (interleaved complex, real)
  double dscale, wscale;
  // integration weights of the GAUSSLEG branch (mcmc_gw.cpp:820-862), times 4
  // and f ln 10 for log10F; null for Simpson's rule (util.h:844-856)
  const double *iw;
  // content key of the whitening weights (what, wscale): streams with equal
  // keys have identical weights (same grid, PSD and integration rule)
  unsigned long long wkey;
};

struct Item {
  int req, k0;
};

constexpr int kAcc = gwt::kMaxDet * gwt::kAccPerDet;  // per-request accumulators

// Tables for the mixed form (device pointers).
struct DevTables {
  gwt::Tables t;
};

// ---- launchers (return cudaError_t of the launch) ----
cudaError_t launch_waveform(const Request &r, const double *freqs, int N, double *hp, double *hc, cudaStream_t s);
cudaError_t launch_response(const Request &r, int det_slot, int apply_shift, const double *freqs, int N, double *out,
                            cudaStream_t s);
// Simpson inner product of given response/data/psd arrays (Log_Likelihood_internal).
cudaError_t launch_inner_product(const double *data, const double *psd, const double *resp, int N, double simpson_df,
                                 double *partials, unsigned *counter, double *out, cudaStream_t s);
// The same with integration weights iw (4 w_i, times f_i ln 10 for log10F).
cudaError_t launch_inner_product_weighted(const double *data, const double *psd, const double *resp, const double *iw,
                                          int N, double *partials, unsigned *counter, double *out, cudaStream_t s);
// Plain form on uniform grids, IMRPhenomD: the waveform from the request's
// FP64 coefficients on the grid (wave64_prologue) and the n-indexed power
// tables instead of the powers, logarithm and cube root of each frequency.
struct PlainTab {
  gwt::WaveF64 w;
  gwt::Tables t;
  const double *tm76d = nullptr;  // n^(-7/6), FP64
  int use = 0;                    // 1: the tables cover every bin of the call
};
// Plain form: one request, FP64, one launch.  out[0] = log L.
cudaError_t launch_plain(const Request &r, const StreamDev *streams, int ndet, double *partials, unsigned *counter,
                         double *out, int *status, cudaStream_t s, const PlainTab *tab = nullptr);
int plain_blocks(int N);
cudaError_t plain_preload();  // loads the plain kernels' module (function-attribute query)

// Work order of a mixed batch: the prologue appends each request's items to
// the bucket of their live 256-bin passes (bucket 0: all live) as soon as it
// knows the request's cut; the bin kernel takes items bucket by bucket.
constexpr int kOrderBuckets = 65;
struct OrderArgs {
  int *fill = nullptr;          // kOrderBuckets counters (zeroed before the prologue); nullptr: no ordering
  int *items = nullptr;         // bucket b's items at items[b * nitems ...]
  const int *item_start = nullptr, *item_count = nullptr;  // per request: first item, number of items
  int nitems = 0, tile = 0;
};
// Batched: prologue (one thread per request) then the fused bin kernel.
cudaError_t launch_prologue(const GenParams *params, const int *approx, int n, const int *handles, int ndet,
                            double T_segment, int tc_from_segment, const StreamDev *streams, const double *qnm,
                            Request *req, MixedReq *mreq, int want_mixed, int *status, cudaStream_t s,
                            const OrderArgs &ord = OrderArgs(), gwt::WaveF64 *w64 = nullptr);
// One thread per request (the reference order of the prologue); kept to check
// the cooperative kernel against.
cudaError_t launch_prologue_serial(const GenParams *params, const int *approx, int n, const int *handles, int ndet,
                            double T_segment, int tc_from_segment, const StreamDev *streams, const double *qnm,
                            Request *req, MixedReq *mreq, int want_mixed, int *status, cudaStream_t s);
cudaError_t launch_mcmc_repack(const double *theta, int dim, int n, int approximant, double gmst, GenParams *out,
                               int *approx_out, cudaStream_t s);
struct BatchArgs {
  const Request *req;
  const MixedReq *mreq;
  const int *handles;  // n * ndet
  int ndet;
  const StreamDev *streams;
  const Item *items;
  const int *bucket_fill;   // work order written by the prologue (nullptr: items as listed);
  const int *bucket_items;  // partials stay indexed by item
  int nitems;
  const int *item_start;  // per request
  const int *item_count;
  int tile;               // bins per item
  unsigned *item_counter;  // dynamic item scheduler (zeroed before launch)
  unsigned *req_done;      // per request finished-item counters (zeroed before launch)
  double *partials;        // nitems * kAcc
  double *out;
  int *status;      // per-request working status (device memory: the bounds flag is set atomically)
  int *status_out;  // where the finalize writes each request's status (status itself, or mapped host memory)
  gwt::Tables tables;
  // FP64 form: per-request coefficients on the grid written by the prologue
  // (IMRPhenomD, uniform grids; null: every bin from the frequency) and the
  // FP64 n^(-7/6) table for n <= tm76d_n
  const gwt::WaveF64 *w64 = nullptr;
  const double *tm76d = nullptr;
  int tm76d_n = 0;
};
// occ: the launch shape's resident blocks per SM (mixed 3 or 4, FP64 2);
// pdl: launched as a programmatic dependent of the kernel before it on s
// (it starts launching while that one runs and waits for its completion).
cudaError_t launch_batch(const BatchArgs &a, int mixed, int grid, int occ, cudaStream_t s, bool pdl);

int batch_default_occ(int mixed);
int batch_block_size(int mixed);
int batch_occupancy(int mixed, int ndet, int occ);  // resident blocks per SM

// ---- device-resident serving loop (mixed form) ----
// The host appends requests to a ring in mapped pinned memory and publishes
// them by advancing `tail`; a persistent kernel claims them in order, runs
// the cooperative prologue for up to kLoopClaim of them per block, and
// publishes each request's live items through its claim word (sequence
// number and next item); blocks take items by compare-and-swap on the claim
// words of the oldest requests (warp-parallel scan, spread over the
// candidates), and the block that finishes a request's last item appends
// its result to a completion queue in mapped memory (tag written last,
// release at system scope).  Every block leaves when it has found no work for
// idle_ns, when the host sets `stop` and it finds no work, or when life_ns
// has passed since the launch; the host relaunches while requests are
// outstanding.  No block waits on another block.  One block in
// kLoopPollEvery reads the host's tail and stop flag at every idle poll, the
// others only after their longest nap.
constexpr int kLoopClaim = 16;
constexpr int kLoopPollEvery = 8;
constexpr int kLoopWindow = 128;  // requests past the oldest unclaimed one scanned for items
// A request's claim word: its sequence number + 1 (low 40 bits), its live
// items and the next unclaimed one (12 bits each).
constexpr int kLoopMaxItems = 4095;
inline __host__ __device__ unsigned long long loop_word(unsigned long long seq, int count, int next) {
  return (((seq + 1) & 0xffffffffffull) << 24) | ((unsigned long long)count << 12) | (unsigned long long)next;
}
struct LoopReq {  // one ring entry (host memory, written by the host)
  GenParams p;
  int approx;
  int handles[gwt::kMaxDet];
  int pad;
};
struct LoopDone {  // one completion (host memory, written by the device)
  unsigned long long tag;  // completion position + 1, written last
  unsigned long long seq;  // the request's sequence number
  double ll;
  int status;      // kernel status code (status_code() maps it)
  int service_ns;  // claimed -> result written, device global timer
};
struct LoopCtl {  // device memory: one counter per 128-byte line
  unsigned long long pro_head, pad0[15];    // requests claimed for the prologue
  unsigned long long tail_dev, pad1[15];    // the largest host tail a block has seen
  unsigned long long scan_head, pad2[15];   // every request below has all its items claimed
  unsigned long long comp_alloc, pad3[15];  // completions written
  unsigned exits[4], pad4[28];              // blocks that left: idle, stop, life
  unsigned stop_dev, pad5[31];              // the launch asked to leave, as seen by a polling block
  // where the blocks' time goes: ns in items, ns in prologues, items,
  // prologue claims, requests claimed
  unsigned long long busy_item_ns, busy_pro_ns, n_item, n_pro, n_pro_req, pad6[11];
};
struct LoopArgs {
  BatchArgs a;  // mreq, handles, ndet, streams, tile, item_start/count, req_done, partials, status, tables
  const LoopReq *ring;             // R entries (device view of mapped host memory)
  LoopDone *comp;                  // R completions (device view of mapped host memory)
  const unsigned long long *tail;  // requests published (mapped)
  const unsigned *stop;            // equal to launch_id: leave when idle (mapped)
  LoopCtl *ctl;
  GenParams *dparams;              // R: claimed requests' parameters (device copy)
  int *dapprox;                    // R
  int *dhandles;                   // R * ndet
  int *dcount;                     // R: live items per request (a.item_count)
  unsigned long long *dwork;       // R: claim word (see loop_word)
  unsigned long long *dseq;        // R: sequence number of the request in each slot
  long long *dclaim;               // R: global timer at the claim
  int R, max_items;
  double T_segment;
  const double *qnm;
  long long idle_ns, life_ns;
  unsigned launch_id;
};
// grid: blocks (at most the resident capacity, serve_loop_blocks_per_sm x SMs)
cudaError_t launch_serve_loop(const LoopArgs &L, int grid, cudaStream_t s);
int serve_loop_blocks_per_sm(int ndet);

// Per-request kernel status -> C ABI status: 0 ok, 1 invalid request (grids of
// different lengths, grid unusable by the mixed form), 4 outside the model
// domain, 5 grid beyond the per-bin power tables.
inline int status_code(int kernel_status) {
  switch (kernel_status) {
    case 0: return GWGPU_OK;
    case 1: return GWGPU_EINVAL;
    case 5: return GWGPU_ETOOLARGE;
    default: return GWGPU_EDOMAIN;
  }
}

// Host-side helpers shared with the C API.
void qnm_host_table(double *out);  // kQnmArrays x kQnmLen: x, fring, fdamp, c_fring, c_fdamp, b/d per interval

}  // namespace gwk
