// capi_internal.h -- the context object behind gwgpu_context* (host only).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/gwgpu.h"
#include "batch_internal.h"
#include "kernels.h"

struct gwgpu_context {
  struct Workspace {
    void *ptr = nullptr;
    size_t bytes = 0;
  };
  struct Stream {
    gwk::StreamDev dev;
    bool live = false;
    std::vector<void *> mem;
    std::vector<double> host_freqs;
    uint64_t psd_hash = 0;  // FNV-1a of the PSD bytes: detectors with equal PSDs share weights
  };
  enum { kWsWave = 0, kWsInner, kWsPlain, kWsBatch, kWsBatchItems, kWsFisher, kWsServe, kWsMaxll, kWsIngest, kWsChirp, kWsChirp32, kWsMaxllRun,
         kWsFisherRef = 40 };
  enum { kHwsPlain = 0, kHwsBatch, kHwsFisher, kHwsInner };

  int device = 0;
  size_t budget = 0, in_use = 0;
  cudaStream_t stream = nullptr;
  std::mutex mu;
  std::string last_error;
  std::map<void *, size_t> sizes;
  std::map<int, Workspace> ws, hws;
  std::vector<double> qnm_host;
  double *qnm_dev = nullptr;
  gwt::Tables tables{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, 0};
  std::vector<void *> table_mem;
  double *tm76d = nullptr;  // FP64 n^(-7/6), built on first Fisher use
  int tm76d_n = 0;
  std::vector<Stream> streams;
  gwk::StreamDev *streams_dev = nullptr;
  size_t streams_dev_cap = 0;
  unsigned *counters = nullptr;
  gwb::Lane lane;                  // scratch of the context-stream batches
  std::map<std::string, int> tuned;      // autotuned tile per (precision, detectors, grid length)
  std::map<std::string, int> tuned_occ;  // and the fused kernel's resident blocks per SM
  int tile_override = 0;
  int occ_override = 0;                  // set while the autotuner times a launch shape
  int occ_user = 0;                      // gwgpu_batch_set_blocks_per_sm (0: autotuned or default)
  int last_shape[3] = {0, 0, 0};         // tile, blocks per SM, grid of the last context-stream batch
  bool use_graphs = true;
  int chirp_n = 0;                 // grid length whose Bluestein kernel the kWsChirp workspace holds
  double chirp_kscale = 0;         // M max|B| of that kernel (the FP32 search's error scale)
  bool maxll_fp64 = false;         // maximised likelihood: FP64 transforms only (no FP32 search)
  bool prologue_serial = false;    // batched prologue: one thread per request instead of the cooperative kernel
  bool order_items = true;         // mixed batch: items in work order (written by the prologue) instead of as listed
  bool pdl = true;                 // batch kernels as programmatic dependents of the prologue
  uint64_t streams_epoch = 0;      // bumped when the device stream table changes
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  bool timing = false;                                   // per-kernel events on context-stream batches
  cudaEvent_t t_ev[3] = {nullptr, nullptr, nullptr};     // before prologue, after prologue, after bin kernel
  gwb::Lane &lane0() {
    lane.stream = stream;
    return lane;
  }

  ~gwgpu_context();
  int fail(cudaError_t e, const char *where);
  int dalloc(void **p, size_t bytes, const char *what);
  void dfree(void *p);
  int workspace(int slot, size_t bytes, void **out);
  int pinned(int slot, size_t bytes, void **out);
  int ensure_tables(int nmax);
  int ensure_tm76d(int nmax);
  int sync_streams_table();
  const Stream *get_stream(int handle) const;
  unsigned *counter(int i);
};
