// batch_internal.h -- host-side state of batched launches: the item plan, the
// per-lane scratch (so several batches can be in flight on separate streams),
// captured CUDA graphs and the tile autotuner's choices.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include "kernels.h"

struct gwgpu_context;

namespace gwb {

struct Plan {
  bool valid = false;  // built for the lane's current batch shape and tile
  int n = 0, ndet = 0, tile = 0, nitems = 0;
  void *mem = nullptr;
  size_t cap = 0;
  gwk::Item *items = nullptr;
  int *item_start = nullptr, *item_count = nullptr, *handles = nullptr;
  int *order = nullptr;  // kOrderBuckets x nitems: the work order the prologue writes for each launch
};

// Scratch of one in-flight batch.  Owned by the context (lane 0, the context
// stream) or by a serving lane.
struct Lane {
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  Plan plan;
  void *work = nullptr;  // Request/MixedReq[n], partials, counters
  size_t work_cap = 0;
  void *hio = nullptr, *dio = nullptr;  // staging for the host-array entry points
  size_t io_cap = 0;
  // captured launch sequences by (pointers, shape), least recently used ones
  // dropped beyond kMaxGraphs: a caller rotating through many buffer sets
  // keeps a bounded number of executable graphs
  struct Graph {
    cudaGraphExec_t exec;
    uint64_t used;
  };
  std::map<std::string, Graph> graphs;
  uint64_t graph_tick = 0;
  size_t bytes = 0;  // device bytes held (budget accounting)
  // the last batch shape (handles, sizes, registration epoch, precision) and
  // its tuning class
  struct Shape {
    std::vector<int> handles;
    int n = -1, ndet = -1, mixed = -1;
    uint64_t epoch = ~0ull;
  } shape;
  std::string tk;
};

constexpr size_t kMaxGraphs = 8;

int default_tile(int mixed);
// Tile for one launch: explicit override, else the autotuned choice for this
// batch's tuning class (key), else the default.
int choose_tile(gwgpu_context *c, int mixed, const std::string &key);
// Key of the tuning tables: precision, detectors, the length class of the
// batch's longest grid, and whether its requests' grids differ.
std::string tune_key(gwgpu_context *c, int mixed, int ndet, const int *h_handles, int n);
int plan_batch(gwgpu_context *c, Lane &L, int n, const int *handles, int ndet, int tile);
// Copies around a launch (pinned host buffers of the lane): before it, the
// inputs host -> device; after it, the outputs device -> host.
struct BatchCopies {
  const void *h2d_src;
  void *h2d_dst;
  size_t h2d_bytes;
  void *d2h_dst;
  const void *d2h_src;
  size_t d2h_bytes;
};
// Enqueue prologue + fused kernel of n requests on L.stream (device arrays).
// use_graph: capture/replay the launch sequence for this exact shape, with
// the copies of io (may be null) inside the same graph.  status_out (null:
// d_status) receives each request's final status; d_status is the working
// array the items flag atomically and must be device memory.
int enqueue_batch(gwgpu_context *c, Lane &L, const gwgpu_gen_params *d_params, const int *d_approx, int n,
                  const int *h_handles, int ndet, double T_segment, int precision, double *d_out, int *d_status,
                  int tile, bool use_graph, const BatchCopies *io = nullptr, int *status_out = nullptr);
void lane_release(gwgpu_context *c, Lane &L);

}  // namespace gwb
