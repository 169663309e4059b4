// batch_internal.h -- host-side plan of a batched launch (item list on the device).
#pragma once

#include <string>

#include "kernels.h"

struct gwgpu_context;

namespace gwb {

struct Plan {
  std::string key;
  int n = 0, ndet = 0, tile = 0, nitems = 0;
  gwk::Item *items = nullptr;
  int *item_start = nullptr, *item_count = nullptr, *handles = nullptr;
};

int default_tile(int mixed);
int plan_batch(gwgpu_context *c, int n, const int *handles, int ndet, int tile, Plan &pl);
int enqueue_batch(gwgpu_context *c, const gwgpu_gen_params *d_params, const int *d_approx, int n,
                  const int *h_handles, int ndet, double T_segment, int tc_from_segment, int precision,
                  double *d_out, int *d_status, int tile);

}  // namespace gwb
