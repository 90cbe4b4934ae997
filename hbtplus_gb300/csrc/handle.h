// handle.h -- the state behind an hbtu_handle (include/hbtu.h).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "device_common.cuh"

struct hbtu_handle {
  hbtu_params params;
  hbtu::DevParams dp;
  int device = 0;
  cudaStream_t own_stream = nullptr, stream = nullptr;
  std::string err;
  char *ws = nullptr;
  size_t ws_bytes = 0;
  hbtu::PassPlan *plan_host = nullptr;
  // tracing
  hbtu_stats stats{};
  bool timing = false;
  // tuning options (hbtu_set_option)
  int64_t opt_leaf_runs = 1;
  int64_t opt_schedule = 0;
  int64_t opt_layout = 1;
  int64_t opt_small = hbtu::kSmallDefault;
  int64_t opt_small_per_sm = 1;
  std::vector<cudaEvent_t> events;  // pool: 4 per pass when timing, 2 per call
};

namespace hbtu {
// The handle's device workspace grown to at least `need` bytes (its contents
// are not kept); the calls on one handle share it.
hbtu_status grow_workspace(hbtu_handle *h, size_t need);
}  // namespace hbtu
