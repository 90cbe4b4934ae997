// driver.h -- host side of the unbinding loop shared by the entry points
// (capi.cu: handle-based calls; noalloc.cu: the allocation-free call).
#pragma once
#include "device_common.cuh"

namespace hbtu {

// Staging buffers of a call (host-located inputs and outputs).
struct Staging {
  float *pos, *vel, *mass;
  long long *id;
  int *type;
  long long *order;
  float *energy;
  double *pot;
  hbtu_result *res;
  float *grad;   // 7 per particle: host-located gradient staging
  double *esum;  // per subhalo
};

// Bytes of device workspace for N particles in S subhaloes, and the carving of
// one allocation (or static array) of that size into the buffers of Ctx.
// `sibling`: also the buffers of the FP32 walk's sibling-block node layout.
size_t workspace_bytes(long long N, long long S, bool sibling = true);
void carve_workspace(char *base, Ctx &c, Staging &sg, long long N, long long S,
                     bool sibling = true);

// Loop state of subhalo s before its first pass.
void init_segment(SegState &g, int off, int n, const hbtu_state &st, long long maxsample);

// Optional tracing of the loop: per-phase marks and counters.
struct LoopHooks {
  hbtu_stats *stats = nullptr;
  virtual void mark() {}
  virtual void collect() {}
  virtual void small_begin() {}
  virtual void small_end() {}
  virtual ~LoopHooks() {}
};

void read_plan(Ctx &c);
void pass_tree_and_energies(Ctx &c, LoopHooks *hk);
void run_passes(Ctx &c, int max_passes, LoopHooks *hk);

}  // namespace hbtu
