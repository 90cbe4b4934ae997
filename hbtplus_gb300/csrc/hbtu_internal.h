// hbtu_internal.h -- shared declarations of the GB300 unbinding library.
//
// Data layout in HBM (one call = one batch of subhaloes, "segments"):
//   particles   pm[i]   float4 {x, y, z, mass}   comoving position, absolute
//               vel[i]  float4 {vx, vy, vz, 0}   physical velocity
//               pseg[i] int32 segment of particle i
//   energy list epid[p] int32 global particle index at list position p
//               eE[p]   float binding energy at list position p
//               (positions of segment s are [off_s, off_s + n_s); the list is
//                the reference's Elist, src/subhalo_unbind.cpp:305-308)
//   tree        per segment 2*ntree node slots in DFS preorder:
//               nd_abs  float4 {x, y, z, m} absolute centre of mass (float,
//                       as the reference stores TreeCell_t::way.s)
//               nd      WNode  32-byte record read by the walks in one load:
//                       p = {x, y, z, m} relative to the segment's frame
//                       centre (wrapped once in double, then cast);
//                       m = {len*len of the cell as float bits (0 for particle
//                       leaves; sign bit set on cells whose children are all
//                       particles), next node after the subtree (kDone when
//                       the subtree ends the tree), 0, 0}
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/hbtu.h"

namespace hbtu {

constexpr int kMaxLevels = 21;  // 63-bit octal keys (3 bits per level)

// Parameters as the reference stores them (src/config_parser.cpp:95-103).
struct DevParams {
  float eps, theta2, box, boxhalf, res, reshalf, G, Hz, a, prec;
  int periodic;
  int refine;
  int minpart;
  int precision;
  long long maxsample;
  double h, h_inv;
};

DevParams derive_params(const hbtu_params &p);

enum SegStatus : int {
  SEG_ACTIVE = 0,
  SEG_CONVERGED = 1,
  SEG_DISRUPTED = 2,
  SEG_TRIVIAL = 3,  // n <= 1: no loop (src/subhalo_unbind.cpp:275-293)
  SEG_FAILED = 4,   // pass limit reached
};
enum SegMode : int { MODE_FULL = 0, MODE_CORRECTION = 1, MODE_REFINE = 2 };

// Per-subhalo state of the unbinding loop, kept on the device.
struct SegState {
  int off, n;          // particle range
  int nbound, nlast;   // Nbound, Nlast of the reference loop
  int status, mode, corr, passes;
  int first_mb;        // first input position with Id == mostbound id
  // tree and targets of the coming pass (positions local to the segment)
  int t0, ntree, ntgt;
  float mfac;
  int nnodes;
  int tgt_mode;         // 0 tree leaves (Morton), 1 last full pass's order, 2 list order
  int coh_n;            // length of that Morton order
  int ub_lo, ub_hi;     // list block removed by the last partition, to be sorted
  int refine;           // RefineBindingEnergyOrder pending (sampling, converged)
  int levels;
  double center[3], len;
  // octal keys in 64-bit fixed point (units of 2^-kscale) when every centre
  // of the subdivision is exact in double (kfast), see k_cube
  long long kc[3], kinc;
  int kscale, kfast;
  float fc[3];  // frame centre of the relative coordinates
  // frames (HBTxyz floats)
  float ref_pos[3], ref_vel[3], old_pos[3], old_vel[3];
  float mb_pos[3], mb_vel[3];
  long long mb_id;
  float dV[3], dK;
  float mbound;
  float e0;  // Elist[0].E at disruption
  long long evals, interactions;
};

// Totals the host reads once per pass.
struct PassPlan {
  int nactive;
  int ntree_total, ntgt_total;
  int nchunks_tree;
  int max_levels;
  int nsort_total;  // elements of the unbound-part sort
  int nchunks_bound;
  int nrefine;
  int error;             // a sort's look-back wait ran out
  int max_nlast;         // longest energy list of an active subhalo
  long long inter_done;  // walk interactions summed so far, all subhaloes
};

#define HBTU_CUDA(x)                                                        \
  do {                                                                      \
    cudaError_t err__ = (x);                                                \
    if (err__ != cudaSuccess) throw ::hbtu::CudaError(err__, #x, __FILE__, __LINE__); \
  } while (0)

// Kernel launches made by the library on this host thread (tracing).
extern thread_local long long g_launches;
#define HBTU_LAUNCHED()                   \
  do {                                    \
    ++::hbtu::g_launches;                 \
    HBTU_CUDA(cudaGetLastError());        \
  } while (0)

struct CudaError {
  cudaError_t err;
  std::string what;
  CudaError(cudaError_t e, const char *expr, const char *file, int line);
};

// Programmatic dependent launch.  The kernels of the unbinding path are
// launched with programmatic stream serialisation (launch_k), so that a
// kernel's launch is processed while its predecessor in the stream still
// runs.  Every such kernel opens with HBTU_KERNEL_PROLOGUE: griddepcontrol.wait
// returns once all prerequisite grids have completed and their memory is
// visible, and only then does the kernel let its own dependents launch (so
// at most one waiting grid sits behind a running one).  For a kernel launched
// the plain way both instructions do nothing.  HBTU_LAUNCH_OVERLAP=0 in the
// environment launches everything the plain way.
#define HBTU_KERNEL_PROLOGUE()                                       \
  do {                                                               \
    asm volatile("griddepcontrol.wait;" ::: "memory");               \
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); \
  } while (0)

bool launch_overlap();  // false when HBTU_LAUNCH_OVERLAP=0 (read once)

// kernel<<<grid, block, smem, st>>>(args...) with programmatic stream
// serialisation; only for kernels that open with HBTU_KERNEL_PROLOGUE.
template <typename... P, typename... A>
inline void launch_k(void (*kernel)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                     A... args)
{
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cfg.attrs = at;
  cfg.numAttrs = launch_overlap() ? 1 : 0;
  HBTU_CUDA(cudaLaunchKernelEx(&cfg, kernel, args...));
}


// ---------------- primitives (prims.cu) ----------------
// Exclusive scan of n int64 values (in may equal out).  tmp: scan_tmp_bytes(n).
size_t scan_tmp_bytes(long long n);
void exclusive_scan_i64(const long long *in, long long *out, long long n, void *tmp,
                        cudaStream_t st);

// Stable LSD radix sort of (hi:uint32, lo:uint64, val:int32) records on the
// digit list given; buffers are ping-ponged, the result lands in *_a.
struct SortBuffers {
  unsigned long long *lo_a, *lo_b;
  unsigned *hi_a, *hi_b;
  int *val_a, *val_b;
  unsigned *os_status;         // sort_status_words(N): per-tile look-back words + tile counter
  unsigned *os_ghist, *os_goff;  // 16 x 256 digit counts and offsets
  int *error;                  // set when a look-back wait ran out (in the pass plan)
};
size_t sort_status_words(long long n);
// passes: list of (word, shift) pairs; word 0 = lo, 1 = hi; LSD order.
void radix_sort(SortBuffers &b, long long n, const int *words, const int *shifts, int npasses,
                cudaStream_t st);

}  // namespace hbtu
