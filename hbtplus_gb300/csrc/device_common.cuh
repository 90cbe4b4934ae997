// device_common.cuh -- device helpers and the per-call context.
//
// Arithmetic that decides the bound set follows the reference's float
// (HBTReal) / double split operation by operation.  nvcc contracts a*b+c into
// FMA by default, which rounds differently from the reference's separate
// multiply and add, so every such operation is spelled with an explicit
// round-to-nearest intrinsic (__fmul_rn, __dadd_rn, ...).
#pragma once
#include "hbtu_internal.h"

namespace hbtu {

constexpr int kChunk = 1024;  // elements per reduction chunk
constexpr int kDone = 0x7fffffff;

// One tree node as the walks read it (32 bytes, one sector): p = {x, y, z,
// mass} relative to the frame centre (sign bit of the mass set on cells),
// m = {len*len bits with the all-particle-children flag in the sign bit, skip
// pointer, sure-open and sure-accept squared distances as float bits}.
struct __align__(32) WNode {
  float4 p;
  int4 m;
};

// Both halves of node i in one 256-bit load.
__device__ __forceinline__ void load_node(const WNode *nd, int i, float4 &p, int4 &m)
{
  asm("ld.global.v8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(p.x), "=f"(p.y), "=f"(p.z), "=f"(p.w), "=r"(m.x), "=r"(m.y), "=r"(m.z), "=r"(m.w)
      : "l"(nd + i));
}

__device__ __forceinline__ void load_node(const WNode *nd, int i, float4 &p, int2 &m)
{
  int4 q;
  load_node(nd, i, p, q);
  m = make_int2(q.x, q.y);
}

__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

// Exact float -> double and round-to-nearest-even double -> float, built
// from the IEEE-754 fields with integer operations: the conversion
// instructions run on the FP64 unit, at 1/64 of the FP32 rate on this GPU.
// Zero, subnormal, infinite and NaN inputs (and results outside the normal
// float range) take the conversion instruction.
__device__ __forceinline__ double f2d(float x)
{
  const unsigned u = __float_as_uint(x);
  const unsigned e = (u >> 23) & 0xffu;
  const unsigned long long s = (unsigned long long)(u >> 31) << 63;
  if ((u & 0x7fffffffu) == 0u) return __longlong_as_double((long long)s);
  if (e == 0u || e == 0xffu) return (double)x;
  return __longlong_as_double((long long)(s | ((unsigned long long)(e + (1023 - 127)) << 52) |
                                          ((unsigned long long)(u & 0x7fffffu) << 29)));
}

__device__ __forceinline__ float d2f(double x)
{
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7ffull) - 1023 + 127;
  if (e <= 0 || e >= 255) return __double2float_rn(x);
  const unsigned long long mant = b & 0xfffffffffffffull;
  unsigned long long r = mant >> 29;
  const unsigned long long rem = mant & 0x1fffffffull, half = 1ull << 28;
  if (rem > half || (rem == half && (r & 1ull))) r++;
  const unsigned bits = (unsigned)(((unsigned long long)e << 23) + r);  // a carry bumps the exponent
  if (((bits >> 23) & 0xffu) == 0xffu) return __double2float_rn(x);
  return __uint_as_float(bits | ((unsigned)(b >> 63) << 31));
}

// NEAREST (src/config_parser.h:142) on a double / a float operand.
__device__ __forceinline__ double nearest_d(double x, const DevParams &P)
{
  return x > (double)P.boxhalf ? dsub(x, (double)P.box)
                               : (x < -(double)P.boxhalf ? dadd(x, (double)P.box) : x);
}
__device__ __forceinline__ float nearest_f(float x, const DevParams &P)
{
  return x > P.boxhalf ? fsub(x, P.box) : (x < -P.boxhalf ? fadd(x, P.box) : x);
}

// Snapshot_t::RelativeVelocity (src/snapshot.h:100-111), float arithmetic.
__device__ __forceinline__ void relvel(const float tp[3], const float tv[3], const float rp[3],
                                       const float rv[3], float dv[3], const DevParams &P)
{
  const float ha = fmul(P.Hz, P.a);
#pragma unroll
  for (int j = 0; j < 3; j++) {
    float dx = fsub(tp[j], rp[j]);
    if (P.periodic) dx = nearest_f(dx, P);
    dv[j] = fadd(fsub(tv[j], rv[j]), fmul(ha, dx));
  }
}

// VecNorm / VecDot (src/mymath.h:20-21) in float.
__device__ __forceinline__ float vdot(const float a[3], const float b[3])
{
  return fadd(fadd(fmul(a[0], b[0]), fmul(a[1], b[1])), fmul(a[2], b[2]));
}

// Relative coordinate of an absolute float coordinate: wrapped once in
// double, then rounded to float.  When the float difference s = x - c is
// exact (a float TwoSum with a zero error term) it equals the double one, and
// for |s| < box the wrap s -+ box is exact in float as in double (Sterbenz:
// box/2 < |s| < 2 box), so the float arithmetic gives the same bits without
// the FP64 pipe (1/64 of the FP32 rate on this GPU); otherwise the double path.
__device__ __forceinline__ float rel_coord(float x, float c, const DevParams &P)
{
  const float s = __fsub_rn(x, c);
  const float bb = __fsub_rn(s, x);
  const float err = __fadd_rn(__fsub_rn(x, __fsub_rn(s, bb)), __fsub_rn(-c, bb));
  if (err == 0.f && !P.periodic) return s;
  if (err == 0.f && fabsf(s) < P.box) return nearest_f(s, P);
  double d = dsub(f2d(x), f2d(c));
  if (P.periodic) d = nearest_d(d, P);
  return d2f(d);
}

// Order-preserving 32-bit key of a float (ascending); -0 sorts as +0.
__device__ __forceinline__ unsigned float_key(float e)
{
  unsigned u = __float_as_uint(e == 0.f ? 0.f : e);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ int upper_bound_i(const int *a, int n, int x)
{
  int lo = 0, hi = n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (a[mid] <= x)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

// The per-call device context: every buffer of the workspace.
struct Ctx {
  DevParams P;
  int N, S;
  cudaStream_t st;
  // particles
  float4 *pm, *vel;
  long long *id;
  int *type, *pseg;
  int *epid, *epid2;
  float *eE, *eE2, *eR;
  int *epos_of_pid, *coh_pid;
  // per segment
  SegState *seg;
  PassPlan *plan, *plan_host;
  int *tree_base, *tgt_base;                 // S+1 each
  int *tchunk_base, *bchunk_base, *ub_base;  // S+1 each
  int4 *plan_cnt, *plan_cnt2;                // S each: gathered plan counters
  long long *plan_inter;                     // S: gathered interaction counts
  int *seg_off;                              // S+1
  int *seg_order;                            // S: subhaloes by size, largest first
  int opt_leaf_runs;                         // warp schedule streams all-particle cells
  int opt_schedule;                          // FP32 walk: 0 one walk per lane, 1 warp schedule
  int *part_info;                            // 8 ints per segment
  unsigned *chunk_bbox;                      // 6 per chunk
  double *chunk_sums;                        // 16 per chunk
  // sort
  SortBuffers sb;
  // tree construction
  int *parentI, *parentL, *rfirst, *rlast, *dnode;
  int *iscell, *cidx, *cskip, *cdepth, *pcell, *pending, *pending0;  // pending: child cells
  int *cslot;  // 8 per cell: node index of the child in each octant, -1 if none
  // moment work lists: cell_list holds the large chunk roots from the front and
  // the top cells from the back, chunk_list the small chunk roots; lvl[0..3]:
  // their counts (large, top), the job counter, the small count
  int *cell_list, *chunk_list, *lvl;
  unsigned long long *mask;
  long long *X;
  // nodes (2 per tree particle)
  float4 *nd_abs;
  WNode *nd;
  // the FP32 walk's layout: the same records with each cell's children in
  // consecutive slots (m.w = first child's slot instead of the upper
  // threshold); null when the workspace has no room for it
  WNode *nd2;
  int *newidx;
  long long *X2;
  void *scan_tmp2;
  int opt_layout;  // 1: the FP32 lane walk uses nd2
  // partition
  long long *pcode, *pX;
  int *Pk, *Qk;
  void *scan_tmp;
  double *pot_out;  // optional: potentials of a full pass (hbtu_binding_energies)
  // adjoint outputs (hbtu_energy_gradient), by input position; grads may be null
  float *grad_pos, *grad_vel, *grad_mass;
  double *e_part;
  // the per-subhalo loop (small.cu): it takes over once every active
  // subhalo's list holds at most small_cap particles (0: never)
  int *small_next;   // work-queue counter
  int small_cap;
  int small_per_sm;  // blocks per SM of its persistent launch
};

// launchers (tree.cu)
void launch_bbox_cube(Ctx &c, int max_chunks);
void launch_tree_build(Ctx &c, const PassPlan &pl);
// launchers (walk.cu)
void launch_walk(Ctx &c, const PassPlan &pl);
void launch_sibling_layout(Ctx &c, const PassPlan &pl);
// The FP32 lane walk over the sibling-block records (the tree build then makes
// them): for trees of at least kSiblingMinTree particles in all, where the
// faster walk pays for the extra pass over the nodes (the small trees of
// correction passes do not).
constexpr int kSiblingMinTree = 1 << 16;
inline bool sibling_walk(const Ctx &c, const PassPlan &pl)
{
  return c.P.precision != HBTU_PRECISION_FP64 && c.opt_schedule == 0 && c.opt_layout && c.nd2 &&
         pl.ntree_total >= kSiblingMinTree;
}
void launch_grad_walk(Ctx &c, const PassPlan &pl);
// per-subhalo sums of a per-particle double array (input positions), deterministic
void launch_segment_sums(Ctx &c, const double *x, double *out);
// (direct.cu) exact FP64 potentials of particles tidx[0..nt) from all n particles
void direct_potential_fp64(const DevParams &P, const float4 *pm, int n, const int *tidx, int nt,
                           double *out, double *partial, int nsplit, cudaStream_t st);
// (small.cu) the remaining passes of every active subhalo, one block per
// subhalo; `cap` bounds their energy lists (at most kSmallCap particles)
constexpr int kSmallCap = 2048;
constexpr int kSmallDefault = 2048;
void launch_small(Ctx &c, int cap, int nactive, int max_passes);
size_t small_smem_bytes(int cap);
// launchers (loop.cu)
void launch_init(Ctx &c, const float *pos, const float *vel, const float *mass,
                 const long long *id);
void launch_plan(Ctx &c, int mode);  // 0 pass, 1 bound chunks, 2 final
void launch_partition(Ctx &c);
void launch_averages_control(Ctx &c, int max_passes);
// which: 0 unbound blocks, 1 bound parts, 2 refined prefixes (keyed by eR)
void launch_block_sort(Ctx &c, int total, int which);
void launch_refine_mode(Ctx &c, int enter);
void launch_finalize(Ctx &c, int64_t *order_out, float *energy_out, hbtu_result *res_dev);

}  // namespace hbtu
