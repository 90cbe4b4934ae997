// walk_ops.cuh -- one target's Barnes-Hut walk and its binding energy, shared
// by the batch walks (walk.cu: one launch per pass over every active
// subhalo's targets) and the per-subhalo loop (small.cu).
//
// Reference: GravityTree_t::EvaluatePotential (src/gravity_tree.cpp:79-164),
// BindingEnergy (:166-175) and the two energy loops of Subhalo_t::Unbind
// (src/subhalo_unbind.cpp:319-328 correction, :341-354 full pass).  A target
// performs exactly the reference's stackless walk: at a cell it opens (goes to
// the first child) when len*len > r*r*theta^2, otherwise it takes the cell's
// monopole and jumps to the skip pointer; particles are never opened.
#pragma once
#include "device_common.cuh"

namespace hbtu {

struct Target {
  int s, epos, pid, nxt, end;
  bool active;
  float q[3];  // position used by the walk (relative for FP32, absolute for FP64)
  float mself;
};

// The walk of particle `pid` at list position `epos` of subhalo s in the
// coming pass: its position (relative to the frame centre for kRel, else
// absolute), the self term it cancels (full and refine passes, if it is in
// the tree), and the node range of the subhalo's tree.
template <bool kRel>
__device__ __forceinline__ void init_target(const Ctx &c, int s, int epos, int pid, bool active,
                                            int root, Target &t)
{
  const SegState &sg = c.seg[s];
  t.s = s;
  t.epos = epos;
  t.pid = pid;
  t.active = active;
  t.nxt = kDone;
  t.end = 0;
  t.mself = 0.f;
  t.q[0] = t.q[1] = t.q[2] = 0.f;
  if (!active) return;
  const float4 a = c.pm[pid];
  if (sg.mode != MODE_CORRECTION && epos - sg.off < sg.ntree) t.mself = fmul(a.w, sg.mfac);
  if (kRel) {
    t.q[0] = rel_coord(a.x, sg.fc[0], c.P);
    t.q[1] = rel_coord(a.y, sg.fc[1], c.P);
    t.q[2] = rel_coord(a.z, sg.fc[2], c.P);
  } else {
    t.q[0] = a.x;
    t.q[1] = a.y;
    t.q[2] = a.z;
  }
  const int nn = sg.ntree > 0 ? min(sg.nnodes, 2 * sg.ntree) : 0;  // node slots of this subhalo
  t.end = root + nn;
  t.nxt = nn > 0 ? root : kDone;
}

// BindingEnergy (full pass) or the correction update, and the store.
__device__ __forceinline__ void finish_target(const Ctx &c, const Target &t, double pot_sum)
{
  if (!t.active) return;
  const DevParams &P = c.P;
  const SegState &sg = c.seg[t.s];
  const double pot = ddiv(dmul(pot_sum, (double)P.G), (double)P.a);
  const float4 a = c.pm[t.pid], v = c.vel[t.pid];
  const float tp[3] = {a.x, a.y, a.z}, tv[3] = {v.x, v.y, v.z};
  float E;
  if (sg.mode != MODE_CORRECTION) {
    float dv[3];
    relvel(tp, tv, sg.ref_pos, sg.ref_vel, dv, P);
    E = __double2float_rn(dadd(dmul((double)vdot(dv, dv), 0.5), pot));
  } else {
    float ov[3];
    relvel(tp, tv, sg.old_pos, sg.old_vel, ov, P);
    const float tt = fadd(vdot(ov, sg.dV), sg.dK);
    E = __double2float_rn(dadd((double)c.eE[t.epos], dsub((double)tt, pot)));
  }
  if (sg.mode == MODE_REFINE)
    c.eR[t.epos] = E;
  else
    c.eE[t.epos] = E;
  if (c.pot_out) c.pot_out[t.epos] = pot;
}

// Adds a warp's interaction counts to its subhaloes' totals (one atomic per
// warp when the warp holds one subhalo).
__device__ __forceinline__ void count_interactions(const Ctx &c, int s, int n)
{
  const unsigned full = 0xffffffffu;
  const int s0 = __shfl_sync(full, s, 0);
  if (__all_sync(full, s == s0)) {
    const int sum = __reduce_add_sync(full, n);
    if ((threadIdx.x & 31) == 0 && sum)
      atomicAdd((unsigned long long *)&c.seg[s0].interactions, (unsigned long long)sum);
  } else if (n) {
    atomicAdd((unsigned long long *)&c.seg[s].interactions, (unsigned long long)n);
  }
}

// Opening test of the reference, len*len > r*r*theta^2: float first, and in
// double with the reference's operation order when within 1e-5 of the edge.
__device__ __forceinline__ bool opens(float4 na, const float q[3], float l2, float r2, float theta2,
                                      double th2d)
{
  const float thr = r2 * theta2;
  bool open = l2 > thr;
  if (l2 > 0.f && fabsf(l2 - thr) <= 1e-5f * thr) {  // particles (l2 = 0) never open
    const double ex = dsub((double)na.x, (double)q[0]);
    const double ey = dsub((double)na.y, (double)q[1]);
    const double ez = dsub((double)na.z, (double)q[2]);
    const double er2 = dadd(dadd(dmul(ex, ex), dmul(ey, ey)), dmul(ez, ez));
    open = (double)l2 > dmul(er2, th2d);
  }
  return open;
}

__device__ __forceinline__ float dist2(float4 na, const float q[3])
{
  const float dx = na.x - q[0], dy = na.y - q[1], dz = na.z - q[2];
  return dx * dx + dy * dy + dz * dz;
}

// FP32 potential sum without double arithmetic in the walk loop (this GPU's
// FP64 rate is 1/64 of its FP32 rate): interactions go into a short float
// partial sum `f`, which is flushed every few steps into a compensated
// (Kahan) float total hi - c.  The total is formed in double once per target.
struct PotAcc {
  float f = 0.f, hi = 0.f, c = 0.f;
  __device__ __forceinline__ void flush()
  {
    const float y = __fsub_rn(f, c);
    const float t = __fadd_rn(hi, y);
    c = __fsub_rn(__fsub_rn(t, hi), y);
    hi = t;
    f = 0.f;
  }
  __device__ __forceinline__ double total(double base) const
  {
    return dadd(dadd(base, (double)hi), dsub((double)f, (double)c));
  }
};

// Softened potential without a division: 1/u = h/r = h * rinv.
__device__ __forceinline__ float softened_fp32(float m, float r2, float rinv, float hf, float hinvf)
{
  const float r = r2 * rinv;
  const float u = r * hinvf;
  float wp;
  if (u < 0.5f)
    wp = -2.8f + u * u * (5.333333333333f + u * u * (6.4f * u - 9.6f));
  else
    wp = -3.2f + 0.066666666667f * (hf * rinv) +
         u * u * (10.666666666667f + u * (-16.0f + u * (9.6f - 2.133333333333f * u)));
  return m * hinvf * wp;
}

// One monopole interaction in FP32: -m/r outside the softening length h,
// the cubic-spline potential inside it (Springel, Yoshida & White 2001).
__device__ __forceinline__ void interact(float4 na, float r2, float &pot_f, float hf, float h2f,
                                         float hinvf)
{
  const float rinv = rsqrtf(fmaxf(r2, 1e-30f));
  const float m = fabsf(na.w);  // cells carry their mass with the sign bit set
  if (r2 >= h2f)
    pot_f = fmaf(-m, rinv, pot_f);
  else
    pot_f += softened_fp32(m, r2, rinv, hf, hinvf);
}

// The reference's opening decision in double, for a target whose float test
// fell within 1e-5 of the threshold.  Not inlined: the compiler would
// otherwise evaluate the double arithmetic on every step and select.
// The target position comes by value, so the walk keeps it in registers.
static __device__ __noinline__ bool exact_open(float4 na, float qx, float qy, float qz, float l2,
                                        double th2d)
{
  const double ex = dsub((double)na.x, (double)qx);
  const double ey = dsub((double)na.y, (double)qy);
  const double ez = dsub((double)na.z, (double)qz);
  const double er2 = dadd(dadd(dmul(ex, ex), dmul(ey, ey)), dmul(ez, ez));
  return (double)l2 > dmul(er2, th2d);
}

// FP32 walk of one target, lane schedule: the opening test is two compares
// against per-cell thresholds precomputed from len^2/theta^2 (the
// reference's double test decides the rare cases in between), every
// interaction goes straight into a compensated float sum, and the walk ends
// when the index leaves the tree (skip pointers that leave it are kDone).
//   kSib = false: preorder records; the next node is cur + 1 on opening, the
//     skip pointer otherwise, so the index strictly grows and the loop ends
//     even on a malformed tree.
//   kSib = true: the sibling-block records (nd2): a cell's children sit in
//     consecutive slots, so the sibling an accepted cell hands on to is
//     usually in the same cache line; the next node is the first-child
//     pointer (m.w) on opening and the skip pointer otherwise, the upper
//     threshold is recomputed from the lower one, and the loop also stops
//     after as many steps as the tree has nodes.  Same nodes, same order,
//     same sums as the preorder walk.
// Returns the potential sum (self term cancelled, before G/a); *ninter counts
// the interactions.
constexpr float kBandRatio = 1.0000200002f;  // (1 + 1e-5) / (1 - 1e-5), rounded up

template <bool kSib>
__device__ __forceinline__ double walk_lean(const WNode *nodes, const Target &t,
                                            const DevParams &P, int *ninter)
{
  const float hf = (float)P.h, hinvf = (float)P.h_inv, h2f = hf * hf;
  const double th2d = (double)P.theta2;
  float hi = 0.f, comp = 0.f;  // Kahan sum
  int iters = 0, nopen = 0;
  int cur = t.nxt;
  const int end = t.end;
  const int steps = kSib ? max(end - t.nxt, 0) : 0;  // the tree's node count
  while (cur < end) {
    float4 na;
    int4 nm;
    load_node(nodes, cur, na, nm);
    const float r2 = dist2(na, t.q);
    const float lo = __int_as_float(nm.z);
    const float up = kSib ? lo * kBandRatio : __int_as_float(nm.w);
    bool open = r2 < lo;
    if (r2 >= lo && r2 <= up)
      open = exact_open(na, t.q[0], t.q[1], t.q[2], __int_as_float(nm.x & 0x7fffffff), th2d);
    const float rinv = rsqrtf(fmaxf(r2, 1e-30f));
    const float mass = fabsf(na.w);
    float contrib = -mass * rinv;
    if (r2 < h2f) contrib = softened_fp32(mass, r2, rinv, hf, hinvf);
    contrib = open ? 0.f : contrib;
    const float y = __fsub_rn(contrib, comp);
    const float s = __fadd_rn(hi, y);
    comp = __fsub_rn(__fsub_rn(s, hi), y);
    hi = s;
    iters++;
    nopen += open ? 1 : 0;
    if (kSib) {
      cur = open ? nm.w : nm.y;
      if (iters >= steps || cur < t.nxt) break;  // malformed pointers: stop
    } else {
      cur = open ? cur + 1 : max(nm.y, cur + 1);
    }
  }
  *ninter = iters - nopen;
  const double base = (double)__fdiv_rn(t.mself, P.eps);  // cancels the self term
  return dadd(dadd(base, (double)hi), -(double)comp);
}

// One FP64 interaction with the reference's arithmetic, operation by operation
// (src/gravity_tree.cpp:136-160).
__device__ __forceinline__ double fp64_contrib(double r2, double mass, const DevParams &P)
{
  const double r = __dsqrt_rn(r2);
  if (r >= P.h) return -ddiv(mass, r);
  const double u = dmul(r, P.h_inv);
  const double uu = dmul(u, u);
  double wp;
  if (u < 0.5)
    wp = dadd(-2.8, dmul(uu, dadd(5.333333333333, dmul(uu, dsub(dmul(6.4, u), 9.6)))));
  else
    wp = dadd(dadd(-3.2, ddiv(0.066666666667, u)),
              dmul(uu, dadd(10.666666666667,
                            dmul(u, dadd(-16.0, dmul(u, dsub(9.6, dmul(2.133333333333, u))))))));
  return dmul(dmul(mass, P.h_inv), wp);
}

// FP64 walk of one target, lane schedule, over the preorder records: absolute
// float coordinates (nd_abs), NEAREST per interaction, the reference's
// arithmetic and summation order.  Returns the potential sum (self term
// cancelled, before G/a).
// NEAREST((double)x - (double)q) for float coordinates, as the reference
// forms a node-target separation.  When the float difference s is exact (a
// float TwoSum with a zero error term) it is the double difference, and for
// |s| < box its wrap is exact in float as well (Sterbenz), so the double pipe
// (1/64 of the FP32 rate on this GPU) only converts the result; otherwise the
// double path.
__device__ __forceinline__ double sep_fp64(float x, float q, const DevParams &P)
{
  const float s = __fsub_rn(x, q);
  const float bb = __fsub_rn(s, x);
  const float err = __fadd_rn(__fsub_rn(x, __fsub_rn(s, bb)), __fsub_rn(-q, bb));
  if (err == 0.f && !P.periodic) return f2d(s);
  if (err == 0.f && fabsf(s) < P.box) return f2d(nearest_f(s, P));
  const double d = dsub(f2d(x), f2d(q));
  return P.periodic ? nearest_d(d, P) : d;
}

__device__ __forceinline__ double walk_fp64(const Ctx &c, const Target &t, int *ninter)
{
  const DevParams &P = c.P;
  double pot_d = (double)__fdiv_rn(t.mself, P.eps);
  const double th2d = (double)P.theta2;
  int n = 0;
  int cur = t.nxt;
  const int end = t.end;
  while (cur < end) {
    const float4 na = c.nd_abs[cur];
    const int2 nm = make_int2(c.nd[cur].m.x, c.nd[cur].m.y);
    const double dx = sep_fp64(na.x, t.q[0], P);
    const double dy = sep_fp64(na.y, t.q[1], P);
    const double dz = sep_fp64(na.z, t.q[2], P);
    const double r2 = dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz));
    if (f2d(__int_as_float(nm.x & 0x7fffffff)) > dmul(r2, th2d)) {
      cur = cur + 1;
    } else {
      const int sk = nm.y;
      cur = (unsigned)(sk - cur - 1) < (unsigned)(end - cur - 1) ? sk : end;
      n++;
      pot_d = dadd(pot_d, fp64_contrib(r2, (double)na.w, P));
    }
  }
  *ninter = n;
  return pot_d;
}

}  // namespace hbtu
