// walk.cu -- binding energies by Barnes-Hut walk (the hot loop).
//
// Reference: GravityTree_t::EvaluatePotential (src/gravity_tree.cpp:79-164),
// BindingEnergy (:166-175), and the two energy loops of Subhalo_t::Unbind
// (src/subhalo_unbind.cpp:319-328 correction, :341-354 full pass).
//
// Each target performs exactly the reference's stackless walk: at a cell it
// opens (goes to the first child, preorder index + 1) when
// len*len > r*r*theta^2, otherwise it takes the cell's monopole and jumps to
// the skip pointer; particles are never opened.  Targets are taken in Morton
// order, subhaloes largest first, so a warp holds neighbouring targets.
//
// FP32 (default): coordinates relative to the subhalo frame centre, wrapped
// once in double, so the per-interaction periodic wrap disappears; opening
// decisions within 1e-5 of the threshold are re-taken in double exactly as
// the reference takes them; the potential is summed in float with
// compensation and formed in double once per target (no double arithmetic in
// the loop: this GPU's FP64 rate is 1/64 of its FP32 rate).  Two schedules:
//   lane (default): every lane walks its own target, one 32-byte node record
//     per step; large blocks keep a block's neighbouring targets on one SM,
//     so the walks share L1;
//   warp: the warp visits the smallest index any of its targets waits at, so
//     each node is a broadcast load (kept as an option for comparison).
// FP64: absolute float coordinates, NEAREST per interaction, every operation
// in the reference's order without fused multiply-add; one walk per lane.
// The per-target walks live in walk_ops.cuh (shared with small.cu).
#include "walk_ops.cuh"

namespace hbtu {
namespace {

constexpr int kWB = 128;

// Target w of this pass: segment, list position, particle, walk range.
template <bool kRel>
__device__ __forceinline__ void load_target(const Ctx &c, int w, int total, Target &t)
{
  if (w >= total) {
    t.s = 0;
    t.epos = -1;
    t.pid = -1;
    t.active = false;
    t.nxt = kDone;
    t.end = 0;
    t.mself = 0.f;
    t.q[0] = t.q[1] = t.q[2] = 0.f;
    return;
  }
  const int k = upper_bound_i(c.tgt_base, c.S + 1, w) - 1;
  const int s = c.seg_order[k];
  const SegState &sg = c.seg[s];
  const int local = w - c.tgt_base[k];
  const int tm = sg.tgt_mode;
  int epos, pid;
  bool active;
  if (tm == 0) {  // full pass: tree leaves in Morton order
    epos = c.sb.val_a[c.tree_base[s] + local];
    pid = c.epid[epos];
    c.coh_pid[sg.off + local] = pid;
    active = true;
  } else if (tm == 1) {  // correction pass: last full pass's Morton order, still bound
    pid = c.coh_pid[sg.off + local];
    epos = c.epos_of_pid[pid];
    active = (epos - sg.off) < sg.ntgt;
  } else {  // list order
    epos = sg.off + local;
    pid = c.epid[epos];
    active = true;
  }
  init_target<kRel>(c, s, epos, pid, active, 2 * c.tree_base[s], t);
}

// FP32 walk, warp schedule.  Leaf runs: when targets open a cell
// whose children are all particles, each of those targets takes every child
// in order (particles are never opened) -- the warp streams the children
// through a loop with no opening test and no scheduling per node.
template <bool kLeafRuns>
__global__ void __launch_bounds__(kWB) k_walk_fp32(Ctx c, int total)
{
  HBTU_KERNEL_PROLOGUE();
  const DevParams &P = c.P;
  const unsigned full = 0xffffffffu;
  Target t;
  load_target<true>(c, blockIdx.x * kWB + threadIdx.x, total, t);
  PotAcc acc;
  const float theta2 = P.theta2;
  const float hf = (float)P.h, hinvf = (float)P.h_inv, h2f = hf * hf;
  const double th2d = (double)P.theta2;
  int ninter = 0;
  unsigned steps = 0;

  int cur = __reduce_min_sync(full, t.nxt);
  float4 na = make_float4(0.f, 0.f, 0.f, 0.f);
  int2 nm = make_int2(0, 0);
  if (cur != kDone) {
    load_node(c.nd, cur, na, nm);
  }
  while (cur != kDone) {
    float4 pa;  // speculative; a spare slot follows the last node
    int2 pmeta;
    load_node(c.nd, cur + 1, pa, pmeta);
    const float l2 = __int_as_float(nm.x & 0x7fffffff);
    const bool bottom = kLeafRuns && nm.x < 0;
    const int sk = nm.y;
    bool run = false;
    if (t.nxt == cur) {
      const float r2 = dist2(na, t.q);
      if (opens(na, t.q, l2, r2, theta2, th2d)) {
        if (bottom)
          run = true;
        else
          t.nxt = cur + 1 < t.end ? cur + 1 : kDone;
      } else {
        t.nxt = (unsigned)(sk - cur - 1) < (unsigned)(t.end - cur - 1) ? sk : kDone;
        ninter++;
        interact(na, r2, acc.f, hf, h2f, hinvf);
      }
    }
    const unsigned runners = kLeafRuns ? __ballot_sync(full, run) : 0u;
    if (runners) {
      // children cur+1 .. sk-1 are particles: stream them (every runner is at
      // cur, in one tree, so the bound is the same for all of them)
      const int last = __shfl_sync(full, min(sk, t.end), __ffs(runners) - 1);
      int j = cur + 1;
      for (; j + 1 < last; j += 2) {
        const float4 a0 = c.nd[j].p, a1 = c.nd[j + 1].p;
        if (run) {
          interact(a0, dist2(a0, t.q), acc.f, hf, h2f, hinvf);
          interact(a1, dist2(a1, t.q), acc.f, hf, h2f, hinvf);
        }
      }
      if (j < last) {
        const float4 a0 = c.nd[j].p;
        if (run) interact(a0, dist2(a0, t.q), acc.f, hf, h2f, hinvf);
      }
      if (run) {
        ninter += last - cur - 1;
        t.nxt = (unsigned)(sk - cur - 1) < (unsigned)(t.end - cur - 1) ? sk : kDone;
      }
      acc.flush();
      cur = __reduce_min_sync(full, t.nxt);
      if (cur != kDone) {
        load_node(c.nd, cur, na, nm);
      }
    } else if (__any_sync(full, t.nxt == cur + 1)) {
      cur = cur + 1;
      na = pa;
      nm = pmeta;
    } else {
      cur = __reduce_min_sync(full, t.nxt);
      if (cur != kDone) {
        load_node(c.nd, cur, na, nm);
      }
    }
    if ((++steps & 7u) == 0u) acc.flush();
  }
  finish_target(c, t, acc.total((double)__fdiv_rn(t.mself, P.eps)));  // + cancels the self term
  count_interactions(c, t.s, ninter);
}

// FP32 walk, lane schedule (walk_lean): blocks of kB neighbouring targets.
template <int kB, bool kSib>
__global__ void __launch_bounds__(kB) k_walk_fp32_lean(Ctx c, int total)
{
  HBTU_KERNEL_PROLOGUE();
  Target t;
  load_target<true>(c, blockIdx.x * kB + threadIdx.x, total, t);
  int ninter = 0;
  const double pot = walk_lean<kSib>(kSib ? c.nd2 : c.nd, t, c.P, &ninter);
  finish_target(c, t, pot);
  count_interactions(c, t.s, ninter);
}

template <bool kSib>
void launch_lean(Ctx &c, int n)
{
  if (n >= 152 * 4 * 512)  // blocks of neighbouring targets share an SM's L1
    launch_k(k_walk_fp32_lean<512, kSib>, (n + 511) / 512, 512, 0, c.st, c, n);
  else if (n >= 152 * 4 * 256)
    launch_k(k_walk_fp32_lean<256, kSib>, (n + 255) / 256, 256, 0, c.st, c, n);
  else
    launch_k(k_walk_fp32_lean<128, kSib>, (n + 127) / 128, 128, 0, c.st, c, n);
}

// FP64: the reference's arithmetic, operation by operation (walk_fp64), one
// walk per lane.
__global__ void __launch_bounds__(kWB) k_walk_fp64(Ctx c, int total)
{
  HBTU_KERNEL_PROLOGUE();
  Target t;
  load_target<false>(c, blockIdx.x * kWB + threadIdx.x, total, t);
  int ninter = 0;
  const double pot = walk_fp64(c, t, &ninter);
  finish_target(c, t, pot);
  count_interactions(c, t.s, ninter);
}

// ---------------------------------------------------------------------------
// Adjoint: gradient of the total binding energy over a fixed particle set,
//   E_tot = sum_i m_i |dv_i|^2 / 2 + (1/2) sum_i m_i phi_i,
// with dv_i the velocity relative to the frame (RelativeVelocity, Hubble flow
// included) and phi_i the walk potential (self term cancelled).  The frame is
// the set's centre of mass, so its dependence on x, v, m cancels (sum m dv = 0):
//   dE/dv_k = m_k dv_k,
//   dE/dx_k = m_k (H a dv_k + grad phi(x_k)),
//   dE/dm_k = |dv_k|^2 / 2 + phi_k.
// grad phi is recomputed by a walk with the reference's opening rule on the same
// tree (nothing of the energy walk is stored); per accepted node
//   far  (r >= h): d(-m/r)/dx_t = -m dx / r^3,
//   near (r < h):  d(m wp(u)/h)/dx_t = -m wp'(u) dx / (h^2 r),  u = r/h,
// with wp' the derivative of the cubic-spline kernel; dx = x_node - x_target.
// The walk is walk_lean's (one target per lane, the same nodes in the same
// order, the potential in the same compensated float sum); the gradient
// terms go into compensated float sums, one per lane, so a target's results do
// not depend on the other targets of the call.  kGrad =
// false computes only the energies (the forward pass of the autograd function).
// s += v in a compensated float sum (Kahan): s - c carries the sum.
__device__ __forceinline__ void kahan_add(float &s, float &c, float v)
{
  const float y = __fsub_rn(v, c);
  const float t = __fadd_rn(s, y);
  c = __fsub_rn(__fsub_rn(t, s), y);
  s = t;
}

template <bool kSib, bool kGrad>
__device__ __forceinline__ double walk_grad(const WNode *nodes, const Target &t,
                                            const DevParams &P, double (&acc)[3])
{
  const float hf = (float)P.h, hinvf = (float)P.h_inv, h2f = hf * hf;
  const double th2d = (double)P.theta2;
  float hi = 0.f, comp = 0.f;  // Kahan sum of the potential
  // compensated (Kahan) float sums of the gradient: no double arithmetic in the
  // loop, where the lanes of a warp drift apart and a double instruction would
  // issue once per drifting group of lanes
  float ax = 0.f, ay = 0.f, az = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
  int iters = 0;
  int cur = t.nxt;
  const int end = t.end;
  const int steps = kSib ? max(end - t.nxt, 0) : 0;
  while (cur < end) {
    float4 na;
    int4 nm;
    load_node(nodes, cur, na, nm);
    const float dx = na.x - t.q[0], dy = na.y - t.q[1], dz = na.z - t.q[2];
    const float r2 = dx * dx + dy * dy + dz * dz;
    const float lo = __int_as_float(nm.z);
    const float up = kSib ? lo * kBandRatio : __int_as_float(nm.w);
    bool open = r2 < lo;
    if (r2 >= lo && r2 <= up)
      open = exact_open(na, t.q[0], t.q[1], t.q[2], __int_as_float(nm.x & 0x7fffffff), th2d);
    const float rinv = rsqrtf(fmaxf(r2, 1e-30f));
    const float mass = fabsf(na.w);  // cells carry their mass with the sign bit set
    float contrib = -mass * rinv;
    if (r2 < h2f) contrib = softened_fp32(mass, r2, rinv, hf, hinvf);
    contrib = open ? 0.f : contrib;
    const float y = __fsub_rn(contrib, comp);
    const float sum = __fadd_rn(hi, y);
    comp = __fsub_rn(__fsub_rn(sum, hi), y);
    hi = sum;
    if (kGrad && !open) {
      float w;  // gradient weight: grad phi -= m * w * dx
      if (r2 >= h2f) {
        w = rinv * rinv * rinv;
      } else {
        const float u = r2 * rinv * hinvf;
        const float iu = hf * rinv;  // 1/u
        const float dwp = u < 0.5f
                              ? u * (10.666666666667f + u * u * (32.0f * u - 38.4f))
                              : -0.066666666667f * iu * iu +
                                    u * (21.333333333333f +
                                         u * (-48.0f + u * (38.4f - 10.666666666667f * u)));
        w = r2 > 0.f ? hinvf * hinvf * dwp * rinv : 0.f;
      }
      const float mw = mass * w;
      kahan_add(ax, cx, mw * dx);
      kahan_add(ay, cy, mw * dy);
      kahan_add(az, cz, mw * dz);
    }
    iters++;
    if (kSib) {
      cur = open ? nm.w : nm.y;
      if (iters >= steps || cur < t.nxt) break;  // malformed pointers: stop
    } else {
      cur = open ? cur + 1 : max(nm.y, cur + 1);
    }
  }
  acc[0] = dsub((double)ax, (double)cx);
  acc[1] = dsub((double)ay, (double)cy);
  acc[2] = dsub((double)az, (double)cz);
  const double base = (double)__fdiv_rn(t.mself, P.eps);  // cancels the self term
  return dadd(dadd(base, (double)hi), -(double)comp);
}

template <int kB, bool kSib, bool kGrad>
__global__ void __launch_bounds__(kB) k_grad_walk(Ctx c, int total)
{
  HBTU_KERNEL_PROLOGUE();
  const DevParams &P = c.P;
  Target t;
  load_target<true>(c, blockIdx.x * kB + threadIdx.x, total, t);
  double acc[3];
  const double pot_sum = walk_grad<kSib, kGrad>(kSib ? c.nd2 : c.nd, t, P, acc);
  if (!t.active) return;
  const SegState &sg = c.seg[t.s];
  const double ga = ddiv((double)P.G, (double)P.a);
  const double pot = dmul(pot_sum, ga);
  const float4 a = c.pm[t.pid], v = c.vel[t.pid];
  const float tp[3] = {a.x, a.y, a.z}, tv[3] = {v.x, v.y, v.z};
  float dv[3];
  relvel(tp, tv, sg.ref_pos, sg.ref_vel, dv, P);
  const double m = (double)a.w;
  const double k2 = (double)dv[0] * dv[0] + (double)dv[1] * dv[1] + (double)dv[2] * dv[2];
  const double ha = (double)P.Hz * (double)P.a;
  const int i = t.pid;  // no list permutation in this call: input position
  if (kGrad) {
    if (c.grad_pos)
      for (int j = 0; j < 3; j++) c.grad_pos[3 * i + j] = (float)(m * (ha * dv[j] - ga * acc[j]));
    if (c.grad_vel)
      for (int j = 0; j < 3; j++) c.grad_vel[3 * i + j] = (float)(m * dv[j]);
    if (c.grad_mass) c.grad_mass[i] = (float)(0.5 * k2 + pot);
  }
  c.e_part[i] = 0.5 * m * k2 + 0.5 * m * pot;
}

template <bool kSib, bool kGrad>
void launch_grad(Ctx &c, int n)
{
  if (n >= 152 * 4 * 512)
    launch_k(k_grad_walk<512, kSib, kGrad>, (n + 511) / 512, 512, 0, c.st, c, n);
  else if (n >= 152 * 4 * 256)
    launch_k(k_grad_walk<256, kSib, kGrad>, (n + 255) / 256, 256, 0, c.st, c, n);
  else
    launch_k(k_grad_walk<128, kSib, kGrad>, (n + 127) / 128, 128, 0, c.st, c, n);
}

}  // namespace

void launch_walk(Ctx &c, const PassPlan &pl)
{
  const int n = pl.ntgt_total;
  if (n <= 0) return;
  const unsigned blocks = (n + kWB - 1) / kWB;
  if (c.P.precision == HBTU_PRECISION_FP64)
    launch_k(k_walk_fp64, blocks, kWB, 0, c.st, c, n);
  else if (c.opt_schedule == 1 && c.opt_leaf_runs)
    launch_k(k_walk_fp32<true>, blocks, kWB, 0, c.st, c, n);
  else if (c.opt_schedule == 1)
    launch_k(k_walk_fp32<false>, blocks, kWB, 0, c.st, c, n);
  else if (sibling_walk(c, pl))  // the tree build made the sibling-block records
    launch_lean<true>(c, n);
  else
    launch_lean<false>(c, n);
  HBTU_LAUNCHED();
}

void launch_grad_walk(Ctx &c, const PassPlan &pl)
{
  const int n = pl.ntgt_total;
  if (n <= 0) return;
  const bool grad = c.grad_pos || c.grad_vel || c.grad_mass;
  const bool sib = sibling_walk(c, pl);  // the tree build made the sibling-block records
  if (sib && grad)
    launch_grad<true, true>(c, n);
  else if (sib)
    launch_grad<true, false>(c, n);
  else if (grad)
    launch_grad<false, true>(c, n);
  else
    launch_grad<false, false>(c, n);
  HBTU_LAUNCHED();
}

}  // namespace hbtu
