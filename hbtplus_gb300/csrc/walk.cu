// walk.cu -- binding energies by Barnes-Hut walk (the hot loop).
//
// Reference: GravityTree_t::EvaluatePotential (src/gravity_tree.cpp:79-164),
// BindingEnergy (:166-175), and the two energy loops of Subhalo_t::Unbind
// (src/subhalo_unbind.cpp:319-328 correction, :341-354 full pass).
//
// Each lane owns one target and performs exactly the reference's stackless
// walk: at a cell it opens (goes to the first child, preorder index + 1) when
// len*len > r*r*theta^2, otherwise it takes the cell's monopole and jumps to
// the skip pointer.  The 32 lanes of a warp walk together: the warp visits
// the smallest preorder index any lane still needs (__reduce_min_sync), so a
// node is fetched once per warp as a broadcast and every lane sums its own
// interactions in its own reference order.  Targets are taken in Morton order
// so the lanes of a warp share most of their path.
//
// FP32 (default): coordinates relative to the subhalo frame centre, wrapped
// once in double, so the per-interaction periodic wrap disappears; opening
// decisions within 1e-5 of the threshold are re-taken in double exactly as
// the reference takes them; the potential is summed in float and flushed to a
// double every 64 warp steps.
// FP64: absolute float coordinates, NEAREST per interaction, every operation
// in the reference's order without fused multiply-add.
#include "device_common.cuh"

namespace hbtu {
namespace {

constexpr int kWB = 128;

template <bool kFP64>
__global__ void __launch_bounds__(kWB) k_walk(Ctx c, int total)
{
  const DevParams &P = c.P;
  const int w = blockIdx.x * kWB + threadIdx.x;
  int s = 0, epos = -1, pid = -1;
  bool active = false;
  if (w < total) {
    s = upper_bound_i(c.tgt_base, c.S + 1, w) - 1;
    const SegState &sg = c.seg[s];
    const int local = w - c.tgt_base[s];
    const int tm = sg.tgt_mode;
    if (tm == 0) {                          // full pass: tree leaves in Morton order
      epos = c.sb.val_a[c.tree_base[s] + local];
      pid = c.epid[epos];
      c.coh_pid[sg.off + local] = pid;
      active = true;
    } else if (tm == 1) {  // correction pass: last full pass's order, still bound
      pid = c.coh_pid[sg.off + local];
      epos = c.epos_of_pid[pid];
      active = (epos - sg.off) < sg.ntgt;
    } else {  // list order
      epos = sg.off + local;
      pid = c.epid[epos];
      active = true;
    }
  }
  const SegState &sg = c.seg[s];
  float tp[3] = {0, 0, 0}, tv[3] = {0, 0, 0}, tq[3] = {0, 0, 0};
  float mself = 0.f;
  int nxt = kDone, end = 0;
  if (active) {
    const float4 a = c.pm[pid];
    const float4 v = c.vel[pid];
    tp[0] = a.x;
    tp[1] = a.y;
    tp[2] = a.z;
    tv[0] = v.x;
    tv[1] = v.y;
    tv[2] = v.z;
    const int local_pos = epos - sg.off;
    if (sg.mode != MODE_CORRECTION && local_pos < sg.ntree) mself = fmul(a.w, sg.mfac);
    if (kFP64) {
      tq[0] = a.x;
      tq[1] = a.y;
      tq[2] = a.z;
    } else {
      tq[0] = rel_coord(a.x, sg.fc[0], P);
      tq[1] = rel_coord(a.y, sg.fc[1], P);
      tq[2] = rel_coord(a.z, sg.fc[2], P);
    }
    const int root = 2 * c.tree_base[s];
    const int nn = sg.ntree > 0 ? min(sg.nnodes, 2 * sg.ntree) : 0;  // node slots of this subhalo
    end = root + nn;
    nxt = nn > 0 ? root : kDone;
  }

  // the self term is cancelled up front: pot = targetMass/SofteningHalo (float)
  double pot_d = (double)__fdiv_rn(mself, P.eps);
  float pot_f = 0.f;
  int ninter = 0;
  unsigned steps = 0;
  const float theta2 = P.theta2;
  const float hf = (float)P.h, hinvf = (float)P.h_inv;
  const double th2d = (double)P.theta2;

  for (;;) {
    const int cur = __reduce_min_sync(0xffffffffu, nxt);
    if (cur == kDone) break;
    const float l2 = c.nd_len2[cur];
    const int sk = c.nd_skip[cur];
    if (!kFP64) {
      const float4 a = c.nd_rel[cur];
      if (nxt == cur) {
        const float dx = a.x - tq[0], dy = a.y - tq[1], dz = a.z - tq[2];
        const float r2 = dx * dx + dy * dy + dz * dz;
        const float thr = r2 * theta2;
        bool open = l2 > thr;
        if (fabsf(l2 - thr) <= 1e-5f * thr) {
          const double ex = dsub((double)a.x, (double)tq[0]);
          const double ey = dsub((double)a.y, (double)tq[1]);
          const double ez = dsub((double)a.z, (double)tq[2]);
          const double er2 = dadd(dadd(dmul(ex, ex), dmul(ey, ey)), dmul(ez, ez));
          open = (double)l2 > dmul(er2, th2d);
        }
        if (open) {
          nxt = cur + 1 < end ? cur + 1 : kDone;
        } else {
          nxt = (sk > cur && sk < end) ? sk : kDone;
          ninter++;
          const float rinv = r2 > 0.f ? rsqrtf(r2) : 0.f;
          const float r = r2 * rinv;
          if (r >= hf) {
            pot_f -= a.w * rinv;
          } else {
            const float u = r * hinvf;
            float wp;
            if (u < 0.5f)
              wp = -2.8f + u * u * (5.333333333333f + u * u * (6.4f * u - 9.6f));
            else
              wp = -3.2f + 0.066666666667f / u +
                   u * u * (10.666666666667f + u * (-16.0f + u * (9.6f - 2.133333333333f * u)));
            pot_f += a.w * hinvf * wp;
          }
        }
      }
      if ((++steps & 63u) == 0u) {
        pot_d += (double)pot_f;
        pot_f = 0.f;
      }
    } else {
      const float4 a = c.nd_abs[cur];
      if (nxt == cur) {
        double dx = dsub((double)a.x, (double)tq[0]);
        double dy = dsub((double)a.y, (double)tq[1]);
        double dz = dsub((double)a.z, (double)tq[2]);
        if (P.periodic) {
          dx = nearest_d(dx, P);
          dy = nearest_d(dy, P);
          dz = nearest_d(dz, P);
        }
        const double r2 = dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz));
        if ((double)l2 > dmul(r2, th2d)) {
          nxt = cur + 1 < end ? cur + 1 : kDone;
        } else {
          nxt = (sk > cur && sk < end) ? sk : kDone;
          ninter++;
          const double mass = (double)a.w;
          const double r = __dsqrt_rn(r2);
          if (r >= P.h) {
            pot_d = dsub(pot_d, ddiv(mass, r));
          } else {
            const double u = dmul(r, P.h_inv);
            const double uu = dmul(u, u);
            double wp;
            if (u < 0.5)
              wp = dadd(-2.8, dmul(uu, dadd(5.333333333333, dmul(uu, dsub(dmul(6.4, u), 9.6)))));
            else
              wp = dadd(dadd(-3.2, ddiv(0.066666666667, u)),
                        dmul(uu, dadd(10.666666666667,
                                      dmul(u, dadd(-16.0, dmul(u, dsub(9.6, dmul(2.133333333333, u))))))));
            pot_d = dadd(pot_d, dmul(dmul(mass, P.h_inv), wp));
          }
        }
      }
    }
  }

  if (active) {
    const double pot_sum = kFP64 ? pot_d : dadd(pot_d, (double)pot_f);
    const double pot = ddiv(dmul(pot_sum, (double)P.G), (double)P.a);
    float E;
    if (sg.mode != MODE_CORRECTION) {
      float dv[3];
      relvel(tp, tv, sg.ref_pos, sg.ref_vel, dv, P);
      E = __double2float_rn(dadd(dmul((double)vdot(dv, dv), 0.5), pot));
    } else {
      float ov[3];
      relvel(tp, tv, sg.old_pos, sg.old_vel, ov, P);
      const float t = fadd(vdot(ov, sg.dV), sg.dK);
      E = __double2float_rn(dadd((double)c.eE[epos], dsub((double)t, pot)));
    }
    if (sg.mode == MODE_REFINE)
      c.eR[epos] = E;
    else
      c.eE[epos] = E;
    if (c.pot_out) c.pot_out[epos] = pot;
  }
  // interaction counts, one atomic per warp when the warp is in one subhalo
  const unsigned full = 0xffffffffu;
  const int s0 = __shfl_sync(full, s, 0);
  if (__all_sync(full, s == s0)) {
    const int sum = __reduce_add_sync(full, ninter);
    if ((threadIdx.x & 31) == 0 && sum) atomicAdd((unsigned long long *)&c.seg[s0].interactions,
                                                  (unsigned long long)sum);
  } else if (ninter) {
    atomicAdd((unsigned long long *)&c.seg[s].interactions, (unsigned long long)ninter);
  }
}

}  // namespace

void launch_walk(Ctx &c, const PassPlan &pl)
{
  const int n = pl.ntgt_total;
  if (n <= 0) return;
  const int blocks = (n + kWB - 1) / kWB;
  if (c.P.precision == HBTU_PRECISION_FP64)
    k_walk<true><<<blocks, kWB, 0, c.st>>>(c, n);
  else
    k_walk<false><<<blocks, kWB, 0, c.st>>>(c, n);
  HBTU_LAUNCHED();
}


}  // namespace hbtu
