// loop_ops.cuh -- steps of the unbinding loop shared by the batch kernels
// (loop.cu) and the per-subhalo loop (small.cu):
//   block_sum        deterministic FP64 sums of a 1024-element chunk by a block
//                    of kLB threads (fixed association, so both callers round
//                    alike);
//   control_segment  one subhalo's decisions after a pass: disruption
//                    (src/subhalo_unbind.cpp:361-379), the sticky correction
//                    flag (:383-392), the frame (AverageVelocity /
//                    AveragePosition from the chunk sums, :108-188),
//                    convergence on the particle count (:395) and the set-up
//                    of the next full (:331-356) or correction (:312-330)
//                    pass.
#pragma once
#include "device_common.cuh"

namespace hbtu {

constexpr int kLB = 256;  // threads of a chunk-sum block
constexpr int kSums = 24;  // doubles per reduction chunk

// One step of a warp reduce-scatter of N doubles: the lanes of each pair
// (lane, lane ^ o) add the same two values as an xor butterfly would, but
// each keeps only half of them (the lane with bit o set keeps the upper
// half, indices h .. N-1 with h = ceil(N/2), padded by one zero when N is
// odd).  Five steps (o = 16 .. 1) leave each sum in one lane, bit-identical
// to the butterfly's result (same pairs, same order of association).
template <int N>
__device__ __forceinline__ void rs_step(const double (&cur)[N], double (&nxt)[(N + 1) / 2], int o,
                                        bool upper)
{
  constexpr int h = (N + 1) / 2;
#pragma unroll
  for (int j = 0; j < h; j++) {
    const double lo = cur[j], hi = (j + h < N) ? cur[j + h] : 0.;
    const double recv = __shfl_xor_sync(0xffffffffu, upper ? lo : hi, o);
    nxt[j] = (upper ? hi : lo) + recv;
  }
}

// Sums of K values over a block of kLB threads into out[0 .. K).  The
// chunk's elements p = threadIdx.x + j*kLB (0 <= p < nvalid) are spread over
// the warps in order, so a warp with 32*w >= nvalid holds only zeros and
// writes them without reducing (small subhaloes leave most warps empty).
template <int K>
__device__ void block_sum(double (&v)[K], double *out, int nvalid)
{
  static_assert(K >= 1 && K <= 32, "one sum per lane at most");
  __shared__ double sh[K][kLB / 32];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (32 * w < nvalid) {
    constexpr int n1 = (K + 1) / 2, n2 = (n1 + 1) / 2, n3 = (n2 + 1) / 2, n4 = (n3 + 1) / 2,
                  n5 = (n4 + 1) / 2;
    double a1[n1], a2[n2], a3[n3], a4[n4], a5[n5];
    rs_step<K>(v, a1, 16, lane & 16);
    rs_step<n1>(a1, a2, 8, lane & 8);
    rs_step<n2>(a2, a3, 4, lane & 4);
    rs_step<n3>(a3, a4, 2, lane & 2);
    rs_step<n4>(a4, a5, 1, lane & 1);
    // the index of the sum this lane holds: the split follows the padded
    // sizes N; n counts the lane's real (unpadded) values
    int base = 0, n = K, N = K;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const int h = (N + 1) / 2;
      if (lane & o) {
        base += h;
        n = max(0, n - h);
      } else {
        n = min(n, h);
      }
      N = h;
    }
    if (n >= 1) sh[base][w] = a5[0];
  } else if (lane < K) {
    sh[lane][w] = 0.;
  }
  __syncthreads();
  if (threadIdx.x < K) {
    double t = 0.;
    for (int j = 0; j < kLB / 32; j++) t += sh[threadIdx.x][j];
    out[threadIdx.x] = t;
  }
}

// NEAREST(x - o) * m in double (AveragePosition's term, src/subhalo_unbind.cpp:
// 139-188), bit for bit, mostly without double arithmetic.  When the float
// difference s = x - o is exact (a float TwoSum with a zero error term) and
// |s| < box, the wrap s -+ box is exact in float too (Sterbenz: box/2 < |s| <
// 2 box), and the product of the two floats is exact as a float product plus
// its fma remainder, added exactly in double: one FP64 add instead of the
// double subtract, wrap and multiply (FP64 runs at 1/64 of the FP32 rate on
// this GPU).  Otherwise the double path.
__device__ __forceinline__ double rel_times_mass(float x, float o, double od, float m, double md,
                                                 const DevParams &P)
{
  const float s = __fsub_rn(x, o);
  const float bb = __fsub_rn(s, x);
  const float err = __fadd_rn(__fsub_rn(x, __fsub_rn(s, bb)), __fsub_rn(-o, bb));
  if (err == 0.f && fabsf(s) < P.box) {
    const float q = s > P.boxhalf ? __fsub_rn(s, P.box) : (s < -P.boxhalf ? __fadd_rn(s, P.box) : s);
    const float p = __fmul_rn(q, m);
    const float r = __fmaf_rn(q, m, -p);  // q*m - p, exact
    return dadd(f2d(p), f2d(r));
  }
  return dmul(nearest_d(dsub(f2d(x), od), P), md);
}

// One bound particle's terms of the frame sums: w[0] += m, w[1..3] += v*m
// (float products), w[4..6] += NEAREST(x - o)*m about the origin o (periodic)
// or x*m (float products).
__device__ __forceinline__ void frame_terms(float4 a, float4 u, float4 o, const double (&od)[3],
                                            const DevParams &P, double (&w)[7])
{
  const float m = a.w;
  const double md = f2d(m);
  w[0] += md;
  w[1] += f2d(fmul(u.x, m));
  w[2] += f2d(fmul(u.y, m));
  w[3] += f2d(fmul(u.z, m));
  if (P.periodic) {
    w[4] += rel_times_mass(a.x, o.x, od[0], m, md, P);
    w[5] += rel_times_mass(a.y, o.y, od[1], m, md, P);
    w[6] += rel_times_mass(a.z, o.z, od[2], m, md, P);
  } else {
    w[4] += f2d(fmul(a.x, m));
    w[5] += f2d(fmul(a.y, m));
    w[6] += f2d(fmul(a.z, m));
  }
}

// The decisions of subhalo s after a pass whose partition kept nb particles
// bound; v[0..6] are the bound block's sums (mass, mass-weighted velocity,
// mass-weighted position about Elist[0]) when nb > 1.
__device__ __forceinline__ void control_segment(const Ctx &c, SegState &sg, int nb,
                                                const double (&v)[7], int max_passes)
{
  const DevParams &P = c.P;
  const int nl = sg.nlast;
  sg.passes++;
  sg.evals += sg.ntgt;
  if (sg.tgt_mode == 0) sg.coh_n = sg.ntgt;
  if (nb < P.minpart) {  // disruption (src/subhalo_unbind.cpp:361-379)
    sg.status = SEG_DISRUPTED;
    sg.e0 = c.eE[sg.off];
    sg.nbound = 1;
    sg.nlast = 1;
    for (int j = 0; j < 3; j++) {
      sg.ref_pos[j] = sg.mb_pos[j];
      sg.ref_vel[j] = sg.mb_vel[j];
    }
    const int k = sg.first_mb < sg.n ? sg.first_mb : 0;
    sg.mbound = c.pm[sg.off + k].w;
    sg.ub_lo = sg.ub_hi = 0;
    return;
  }
  sg.ub_lo = nb;
  sg.ub_hi = nl;
  const int ndiff = nl - nb;
  if (ndiff < nb && (P.maxsample <= 0 || ndiff < P.maxsample)) {  // :383-392
    sg.corr = 1;
    for (int j = 0; j < 3; j++) {
      sg.old_pos[j] = sg.ref_pos[j];
      sg.old_vel[j] = sg.ref_vel[j];
    }
  }
  if (nb == 1) {  // AverageVelocity / AveragePosition with one particle
    const int pid = c.epid[sg.off];
    const float4 a = c.pm[pid], u = c.vel[pid];
    sg.mbound = a.w;
    sg.ref_vel[0] = u.x;
    sg.ref_vel[1] = u.y;
    sg.ref_vel[2] = u.z;
    sg.ref_pos[0] = a.x;
    sg.ref_pos[1] = a.y;
    sg.ref_pos[2] = a.z;
  } else if (nb > 1) {
    const double msum = v[0];
    sg.mbound = (float)msum;
    for (int j = 0; j < 3; j++) sg.ref_vel[j] = __double2float_rn(ddiv(v[1 + j], msum));
    const float4 o = c.pm[c.epid[sg.off]];
    const double org[3] = {o.x, o.y, o.z};
    for (int j = 0; j < 3; j++) {
      double x = ddiv(v[4 + j], msum);
      if (P.periodic) x = dadd(x, org[j]);
      sg.ref_pos[j] = __double2float_rn(x);
    }
  } else {
    sg.mbound = 0.f;
  }
  if (__int2float_rn(nb) >= fmul(__int2float_rn(nl), P.prec)) {  // :395
    sg.status = SEG_CONVERGED;
    sg.nbound = nb;
    sg.refine = P.refine && nb > P.maxsample;  // :406-407
    return;
  }
  sg.nbound = nb;
  if (sg.corr) {  // correction pass over the removed block (:312-330)
    sg.mode = MODE_CORRECTION;
    sg.t0 = nb;
    sg.ntree = nl - nb;
    sg.ntgt = nb;
    sg.mfac = 1.f;
    relvel(sg.old_pos, sg.old_vel, sg.ref_pos, sg.ref_vel, sg.dV, P);
    sg.dK = __double2float_rn(dmul(0.5, (double)vdot(sg.dV, sg.dV)));
    sg.tgt_mode = sg.coh_n > 0 ? 1 : 2;
  } else {  // full pass (:331-356)
    sg.mode = MODE_FULL;
    sg.t0 = 0;
    sg.ntgt = nb;
    if (P.maxsample > 0 && nb > P.maxsample) {
      sg.ntree = (int)P.maxsample;
      sg.mfac = __fdiv_rn(__int2float_rn(nb), (float)P.maxsample);
      sg.tgt_mode = 2;
    } else {
      sg.ntree = nb;
      sg.mfac = 1.f;
      sg.tgt_mode = 0;
    }
  }
  sg.nlast = nb;
  if (sg.passes >= max_passes) sg.status = SEG_FAILED;
}

}  // namespace hbtu
