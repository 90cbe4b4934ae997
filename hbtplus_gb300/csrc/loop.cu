// loop.cu -- the iterate-until-converged loop of Subhalo_t::Unbind
// (src/subhalo_unbind.cpp:263-431), for every subhalo of a batch at once.
//
// One pass = tree build (tree.cu) + energies (walk.cu) + the kernels here:
//   partition   PartitionBindingEnergy (:21-58) reproduced exactly: its
//               two-pointer exchange is a fixed function of the sign pattern
//               (k-th positive from the left trades with the k-th negative
//               from the right), computed with prefix counts, no serial scan;
//   averages    AverageVelocity / AveragePosition (:108-188) as deterministic
//               FP64 chunk reductions;
//   control     disruption (:361-379), the sticky correction flag (:383-392),
//               convergence on the particle count (:395), and the set-up of
//               the next pass (full :331-356 or correction :312-330);
//   block sorts the stable energy sorts of the unbound block (:382) and, at
//               the end, of the bound block (:405);
//   finalize    the permuted particle order (:409-418), AverageKinematics
//               (:189-232) and CountParticleTypes (src/subhalo.cpp:400-444).
#include "loop_ops.cuh"

namespace hbtu {
namespace {

constexpr int kPlanThreads = 1024;

inline unsigned nblk(long long n, int b = kLB) { return (unsigned)((n + b - 1) / b); }

// Exclusive scan over segments of up to 4 counters, one block of 1024 threads,
// each thread owning a contiguous run of segments (a few, for up to a few
// thousand subhaloes).  The getter is a template argument so it inlines: each
// thread's segments are then read with independent loads in flight (an
// indirect call per segment serialises them).
template <int (*getter)(const Ctx &, int, int *)>
__device__ void plan_scan4_thread(int S, const Ctx &c, int *out0, int *out1, int *out2, int *out3,
                           int *tot)
{
  __shared__ int wsum[4][kPlanThreads / 32];
  const int per = (S + kPlanThreads - 1) / kPlanThreads;
  const int b = threadIdx.x * per, e = min(S, b + per);
  int loc[4] = {0, 0, 0, 0}, v[4];
  constexpr int kKeep = 4;  // segments per thread whose counters stay in registers
  int kept[kKeep][4];
#pragma unroll
  for (int q = 0; q < kKeep; q++)
    if (b + q < e) {
      getter(c, b + q, kept[q]);
      for (int k = 0; k < 4; k++) loc[k] += kept[q][k];
    }
  for (int s = b + kKeep; s < e; s++) {
    getter(c, s, v);
    for (int k = 0; k < 4; k++) loc[k] += v[k];
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int inc[4];
  for (int k = 0; k < 4; k++) {
    int x = loc[k];
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    inc[k] = x;
    if (lane == 31) wsum[k][w] = x;
  }
  __syncthreads();
  if (w == 0) {
    for (int k = 0; k < 4; k++) {
      int x = wsum[k][lane];
      for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
      }
      wsum[k][lane] = x;
    }
  }
  __syncthreads();
  int run[4];
  for (int k = 0; k < 4; k++) run[k] = (w > 0 ? wsum[k][w - 1] : 0) + inc[k] - loc[k];
  int *outs[4] = {out0, out1, out2, out3};
#pragma unroll
  for (int q = 0; q < kKeep; q++)
    if (b + q < e)
      for (int k = 0; k < 4; k++) {
        if (outs[k]) outs[k][b + q] = run[k];
        run[k] += kept[q][k];
      }
  for (int s = b + kKeep; s < e; s++) {
    getter(c, s, v);
    for (int k = 0; k < 4; k++) {
      if (outs[k]) outs[k][s] = run[k];
      run[k] += v[k];
    }
  }
  if (threadIdx.x == kPlanThreads - 1) {
    for (int k = 0; k < 4; k++) {
      tot[k] = run[k];
      if (outs[k]) outs[k][S] = run[k];
    }
  }
  __syncthreads();
}

// The same scan for many subhaloes (the gathered plans): warp w owns a
// contiguous run of segments (a multiple of 32 long) and its
// lanes read consecutive segments, so a warp's loads are coalesced and
// independent: a first sweep sums the run, one warp scans the 32 run totals,
// a second sweep scans the run 32 segments at a time on top of its start.  The
// getter is a template argument so it inlines.
template <int (*getter)(const Ctx &, int, int *)>
__device__ void plan_scan4_warp(int S, const Ctx &c, int *out0, int *out1, int *out2, int *out3,
                                int *tot)
{
  constexpr int kWarps = kPlanThreads / 32;
  static_assert(kWarps == 32, "one lane of warp 0 per warp");
  constexpr unsigned kFull = 0xffffffffu;
  __shared__ int wsum[4][kWarps];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int per = ((S + kWarps - 1) / kWarps + 31) & ~31;
  const int b = w * per, e = min(S, b + per);
  int loc[4] = {0, 0, 0, 0}, v[4];
  for (int s = b + lane; s < e; s += 32) {
    getter(c, s, v);
    for (int k = 0; k < 4; k++) loc[k] += v[k];
  }
  for (int k = 0; k < 4; k++) {
    loc[k] = __reduce_add_sync(kFull, loc[k]);
    if (lane == 0) wsum[k][w] = loc[k];
  }
  __syncthreads();
  if (w == 0) {
    for (int k = 0; k < 4; k++) {
      const int t = wsum[k][lane];
      int x = t;
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(kFull, x, o);
        if (lane >= o) x += y;
      }
      wsum[k][lane] = x - t;  // start of warp lane's run
      if (lane == 31) tot[k] = x;
    }
  }
  __syncthreads();
  int *outs[4] = {out0, out1, out2, out3};
  int run[4];
  for (int k = 0; k < 4; k++) run[k] = wsum[k][w];
  for (int s0 = b; s0 < e; s0 += 32) {
    const int s = s0 + lane;
    int x[4] = {0, 0, 0, 0};
    if (s < e) getter(c, s, x);
    for (int k = 0; k < 4; k++) {
      int inc = x[k];
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(kFull, inc, o);
        if (lane >= o) inc += y;
      }
      if (s < e && outs[k]) outs[k][s] = run[k] + inc - x[k];
      run[k] += __shfl_sync(kFull, inc, 31);
    }
  }
  if (threadIdx.x == 0)
    for (int k = 0; k < 4; k++)
      if (outs[k]) outs[k][S] = tot[k];
  __syncthreads();
}

// ---------------------------------------------------------------- init
__global__ void k_init(Ctx c, const float *pos, const float *vel, const float *mass,
                       const long long *id)
{
  HBTU_KERNEL_PROLOGUE();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.N) return;
  const int s = upper_bound_i(c.seg_off, c.S + 1, i) - 1;
  c.pseg[i] = s;
  c.pm[i] = make_float4(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], mass[i]);
  c.vel[i] = make_float4(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2], 0.f);
  c.epid[i] = i;
  c.eE[i] = 0.f;
  c.epos_of_pid[i] = i;
  SegState &sg = c.seg[s];
  if (id[i] == sg.mb_id) atomicMin(&sg.first_mb, i - sg.off);
}

// ---------------------------------------------------------------- plans
__device__ int get_pass(const Ctx &c, int s, int *v)
{
  const SegState &sg = c.seg[s];
  const bool act = sg.status == SEG_ACTIVE;
  v[0] = act ? sg.ntree : 0;
  v[1] = act ? (sg.ntree + kChunk - 1) / kChunk : 0;
  v[2] = act ? (sg.tgt_mode == 1 ? sg.coh_n : sg.ntgt) : 0;
  v[3] = sg.ub_hi - sg.ub_lo;
  return 0;
}
// targets of the pass, subhaloes in size order (largest first)
__device__ int get_targets_sorted(const Ctx &c, int k, int *v)
{
  const SegState &sg = c.seg[c.seg_order[k]];
  const bool act = sg.status == SEG_ACTIVE;
  v[0] = act ? (sg.tgt_mode == 1 ? sg.coh_n : sg.ntgt) : 0;
  v[1] = v[2] = v[3] = 0;
  return 0;
}
__device__ int get_bound(const Ctx &c, int s, int *v)
{
  const bool act = c.seg[s].status == SEG_ACTIVE;
  const int nb = act ? c.part_info[8 * s + 7] : 0;
  v[0] = (nb + kChunk - 1) / kChunk;
  v[1] = v[2] = v[3] = 0;
  return 0;
}
__device__ int get_final(const Ctx &c, int s, int *v)
{
  const SegState &sg = c.seg[s];
  const bool conv = sg.status == SEG_CONVERGED || sg.status == SEG_FAILED;
  const int nb = conv ? sg.nbound : 0;
  v[0] = (nb + kChunk - 1) / kChunk;
  v[1] = nb;  // bound block to sort
  v[2] = sg.refine ? 1 : 0;
  v[3] = 0;
  return 0;
}
__device__ int get_refine(const Ctx &c, int s, int *v)
{
  const SegState &sg = c.seg[s];
  v[0] = sg.refine ? (int)min((long long)sg.nbound, c.P.maxsample) : 0;
  v[1] = v[2] = v[3] = 0;
  return 0;
}

// Large batches: the per-subhalo counters are first gathered into dense
// arrays by a grid of threads, so the one-block scans read them coalesced
// (read from the subhalo records, one block's loads serialise on one SM).
constexpr int kPlanGatherMin = 4096;

template <int (*getter)(const Ctx &, int, int *)>
__device__ __forceinline__ int4 counts_of(const Ctx &c, int s)
{
  int v[4];
  getter(c, s, v);
  return make_int4(v[0], v[1], v[2], v[3]);
}

__global__ void k_plan_gather(Ctx c, int mode)
{
  HBTU_KERNEL_PROLOGUE();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= c.S) return;
  if (mode == 0) {
    c.plan_cnt[s] = counts_of<get_pass>(c, s);
    int4 t = counts_of<get_targets_sorted>(c, s);  // by position in size order
    t.y = c.seg[s].status == SEG_ACTIVE;           // summed only
    t.z = t.y ? c.seg[s].nlast : 0;                // maximum only
    c.plan_cnt2[s] = t;
    c.plan_inter[s] = c.seg[s].interactions;
  } else if (mode == 1) {
    c.plan_cnt[s] = counts_of<get_bound>(c, s);
  } else if (mode == 2) {
    c.plan_cnt[s] = counts_of<get_final>(c, s);
  } else {
    c.plan_cnt[s] = counts_of<get_refine>(c, s);
  }
}

__device__ int get_cnt(const Ctx &c, int s, int *v)
{
  const int4 q = c.plan_cnt[s];
  v[0] = q.x;
  v[1] = q.y;
  v[2] = q.z;
  v[3] = q.w;
  return 0;
}
__device__ int get_cnt2(const Ctx &c, int s, int *v)
{
  const int4 q = c.plan_cnt2[s];
  v[0] = q.x;
  v[1] = q.y;
  v[2] = q.z;
  v[3] = q.w;
  return 0;
}

__global__ void __launch_bounds__(kPlanThreads) k_plan(Ctx c, int mode, int gathered)
{
  HBTU_KERNEL_PROLOGUE();
  __shared__ int tot[4];
  __shared__ int nact;
  if (threadIdx.x == 0) nact = 0;
  __syncthreads();
  if (mode == 0) {
    __shared__ unsigned long long inter;
    if (threadIdx.x == 0) inter = 0;
    __syncthreads();
    __shared__ int maxn;
    if (threadIdx.x == 0) maxn = 0;
    __syncthreads();
    int cnt = 0, mx = 0;
    unsigned long long it = 0;
    for (int s = threadIdx.x; s < c.S; s += kPlanThreads) {
      if (gathered) {
        it += (unsigned long long)c.plan_inter[s];
        mx = max(mx, c.plan_cnt2[s].z);
      } else {
        const SegState &sg = c.seg[s];
        const bool act = sg.status == SEG_ACTIVE;
        cnt += act;
        mx = max(mx, act ? sg.nlast : 0);
        it += (unsigned long long)sg.interactions;
      }
    }
    // warp sums first: one shared atomic per warp, not per thread
    cnt = __reduce_add_sync(0xffffffffu, cnt);
    mx = __reduce_max_sync(0xffffffffu, mx);
    for (int o = 16; o > 0; o >>= 1) it += __shfl_xor_sync(0xffffffffu, it, o);
    if ((threadIdx.x & 31) == 0) {
      atomicAdd(&nact, cnt);
      atomicAdd(&inter, it);
      atomicMax(&maxn, mx);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      c.plan->inter_done = (long long)inter;
      c.plan->max_nlast = maxn;
    }
    if (gathered)
      plan_scan4_warp<get_cnt>(c.S, c, c.tree_base, c.tchunk_base, nullptr, c.ub_base, tot);
    else
      plan_scan4_thread<get_pass>(c.S, c, c.tree_base, c.tchunk_base, nullptr, c.ub_base, tot);
    if (threadIdx.x == 0) {
      c.plan->ntree_total = tot[0];
      c.plan->nchunks_tree = tot[1];
      c.plan->nsort_total = tot[3];
      c.plan->max_levels = 0;
    }
    __syncthreads();
    if (gathered) {
      plan_scan4_warp<get_cnt2>(c.S, c, c.tgt_base, nullptr, nullptr, nullptr, tot);
      if (threadIdx.x == 0) {
        c.plan->ntgt_total = tot[0];
        c.plan->nactive = tot[1];
      }
    } else {
      plan_scan4_thread<get_targets_sorted>(c.S, c, c.tgt_base, nullptr, nullptr, nullptr, tot);
      if (threadIdx.x == 0) {
        c.plan->ntgt_total = tot[0];
        c.plan->nactive = nact;
      }
    }
  } else if (mode == 1) {
    if (gathered)
      plan_scan4_warp<get_cnt>(c.S, c, c.bchunk_base, nullptr, nullptr, nullptr, tot);
    else
      plan_scan4_thread<get_bound>(c.S, c, c.bchunk_base, nullptr, nullptr, nullptr, tot);
    if (threadIdx.x == 0) c.plan->nchunks_bound = tot[0];
  } else if (mode == 2) {
    if (gathered)
      plan_scan4_warp<get_cnt>(c.S, c, c.bchunk_base, c.ub_base, nullptr, nullptr, tot);
    else
      plan_scan4_thread<get_final>(c.S, c, c.bchunk_base, c.ub_base, nullptr, nullptr, tot);
    if (threadIdx.x == 0) {
      c.plan->nchunks_bound = tot[0];
      c.plan->nsort_total = tot[1];
      c.plan->nrefine = tot[2];
    }
  } else {
    if (gathered)
      plan_scan4_warp<get_cnt>(c.S, c, c.ub_base, nullptr, nullptr, nullptr, tot);
    else
      plan_scan4_thread<get_refine>(c.S, c, c.ub_base, nullptr, nullptr, nullptr, tot);
    if (threadIdx.x == 0) c.plan->nsort_total = tot[0];
  }
}

// ---------------------------------------------------------------- partition
// part_info[8s+]: 0 nPos, 1 nNeg, 2 firstF, 3 firstG, 4 m_b, 5 m_f, 6 void, 7 Nbound
__global__ void __launch_bounds__(kLB) k_part_codes(Ctx c)
{
  HBTU_KERNEL_PROLOGUE();
  const int p = blockIdx.x * kLB + threadIdx.x;
  if (p > c.N) return;
  if (p == c.N) {
    c.pcode[p] = 0;
    return;
  }
  const int s = c.pseg[p];
  const SegState &sg = c.seg[s];
  const int l = p - sg.off;
  long long code = 0;
  if (sg.status == SEG_ACTIVE && l >= 1 && l < sg.nlast) {
    const float e = c.eE[p];
    code = (e < 0.f ? (1ll << 32) : 0ll) | (e > 0.f ? 1ll : 0ll);
  }
  c.pcode[p] = code;
  if (l == 0) {
    c.part_info[8 * s + 2] = 0x7fffffff;
    c.part_info[8 * s + 3] = 0x7fffffff;
  }
}

__device__ __forceinline__ int lo32(long long x) { return (int)(x & 0xffffffffll); }
__device__ __forceinline__ int hi32(long long x) { return (int)(x >> 32); }

__global__ void __launch_bounds__(kLB) k_part_pq(Ctx c)
{
  HBTU_KERNEL_PROLOGUE();
  const int p = blockIdx.x * kLB + threadIdx.x;
  if (p >= c.N) return;
  const int s = c.pseg[p];
  const SegState &sg = c.seg[s];
  const int l = p - sg.off;
  if (sg.status != SEG_ACTIVE || sg.nlast < 2) return;
  const long long x1 = c.pX[sg.off + 1], xe = c.pX[sg.off + sg.nlast];
  if (l == 0) {
    c.part_info[8 * s + 0] = lo32(xe - x1);
    c.part_info[8 * s + 1] = hi32(xe - x1);
  }
  if (l < 1 || l >= sg.nlast) return;
  const float e = c.eE[p];
  if (e > 0.f) c.Pk[sg.off + lo32(c.pX[p] - x1)] = l;
  if (e < 0.f) c.Qk[sg.off + hi32(xe - c.pX[p]) - 1] = l;
}

__global__ void __launch_bounds__(kLB) k_part_fg(Ctx c)
{
  HBTU_KERNEL_PROLOGUE();
  const int p = blockIdx.x * kLB + threadIdx.x;
  if (p >= c.N) return;
  const int s = c.pseg[p];
  const SegState &sg = c.seg[s];
  const int l = p - sg.off;
  if (sg.status != SEG_ACTIVE || sg.nlast < 2 || l < 1 || l >= sg.nlast) return;
  if (!(c.eE[p] > 0.f)) return;
  const int k = lo32(c.pX[p] - c.pX[sg.off + 1]) + 1;
  const int nPos = c.part_info[8 * s + 0], nNeg = c.part_info[8 * s + 1];
  const int mn = min(nPos, nNeg);
  if (k > mn) return;
  const int Pk = l, Qk = c.Qk[sg.off + k - 1];
  if (Pk >= Qk) atomicMin(&c.part_info[8 * s + 2], k);
  if (k + 1 > nNeg || Pk >= c.Qk[sg.off + k]) atomicMin(&c.part_info[8 * s + 3], k);
}

__global__ void k_part_seg(Ctx c)
{
  HBTU_KERNEL_PROLOGUE();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= c.S) return;
  const SegState &sg = c.seg[s];
  if (sg.status != SEG_ACTIVE) return;
  int *pi = c.part_info + 8 * s;
  const float e0 = c.eE[sg.off];
  if (sg.nlast < 2) {
    pi[4] = pi[5] = pi[6] = 0;
    pi[7] = sg.nlast == 1 ? (e0 < 0.f) : 0;
    return;
  }
  const int nPos = pi[0], nNeg = pi[1], mn = min(nPos, nNeg);
  const int F = min(pi[2], mn + 1) - 1;
  const int G = min(pi[3] - 1, F);
  int mb = 0, mf = 0, vd = 0;
  if (nNeg > 0) {
    mb = 1 + G;
    mf = G + (G + 1 <= F ? 1 : 0);
    vd = (mf == mb) ? c.Pk[sg.off + mf - 1] : c.Qk[sg.off + mb - 1];
  }
  pi[4] = mb;
  pi[5] = mf;
  pi[6] = vd;
  pi[7] = vd + (e0 < 0.f);
}

__global__ void __launch_bounds__(kLB) k_part_gather(Ctx c)
{
  HBTU_KERNEL_PROLOGUE();
  const int p = blockIdx.x * kLB + threadIdx.x;
  if (p >= c.N) return;
  const int s = c.pseg[p];
  const SegState &sg = c.seg[s];
  const int l = p - sg.off;
  if (sg.status != SEG_ACTIVE || l >= sg.nlast) return;
  int src = l;
  if (sg.nlast >= 2) {
    const int *pi = c.part_info + 8 * s;
    const int nNeg = pi[1], mb = pi[4], mf = pi[5], vd = pi[6];
    const float e = c.eE[p];
    if (l == vd) {
      src = 0;
    } else if (l == 0) {
      src = nNeg >= 1 ? c.Qk[sg.off] : 0;
    } else if (e < 0.f) {
      const int kq = hi32(c.pX[sg.off + sg.nlast] - c.pX[p]);
      if (kq <= mf) src = c.Pk[sg.off + kq - 1];
    } else if (e > 0.f) {
      const int kp = lo32(c.pX[p] - c.pX[sg.off + 1]) + 1;
      if (kp <= mb - 1) src = c.Qk[sg.off + kp];
    }
  }
  c.epid2[p] = c.epid[sg.off + src];
  c.eE2[p] = c.eE[sg.off + src];
}

__global__ void __launch_bounds__(kLB) k_part_copyback(Ctx c)
{
  HBTU_KERNEL_PROLOGUE();
  const int p = blockIdx.x * kLB + threadIdx.x;
  if (p >= c.N) return;
  const SegState &sg = c.seg[c.pseg[p]];
  if (sg.status != SEG_ACTIVE || p - sg.off >= sg.nlast) return;
  const int q = c.epid2[p];
  c.epid[p] = q;
  c.eE[p] = c.eE2[p];
  c.epos_of_pid[q] = p;
}

// ---------------------------------------------------------------- averages
__global__ void __launch_bounds__(kLB) k_avg_chunks(Ctx c)
{
  HBTU_KERNEL_PROLOGUE();
  const int b = blockIdx.x;
  if (b >= c.bchunk_base[c.S]) return;
  const int s = upper_bound_i(c.bchunk_base, c.S + 1, b) - 1;
  const SegState &sg = c.seg[s];
  const int nb = c.part_info[8 * s + 7];
  const int ci = b - c.bchunk_base[s];
  const int lo = ci * kChunk, hi = min(lo + kChunk, nb);
  const float4 o = c.pm[c.epid[sg.off]];
  const double od[3] = {f2d(o.x), f2d(o.y), f2d(o.z)};
  double v[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int p = lo + threadIdx.x; p < hi; p += kLB) {
    const int pid = c.epid[sg.off + p];
    frame_terms(c.pm[pid], c.vel[pid], o, od, c.P, v);
  }
  block_sum<7>(v, c.chunk_sums + (size_t)b * kSums, hi - lo);
}

// ---------------------------------------------------------------- control
__global__ void k_control(Ctx c, int max_passes)
{
  HBTU_KERNEL_PROLOGUE();
  // one warp per subhalo: lanes 0..6 add the 7 chunk sums in chunk order
  // (each an independent chain), lane 0 then takes the decisions
  const int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (s >= c.S) return;
  SegState &sg = c.seg[s];
  if (sg.status != SEG_ACTIVE) return;
  const int nb = c.part_info[8 * s + 7];
  double part = 0.;
  if (nb > 1 && lane < 7)
    for (int b = c.bchunk_base[s]; b < c.bchunk_base[s + 1]; b++)
      part += c.chunk_sums[(size_t)b * kSums + lane];
  double v[7];
#pragma unroll
  for (int k = 0; k < 7; k++) v[k] = __shfl_sync(0xffffffffu, part, k);
  if (lane != 0) return;
  control_segment(c, sg, nb, v, max_passes);
}

// ---------------------------------------------------------------- block sorts
// which 0: [ub_lo, ub_hi) of every subhalo; which 1: [0, nbound) of converged.
__device__ __forceinline__ bool block_of(const SegState &sg, int which, int &lo, int &hi,
                                         long long c_maxsample)
{
  if (which == 0) {
    lo = sg.ub_lo;
    hi = sg.ub_hi;
  } else if (which == 2) {
    lo = 0;
    hi = sg.refine ? (int)min((long long)sg.nbound, c_maxsample) : 0;
  } else {
    lo = 0;
    hi = (sg.status == SEG_CONVERGED || sg.status == SEG_FAILED) ? sg.nbound : 0;
  }
  return hi > lo;
}

__global__ void __launch_bounds__(kLB) k_blk_gather(Ctx c, int which)
{
  HBTU_KERNEL_PROLOGUE();
  const int p = blockIdx.x * kLB + threadIdx.x;
  if (p >= c.N) return;
  const int s = c.pseg[p];
  const SegState &sg = c.seg[s];
  int lo, hi;
  if (!block_of(sg, which, lo, hi, c.P.maxsample)) return;
  const int l = p - sg.off;
  if (l < lo || l >= hi) return;
  const int e = c.ub_base[s] + (l - lo);
  c.sb.hi_a[e] = (unsigned)s;
  c.sb.lo_a[e] = (unsigned long long)float_key(which == 2 ? c.eR[p] : c.eE[p]) << 32;
  c.sb.val_a[e] = p;
}

__global__ void __launch_bounds__(kLB) k_blk_scatter(Ctx c, int which, int total)
{
  HBTU_KERNEL_PROLOGUE();
  const int e = blockIdx.x * kLB + threadIdx.x;
  if (e >= total) return;
  const int s = c.sb.hi_a[e];
  const SegState &sg = c.seg[s];
  int lo, hi;
  block_of(sg, which, lo, hi, c.P.maxsample);
  const int dst = sg.off + lo + (e - c.ub_base[s]);
  const int src = c.sb.val_a[e];
  c.epid2[dst] = c.epid[src];
  c.eE2[dst] = c.eE[src];
}

__global__ void __launch_bounds__(kLB) k_blk_copyback(Ctx c, int which, int total)
{
  HBTU_KERNEL_PROLOGUE();
  const int e = blockIdx.x * kLB + threadIdx.x;
  if (e >= total) return;
  const int s = c.sb.hi_a[e];
  SegState &sg = c.seg[s];
  int lo, hi;
  block_of(sg, which, lo, hi, c.P.maxsample);
  const int dst = sg.off + lo + (e - c.ub_base[s]);
  const int q = c.epid2[dst];
  c.epid[dst] = q;
  c.eE[dst] = c.eE2[dst];
  c.epos_of_pid[q] = dst;
}

// RefineBindingEnergyOrder (src/subhalo_unbind.cpp:234-262): one more full
// pass over the first MaxSampleSize bound particles with their own masses;
// energies go to eR and only reorder the list (its stored energies stay).
__global__ void k_refine_mode(Ctx c, int enter)
{
  HBTU_KERNEL_PROLOGUE();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= c.S) return;
  SegState &sg = c.seg[s];
  if (!sg.refine) return;
  if (enter) {
    sg.status = SEG_ACTIVE;
    sg.mode = MODE_REFINE;
    sg.t0 = 0;
    sg.ntree = (int)min((long long)sg.nbound, c.P.maxsample);
    sg.ntgt = sg.ntree;
    sg.mfac = 1.f;
    sg.tgt_mode = 0;
    sg.evals += sg.ntgt;
  } else {
    sg.status = SEG_CONVERGED;
  }
}

__global__ void k_blk_clear(Ctx c)
{
  HBTU_KERNEL_PROLOGUE();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= c.S) return;
  c.seg[s].ub_lo = c.seg[s].ub_hi = 0;
}

// ---------------------------------------------------------------- finalize
__global__ void __launch_bounds__(kLB) k_kin_chunks(Ctx c)
{
  HBTU_KERNEL_PROLOGUE();
  const int b = blockIdx.x;
  if (b >= c.bchunk_base[c.S]) return;
  const int s = upper_bound_i(c.bchunk_base, c.S + 1, b) - 1;
  const SegState &sg = c.seg[s];
  const DevParams &P = c.P;
  const int nb = sg.nbound;
  const int ci = b - c.bchunk_base[s];
  const int lo = ci * kChunk, hi = min(lo + kChunk, nb);
  double v[18];
  for (int k = 0; k < 18; k++) v[k] = 0.;
  int cnt[6] = {0, 0, 0, 0, 0, 0};
  const double Pa = (double)P.a, PHz = (double)P.Hz;
  for (int p = lo + threadIdx.x; p < hi; p += kLB) {
    const int pid = c.epid[sg.off + p];
    const float4 a = c.pm[pid], u = c.vel[pid];
    const float m = a.w;
    const float x[3] = {a.x, a.y, a.z}, w[3] = {u.x, u.y, u.z};
    const double md = f2d(m);
    v[0] += f2d(fmul(c.eE[sg.off + p], m));
    double dx[3], dv[3];
    for (int j = 0; j < 3; j++) {
      // the wrap of a float difference below the box size is exact in float
      // (Sterbenz), so it gives the double wrap's bits without the FP64 pipe
      const float d = fsub(x[j], sg.ref_pos[j]);
      if (!P.periodic)
        dx[j] = f2d(d);
      else if (fabsf(d) < P.box)
        dx[j] = f2d(nearest_f(d, P));
      else
        dx[j] = nearest_d(f2d(d), P);
      dx[j] = dmul(dx[j], Pa);
      dv[j] = dadd(f2d(fsub(w[j], sg.ref_vel[j])), dmul(PHz, dx[j]));
      v[1] += dmul(dmul(dv[j], dv[j]), md);
    }
    v[2] += dmul(dsub(dmul(dx[1], dv[2]), dmul(dx[2], dv[1])), md);
    v[3] += dmul(dsub(dmul(dx[2], dv[0]), dmul(dx[0], dv[2])), md);
    v[4] += dmul(dsub(dmul(dx[0], dv[1]), dmul(dx[1], dv[0])), md);
    v[5] += md;
    const int t = c.type ? c.type[pid] : 1;
    const bool skip = (nb <= 100 && c.id[pid] == -1) || t < 0 || t > 5;
    if (!skip) {
      switch (t) {  // one double add per particle (the type is nearly always warp-uniform)
        case 0: cnt[0]++; v[12] += md; break;
        case 1: cnt[1]++; v[13] += md; break;
        case 2: cnt[2]++; v[14] += md; break;
        case 3: cnt[3]++; v[15] += md; break;
        case 4: cnt[4]++; v[16] += md; break;
        default: cnt[5]++; v[17] += md; break;
      }
    }
  }
#pragma unroll
  for (int q = 0; q < 6; q++) v[6 + q] = (double)cnt[q];  // exact: counts < 2^53
  block_sum<18>(v, c.chunk_sums + (size_t)b * kSums, hi - lo);
}

__global__ void k_final_seg(Ctx c, hbtu_result *res)
{
  HBTU_KERNEL_PROLOGUE();
  // one warp per subhalo: lanes 0..17 add the 18 chunk sums in chunk order,
  // lane 0 then writes the result
  const int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (s >= c.S) return;
  const SegState &sg = c.seg[s];
  const DevParams &P = c.P;
  const bool summed = sg.status != SEG_TRIVIAL && sg.status != SEG_DISRUPTED;
  double part = 0.;
  if (summed && lane < 18)
    for (int b = c.bchunk_base[s]; b < c.bchunk_base[s + 1]; b++)
      part += c.chunk_sums[(size_t)b * kSums + lane];
  double v[18];
#pragma unroll
  for (int k = 0; k < 18; k++) v[k] = __shfl_sync(0xffffffffu, part, k);
  if (lane != 0) return;
  hbtu_result r;
  memset(&r, 0, sizeof(r));
  r.too_few = sg.n < P.minpart;
  r.iterations = sg.passes;
  r.evaluations = sg.evals;
  r.interactions = sg.interactions;
  for (int j = 0; j < 3; j++) {
    r.ref_pos[j] = sg.ref_pos[j];
    r.ref_vel[j] = sg.ref_vel[j];
    r.mostbound_pos[j] = sg.mb_pos[j];
    r.mostbound_vel[j] = sg.mb_vel[j];
  }
  if (sg.status == SEG_TRIVIAL) {  // src/subhalo_unbind.cpp:275-293 + CountParticles
    r.nbound = sg.n;
    if (sg.n == 1) {
      const int t = c.type ? c.type[sg.off] : 1;
      const float m = c.pm[sg.off].w;
      if (t >= 0 && t <= 5) {
        r.nbound_type[t] = 1;
        r.mbound_type[t] = m;
      }
      float acc = 0.f;
      for (int k = 0; k < 6; k++) acc = fadd(acc, r.mbound_type[k]);
      r.mbound = acc;
    }
  } else if (sg.status == SEG_DISRUPTED) {
    r.disrupted = 1;
    r.nbound = 1;
    r.mbound = sg.mbound;
    const int k = sg.first_mb < sg.n ? sg.first_mb : 0;
    const int t = c.type ? c.type[sg.off + k] : 1;
    const bool skip = c.id[sg.off + k] == -1 || t < 0 || t > 5;
    if (!skip) {
      r.nbound_type[t] = 1;
      r.mbound_type[t] = c.pm[sg.off + k].w;
    }
  } else {
    r.converged = sg.status == SEG_CONVERGED;
    if (sg.status == SEG_FAILED) r.status = HBTU_ERR_NOT_CONVERGED;
    r.nbound = sg.nbound;
    r.mbound = sg.mbound;
    if (sg.nbound > 0) {
      const int pid = c.epid[sg.off];
      const float4 a = c.pm[pid], u = c.vel[pid];
      r.mostbound_pos[0] = a.x;
      r.mostbound_pos[1] = a.y;
      r.mostbound_pos[2] = a.z;
      r.mostbound_vel[0] = u.x;
      r.mostbound_vel[1] = u.y;
      r.mostbound_vel[2] = u.z;
    }
    if (sg.nbound > 1) {
      const double M = v[5];
      const double E = ddiv(v[0], M);
      const double K = dmul(v[1], ddiv(0.5, M));
      r.specific_potential = __double2float_rn(dsub(E, K));
      r.specific_kinetic = __double2float_rn(K);
      for (int j = 0; j < 3; j++) r.specific_angmom[j] = __double2float_rn(ddiv(v[2 + j], M));
    }
    for (int t = 0; t < 6; t++) {
      r.nbound_type[t] = (int64_t)v[6 + t];
      r.mbound_type[t] = (float)v[12 + t];
    }
  }
  res[s] = r;
}

__global__ void __launch_bounds__(kLB) k_final_out(Ctx c, int64_t *order, float *energy)
{
  HBTU_KERNEL_PROLOGUE();
  const int p = blockIdx.x * kLB + threadIdx.x;
  if (p >= c.N) return;
  const SegState &sg = c.seg[c.pseg[p]];
  const int l = p - sg.off;
  if (sg.status == SEG_TRIVIAL) {
    order[p] = l;
    energy[p] = 0.f;
  } else if (sg.status == SEG_DISRUPTED) {
    const int k = sg.first_mb < sg.n ? sg.first_mb : 0;
    order[p] = l == 0 ? k : (l == k ? 0 : l);
    energy[p] = l == 0 ? sg.e0 : __int_as_float(0x7fc00000);
  } else {
    order[p] = c.epid[p] - sg.off;
    energy[p] = c.eE[p];
  }
}

// Deterministic per-subhalo sums of x[off_s .. off_s + n_s): one block per
// 1024-element chunk (fixed-order tree), then the chunks of each subhalo in order.
__global__ void __launch_bounds__(kLB) k_segsum_chunks(Ctx c, const double *x)
{
  HBTU_KERNEL_PROLOGUE();
  const int b = blockIdx.x;
  if (b >= c.bchunk_base[c.S]) return;
  const int s = upper_bound_i(c.bchunk_base, c.S + 1, b) - 1;
  const SegState &sg = c.seg[s];
  const int lo = (b - c.bchunk_base[s]) * kChunk, hi = min(lo + kChunk, sg.n);
  double v[1] = {0.};
  for (int p = lo + threadIdx.x; p < hi; p += kLB) v[0] += x[sg.off + p];
  block_sum<1>(v, c.chunk_sums + (size_t)b * kSums, hi - lo);
}

__global__ void k_segsum_combine(Ctx c, double *out)
{
  HBTU_KERNEL_PROLOGUE();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= c.S) return;
  double t = 0.;
  for (int b = c.bchunk_base[s]; b < c.bchunk_base[s + 1]; b++) t += c.chunk_sums[(size_t)b * kSums];
  out[s] = t;
}

__device__ int get_all_chunks(const Ctx &c, int s, int *v)
{
  v[0] = (c.seg[s].n + kChunk - 1) / kChunk;
  v[1] = v[2] = v[3] = 0;
  return 0;
}

__global__ void __launch_bounds__(kPlanThreads) k_plan_all(Ctx c)
{
  HBTU_KERNEL_PROLOGUE();
  __shared__ int tot[4];
  if (c.S >= kPlanGatherMin)
    plan_scan4_warp<get_all_chunks>(c.S, c, c.bchunk_base, nullptr, nullptr, nullptr, tot);
  else
    plan_scan4_thread<get_all_chunks>(c.S, c, c.bchunk_base, nullptr, nullptr, nullptr, tot);
}

}  // namespace

// ---------------------------------------------------------------- launchers
void launch_segment_sums(Ctx &c, const double *x, double *out)
{
  launch_k(k_plan_all, 1, kPlanThreads, 0, c.st, c);
  HBTU_LAUNCHED();
  const int max_chunks = (c.N + kChunk - 1) / kChunk + c.S;
  if (max_chunks > 0) {
    launch_k(k_segsum_chunks, max_chunks, kLB, 0, c.st, c, x);
    HBTU_LAUNCHED();
  }
  launch_k(k_segsum_combine, nblk(c.S, 128), 128, 0, c.st, c, out);
  HBTU_LAUNCHED();
}
void launch_init(Ctx &c, const float *pos, const float *vel, const float *mass,
                 const long long *id)
{
  launch_k(k_init, nblk(c.N), kLB, 0, c.st, c, pos, vel, mass, id);
  HBTU_LAUNCHED();
}

void launch_plan(Ctx &c, int mode)
{
  const int gathered = c.S >= kPlanGatherMin;
  if (gathered) {
    launch_k(k_plan_gather, nblk(c.S, 256), 256, 0, c.st, c, mode);
    HBTU_LAUNCHED();
  }
  launch_k(k_plan, 1, kPlanThreads, 0, c.st, c, mode, gathered);
  HBTU_LAUNCHED();
}

void launch_partition(Ctx &c)
{
  launch_k(k_part_codes, nblk(c.N + 1), kLB, 0, c.st, c);
  HBTU_LAUNCHED();
  exclusive_scan_i64(c.pcode, c.pX, c.N + 1, c.scan_tmp, c.st);
  launch_k(k_part_pq, nblk(c.N), kLB, 0, c.st, c);
  HBTU_LAUNCHED();
  launch_k(k_part_fg, nblk(c.N), kLB, 0, c.st, c);
  HBTU_LAUNCHED();
  launch_k(k_part_seg, nblk(c.S, 128), 128, 0, c.st, c);
  HBTU_LAUNCHED();
  launch_k(k_part_gather, nblk(c.N), kLB, 0, c.st, c);
  HBTU_LAUNCHED();
  launch_k(k_part_copyback, nblk(c.N), kLB, 0, c.st, c);
  HBTU_LAUNCHED();
}

void launch_averages_control(Ctx &c, int max_passes)
{
  launch_plan(c, 1);
  const int max_chunks = (c.N + kChunk - 1) / kChunk + c.S;
  launch_k(k_avg_chunks, max_chunks, kLB, 0, c.st, c);
  HBTU_LAUNCHED();
  launch_k(k_control, nblk(32ll * c.S, 128), 128, 0, c.st, c, max_passes);
  HBTU_LAUNCHED();
}

void launch_block_sort(Ctx &c, int total, int which)
{
  if (total > 0) {
    launch_k(k_blk_gather, nblk(c.N), kLB, 0, c.st, c, which);
    HBTU_LAUNCHED();
    int words[8], shifts[8], np = 0;
    for (int p = 0; p < 4; p++) {
      words[np] = 0;
      shifts[np++] = 32 + 8 * p;
    }
    int sbits = 0;
    while ((1 << sbits) < c.S) sbits++;
    for (int p = 0; p < (sbits + 7) / 8; p++) {
      words[np] = 1;
      shifts[np++] = 8 * p;
    }
    radix_sort(c.sb, total, words, shifts, np, c.st);
    launch_k(k_blk_scatter, nblk(total), kLB, 0, c.st, c, which, total);
    HBTU_LAUNCHED();
    launch_k(k_blk_copyback, nblk(total), kLB, 0, c.st, c, which, total);
    HBTU_LAUNCHED();
  }
  if (which == 0) {
    launch_k(k_blk_clear, nblk(c.S, 128), 128, 0, c.st, c);
    HBTU_LAUNCHED();
  }
}

void launch_refine_mode(Ctx &c, int enter)
{
  launch_k(k_refine_mode, nblk(c.S, 128), 128, 0, c.st, c, enter);
  HBTU_LAUNCHED();
}

void launch_finalize(Ctx &c, int64_t *order_out, float *energy_out, hbtu_result *res_dev)
{
  const int max_chunks = (c.N + kChunk - 1) / kChunk + c.S;
  launch_k(k_kin_chunks, max_chunks, kLB, 0, c.st, c);
  HBTU_LAUNCHED();
  launch_k(k_final_seg, nblk(32ll * c.S, 128), 128, 0, c.st, c, res_dev);
  HBTU_LAUNCHED();
  if (c.N > 0) {
    launch_k(k_final_out, nblk(c.N), kLB, 0, c.st, c, order_out, energy_out);
    HBTU_LAUNCHED();
  }
}

}  // namespace hbtu
