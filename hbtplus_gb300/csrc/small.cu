// small.cu -- the rest of the unbinding loop of small subhaloes, one thread
// block per subhalo.
//
// Subhalo_t::Unbind (src/subhalo_unbind.cpp:263-431) iterates until the bound
// count converges.  The batch path (loop.cu, tree.cu, walk.cu) advances every
// active subhalo of a call by one pass per round of ~40 launches, so the round
// count is set by the slowest subhalo.  In the 2000-subhalo workload the
// subhaloes of 512 particles or more converge in 2-3 passes, while a few dozen
// of under 512 particles need 4-7: rounds 4-7 exist for them alone.
//
// At the first round where every active subhalo's energy list holds at most
// `cap` particles, one persistent launch finishes them all: blocks take the
// subhaloes from a queue in size order (largest first; an atomic counter
// hands out the next), and one block runs a subhalo's remaining passes to the
// end on the device -- tree, walk, partition, averages and decisions, one step
// after another with block barriers between them.  A call whose subhaloes are
// all small (the one-subhalo form, for one) hands over at the first round.
// The steps are the batch kernels' own per-element functions (tree_ops.cuh,
// walk_ops.cuh, loop_ops.cuh) on the subhalo's slice of the same buffers, so
// every result is bit for bit the batch path's:
//   * the tree keys are sorted by rank (the count of smaller keys, ties by
//     position): the order of the batch path's stable radix sort;
//   * the unbound block of each pass is sorted the same way on its energy
//     keys at the start of the next pass;
//   * the cells' moments are taken one octal depth at a time, deepest first;
//   * the frame sums are the 1024-element chunk sums of k_avg_chunks,
//     added in chunk order as k_control does.
// The block has kLB (256) threads, the chunk-sum block size, so block_sum
// associates exactly as in the batch kernel.  One block per SM keeps the FP64
// pipe (moments, frames; 1/64 of the FP32 rate) to one subhalo at a time.
#include "loop_ops.cuh"
#include "tree_ops.cuh"
#include "walk_ops.cuh"

#include <algorithm>

namespace hbtu {
namespace {

constexpr int kSB = kLB;
static_assert(kSB == 256, "chunk sums and the per-digit scans assume 256 threads");
constexpr int kPerThread = kSmallCap / kSB;  // list entries a thread holds while permuting

// Shared memory of one block, for subhaloes of up to `cap` particles.
struct SmallLayout {
  size_t key0, key1, val0, val1, sums, bytes;
  explicit __host__ __device__ SmallLayout(int cap)
  {
    const size_t n1 = (size_t)cap + 1;
    key0 = 0;
    key1 = key0 + 8 * n1;
    val0 = key1 + 8 * n1;
    val1 = val0 + 4 * n1;
    sums = (val1 + 4 * n1 + 7) / 8 * 8;
    bytes = sums + sizeof(double) * kSums * (size_t)(cap / kChunk + 1);
  }
};

// Exclusive block scan of one value per thread (kSB threads); *total gets the sum.
__device__ __forceinline__ long long block_excl_scan(long long v, long long *total)
{
  __shared__ long long ws[kSB / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  long long x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[w] = x;
  __syncthreads();
  long long before = 0, all = 0;
#pragma unroll
  for (int k = 0; k < kSB / 32; k++) {
    before += k < w ? ws[k] : 0;
    all += ws[k];
  }
  __syncthreads();
  if (total) *total = all;
  return before + x - v;
}

// Exclusive scan of n+1 values in[0..n] (in may alias out), each thread
// taking a contiguous run.
__device__ void block_scan_array(const long long *in, long long *out, int n1)
{
  const int per = (n1 + kSB - 1) / kSB;
  const int b = threadIdx.x * per, e = min(n1, b + per);
  long long loc = 0;
  for (int k = b; k < e; k++) loc += in[k];
  long long run = block_excl_scan(loc, nullptr);
  for (int k = b; k < e; k++) {
    const long long v = in[k];
    out[k] = run;
    run += v;
  }
  __syncthreads();
}

// The unbound block [lo, hi) of the list sorted by energy, stable (the batch
// path's k_blk_* with the radix sort, which = 0).
__device__ void sort_unbound_block(const Ctx &c, int P0, int lo, int hi, unsigned *key)
{
  for (int l = lo + (int)threadIdx.x; l < hi; l += kSB) key[l - lo] = float_key(c.eE[P0 + l]);
  __syncthreads();
  const int m = hi - lo;
  int pid[kPerThread], dst[kPerThread];
  float E[kPerThread];
#pragma unroll
  for (int k = 0; k < kPerThread; k++) {
    const int i = threadIdx.x + k * kSB;
    if (i >= m) break;
    const unsigned ki = key[i];
    int r = 0;
    for (int j = 0; j < m; j++) {
      const unsigned kj = key[j];
      r += (kj < ki) | ((kj == ki) & (j < i));
    }
    dst[k] = lo + r;
    pid[k] = c.epid[P0 + lo + i];
    E[k] = c.eE[P0 + lo + i];
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < kPerThread; k++) {
    if ((int)threadIdx.x + k * kSB >= m) break;
    c.epid[P0 + dst[k]] = pid[k];
    c.eE[P0 + dst[k]] = E[k];
    c.epos_of_pid[pid[k]] = P0 + dst[k];
  }
  __syncthreads();
}

// One pass's octree over list positions [t0, t0 + ntree) of subhalo s, in the
// element arrays from P0 and node slots from 2*P0.  Leaves the sorted keys in
// skey and the list positions in Morton order in sval.
__device__ void build_tree(const Ctx &c, SegState &sg, int P0, unsigned long long *ukey,
                           unsigned long long *skey, int *uval, int *sval)
{
  int *const clist = uval;  // free once the keys are sorted
  __shared__ float bb[6][kSB / 32];
  __shared__ int maxdepth;
  const int n = sg.ntree, t0 = sg.t0;
  float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int i = threadIdx.x; i < n; i += kSB) {
    const float4 a = c.pm[c.epid[P0 + t0 + i]];
    mn[0] = fminf(mn[0], a.x);
    mn[1] = fminf(mn[1], a.y);
    mn[2] = fminf(mn[2], a.z);
    mx[0] = fmaxf(mx[0], a.x);
    mx[1] = fmaxf(mx[1], a.y);
    mx[2] = fmaxf(mx[2], a.z);
    const int e = P0 + i;
    c.mask[e] = 0ull;
    c.pending[e] = 0;
    int4 *slot = reinterpret_cast<int4 *>(c.cslot + 8 * (size_t)e);
    slot[0] = make_int4(-1, -1, -1, -1);
    slot[1] = make_int4(-1, -1, -1, -1);
  }
#pragma unroll
  for (int j = 0; j < 3; j++)
    for (int o = 16; o > 0; o >>= 1) {
      mn[j] = fminf(mn[j], __shfl_xor_sync(0xffffffffu, mn[j], o));
      mx[j] = fmaxf(mx[j], __shfl_xor_sync(0xffffffffu, mx[j], o));
    }
  if ((threadIdx.x & 31) == 0)
    for (int j = 0; j < 3; j++) {
      bb[j][threadIdx.x >> 5] = mn[j];
      bb[3 + j][threadIdx.x >> 5] = mx[j];
    }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int j = 0; j < 3; j++) {
      float a = bb[j][0], b = bb[3 + j][0];
      for (int w = 1; w < kSB / 32; w++) {
        a = fminf(a, bb[j][w]);
        b = fmaxf(b, bb[3 + j][w]);
      }
      mn[j] = a;
      mx[j] = b;
    }
    seg_cube(sg, mn, mx, n == 0, c.P);
    maxdepth = 0;
  }
  __syncthreads();
  // keys, then the stable order by rank
  for (int e = threadIdx.x; e < n; e += kSB) {
    const int epos = P0 + t0 + e;
    ukey[e] = seg_key(sg, c.pm[c.epid[epos]]);
    uval[e] = epos;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += kSB) {
    const unsigned long long ki = ukey[i];
    int r = 0;
    for (int j = 0; j < n; j++) {
      const unsigned long long kj = ukey[j];
      r += (kj < ki) | ((kj == ki) & (j < i));
    }
    skey[r] = ki;
    sval[r] = uval[i];
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n - 1; i += kSB) karras_elem(c, skey, P0, n, i);
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += kSB) cells_elem(c, P0, n, P0 + i, sg.levels);
  __syncthreads();
  // prefix counts of the cells starting at each key (the batch path's k_popc +
  // scan), kept in shared memory: entry n of this subhalo's scan would be
  // entry 0 of the next subhalo's in the global array
  long long *pc = reinterpret_cast<long long *>(ukey);
  for (int i = threadIdx.x; i <= n; i += kSB) pc[i] = i < n ? __popcll(c.mask[P0 + i]) : 0;
  __syncthreads();
  block_scan_array(pc, pc, n + 1);
  for (int i = threadIdx.x; i < n; i += kSB)
    leaves_elem(c, sg, P0, n, P0 + i, c.pm[c.epid[sval[i]]], skey[i], pc);
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += kSB) {
    const int e = P0 + i;
    if (c.iscell[e]) {
      cellnodes_elem(c, sg, P0, n, e, skey, pc);
      atomicMax(&maxdepth, c.cdepth[e]);
    } else {
      c.cdepth[e] = -1;
    }
  }
  __syncthreads();
  // moments one octal depth at a time, deepest first, over dense per-depth
  // lists of the cells so that every lane of a warp works on a cell (a warp's
  // double instruction costs the same however few lanes run it)
  __shared__ int dcount[kMaxLevels + 2], dstart[kMaxLevels + 2];
  if (threadIdx.x < kMaxLevels + 2) dcount[threadIdx.x] = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += kSB) {
    const int d = c.cdepth[P0 + i];
    if (d >= 0) atomicAdd(&dcount[d], 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int d = 0; d <= maxdepth; d++) {
      dstart[d] = run;
      run += dcount[d];
      dcount[d] = dstart[d];  // cursor
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += kSB) {
    const int d = c.cdepth[P0 + i];
    if (d >= 0) clist[atomicAdd(&dcount[d], 1)] = P0 + i;
  }
  __syncthreads();
  for (int d = maxdepth; d >= 0; d--) {
    const int first = dstart[d], last = dcount[d];
    for (int k = first + (int)threadIdx.x; k < last; k += kSB) {
      const int e = clist[k];
      if (c.pending[e] == 0) c.nd[c.cidx[e]].m.x |= (int)0x80000000;
      cell_moment<false>(c, sg, e, d);
    }
    __syncthreads();
  }
}

// The pass's energies: every target's walk and BindingEnergy (or the
// correction update), as the batch walk does for its targets.
template <bool kFP64>
__device__ void walk_targets(const Ctx &c, int s, SegState &sg, int P0, const int *sval)
{
  const int tm = sg.tgt_mode;
  const int count = tm == 1 ? sg.coh_n : sg.ntgt;
  const int rounds = (count + kSB - 1) / kSB;
  for (int r = 0; r < rounds; r++) {
    const int w = r * kSB + threadIdx.x;
    int epos = -1, pid = -1;
    bool active = false;
    if (w < count) {
      if (tm == 0) {  // full pass: tree leaves in Morton order
        epos = sval[w];
        pid = c.epid[epos];
        c.coh_pid[P0 + w] = pid;
        active = true;
      } else if (tm == 1) {  // correction pass: the last full pass's order, still bound
        pid = c.coh_pid[P0 + w];
        epos = c.epos_of_pid[pid];
        active = (epos - P0) < sg.ntgt;
      } else {
        epos = P0 + w;
        pid = c.epid[epos];
        active = true;
      }
    }
    Target t;
    init_target<!kFP64>(c, s, epos, pid, active, 2 * P0, t);
    int ninter = 0;
    const double pot = kFP64 ? walk_fp64(c, t, &ninter) : walk_lean<false>(c.nd, t, c.P, &ninter);
    finish_target(c, t, pot);
    count_interactions(c, s, ninter);
  }
  __syncthreads();
}

// PartitionBindingEnergy (src/subhalo_unbind.cpp:21-58) in closed form, as
// k_part_codes .. k_part_copyback do; returns Nbound.
__device__ int partition(const Ctx &c, SegState &sg, int P0, long long *px, int *Pk, int *Qk)
{
  __shared__ int F, G, nb_s, info[4];
  const int nl = sg.nlast;
  if (threadIdx.x == 0) {
    F = 0x7fffffff;
    G = 0x7fffffff;
  }
  for (int l = threadIdx.x; l <= nl; l += kSB) {
    long long code = 0;
    if (l >= 1 && l < nl) {
      const float e = c.eE[P0 + l];
      code = (e < 0.f ? (1ll << 32) : 0ll) | (e > 0.f ? 1ll : 0ll);
    }
    px[l] = code;
  }
  __syncthreads();
  block_scan_array(px, px, nl + 1);
  const long long x1 = nl >= 2 ? px[1] : 0, xe = nl >= 2 ? px[nl] : 0;
  const int nPos = (int)((xe - x1) & 0xffffffffll), nNeg = (int)((xe - x1) >> 32);
  if (nl >= 2)
    for (int l = 1 + threadIdx.x; l < nl; l += kSB) {
      const float e = c.eE[P0 + l];
      if (e > 0.f) Pk[(int)((px[l] - x1) & 0xffffffffll)] = l;
      if (e < 0.f) Qk[(int)((xe - px[l]) >> 32) - 1] = l;
    }
  __syncthreads();
  if (nl >= 2)
    for (int l = 1 + threadIdx.x; l < nl; l += kSB) {
      if (!(c.eE[P0 + l] > 0.f)) continue;
      const int k = (int)((px[l] - x1) & 0xffffffffll) + 1;
      if (k > min(nPos, nNeg)) continue;
      const int qk = Qk[k - 1];
      if (l >= qk) atomicMin(&F, k);
      if (k + 1 > nNeg || l >= Qk[k]) atomicMin(&G, k);
    }
  __syncthreads();
  if (threadIdx.x == 0) {
    const float e0 = c.eE[P0];
    if (nl < 2) {
      info[0] = info[1] = info[2] = 0;
      nb_s = nl == 1 ? (e0 < 0.f) : 0;
    } else {
      const int mn = min(nPos, nNeg);
      const int Fk = min(F, mn + 1) - 1;
      const int Gk = min(G - 1, Fk);
      int mb = 0, mf = 0, vd = 0;
      if (nNeg > 0) {
        mb = 1 + Gk;
        mf = Gk + (Gk + 1 <= Fk ? 1 : 0);
        vd = (mf == mb) ? Pk[mf - 1] : Qk[mb - 1];
      }
      info[0] = mb;
      info[1] = mf;
      info[2] = vd;
      nb_s = vd + (e0 < 0.f);
    }
  }
  __syncthreads();
  const int mb = info[0], mf = info[1], vd = info[2];
  int pid[kPerThread];
  float E[kPerThread];
#pragma unroll
  for (int k = 0; k < kPerThread; k++) {
    const int l = threadIdx.x + k * kSB;
    if (l >= nl) break;
    int src = l;
    if (nl >= 2) {
      const float e = c.eE[P0 + l];
      if (l == vd) {
        src = 0;
      } else if (l == 0) {
        src = nNeg >= 1 ? Qk[0] : 0;
      } else if (e < 0.f) {
        const int kq = (int)((xe - px[l]) >> 32);
        if (kq <= mf) src = Pk[kq - 1];
      } else if (e > 0.f) {
        const int kp = (int)((px[l] - x1) & 0xffffffffll) + 1;
        if (kp <= mb - 1) src = Qk[kp];
      }
    }
    pid[k] = c.epid[P0 + src];
    E[k] = c.eE[P0 + src];
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < kPerThread; k++) {
    const int l = threadIdx.x + k * kSB;
    if (l >= nl) break;
    c.epid[P0 + l] = pid[k];
    c.eE[P0 + l] = E[k];
    c.epos_of_pid[pid[k]] = P0 + l;
  }
  __syncthreads();
  return nb_s;
}

// AverageVelocity / AveragePosition sums of the bound block [0, nb): the
// chunk sums of k_avg_chunks, added in chunk order.
__device__ void frame_sums(const Ctx &c, const SegState &sg, int nb, double *chunk, double (&v)[7])
{
  for (int k = 0; k < 7; k++) v[k] = 0.;
  if (nb <= 1) return;
  const float4 o = c.pm[c.epid[sg.off]];
  const double od[3] = {f2d(o.x), f2d(o.y), f2d(o.z)};
  const int nch = (nb + kChunk - 1) / kChunk;
  for (int ci = 0; ci < nch; ci++) {
    const int lo = ci * kChunk, hi = min(lo + kChunk, nb);
    double w[7] = {0, 0, 0, 0, 0, 0, 0};
    for (int p = lo + threadIdx.x; p < hi; p += kLB) {
      const int pid = c.epid[sg.off + p];
      frame_terms(c.pm[pid], c.vel[pid], o, od, c.P, w);
    }
    block_sum<7>(w, chunk + (size_t)ci * kSums, hi - lo);
    __syncthreads();
  }
  for (int ci = 0; ci < nch; ci++)
    for (int k = 0; k < 7; k++) v[k] += chunk[(size_t)ci * kSums + k];
}

template <bool kFP64>
__global__ void __launch_bounds__(kSB) k_unbind_small(Ctx c, int cap, int max_passes)
{
  HBTU_KERNEL_PROLOGUE();
  extern __shared__ __align__(16) unsigned char smem[];
  const SmallLayout L(cap);
  unsigned long long *key0 = reinterpret_cast<unsigned long long *>(smem + L.key0);
  unsigned long long *key1 = reinterpret_cast<unsigned long long *>(smem + L.key1);
  int *val0 = reinterpret_cast<int *>(smem + L.val0);
  int *val1 = reinterpret_cast<int *>(smem + L.val1);
  double *chunk = reinterpret_cast<double *>(smem + L.sums);
  __shared__ int job;
  for (;;) {
    if (threadIdx.x == 0) {
      int k, s = -1;
      // the next active subhalo in size order (inactive ones are passed over)
      while ((k = atomicAdd(c.small_next, 1)) < c.S) {
        s = c.seg_order[k];
        if (c.seg[s].status == SEG_ACTIVE) break;
        s = -1;
      }
      job = s;
    }
    __syncthreads();
    const int s = job;
    __syncthreads();
    if (s < 0) break;
    SegState &sg = c.seg[s];
    const int P0 = sg.off;
    for (;;) {
      // the unbound block of the last pass (the batch path sorts it at the
      // start of the next round, also after convergence)
      const int lo = sg.ub_lo, hi = sg.ub_hi;
      if (hi > lo) sort_unbound_block(c, P0, lo, hi, reinterpret_cast<unsigned *>(key0));
      __syncthreads();
      if (threadIdx.x == 0) sg.ub_lo = sg.ub_hi = 0;
      const bool active = sg.status == SEG_ACTIVE;
      __syncthreads();
      if (!active) break;
      build_tree(c, sg, P0, key0, key1, val0, val1);
      walk_targets<kFP64>(c, s, sg, P0, val1);
      const int nb = partition(c, sg, P0, reinterpret_cast<long long *>(key0), val0, val1);
      double v[7];
      frame_sums(c, sg, nb, chunk, v);
      if (threadIdx.x == 0) control_segment(c, sg, nb, v, max_passes);
      __syncthreads();
    }
  }
}

}  // namespace

size_t small_smem_bytes(int cap) { return SmallLayout(cap).bytes; }

void launch_small(Ctx &c, int cap, int nactive, int max_passes)
{
  if (nactive <= 0) return;
  const size_t smem = SmallLayout(cap).bytes;
  int dev = 0, sms = 0;
  HBTU_CUDA(cudaGetDevice(&dev));
  HBTU_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  HBTU_CUDA(cudaMemsetAsync(c.small_next, 0, sizeof(int), c.st));
  const bool fp64 = c.P.precision == HBTU_PRECISION_FP64;
  if (fp64)
    HBTU_CUDA(cudaFuncSetAttribute(k_unbind_small<true>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  else
    HBTU_CUDA(cudaFuncSetAttribute(k_unbind_small<false>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int grid = std::max(1, std::min(nactive, sms * c.small_per_sm));
  if (fp64)
    launch_k(k_unbind_small<true>, grid, kSB, smem, c.st, c, cap, max_passes);
  else
    launch_k(k_unbind_small<false>, grid, kSB, smem, c.st, c, cap, max_passes);
  HBTU_LAUNCHED();
}

}  // namespace hbtu
