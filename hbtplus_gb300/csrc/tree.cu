// tree.cu -- octree build for every active subhalo of a batch.
//
// Reproduces the cells of the reference's OctTree_t::Build
// (src/oct_tree.tpp:16-144) without its serial insertion:
//   1. bounding cube per subhalo: centre = box midpoint, side = largest extent,
//      in double on the float positions (tpp:30-51);
//   2. octal key of each particle: the octant chosen at each level by the
//      reference's own test x > centre with centres halved in double
//      (tpp:67-95), down to the level whose side drops below
//      TreeNodeResolution (below it the reference places particles in random
//      octants, tpp:112-123; here such particles share one bucket cell);
//   3. stable LSD radix sort by (subhalo, key): DFS order with octants 0..7,
//      which is the reference's nextnode/sibling order
//      (src/gravity_tree.cpp:48-77);
//   4. Karras binary radix tree on the sorted keys, collapsed to the octree
//      cells where a key prefix branches.  A cell with one child cell has the
//      same mass and centre of mass as that child (exact in double), so the
//      collapsed cell, given the smaller child's side, makes the same walk;
//   5. DFS preorder numbering and skip pointers from prefix counts (a skip
//      pointer that leaves the tree is stored as kDone);
//   6. bottom-up mass and centre of mass over each cell's children in octant
//      order, in double, rounded to float per cell as the reference does
//      (ProcessNode / FillNodeCenter, src/gravity_tree.cpp:18-46): the
//      subtrees of at most kChunkKeys particles in batches per thread block,
//      one level per step between block barriers, then an atomic-countdown
//      climb over the few cells above those subtrees.
#include <algorithm>

#include "tree_ops.cuh"

namespace hbtu {
namespace {

constexpr int kTB = 256;
// Moments: a cell whose subtree holds at most kChunkKeys particles and whose
// parent's holds more (or that is a root) is a chunk root, and a block
// computes the cells of its chunks.  Cells above the chunk roots are top
// cells.
constexpr int kChunkKeys = 2048;
constexpr int kChunkThreads = 256;
// Chunks of more than kSmallChunkKeys particles are computed one per block,
// the others kBatch at a time, so that a block's work stays within 2x of
// another's.
constexpr int kSmallChunkKeys = 256;
constexpr int kBatch = 16;
constexpr int kDepthBins = 32;  // octal depths 0 .. kMaxLevels

__global__ void __launch_bounds__(kTB) k_bbox_chunks(Ctx c)
{
  HBTU_KERNEL_PROLOGUE();
  const int b = blockIdx.x;
  const int total = c.tchunk_base[c.S];
  if (b >= total) return;
  const int s = upper_bound_i(c.tchunk_base, c.S + 1, b) - 1;
  const SegState &sg = c.seg[s];
  const int ci = b - c.tchunk_base[s];
  const int lo = sg.t0 + ci * kChunk, hi = min(sg.t0 + (ci + 1) * kChunk, sg.t0 + sg.ntree);
  float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int p = lo + threadIdx.x; p < hi; p += kTB) {
    const float4 a = c.pm[c.epid[sg.off + p]];
    mn[0] = fminf(mn[0], a.x);
    mn[1] = fminf(mn[1], a.y);
    mn[2] = fminf(mn[2], a.z);
    mx[0] = fmaxf(mx[0], a.x);
    mx[1] = fmaxf(mx[1], a.y);
    mx[2] = fmaxf(mx[2], a.z);
  }
  __shared__ float sh[6][kTB / 32];
#pragma unroll
  for (int j = 0; j < 3; j++) {
    for (int o = 16; o > 0; o >>= 1) {
      mn[j] = fminf(mn[j], __shfl_xor_sync(0xffffffffu, mn[j], o));
      mx[j] = fmaxf(mx[j], __shfl_xor_sync(0xffffffffu, mx[j], o));
    }
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0)
    for (int j = 0; j < 3; j++) {
      sh[j][w] = mn[j];
      sh[3 + j][w] = mx[j];
    }
  __syncthreads();
  if (threadIdx.x < 6) {
    const int j = threadIdx.x;
    float v = sh[j][0];
    for (int k = 1; k < kTB / 32; k++) v = j < 3 ? fminf(v, sh[j][k]) : fmaxf(v, sh[j][k]);
    c.chunk_bbox[(size_t)b * 6 + j] = __float_as_uint(v);
  }
}

// Root cube of each active subhalo (seg_cube) from its chunks' boxes.
__global__ void k_cube(Ctx c)
{
  HBTU_KERNEL_PROLOGUE();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= c.S) return;
  SegState &sg = c.seg[s];
  if (sg.status != SEG_ACTIVE) return;
  float mn[3], mx[3];
  const int b0 = c.tchunk_base[s], b1 = c.tchunk_base[s + 1];
  for (int j = 0; j < 3; j++) {
    mn[j] = INFINITY;
    mx[j] = -INFINITY;
    for (int b = b0; b < b1; b++) {
      mn[j] = fminf(mn[j], __uint_as_float(c.chunk_bbox[(size_t)b * 6 + j]));
      mx[j] = fmaxf(mx[j], __uint_as_float(c.chunk_bbox[(size_t)b * 6 + 3 + j]));
    }
  }
  const int levels = seg_cube(sg, mn, mx, b1 == b0, c.P);
  atomicMax(&c.plan->max_levels, levels);
}

// Octal key of every tree particle of every active subhalo.  Also clears the
// element's prefix-depth bits, child-cell counts and octant slots (-1) for the
// cell stages, and the moment work-list counters.
__global__ void __launch_bounds__(kTB) k_keys(Ctx c, int ntotal)
{
  HBTU_KERNEL_PROLOGUE();
  const int e = blockIdx.x * kTB + threadIdx.x;
  if (e == 0)
    for (int k = 0; k < 4; k++) c.lvl[k] = 0;
  if (e >= ntotal) return;
  c.mask[e] = 0ull;
  c.pending[e] = 0;
  c.pending0[e] = 0;
  int4 *slot = reinterpret_cast<int4 *>(c.cslot + 8 * (size_t)e);
  slot[0] = make_int4(-1, -1, -1, -1);
  slot[1] = make_int4(-1, -1, -1, -1);
  const int s = upper_bound_i(c.tree_base, c.S + 1, e) - 1;
  const SegState &sg = c.seg[s];
  const int epos = sg.off + sg.t0 + (e - c.tree_base[s]);
  c.sb.lo_a[e] = seg_key(sg, c.pm[c.epid[epos]]);
  c.sb.hi_a[e] = (unsigned)s;
  c.sb.val_a[e] = epos;
}

__global__ void __launch_bounds__(kTB) k_karras(Ctx c, int ntotal)
{
  HBTU_KERNEL_PROLOGUE();
  const int e = blockIdx.x * kTB + threadIdx.x;
  if (e >= ntotal) return;
  const int s = c.sb.hi_a[e];
  const int base = c.tree_base[s], n = c.tree_base[s + 1] - base;
  const int i = e - base;
  if (i >= n - 1) return;
  karras_elem(c, c.sb.lo_a + base, base, n, i);
}

__global__ void __launch_bounds__(kTB) k_cells(Ctx c, int ntotal)
{
  HBTU_KERNEL_PROLOGUE();
  const int e = blockIdx.x * kTB + threadIdx.x;
  if (e >= ntotal) return;
  const int s = c.sb.hi_a[e];
  const int base = c.tree_base[s], n = c.tree_base[s + 1] - base;
  cells_elem(c, base, n, e, c.seg[s].levels);
}

__global__ void __launch_bounds__(kTB) k_popc(Ctx c, int ntotal)
{
  HBTU_KERNEL_PROLOGUE();
  const int e = blockIdx.x * kTB + threadIdx.x;
  if (e > ntotal) return;
  c.pcode[e] = e < ntotal ? __popcll(c.mask[e]) : 0;
}

// sib: the sibling-block layout follows; clear its slot counts (X2) and new
// slot numbers (newidx, -1) here, two slots per element.
__global__ void __launch_bounds__(kTB) k_leaves(Ctx c, int ntotal, int sib)
{
  HBTU_KERNEL_PROLOGUE();
  const int e = blockIdx.x * kTB + threadIdx.x;
  if (sib && e <= ntotal) {
    c.X2[2 * (size_t)e] = 0;
    if (e < ntotal) {
      c.X2[2 * (size_t)e + 1] = 0;
      c.newidx[2 * (size_t)e] = -1;
      c.newidx[2 * (size_t)e + 1] = -1;
    }
  }
  if (e >= ntotal) return;
  const int s = c.sb.hi_a[e];
  const int base = c.tree_base[s], n = c.tree_base[s + 1] - base;
  leaves_elem(c, c.seg[s], base, n, e, c.pm[c.epid[c.sb.val_a[e]]], c.sb.lo_a[e], c.X + base);
}

__global__ void __launch_bounds__(kTB) k_cellnodes(Ctx c, int ntotal)
{
  HBTU_KERNEL_PROLOGUE();
  const int e = blockIdx.x * kTB + threadIdx.x;
  if (e >= ntotal) return;
  if (!c.iscell[e]) {
    c.cdepth[e] = -1;
    return;
  }
  const int s = c.sb.hi_a[e];
  const int base = c.tree_base[s], n = c.tree_base[s + 1] - base;
  cellnodes_elem(c, c.seg[s], base, n, e, c.sb.lo_a + base, c.X + base);
  // moment work lists: large chunk roots at the front of cell_list (count
  // lvl[0]), top cells at its back (count lvl[1]), small chunk roots in
  // chunk_list (count lvl[3]).  pending0 of a top cell counts its top child
  // cells twice over: in the high half (kept) and in the low half (counted
  // down by the climb).
  const int p = c.pcell[e];
  const int keys = c.rlast[e] - c.rfirst[e] + 1;
  if (keys > kChunkKeys) {
    if (p >= 0) atomicAdd(&c.pending0[p], 0x10001);
    c.cell_list[ntotal - 1 - atomicAdd(&c.lvl[1], 1)] = e;
  } else if (p < 0 || c.rlast[p] - c.rfirst[p] + 1 > kChunkKeys) {
    if (keys > kSmallChunkKeys)
      c.cell_list[atomicAdd(&c.lvl[0], 1)] = e;
    else
      c.chunk_list[atomicAdd(&c.lvl[3], 1)] = e;
  }
}

// A cell of a moment step: its slot, skip, octant slots, subhalo frame centre.
struct MomCell {
  int idx, end;
  bool bucket, mark;
  int4 s0, s1;
  float fc[3];
};

// Moments of the chunks.  The double arithmetic of a cell issues per warp
// instruction whatever the number of active lanes, at 1/64 of the FP32 rate on
// this GPU, so the cells computed together must fill the lanes: a persistent
// block takes one large chunk or kBatch small ones at a time and aligns their
// subtrees at the bottom, so that step t computes, in every chunk, the cells t
// levels above its deepest ones, all of them spread over the block's threads,
// with one barrier per step (every cell's child cells are deeper, so done
// before it).
// The internal nodes of the Karras subtree over keys [first, last] rooted at
// node i are nodes first..last-1 when i == first, first+1..last when i == last;
// a warp lists the octree cells among them by depth in the chunk's own element
// range of a scratch array (chunks' ranges are disjoint).  A cell without
// child cells is marked for the walk's leaf runs (sign bit of len*len).
__global__ void __launch_bounds__(kChunkThreads) k_moments_chunks(Ctx c)
{
  HBTU_KERNEL_PROLOGUE();
  constexpr unsigned kFull = 0xffffffffu;
  constexpr int kWarps = kChunkThreads / 32;
  __shared__ int s_first, s_steps;
  __shared__ int s_maxd[kBatch], s_pre[kDepthBins][kBatch + 1];
  __shared__ int s_cnt[kBatch][kDepthBins], s_start[kBatch][kDepthBins];
  __shared__ int s_back[kChunkThreads / 32][kDepthBins];  // fill cursors from the back
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int *glist = reinterpret_cast<int *>(c.X);  // the cell-slot scan is no longer needed
  const int nlarge = c.lvl[0], nsmall = c.lvl[3];
  const int njobs = nlarge + (nsmall + kBatch - 1) / kBatch;
  for (;;) {
    if (threadIdx.x == 0) {
      s_first = atomicAdd(&c.lvl[2], 1);  // a large chunk, or a batch of small ones
      s_steps = 0;
    }
    __syncthreads();
    const int job = s_first;
    if (job >= njobs) return;
    const int *roots = job < nlarge ? c.cell_list + job : c.chunk_list + (job - nlarge) * kBatch;
    const int nb = job < nlarge ? 1 : min(kBatch, nsmall - (job - nlarge) * kBatch);
    // each warp lists the cells of its chunks by depth below the chunk root
    for (int j = w; j < nb; j += kWarps) {
      int *cnt = s_cnt[j], *start = s_start[j];
      const int e0 = roots[j];
      const int base = c.tree_base[c.sb.hi_a[e0]];
      const int first = c.rfirst[e0], last = c.rlast[e0];
      const int lo = base + (e0 - base == first ? first : first + 1);
      const int nint = last - first;  // internal nodes of the subtree
      const int d0 = c.cdepth[e0];
      cnt[lane] = 0;
      __syncwarp();
      int maxd = 0;
      for (int k = lane; k < nint; k += 32) {
        const int d = c.cdepth[lo + k];  // -1: not a cell
        if (d >= 0) {
          const int r = min(max(d - d0, 0), kDepthBins - 1);
          atomicAdd(&cnt[r], 1);
          maxd = max(maxd, r);
        }
      }
      maxd = __reduce_max_sync(kFull, maxd);
      __syncwarp();
      const int v = cnt[lane];
      int incl = v;
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += t;
      }
      start[lane] = lo + incl - v;
      cnt[lane] = 0;
      __syncwarp();
      // each depth's cells of two children first, the others from the back,
      // so that a warp's lanes mostly add the same number of children
      int *back = s_back[w];
      back[lane] = v;
      __syncwarp();
      for (int k = lane; k < nint; k += 32) {
        const int e = lo + k;
        const int d = c.cdepth[e];
        if (d >= 0) {
          const int r = min(max(d - d0, 0), kDepthBins - 1);
          const int4 *slot = reinterpret_cast<const int4 *>(c.cslot + 8 * e);
          const int4 a = slot[0], b = slot[1];
          const int kids = (a.x >= 0) + (a.y >= 0) + (a.z >= 0) + (a.w >= 0) + (b.x >= 0) +
                           (b.y >= 0) + (b.z >= 0) + (b.w >= 0);
          if (kids == 2)
            glist[start[r] + atomicAdd(&cnt[r], 1)] = e;
          else
            glist[start[r] + atomicSub(&back[r], 1) - 1] = e;
        }
      }
      __syncwarp();
      cnt[lane] = v;
      if (lane == 0) {
        s_maxd[j] = maxd;
        atomicMax(&s_steps, maxd + 1);
      }
    }
    __syncthreads();
    const int steps = s_steps;
    if (w == 0) {  // per step: where each chunk's cells start in the step's list
      for (int t = 0; t < steps; t++) {
        int v = 0;
        if (lane < nb) {
          const int r = s_maxd[lane] - t;
          v = r >= 0 ? s_cnt[lane][r] : 0;
        }
        int incl = v;
        for (int o = 1; o < 32; o <<= 1) {
          const int u = __shfl_up_sync(kFull, incl, o);
          if (lane >= o) incl += u;
        }
        if (lane < kBatch) s_pre[t][lane + 1] = incl;
        if (lane == 0) s_pre[t][0] = 0;
      }
    }
    __syncthreads();
    // A cell's records (slots, children's slots, subhalo) do not depend on the
    // cells below it: each thread loads those of its next step's first cell
    // before computing this step's, so a step waits only for the children's
    // moments.
    auto load_cell = [&](int t, int i, MomCell &q) {
      const int *pre = s_pre[t];
      int j = 0;  // the chunk: pre[j] <= i < pre[j + 1]
#pragma unroll
      for (int step = kBatch / 2; step > 0; step >>= 1)
        if (j + step < nb && pre[j + step] <= i) j += step;
      const int e = glist[s_start[j][s_maxd[j] - t] + (i - pre[j])];
      const SegState &sg = c.seg[c.sb.hi_a[e]];
      q.idx = c.cidx[e];
      q.end = c.cskip[e];
      q.bucket = c.cdepth[e] >= sg.levels;
      q.mark = c.pending[e] == 0;
      const int4 *slot = reinterpret_cast<const int4 *>(c.cslot + 8 * e);
      q.s0 = slot[0];
      q.s1 = slot[1];
      q.fc[0] = sg.fc[0];
      q.fc[1] = sg.fc[1];
      q.fc[2] = sg.fc[2];
    };
    auto do_cell = [&](const MomCell &q) {
      if (q.mark) c.nd[q.idx].m.x |= (int)0x80000000;
      const float4 m = cell_moment_slots(q.bucket, q.idx, q.end, q.s0, q.s1,
                                         [&](int k2) { return c.nd_abs[k2]; });
      c.nd_abs[q.idx] = m;
      store_cell_rel(c, q.fc, q.idx, m);
    };
    MomCell cur;
    bool have = threadIdx.x < s_pre[0][nb];
    if (have) load_cell(0, threadIdx.x, cur);
    for (int t = 0; t < steps; t++) {
      MomCell nxt;
      const bool have_next = t + 1 < steps && (int)threadIdx.x < s_pre[t + 1][nb];
      if (have_next) load_cell(t + 1, threadIdx.x, nxt);
      if (have) do_cell(cur);
      for (int i = threadIdx.x + kChunkThreads; i < s_pre[t][nb]; i += kChunkThreads) {
        MomCell q;
        load_cell(t, i, q);
        do_cell(q);
      }
      __syncthreads();
      cur = nxt;
      have = have_next;
    }
  }
}

// Atomic add with acquire-release ordering at device scope: the adder's
// earlier writes are visible to whoever reads the counter's new value.
__device__ __forceinline__ int atomic_add_acq_rel(int *p, int v)
{
  int old;
  asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], %2;"
               : "=r"(old)
               : "l"(p), "r"(v)
               : "memory");
  return old;
}

// Moments of the top cells (above the chunk roots, few): a cell is summed
// once all its top child cells are, by the thread that finished the last one
// (atomic countdown on the low half of pending0; the high half, never
// changed, says whether the cell waits for any).  Children written during this
// launch are read through L2.
__global__ void __launch_bounds__(kTB) k_moments_top(Ctx c, int ntotal)
{
  HBTU_KERNEL_PROLOGUE();
  const int i = blockIdx.x * kTB + threadIdx.x;
  if (i >= c.lvl[1]) return;
  int e = c.cell_list[ntotal - 1 - i];
  if ((c.pending0[e] >> 16) != 0) return;  // a child's climb computes it
  for (int guard = 0; guard <= 2 * kMaxLevels + 2; guard++) {
    if (c.pending[e] == 0) c.nd[c.cidx[e]].m.x |= (int)0x80000000;
    cell_moment<true>(c, c.seg[c.sb.hi_a[e]], e, c.cdepth[e]);
    const int p = c.pcell[e];
    if (p < 0) break;
    if ((atomic_add_acq_rel(&c.pending0[p], -1) & 0xffff) != 1) break;
    e = p;
  }
}

inline unsigned nblk(long long n) { return (unsigned)((n + kTB - 1) / kTB); }

}  // namespace

void launch_bbox_cube(Ctx &c, int max_chunks)
{
  if (max_chunks > 0) launch_k(k_bbox_chunks, max_chunks, kTB, 0, c.st, c);
  HBTU_LAUNCHED();
  launch_k(k_cube, (c.S + 127) / 128, 128, 0, c.st, c);
  HBTU_LAUNCHED();
}

void launch_tree_build(Ctx &c, const PassPlan &pl)
{
  const int n = pl.ntree_total;
  if (n <= 0) return;
  launch_k(k_keys, nblk(n), kTB, 0, c.st, c, n);
  HBTU_LAUNCHED();
  // LSD passes: octal-key digits (top 3*levels bits), then subhalo index
  int words[16], shifts[16], np = 0;
  const int kbits = 3 * pl.max_levels;
  const int kp = (kbits + 7) / 8;
  for (int p = 0; p < kp; p++) {
    words[np] = 0;
    shifts[np++] = 64 - 8 * kp + 8 * p;
  }
  int sbits = 0;
  while ((1 << sbits) < c.S) sbits++;
  for (int p = 0; p < (sbits + 7) / 8; p++) {
    words[np] = 1;
    shifts[np++] = 8 * p;
  }
  radix_sort(c.sb, n, words, shifts, np, c.st);
  launch_k(k_karras, nblk(n), kTB, 0, c.st, c, n);
  HBTU_LAUNCHED();
  launch_k(k_cells, nblk(n), kTB, 0, c.st, c, n);
  HBTU_LAUNCHED();
  launch_k(k_popc, nblk(n + 1), kTB, 0, c.st, c, n);
  HBTU_LAUNCHED();
  exclusive_scan_i64(c.pcode, c.X, n + 1, c.scan_tmp, c.st);
  const int sib = sibling_walk(c, pl) ? 1 : 0;
  launch_k(k_leaves, nblk(n + 1), kTB, 0, c.st, c, n, sib);
  HBTU_LAUNCHED();
  launch_k(k_cellnodes, nblk(n), kTB, 0, c.st, c, n);
  HBTU_LAUNCHED();
  int dev = 0, sms = 0, per_sm = 0;  // a persistent grid: the resident blocks
  HBTU_CUDA(cudaGetDevice(&dev));
  HBTU_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  HBTU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_moments_chunks,
                                                          kChunkThreads, 0));
  const int njob_max = std::max(1, n / 2);  // a chunk root holds at least 2 particles
  launch_k(k_moments_chunks, std::min(sms * std::max(per_sm, 1), njob_max), kChunkThreads, 0,
           c.st, c);
  HBTU_LAUNCHED();
  // top cells hold more than kChunkKeys particles each, at most n / kChunkKeys per depth
  const int ntop_max = std::max(1, (n / kChunkKeys) * (pl.max_levels + 1));
  launch_k(k_moments_top, nblk(std::min(ntop_max, n)), kTB, 0, c.st, c, n);
  HBTU_LAUNCHED();
  if (sibling_walk(c, pl)) launch_sibling_layout(c, pl);
}


// ---------------------------------------------------------------------------
// Sibling-block layout for the FP32 lane walk.  The preorder numbering puts a
// cell's next sibling after the whole subtree of the cell, so a walk that
// accepts a cell jumps to a far slot.  This copy places the children of every
// cell in consecutive slots (the children blocks follow the preorder of their
// cells), keeps each segment's slots, and stores with each cell the slot of
// its first child; the walk then follows child (open) or skip (accept)
// pointers: the same nodes in the same order, at other addresses.
namespace {

// children per node slot, as int64 for the scan (cells only; particles and
// empty slots keep 0)
__global__ void __launch_bounds__(kTB) k_sib_count(Ctx c, int ntotal)
{
  HBTU_KERNEL_PROLOGUE();
  const int e = blockIdx.x * kTB + threadIdx.x;
  if (e >= ntotal || !c.iscell[e]) return;
  const int s = c.sb.hi_a[e];
  const int idx = c.cidx[e], end = c.cskip[e];
  int k = 0;
  if (c.cdepth[e] < c.seg[s].levels) {
    for (int j = 0; j < 8; j++) {
      const int sl = c.cslot[8 * e + j];
      k += (sl > idx && sl < end);
    }
  } else {  // a bucket: its particles follow it, one after another
    k = end - idx - 1;
  }
  c.X2[idx] = k;
}

// the slots of every cell's children: its block starts after the blocks of
// the cells before it in preorder
__global__ void __launch_bounds__(kTB) k_sib_assign(Ctx c, int ntotal)
{
  HBTU_KERNEL_PROLOGUE();
  const int e = blockIdx.x * kTB + threadIdx.x;
  if (e >= ntotal || !c.iscell[e]) return;
  const int s = c.sb.hi_a[e];
  const int root = 2 * c.tree_base[s];
  const int idx = c.cidx[e], end = c.cskip[e];
  const int base = root + 1 + (int)(c.X2[idx] - c.X2[root]);
  if (idx == root) c.newidx[root] = root;
  int k = 0;
  if (c.cdepth[e] < c.seg[s].levels) {
    for (int j = 0; j < 8; j++) {
      const int sl = c.cslot[8 * e + j];
      if (sl > idx && sl < end) c.newidx[sl] = base + k++;
    }
  } else {
    for (int d = idx + 1; d < end; d++) c.newidx[d] = base + k++;
  }
}

// a segment of one particle has no cell records: its two nodes keep their slots
__global__ void k_sib_single(Ctx c)
{
  HBTU_KERNEL_PROLOGUE();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= c.S) return;
  const SegState &sg = c.seg[s];
  if (sg.status != SEG_ACTIVE || c.tree_base[s + 1] - c.tree_base[s] != 1) return;
  const int root = 2 * c.tree_base[s];
  c.newidx[root] = root;
  c.newidx[root + 1] = root + 1;
}

// every live node slot: its record at its new slot, pointers renumbered
__global__ void __launch_bounds__(kTB) k_sib_copy(Ctx c, int nslots)
{
  HBTU_KERNEL_PROLOGUE();
  const int d = blockIdx.x * kTB + threadIdx.x;
  if (d >= nslots) return;
  const int s = upper_bound_i(c.tree_base, c.S + 1, d >> 1) - 1;
  if (s < 0 || s >= c.S) return;
  const int root = 2 * c.tree_base[s];
  const int nn = c.seg[s].nnodes;
  if (d - root >= nn || c.tree_base[s + 1] == c.tree_base[s]) return;
  const int nd = c.newidx[d];
  if (nd < root || nd >= root + nn) return;  // never written: leave the slot alone
  WNode w = c.nd[d];
  const int skip = w.m.y;
  w.m.y = (skip >= root && skip < root + nn) ? c.newidx[skip] : kDone;
  const bool cell = signbit(w.p.w) != 0;
  w.m.w = (cell && d + 1 < root + nn) ? c.newidx[d + 1] : kDone;
  c.nd2[nd] = w;
}

}  // namespace

void launch_sibling_layout(Ctx &c, const PassPlan &pl)
{
  const int n = pl.ntree_total;
  if (n <= 0 || !c.nd2) return;
  const int nslots = 2 * n;  // X2 and newidx were cleared by k_leaves
  launch_k(k_sib_count, nblk(n), kTB, 0, c.st, c, n);
  HBTU_LAUNCHED();
  exclusive_scan_i64(c.X2, c.X2, nslots + 1, c.scan_tmp2, c.st);
  launch_k(k_sib_assign, nblk(n), kTB, 0, c.st, c, n);
  HBTU_LAUNCHED();
  launch_k(k_sib_single, (c.S + 127) / 128, 128, 0, c.st, c);
  HBTU_LAUNCHED();
  launch_k(k_sib_copy, nblk(nslots), kTB, 0, c.st, c, nslots);
  HBTU_LAUNCHED();
}

}  // namespace hbtu
