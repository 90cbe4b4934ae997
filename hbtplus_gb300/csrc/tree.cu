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
//      (ProcessNode / FillNodeCenter, src/gravity_tree.cpp:18-46).
#include "tree_ops.cuh"

namespace hbtu {
namespace {

constexpr int kTB = 256;
constexpr int kLevelSyncMin = 1 << 18;  // tree particles from which moments go level by level

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

// Octal key of every tree particle of every active subhalo.
__global__ void __launch_bounds__(kTB) k_keys(Ctx c, int ntotal)
{
  HBTU_KERNEL_PROLOGUE();
  const int e = blockIdx.x * kTB + threadIdx.x;
  if (e >= ntotal) return;
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

__global__ void __launch_bounds__(kTB) k_leaves(Ctx c, int ntotal)
{
  HBTU_KERNEL_PROLOGUE();
  const int e = blockIdx.x * kTB + threadIdx.x;
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
}

// Bottom-up moments (cell_moment): a cell is summed once all its child cells
// are, by the thread that finished the last child (atomic countdown, no
// waiting).  A cell without child cells is marked for the walk's leaf runs
// (sign bit of len*len).
__global__ void __launch_bounds__(kTB) k_moments(Ctx c, int ntotal)
{
  HBTU_KERNEL_PROLOGUE();
  int e = blockIdx.x * kTB + threadIdx.x;
  if (e >= ntotal || !c.iscell[e] || c.pending0[e] != 0) return;
  c.nd[c.cidx[e]].m.x |= (int)0x80000000;
  for (int level = 0; level <= 2 * kMaxLevels + 2; level++) {
    const int s = c.sb.hi_a[e];
    cell_moment<true>(c, c.seg[s], e, c.cdepth[e]);
    __threadfence();
    const int p = c.pcell[e];
    if (p < 0) break;
    if (atomicSub(&c.pending[p], 1) != 1) break;
    __threadfence();
    e = p;
  }
}

// Large trees: the same moments one octal depth at a time, deepest first,
// over a dense list of the cells of each depth, so a warp's 32 lanes work on
// 32 cells (double arithmetic issues per warp instruction whatever the number
// of active lanes, and runs at 1/64 of the FP32 rate on this GPU).
constexpr int kDepthBins = 32;  // octal depths 0 .. kMaxLevels

__global__ void __launch_bounds__(kTB) k_depth_count(Ctx c, int ntotal)
{
  HBTU_KERNEL_PROLOGUE();
  __shared__ int h[kDepthBins];
  if (threadIdx.x < kDepthBins) h[threadIdx.x] = 0;
  __syncthreads();
  const int e = blockIdx.x * kTB + threadIdx.x;
  if (e < ntotal && c.cdepth[e] >= 0) atomicAdd(&h[c.cdepth[e]], 1);
  __syncthreads();
  if (threadIdx.x < kDepthBins && h[threadIdx.x]) atomicAdd(&c.lvl[threadIdx.x], h[threadIdx.x]);
}

// lvl[0..31] counts per depth, lvl[32..63] list start per depth, lvl[64..95] cursors
__global__ void __launch_bounds__(kTB) k_depth_fill(Ctx c, int ntotal)
{
  HBTU_KERNEL_PROLOGUE();
  __shared__ int h[kDepthBins], start[kDepthBins];
  if (threadIdx.x < kDepthBins) h[threadIdx.x] = 0;
  __syncthreads();
  const int e = blockIdx.x * kTB + threadIdx.x;
  const int d = e < ntotal ? c.cdepth[e] : -1;
  int rank = 0;
  if (d >= 0) rank = atomicAdd(&h[d], 1);
  __syncthreads();
  if (threadIdx.x < kDepthBins) {
    int off = 0;
    for (int k = 0; k < (int)threadIdx.x; k++) off += c.lvl[k];
    if (blockIdx.x == 0) c.lvl[kDepthBins + threadIdx.x] = off;
    start[threadIdx.x] = h[threadIdx.x] ? off + atomicAdd(&c.lvl[2 * kDepthBins + threadIdx.x],
                                                          h[threadIdx.x])
                                        : 0;
  }
  __syncthreads();
  if (d >= 0) c.cell_list[start[d] + rank] = e;
}

__global__ void __launch_bounds__(kTB) k_moments_level(Ctx c, int depth)
{
  HBTU_KERNEL_PROLOGUE();
  const int count = c.lvl[depth], first = c.lvl[kDepthBins + depth];
  for (int i = blockIdx.x * kTB + threadIdx.x; i < count; i += gridDim.x * kTB) {
    const int e = c.cell_list[first + i];
    if (c.pending[e] == 0) c.nd[c.cidx[e]].m.x |= (int)0x80000000;
    cell_moment<false>(c, c.seg[c.sb.hi_a[e]], e, depth);
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
  HBTU_CUDA(cudaMemsetAsync(c.mask, 0, sizeof(unsigned long long) * (size_t)n, c.st));
  HBTU_CUDA(cudaMemsetAsync(c.pending, 0, sizeof(int) * (size_t)n, c.st));
  HBTU_CUDA(cudaMemsetAsync(c.cslot, 0xff, sizeof(int) * 8 * (size_t)n, c.st));
  launch_k(k_karras, nblk(n), kTB, 0, c.st, c, n);
  HBTU_LAUNCHED();
  launch_k(k_cells, nblk(n), kTB, 0, c.st, c, n);
  HBTU_LAUNCHED();
  launch_k(k_popc, nblk(n + 1), kTB, 0, c.st, c, n);
  HBTU_LAUNCHED();
  exclusive_scan_i64(c.pcode, c.X, n + 1, c.scan_tmp, c.st);
  launch_k(k_leaves, nblk(n), kTB, 0, c.st, c, n);
  HBTU_LAUNCHED();
  launch_k(k_cellnodes, nblk(n), kTB, 0, c.st, c, n);
  HBTU_LAUNCHED();
  if (n < kLevelSyncMin) {  // small trees: one launch, climbing by atomic countdown
    HBTU_CUDA(cudaMemcpyAsync(c.pending0, c.pending, sizeof(int) * (size_t)n,
                              cudaMemcpyDeviceToDevice, c.st));
    launch_k(k_moments, nblk(n), kTB, 0, c.st, c, n);
    HBTU_LAUNCHED();
  } else {  // large trees: dense per-depth cell lists, one launch per depth
    HBTU_CUDA(cudaMemsetAsync(c.lvl, 0, sizeof(int) * 3 * kDepthBins, c.st));
    launch_k(k_depth_count, nblk(n), kTB, 0, c.st, c, n);
    HBTU_LAUNCHED();
    launch_k(k_depth_fill, nblk(n), kTB, 0, c.st, c, n);
    HBTU_LAUNCHED();
    for (int d = pl.max_levels; d >= 0; d--) {
      launch_k(k_moments_level, 152 * 2, kTB, 0, c.st, c, d);
      HBTU_LAUNCHED();
    }
  }
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
  const int nslots = 2 * n;
  HBTU_CUDA(cudaMemsetAsync(c.X2, 0, sizeof(long long) * (size_t)(nslots + 1), c.st));
  HBTU_CUDA(cudaMemsetAsync(c.newidx, 0xff, sizeof(int) * (size_t)nslots, c.st));  // -1
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
