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
#include "device_common.cuh"

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

// Fixed-point form of the key computation.  The reference halves the cube in
// double: centre_k = centre_{k-1} +- len / 2^(k+1).  When the centre, len/4
// and every later increment are integers in units of 2^-E, and every centre
// fits in 53 significant bits, none of those double operations rounds, so the
// same comparisons x > centre_k can be made exactly on 64-bit integers
// (a tenth of the cost: double runs at 1/64 of the FP32 rate on this GPU).
__device__ __forceinline__ int ll_tz(long long v) { return v ? __ffsll(v) - 1 : 64; }

__device__ void fixed_point_cube(SegState &sg, int levels)
{
  sg.kfast = 0;
  if (levels <= 0 || !(sg.len > 0.)) return;
  double M = sg.len;
  for (int j = 0; j < 3; j++) M = fmax(M, fabs(sg.center[j]) + sg.len);
  int top;
  frexp(M, &top);                // M < 2^top
  const int E = 61 - top;        // |values| < 2^61 in fixed point
  const double l4 = ldexp(sg.len, E - 2);
  const double lmin = ldexp(sg.len, E - levels - 1);
  if (l4 != trunc(l4) || lmin != trunc(lmin) || l4 >= 0x1p62) return;
  const long long inc = (long long)l4;
  int g = ll_tz(inc >> (levels - 1));  // trailing zeros of the smallest increment
  for (int j = 0; j < 3; j++) {
    const double cj = ldexp(sg.center[j], E);
    if (cj != trunc(cj) || fabs(cj) >= 0x1p62) return;
    sg.kc[j] = (long long)cj;
    g = min(g, ll_tz(sg.kc[j]));
  }
  if (top + E - g > 53) return;  // some centre would need more than 53 bits
  sg.kinc = inc;
  sg.kscale = E;
  sg.kfast = 1;
}

// A float position in units of 2^-E, if exact (else false).
__device__ __forceinline__ bool float_fixed(float x, int E, long long &X)
{
  const unsigned b = __float_as_uint(x);
  const int ex = (int)((b >> 23) & 255u);
  if (ex == 0) {  // zero (denormals take the double path)
    X = 0;
    return (b & 0x7fffffffu) == 0u;
  }
  if (ex == 255) return false;
  const long long mant = (long long)((b & 0x7fffffu) | 0x800000u);
  const int sh = ex - 150 + E;  // x = mant * 2^(ex - 150)
  long long v;
  if (sh >= 0) {
    if (sh > 37) return false;  // would pass 2^61
    v = mant << sh;
  } else {
    if (-sh > 24 || (mant & ((1ll << -sh) - 1)) != 0) return false;
    v = mant >> -sh;
  }
  X = (b >> 31) ? -v : v;
  return true;
}

// Root cube of each active subhalo (src/oct_tree.tpp:30-51) and its depth of
// geometric subdivision: the first level whose side is below TreeNodeResolution
// (the len halving rule of src/gravity_tree.cpp:37-40).
__global__ void k_cube(Ctx c)
{
  HBTU_KERNEL_PROLOGUE();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= c.S) return;
  SegState &sg = c.seg[s];
  if (sg.status != SEG_ACTIVE) return;
  double xmin[3] = {0, 0, 0}, xmax[3] = {0, 0, 0};
  const int b0 = c.tchunk_base[s], b1 = c.tchunk_base[s + 1];
  for (int j = 0; j < 3; j++) {
    float mn = INFINITY, mx = -INFINITY;
    for (int b = b0; b < b1; b++) {
      mn = fminf(mn, __uint_as_float(c.chunk_bbox[(size_t)b * 6 + j]));
      mx = fmaxf(mx, __uint_as_float(c.chunk_bbox[(size_t)b * 6 + 3 + j]));
    }
    xmin[j] = mn;
    xmax[j] = mx;
  }
  double Len = dsub(xmax[0], xmin[0]);
  for (int j = 1; j < 3; j++) {
    const double e = dsub(xmax[j], xmin[j]);
    if (e > Len) Len = e;
  }
  for (int j = 0; j < 3; j++) sg.center[j] = dmul(0.5, dadd(xmax[j], xmin[j]));
  if (b1 == b0) Len = 0.;
  sg.len = Len;
  int levels = 0;
  double L = Len;
  while (L >= (double)c.P.res && levels < kMaxLevels) {
    L = dmul(L, 0.5);
    levels++;
  }
  sg.levels = levels;
  fixed_point_cube(sg, levels);
  for (int j = 0; j < 3; j++) sg.fc[j] = sg.ref_pos[j];
  atomicMax(&c.plan->max_levels, levels);
}

// Octal key: digit k (k = 1..levels) is the octant at depth k, found with the
// reference's comparisons against centres halved in double.  Left-aligned.
__global__ void __launch_bounds__(kTB) k_keys(Ctx c, int ntotal)
{
  HBTU_KERNEL_PROLOGUE();
  const int e = blockIdx.x * kTB + threadIdx.x;
  if (e >= ntotal) return;
  const int s = upper_bound_i(c.tree_base, c.S + 1, e) - 1;
  const SegState &sg = c.seg[s];
  const int epos = sg.off + sg.t0 + (e - c.tree_base[s]);
  const float4 a = c.pm[c.epid[epos]];
  const float x[3] = {a.x, a.y, a.z};
  unsigned long long key = 0;
  long long X[3];
  if (sg.kfast && float_fixed(x[0], sg.kscale, X[0]) && float_fixed(x[1], sg.kscale, X[1]) &&
      float_fixed(x[2], sg.kscale, X[2])) {
    long long cen[3] = {sg.kc[0], sg.kc[1], sg.kc[2]};
    long long inc = sg.kinc;
    for (int k = 0; k < sg.levels; k++) {
      unsigned d = 0;
#pragma unroll
      for (int j = 0; j < 3; j++) {
        const bool gt = X[j] > cen[j];
        cen[j] += gt ? inc : -inc;
        d |= (unsigned)gt << j;
      }
      inc >>= 1;
      key = (key << 3) | d;
    }
    if (sg.levels > 0) key <<= (64 - 3 * sg.levels);
    c.sb.lo_a[e] = key;
    c.sb.hi_a[e] = (unsigned)s;
    c.sb.val_a[e] = epos;
    return;
  }
  double cen[3] = {sg.center[0], sg.center[1], sg.center[2]};
  double lenhalf = dmul(0.5, sg.len);
  for (int k = 0; k < sg.levels; k++) {
    lenhalf = dmul(lenhalf, 0.5);
    unsigned d = 0;
#pragma unroll
    for (int j = 0; j < 3; j++) {
      if ((double)x[j] > cen[j]) {
        cen[j] = dadd(cen[j], lenhalf);
        d |= 1u << j;
      } else {
        cen[j] = dsub(cen[j], lenhalf);
      }
    }
    key = (key << 3) | d;
  }
  if (sg.levels > 0) key <<= (64 - 3 * sg.levels);
  c.sb.lo_a[e] = key;
  c.sb.hi_a[e] = (unsigned)s;
  c.sb.val_a[e] = epos;
}

__device__ __forceinline__ int kdelta(const unsigned long long *keys, int n, int i, int j)
{
  if (j < 0 || j >= n) return -1;
  const unsigned long long a = keys[i], b = keys[j];
  if (a != b) return __clzll(a ^ b);
  return 64 + __clz((unsigned)(i ^ j));
}

// Karras (2012) binary radix tree over each subhalo's sorted keys.
// Child codes: internal node -> its element index; leaf -> ~element index.
__global__ void __launch_bounds__(kTB) k_karras(Ctx c, int ntotal)
{
  HBTU_KERNEL_PROLOGUE();
  const int e = blockIdx.x * kTB + threadIdx.x;
  if (e >= ntotal) return;
  const int s = c.sb.hi_a[e];
  const int base = c.tree_base[s], n = c.tree_base[s + 1] - base;
  const int i = e - base;
  if (i >= n - 1) return;
  const unsigned long long *keys = c.sb.lo_a + base;
  const int d = (kdelta(keys, n, i, i + 1) - kdelta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
  const int dmin = kdelta(keys, n, i, i - d);
  int lmax = 2;
  while (kdelta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
  int l = 0;
  for (int t = lmax >> 1; t >= 1; t >>= 1)
    if (kdelta(keys, n, i, i + (l + t) * d) > dmin) l += t;
  const int j = i + l * d;
  const int dn = kdelta(keys, n, i, j);
  int sp = 0, t = l;
  do {
    t = (t + 1) >> 1;
    if (kdelta(keys, n, i, i + (sp + t) * d) > dn) sp += t;
  } while (t > 1);
  const int gamma = i + sp * d + min(d, 0);
  const int first = min(i, j), last = max(i, j);
  c.rfirst[e] = first;
  c.rlast[e] = last;
  c.dnode[e] = dn;
  if (first == gamma) {
    c.childL[e] = ~(base + gamma);
    c.parentL[base + gamma] = e;
  } else {
    c.childL[e] = base + gamma;
    c.parentI[base + gamma] = e;
  }
  if (last == gamma + 1) {
    c.childR[e] = ~(base + gamma + 1);
    c.parentL[base + gamma + 1] = e;
  } else {
    c.childR[e] = base + gamma + 1;
    c.parentI[base + gamma + 1] = e;
  }
  if (i == 0) c.parentI[e] = -1;
}

__device__ __forceinline__ int oct_depth(int dn, int levels) { return min(dn / 3, levels); }

// Octant digit at depth k (1-based) of a left-aligned key.
__device__ __forceinline__ int octant_at(unsigned long long key, int k)
{
  return (int)(key >> (64 - 3 * k)) & 7;
}

// An internal node is an octree cell when its octal depth exceeds its
// parent's (the root always is).  Record depth bits per first key.
__global__ void __launch_bounds__(kTB) k_cells(Ctx c, int ntotal)
{
  HBTU_KERNEL_PROLOGUE();
  const int e = blockIdx.x * kTB + threadIdx.x;
  if (e >= ntotal) return;
  const int s = c.sb.hi_a[e];
  const int base = c.tree_base[s], n = c.tree_base[s + 1] - base;
  if (e - base >= n - 1) {
    c.iscell[e] = 0;
    return;
  }
  const int L = c.seg[s].levels;
  const int od = oct_depth(c.dnode[e], L);
  const int p = c.parentI[e];
  const int odp = p < 0 ? -1 : oct_depth(c.dnode[p], L);
  const int cell = od > odp;
  c.iscell[e] = cell;
  if (cell) atomicOr(&c.mask[base + c.rfirst[e]], 1ull << od);
}

__global__ void __launch_bounds__(kTB) k_popc(Ctx c, int ntotal)
{
  HBTU_KERNEL_PROLOGUE();
  const int e = blockIdx.x * kTB + threadIdx.x;
  if (e > ntotal) return;
  c.pcode[e] = e < ntotal ? __popcll(c.mask[e]) : 0;
}

// Walk record meta of a cell with side^2 = l2 (float, as the reference
// computes len*len): the squared distances below which the cell surely opens
// and above which it surely does not, l2/theta^2 (1 -+ 1e-5); in between the
// walk takes the reference's decision in double.  Particles (never opened)
// get -1 for both.
__device__ __forceinline__ int4 cell_meta(float l2, int skip, const DevParams &P)
{
  const double q = (double)l2 / (double)P.theta2;
  const float lo = (float)(q * (1.0 - 1e-5)), hi = (float)(q * (1.0 + 1e-5));
  return make_int4(__float_as_int(l2), skip, __float_as_int(lo), __float_as_int(hi));
}

__device__ __forceinline__ int4 particle_meta(int skip)
{
  return make_int4(0, skip, __float_as_int(-1.f), __float_as_int(-1.f));
}

__device__ __forceinline__ float4 make_rel(float4 a, const float fc[3], const DevParams &P)
{
  return make_float4(rel_coord(a.x, fc[0], P), rel_coord(a.y, fc[1], P), rel_coord(a.z, fc[2], P),
                     a.w);
}

// Particle leaves: preorder index = j + #cells starting at or before key j.
__global__ void __launch_bounds__(kTB) k_leaves(Ctx c, int ntotal)
{
  HBTU_KERNEL_PROLOGUE();
  const int e = blockIdx.x * kTB + threadIdx.x;
  if (e >= ntotal) return;
  const int s = c.sb.hi_a[e];
  SegState &sg = c.seg[s];
  const int base = c.tree_base[s], n = c.tree_base[s + 1] - base;
  const int j = e - base;
  const int nb = 2 * base;
  const float4 a0 = c.pm[c.epid[c.sb.val_a[e]]];
  const float4 a = make_float4(a0.x, a0.y, a0.z, fmul(a0.w, sg.mfac));
  if (n == 1) {  // a root cell of side 0 holding the particle (tpp:56-102 with one particle)
    const float4 r = make_rel(a, sg.fc, c.P);
    c.nd_abs[nb] = a;
    c.nd[nb].p = make_float4(r.x, r.y, r.z, -r.w);  // the sign bit marks a cell
    c.nd[nb].m = cell_meta(fmul((float)sg.len, (float)sg.len), kDone, c.P);
    c.nd_abs[nb + 1] = a;
    c.nd[nb + 1].p = r;
    c.nd[nb + 1].m = particle_meta(kDone);
    sg.nnodes = 2;
    return;
  }
  const long long xb = c.X[base];
  const int idx = j + (int)(c.X[e + 1] - xb);
  const int nnodes = n + (int)(c.X[base + n] - xb);
  c.nd_abs[nb + idx] = a;
  c.nd[nb + idx].p = make_rel(a, sg.fc, c.P);
  c.nd[nb + idx].m = particle_meta(idx + 1 < nnodes ? nb + idx + 1 : kDone);
  if (j == 0) sg.nnodes = nnodes;
  // the octant slot in the lowest cell holding this particle (none in a bucket)
  int p = c.parentL[e];
  for (int guard = 0; p >= 0 && !c.iscell[p] && guard < 256; guard++) p = c.parentI[p];
  if (p >= 0 && c.iscell[p]) {
    const int odp = oct_depth(c.dnode[p], sg.levels);
    if (odp < sg.levels) c.cslot[8 * p + octant_at(c.sb.lo_a[e], odp + 1)] = nb + idx;
  }
}

// Cells: preorder index, skip pointer, side (len*len in float), octal depth,
// and a count of child cells on the parent.
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
  const SegState &sg = c.seg[s];
  const int base = c.tree_base[s];
  const int nb = 2 * base;
  const int od = oct_depth(c.dnode[e], sg.levels);
  const int lo = c.rfirst[e], hi = c.rlast[e];
  const unsigned long long m = c.mask[base + lo];
  const int rank = __popcll(m & ((1ull << od) - 1ull));
  const long long xb = c.X[base];
  const int idx = lo + (int)(c.X[base + lo] - xb) + rank;
  const int skip = hi + 1 + (int)(c.X[base + hi + 1] - xb);
  double len = sg.len;
  for (int k = 0; k < od; k++)
    if (len >= (double)c.P.res) len = dmul(len, 0.5);
  const float lf = (float)len;
  const int n = c.tree_base[s + 1] - base;
  c.nd[nb + idx].m = cell_meta(fmul(lf, lf), hi + 1 < n ? nb + skip : kDone, c.P);
  c.cidx[e] = nb + idx;
  c.cskip[e] = nb + skip;
  c.cdepth[e] = od;
  int p = c.parentI[e];
  for (int guard = 0; p >= 0 && !c.iscell[p] && guard < 256; guard++) p = c.parentI[p];
  if (p >= 0 && !c.iscell[p]) p = -1;  // malformed tree: never climb past it
  c.pcell[e] = p;
  if (p >= 0) {
    atomicAdd(&c.pending[p], 1);
    const int odp = oct_depth(c.dnode[p], sg.levels);
    c.cslot[8 * p + octant_at(c.sb.lo_a[base + lo], odp + 1)] = nb + idx;
  }
}

// Bottom-up moments: a cell is summed once all its child cells are, by the
// thread that finished the last child (atomic countdown, no waiting): mass
// and centre of mass over the children in octant order, in double, rounded
// to float per cell as the reference does.  The children are read from the
// cell's eight octant slots with independent loads; a bucket cell (particles
// sharing the whole key) walks its children by skip pointers.  A cell
// without child cells is marked for the walk's leaf runs (sign bit of
// len*len).
__device__ __forceinline__ void add_child(const Ctx &c, int k, double &m, double &cx, double &cy,
                                          double &cz)
{
  // a product of two floats is exact in double, so one fused multiply-add
  // rounds exactly as the reference's multiply-then-add
  const float4 a = __ldcg(&c.nd_abs[k]);
  const double w = f2d(a.w);
  m = dadd(m, w);
  cx = __fma_rn(f2d(a.x), w, cx);
  cy = __fma_rn(f2d(a.y), w, cy);
  cz = __fma_rn(f2d(a.z), w, cz);
}

__global__ void __launch_bounds__(kTB) k_moments(Ctx c, int ntotal)
{
  HBTU_KERNEL_PROLOGUE();
  int e = blockIdx.x * kTB + threadIdx.x;
  if (e >= ntotal || !c.iscell[e] || c.pending0[e] != 0) return;
  c.nd[c.cidx[e]].m.x |= (int)0x80000000;
  for (int level = 0; level <= 2 * kMaxLevels + 2; level++) {
    const int s = c.sb.hi_a[e];
    const SegState &sg = c.seg[s];
    const int idx = c.cidx[e], end = c.cskip[e];
    double m = 0., cx = 0., cy = 0., cz = 0.;
    if (c.cdepth[e] < sg.levels) {
      const int4 s0 = __ldcg(reinterpret_cast<const int4 *>(c.cslot + 8 * e));
      const int4 s1 = __ldcg(reinterpret_cast<const int4 *>(c.cslot + 8 * e) + 1);
      const int sl[8] = {s0.x, s0.y, s0.z, s0.w, s1.x, s1.y, s1.z, s1.w};
#pragma unroll
      for (int j = 0; j < 8; j++)
        if (sl[j] > idx && sl[j] < end) add_child(c, sl[j], m, cx, cy, cz);
    } else {
      for (int k = idx + 1; k < end;) {
        add_child(c, k, m, cx, cy, cz);
        const int nk = c.nd[k].m.y;
        k = nk > k ? nk : end;  // skip pointers always move forward
      }
    }
    const float4 r = make_float4(d2f(ddiv(cx, m)), d2f(ddiv(cy, m)), d2f(ddiv(cz, m)), d2f(m));
    __stcg(&c.nd_abs[idx], r);
    float4 rel = make_rel(r, sg.fc, c.P);
    rel.w = -rel.w;  // the sign bit marks a cell for the walks
    c.nd[idx].p = rel;
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
    const int s = c.sb.hi_a[e];
    const SegState &sg = c.seg[s];
    const int idx = c.cidx[e], end = c.cskip[e];
    if (c.pending[e] == 0) c.nd[idx].m.x |= (int)0x80000000;
    double m = 0., cx = 0., cy = 0., cz = 0.;
    if (depth < sg.levels) {
      const int4 s0 = reinterpret_cast<const int4 *>(c.cslot + 8 * e)[0];
      const int4 s1 = reinterpret_cast<const int4 *>(c.cslot + 8 * e)[1];
      const int sl[8] = {s0.x, s0.y, s0.z, s0.w, s1.x, s1.y, s1.z, s1.w};
#pragma unroll
      for (int j = 0; j < 8; j++)
        if (sl[j] > idx && sl[j] < end) add_child(c, sl[j], m, cx, cy, cz);
    } else {
      for (int k = idx + 1; k < end;) {
        add_child(c, k, m, cx, cy, cz);
        const int nk = c.nd[k].m.y;
        k = nk > k ? nk : end;  // skip pointers always move forward
      }
    }
    const float4 r = make_float4(d2f(ddiv(cx, m)), d2f(ddiv(cy, m)), d2f(ddiv(cz, m)), d2f(m));
    c.nd_abs[idx] = r;
    float4 rel = make_rel(r, sg.fc, c.P);
    rel.w = -rel.w;  // the sign bit marks a cell for the walks
    c.nd[idx].p = rel;
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
