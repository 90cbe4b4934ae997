// tree_ops.cuh -- the per-element steps of the octree build, shared by the
// batch kernels (tree.cu: one thread per element of every active subhalo) and
// the per-subhalo loop (small.cu: one block walks one subhalo through them).
//
// Reference: OctTree_t::Build (src/oct_tree.tpp:16-144) and
// GravityTree_t::UpdateInternalNodes / ProcessNode / FillNodeCenter
// (src/gravity_tree.cpp:18-77).  The steps:
//   seg_cube       bounding cube and depth of geometric subdivision;
//   seg_key        octal key of one particle (the reference's comparisons
//                  x > centre with centres halved in double);
//   karras_elem    one internal node of the Karras (2012) radix tree over a
//                  subhalo's sorted keys;
//   cells_elem     whether an internal node is an octree cell;
//   leaves_elem    preorder slot and record of one particle leaf;
//   cellnodes_elem preorder slot, skip pointer and side of one cell;
//   cell_moment    mass and centre of mass of one cell from its children,
//                  in octant order, in double, rounded to float per cell.
// Element e of a subhalo's tree is its e-th key in sorted order; `base` is the
// index of its first element in the element arrays, and its node slots are
// [2*base, 2*base + 2*n).
#pragma once
#include "device_common.cuh"

namespace hbtu {

__device__ __forceinline__ int ll_tz(long long v) { return v ? __ffsll(v) - 1 : 64; }

// Fixed-point form of the key computation.  The reference halves the cube in
// double: centre_k = centre_{k-1} +- len / 2^(k+1).  When the centre, len/4
// and every later increment are integers in units of 2^-E, and every centre
// fits in 53 significant bits, none of those double operations rounds, so the
// same comparisons x > centre_k can be made exactly on 64-bit integers
// (a tenth of the cost: double runs at 1/64 of the FP32 rate on this GPU).
__device__ __forceinline__ void fixed_point_cube(SegState &sg, int levels)
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

// Root cube of a subhalo from the float bounding box of its tree particles
// (src/oct_tree.tpp:30-51; an empty box gives a cube of side 0) and its depth
// of geometric subdivision: the first level whose side is below
// TreeNodeResolution (the len halving rule of src/gravity_tree.cpp:37-40).
// The frame centre of the relative coordinates is the subhalo's frame.
__device__ __forceinline__ int seg_cube(SegState &sg, const float mn[3], const float mx[3],
                                        bool empty, const DevParams &P)
{
  double xmin[3], xmax[3];
  for (int j = 0; j < 3; j++) {
    xmin[j] = mn[j];
    xmax[j] = mx[j];
  }
  double Len = dsub(xmax[0], xmin[0]);
  for (int j = 1; j < 3; j++) {
    const double e = dsub(xmax[j], xmin[j]);
    if (e > Len) Len = e;
  }
  for (int j = 0; j < 3; j++) sg.center[j] = dmul(0.5, dadd(xmax[j], xmin[j]));
  if (empty) Len = 0.;
  sg.len = Len;
  int levels = 0;
  double L = Len;
  while (L >= (double)P.res && levels < kMaxLevels) {
    L = dmul(L, 0.5);
    levels++;
  }
  sg.levels = levels;
  fixed_point_cube(sg, levels);
  for (int j = 0; j < 3; j++) sg.fc[j] = sg.ref_pos[j];
  return levels;
}

// Octal key: digit k (k = 1..levels) is the octant at depth k, found with the
// reference's comparisons against centres halved in double (tpp:67-95).
// Left-aligned in 64 bits.
__device__ __forceinline__ unsigned long long seg_key(const SegState &sg, float4 a)
{
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
    return key;
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
  return key;
}

// Longest common prefix of sorted keys i and j (index tie-break for equal keys).
__device__ __forceinline__ int kdelta(const unsigned long long *keys, int n, int i, int j)
{
  if (j < 0 || j >= n) return -1;
  const unsigned long long a = keys[i], b = keys[j];
  if (a != b) return __clzll(a ^ b);
  return 64 + __clz((unsigned)(i ^ j));
}

// Internal node i (0 <= i < n-1) of the Karras (2012) binary radix tree over
// a subhalo's sorted keys: its key range, split depth, and the parent links of
// its two children (parentI for an internal child, parentL for a leaf).
__device__ __forceinline__ void karras_elem(const Ctx &c, const unsigned long long *keys, int base,
                                            int n, int i)
{
  const int e = base + i;
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
  if (first == gamma)  // the left child is a leaf (key gamma) or internal node gamma
    c.parentL[base + gamma] = e;
  else
    c.parentI[base + gamma] = e;
  if (last == gamma + 1)  // the right child: leaf or internal node gamma + 1
    c.parentL[base + gamma + 1] = e;
  else
    c.parentI[base + gamma + 1] = e;
  if (i == 0) c.parentI[e] = -1;
}

__device__ __forceinline__ int oct_depth(int dn, int levels) { return min(dn / 3, levels); }

// Octant digit at depth k (1-based) of a left-aligned key.
__device__ __forceinline__ int octant_at(unsigned long long key, int k)
{
  return (int)(key >> (64 - 3 * k)) & 7;
}

// An internal node is an octree cell when its octal depth exceeds its
// parent's (the root always is).  Records the depth bits per first key.
__device__ __forceinline__ void cells_elem(const Ctx &c, int base, int n, int e, int levels)
{
  if (e - base >= n - 1) {
    c.iscell[e] = 0;
    return;
  }
  const int od = oct_depth(c.dnode[e], levels);
  const int p = c.parentI[e];
  const int odp = p < 0 ? -1 : oct_depth(c.dnode[p], levels);
  const int cell = od > odp;
  c.iscell[e] = cell;
  if (cell) atomicOr(&c.mask[base + c.rfirst[e]], 1ull << od);
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

// Particle leaf j of a subhalo's tree (element e = base + j): preorder index
// j + #cells starting at or before key j; a0 is its particle {x, y, z, m}
// (mass not yet scaled by the sampling factor).  Xs[0..n]: the exclusive scan
// of the cells starting at each of the subhalo's keys (any common offset).
// The subhalo of one particle gets a root cell of side 0 holding it
// (tpp:56-102 with one particle).
__device__ __forceinline__ void leaves_elem(const Ctx &c, SegState &sg, int base, int n, int e,
                                            float4 a0, unsigned long long key,
                                            const long long *Xs)
{
  const int j = e - base;
  const int nb = 2 * base;
  const float4 a = make_float4(a0.x, a0.y, a0.z, fmul(a0.w, sg.mfac));
  if (n == 1) {
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
  const long long xb = Xs[0];
  const int idx = j + (int)(Xs[j + 1] - xb);
  const int nnodes = n + (int)(Xs[n] - xb);
  c.nd_abs[nb + idx] = a;
  c.nd[nb + idx].p = make_rel(a, sg.fc, c.P);
  c.nd[nb + idx].m = particle_meta(idx + 1 < nnodes ? nb + idx + 1 : kDone);
  if (j == 0) sg.nnodes = nnodes;
  // the octant slot in the lowest cell holding this particle (none in a bucket)
  int p = c.parentL[e];
  for (int guard = 0; p >= 0 && !c.iscell[p] && guard < 256; guard++) p = c.parentI[p];
  if (p >= 0 && c.iscell[p]) {
    const int odp = oct_depth(c.dnode[p], sg.levels);
    if (odp < sg.levels) c.cslot[8 * p + octant_at(key, odp + 1)] = nb + idx;
  }
}

// Cell e (an internal node with iscell[e] set): preorder index, skip pointer,
// side (len*len in float), octal depth, and a count of child cells on the
// parent.  keys: the subhalo's sorted keys, element-indexed from `base`; Xs
// as for leaves_elem.
__device__ __forceinline__ void cellnodes_elem(const Ctx &c, const SegState &sg, int base, int n,
                                               int e, const unsigned long long *keys,
                                               const long long *Xs)
{
  const int nb = 2 * base;
  const int od = oct_depth(c.dnode[e], sg.levels);
  const int lo = c.rfirst[e], hi = c.rlast[e];
  const unsigned long long m = c.mask[base + lo];
  const int rank = __popcll(m & ((1ull << od) - 1ull));
  const long long xb = Xs[0];
  const int idx = lo + (int)(Xs[lo] - xb) + rank;
  const int skip = hi + 1 + (int)(Xs[hi + 1] - xb);
  double len = sg.len;
  for (int k = 0; k < od; k++)
    if (len >= (double)c.P.res) len = dmul(len, 0.5);
  const float lf = (float)len;
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
    c.cslot[8 * p + octant_at(keys[lo], odp + 1)] = nb + idx;
  }
}

// 1/m to within a few units in the last place: the hardware's approximate
// double reciprocal refined by two Newton-Raphson steps r <- r + r (1 - m r)
// (each step squares the relative error).  ok: the residual 1 - m r, taken
// once more, shows a relative error below 2^-49 (else r is not used).
__device__ __forceinline__ double recip_refined(double m, bool &ok)
{
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(m));
  r = __fma_rn(r, __fma_rn(-m, r, 1.0), r);
  r = __fma_rn(r, __fma_rn(-m, r, 1.0), r);
  ok = fabs(__fma_rn(-m, r, 1.0)) < 0x1p-49;
  return r;
}

// float(c / m) with the quotient first rounded to double, as the reference
// rounds its double centre of mass to float, given r ~ 1/m (ok as above).
// q = c * r then lies within a few double units in the last place of the
// correctly rounded quotient, so both round to the same float unless q lies
// within 64 units of a point halfway between two floats (its low 29 mantissa
// bits near 2^28), or outside the range of normal floats; those take the
// exact division.
__device__ __forceinline__ float quot_float(double c, double m, double r, bool ok)
{
  const double q = dmul(c, r);
  const unsigned long long b = (unsigned long long)__double_as_longlong(q);
  const int ex = (int)((b >> 52) & 0x7ffull);
  const unsigned rem = (unsigned)(b & 0x1fffffffull);
  if (ok && ex >= 1023 - 125 && ex <= 1023 + 126 && rem - (0x10000000u - 64u) > 128u)
    return d2f(q);
  return d2f(ddiv(c, m));
}

// Bottom-up moments of one cell: mass and centre of mass over its children in
// octant order, in double, rounded to float as the reference does.  The
// children come from the cell's eight octant slots; the children of a bucket
// cell (particles sharing the whole key, depth == levels) hold the slots that
// follow it, in preorder, so they are read one after another.  src(k) gives
// the moment {x, y, z, m} of node slot k (global memory, or a block's copy).
// A product of two floats is exact in double, so one fused multiply-add
// rounds exactly as the reference's multiply-then-add.
// The same with the cell's octant slots s0, s1 (cslot) already loaded;
// bucket: the cell is a bucket (depth == levels).
template <class Src>
__device__ __forceinline__ float4 cell_moment_slots(bool bucket, int idx, int end, int4 s0,
                                                    int4 s1, Src src)
{
  double m = 0., cx = 0., cy = 0., cz = 0.;
  auto add = [&](int k) {
    const float4 a = src(k);
    const double w = f2d(a.w);
    m = dadd(m, w);
    cx = __fma_rn(f2d(a.x), w, cx);
    cy = __fma_rn(f2d(a.y), w, cy);
    cz = __fma_rn(f2d(a.z), w, cz);
  };
  if (!bucket) {
    // the occupied octants in ascending order; a warp then issues as many
    // (double) additions as its lanes' largest number of children, not eight
    const int sl[8] = {s0.x, s0.y, s0.z, s0.w, s1.x, s1.y, s1.z, s1.w};
    unsigned occ = 0;
#pragma unroll
    for (int j = 0; j < 8; j++) occ |= (sl[j] > idx && sl[j] < end ? 1u : 0u) << j;
    while (occ) {
      const int j = __ffs(occ) - 1;
      occ &= occ - 1;
      const int4 h = j < 4 ? s0 : s1;
      const int q = j & 3;
      add(q == 0 ? h.x : (q == 1 ? h.y : (q == 2 ? h.z : h.w)));
    }
  } else {
#pragma unroll 4
    for (int k = idx + 1; k < end; k++) add(k);
  }
  bool ok;
  const double r = recip_refined(m, ok);
  return make_float4(quot_float(cx, m, r, ok), quot_float(cy, m, r, ok), quot_float(cz, m, r, ok),
                     d2f(m));
}

template <bool kCG, class Src>
__device__ __forceinline__ float4 cell_moment_of(const Ctx &c, const SegState &sg, int e,
                                                 int depth, int idx, int end, Src src)
{
  int4 s0 = make_int4(-1, -1, -1, -1), s1 = s0;
  const bool bucket = depth >= sg.levels;
  if (!bucket) {
    const int4 *slot = reinterpret_cast<const int4 *>(c.cslot + 8 * e);
    s0 = kCG ? __ldcg(slot) : slot[0];
    s1 = kCG ? __ldcg(slot + 1) : slot[1];
  }
  return cell_moment_slots(bucket, idx, end, s0, s1, src);
}

// The walk record's position and mass of a cell from its moment (fc: the
// subhalo's frame centre).
__device__ __forceinline__ void store_cell_rel(const Ctx &c, const float fc[3], int idx, float4 r)
{
  float4 rel = make_rel(r, fc, c.P);
  rel.w = -rel.w;  // the sign bit marks a cell for the walks
  c.nd[idx].p = rel;
}

// cell_moment_of over the moments in global memory (kCG: through L2, for
// callers whose children were written by other blocks during the same
// launch); stores the cell's moment and record.
template <bool kCG>
__device__ __forceinline__ void cell_moment(const Ctx &c, const SegState &sg, int e, int depth)
{
  const int idx = c.cidx[e], end = c.cskip[e];
  const float4 r = cell_moment_of<kCG>(c, sg, e, depth, idx, end, [&](int k) {
    return kCG ? __ldcg(&c.nd_abs[k]) : c.nd_abs[k];
  });
  if (kCG)
    __stcg(&c.nd_abs[idx], r);
  else
    c.nd_abs[idx] = r;
  store_cell_rel(c, sg.fc, idx, r);
}

}  // namespace hbtu
