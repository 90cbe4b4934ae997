// props.cu -- post-unbinding properties of every subhalo of a batch.
//
// Reference: Subhalo_t::CalculateProfileProperties (src/subhalo.cpp:242-335)
// with Snapshot_t::SphericalOverdensitySize and HaloVirialFactors
// (src/snapshot.cpp:259-281, :328-336), and Subhalo_t::CalculateShape
// (src/subhalo.cpp:337-398), on the bound particles an unbinding left in
// front of each subhalo's list.
//   profile: the distance of every bound particle to the most-bound one
//     (PeriodicDistance, src/config_parser.h:143-156, in float), a stable
//     radix sort by (subhalo, distance), the cumulative mass, the radius
//     floored at the softening, v^2 = m / r and its first maximum, the
//     half-mass and 95.5% radii, and the outermost radius inside which the
//     mean density exceeds 200 times critical;
//   shape: the inertia tensors, float terms summed in double per 256-particle
//     chunk (one warp: lane-strided sums, then a fixed shuffle tree), then over
//     the chunks in order.
// Exactness.  The reference sums the cumulative mass sequentially in double.
// Here it is summed exactly in 64-bit fixed point (units of the lowest mass
// bit of the batch), which equals the sequential double sum whenever that sum
// never rounds: a subhalo whose total stays below 2^53 units.  Other subhaloes
// (and every subhalo when a mass is negative or the masses span too many
// binary orders) take a sequential double sum, one thread per subhalo.  Ties
// in distance keep the unbinding order (the reference's std::sort leaves them
// unspecified).  The shape sums run in another order than the reference's
// sequential loop; the float results can differ from it by one unit in the
// last place when a double sum lies within rounding error of a float
// rounding boundary.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "device_common.cuh"
#include "handle.h"

namespace hbtu {
namespace {

constexpr int kPB = 256;
constexpr int kPChunk = 256;  // shape particles per warp-chunk
constexpr long long kExact = 1ll << 53;

struct PropSeg {
  int64_t off;   // first particle of the subhalo in the batch
  int64_t boff;  // first bound element in the flat bound index space
  int64_t nb;    // Nbound (0 when <= 1: no properties)
  int64_t n;     // particles of the subhalo
  float cen[3];  // ComovingMostBoundPosition
  float mbound;
  int chunk0, nchunk;  // shape chunks
};

// Flags of one call (device): [0] sort look-back error, [1] lowest set bit of
// any mass (power of two), [2] highest, [3] a negative or non-finite mass,
// [4] an order entry outside its subhalo.
enum { F_SORT = 0, F_LOW = 1, F_HIGH = 2, F_NEG = 3, F_ORDER = 4, F_WORDS = 5 };

// Particle at bound position k of subhalo g (an order entry outside the
// subhalo reads its first particle; k_pr_elem reports it).
__device__ __forceinline__ int64_t bound_particle(const PropSeg &g, const int64_t *order,
                                                  int64_t k, int64_t n)
{
  const int64_t o = order[g.off + k];
  return g.off + ((o >= 0 && o < n) ? o : 0);
}

__device__ __forceinline__ int seg_of(const int64_t *boff, int S, int64_t j)
{
  int lo = 0, hi = S;  // last s with boff[s] <= j
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (boff[mid] <= j)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

// Fixed-point scale of the batch: every mass is an integer multiple of 2^-K,
// and every prefix sum fits an int64.  false: no usable scale.
__device__ __forceinline__ bool fix_scale(const int *flags, int64_t T, int *K)
{
  const int lo = flags[F_LOW], hi = flags[F_HIGH];
  *K = 0;
  if (flags[F_NEG]) return false;
  if (lo == 0x7fffffff) return true;  // every mass is zero
  int lt = 0;
  while ((1ll << lt) <= T) lt++;
  if (hi - lo + 1 + lt > 62) return false;
  *K = -lo;
  return true;
}

__device__ __forceinline__ float periodic_distance(const float x[3], const float c[3],
                                                   const DevParams &P)
{
  float d[3];
  for (int j = 0; j < 3; j++) {
    d[j] = fsub(x[j], c[j]);
    if (P.periodic) d[j] = nearest_f(d[j], P);
  }
  return __fsqrt_rn(fadd(fadd(fmul(d[0], d[0]), fmul(d[1], d[1])), fmul(d[2], d[2])));
}

// Per bound element: distance, sort record, binary range of the masses (the
// range reduced over the warp before its one atomic).
__global__ void __launch_bounds__(kPB) k_pr_elem(const PropSeg *seg, const int64_t *boff, int S,
                                                 int64_t T, const float *pos, const float *mass,
                                                 const int64_t *order, unsigned long long *lo,
                                                 unsigned *hi, int *val, int *flags, DevParams P)
{
  HBTU_KERNEL_PROLOGUE();
  const int64_t j = (int64_t)blockIdx.x * kPB + threadIdx.x;
  int lowbit = 0x7fffffff, highbit = -0x7fffffff;
  if (j < T) {
    const int s = seg_of(boff, S, j);
    const PropSeg g = seg[s];
    const int64_t o = order[g.off + (j - g.boff)];
    if (o < 0 || o >= g.n) atomicOr(&flags[F_ORDER], 1);
    const int64_t pid = bound_particle(g, order, j - g.boff, g.n);
    const float x[3] = {pos[3 * pid], pos[3 * pid + 1], pos[3 * pid + 2]};
    const float r = periodic_distance(x, g.cen, P);
    lo[j] = (unsigned long long)__float_as_uint(r);  // r >= 0: bits sort as values
    hi[j] = (unsigned)s;
    val[j] = (int)j;
    const unsigned b = __float_as_uint(mass[pid]);
    const int ex = (int)((b >> 23) & 255u);
    const unsigned m = ex ? ((b & 0x7fffffu) | 0x800000u) : (b & 0x7fffffu);
    if (((b >> 31) && (b & 0x7fffffffu)) || ex == 255) atomicOr(&flags[F_NEG], 1);
    if (m && ex != 255) {
      const int e0 = (ex ? ex : 1) - 150;  // value = m * 2^e0
      lowbit = e0 + __ffs(m) - 1;
      highbit = e0 + 31 - __clz(m);
    }
  }
  lowbit = __reduce_min_sync(0xffffffffu, lowbit);
  highbit = __reduce_max_sync(0xffffffffu, highbit);
  if ((threadIdx.x & 31) == 0 && lowbit != 0x7fffffff) {
    atomicMin(&flags[F_LOW], lowbit);
    atomicMax(&flags[F_HIGH], highbit);
  }
}

// Masses in sorted order: as floats, and as fixed-point integers (0 when no
// scale exists).
__global__ void __launch_bounds__(kPB) k_pr_fix(const PropSeg *seg, const int64_t *boff, int S,
                                                int64_t T, const int *val, const float *mass,
                                                const int64_t *order, const int *flags,
                                                float *msorted, long long *mfix)
{
  HBTU_KERNEL_PROLOGUE();
  const int64_t q = (int64_t)blockIdx.x * kPB + threadIdx.x;
  if (q > T) return;
  if (q == T) {
    mfix[q] = 0;
    return;
  }
  const int64_t j = val[q];
  const int s = seg_of(boff, S, j);
  const PropSeg g = seg[s];
  const float m = mass[bound_particle(g, order, j - g.boff, g.n)];
  msorted[q] = m;
  int K;
  mfix[q] = fix_scale(flags, T, &K) ? (long long)ldexp((double)m, K) : 0;  // exact: below 2^62
}

__device__ __forceinline__ bool seg_exact(const PropSeg &g, const long long *cum, bool scaled)
{
  return scaled && cum[g.boff + g.nb] - cum[g.boff] < kExact;
}

// Sequential cumulative mass (double, as the reference) of the subhaloes the
// fixed-point sum does not cover; one thread per subhalo.
__global__ void k_pr_seq(const PropSeg *__restrict__ seg, int S, int64_t T,
                         const float *__restrict__ msorted, const int *__restrict__ flags,
                         const long long *__restrict__ cum, float *__restrict__ mc)
{
  HBTU_KERNEL_PROLOGUE();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= S) return;
  const PropSeg g = seg[s];
  int K;
  const bool scaled = fix_scale(flags, T, &K);
  if (g.nb == 0 || seg_exact(g, cum, scaled)) return;
  const float *m = msorted + g.boff;
  float *out = mc + g.boff;
  double c = 0.;
  for (int64_t k = 0; k < g.nb; k++) {
    c = dadd(c, f2d(m[k]));
    out[k] = d2f(c);
  }
}

// Maximum over the lanes of each run of equal s (runs are contiguous: the
// elements are sorted by subhalo), left in the run's first lane.
__device__ __forceinline__ unsigned long long run_max(unsigned long long v, int s)
{
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long w = __shfl_down_sync(0xffffffffu, v, o);
    const int ws = __shfl_down_sync(0xffffffffu, s, o);
    if (lane + o < 32 && ws == s) v = max(v, w);
  }
  return v;
}

// Per sorted element: cumulative mass, floored radius, v^2, the per-subhalo
// first maximum, the overdensity radius and the two quantile radii.  The
// maxima are reduced over each warp's runs of one subhalo before the atomics.
__global__ void __launch_bounds__(kPB) k_pr_prof(const PropSeg *seg, const int64_t *boff, int S,
                                                 int64_t T, const unsigned long long *rsorted,
                                                 const long long *mfix, const long long *cum,
                                                 const int *flags, float eps, float rho_vir,
                                                 float *rc, float *mc, unsigned long long *vmax,
                                                 long long *so, float *quant)
{
  HBTU_KERNEL_PROLOGUE();
  const int64_t q = (int64_t)blockIdx.x * kPB + threadIdx.x;
  const int lane = threadIdx.x & 31;
  int s = -1 - lane;  // a run of its own for lanes past the end
  unsigned long long vkey = 0ull, sokey = 0ull;  // so index + 1, 0: none
  if (q < T) {
    s = seg_of(boff, S, q);  // sorted by subhalo first: the same ranges
    const PropSeg g = seg[s];
    const int64_t k = q - g.boff;
    int K;
    const bool scaled = fix_scale(flags, T, &K);
    float m;
    if (seg_exact(g, cum, scaled))
      m = d2f(ldexp((double)(cum[q] + mfix[q] - cum[g.boff]), -K));  // exact below 2^53
    else
      m = mc[q];
    float r = __uint_as_float((unsigned)rsorted[q]);
    if (r < eps) r = eps;
    const float v = __fdiv_rn(m, r);
    rc[q] = r;
    mc[q] = m;
    vkey = ((unsigned long long)__float_as_uint(v) << 32) |
           (unsigned long long)(0xffffffffu - (unsigned)k);
    if (m > fmul(fmul(fmul(rho_vir, r), r), r)) sokey = (unsigned long long)k + 1ull;
    if (k == g.nb / 2) quant[2 * s] = r;
    if (k == (int64_t)((double)g.nb * 0.955)) quant[2 * s + 1] = r;
  }
  vkey = run_max(vkey, s);
  sokey = run_max(sokey, s);
  const int prev = __shfl_up_sync(0xffffffffu, s, 1);
  if (q < T && (lane == 0 || prev != s)) {
    atomicMax(&vmax[s], vkey);
    if (sokey) atomicMax(&so[s], (long long)sokey - 1);
  }
}

// Shape: the 12 tensor sums of one 256-particle chunk (particles 1 .. Nbound-1
// in bound order) per warp: each lane over a strided subset, then a fixed
// shuffle tree; eight chunks per block.
__global__ void __launch_bounds__(kPB) k_pr_shape(const PropSeg *seg, const int *chunk_seg, int nch,
                                                  const float *pos, const float *mass,
                                                  const int64_t *order, double *csum, DevParams P)
{
  HBTU_KERNEL_PROLOGUE();
  const int b = (int)(((int64_t)blockIdx.x * kPB + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (b >= nch) return;  // whole warps leave together
  const int s = chunk_seg[b];
  const PropSeg g = seg[s];
  const int64_t lo = 1 + (int64_t)(b - g.chunk0) * kPChunk;
  const int64_t hi = min(lo + kPChunk, g.nb);
  double v[12];
  for (int k = 0; k < 12; k++) v[k] = 0.;
  for (int64_t i = lo + lane; i < hi; i += 32) {
    const int64_t pid = bound_particle(g, order, i, g.n);
    const float m = mass[pid];
    float dx = fsub(pos[3 * pid], g.cen[0]), dy = fsub(pos[3 * pid + 1], g.cen[1]),
          dz = fsub(pos[3 * pid + 2], g.cen[2]);
    if (P.periodic) {
      dx = nearest_f(dx, P);
      dy = nearest_f(dy, P);
      dz = nearest_f(dz, P);
    }
    const float dx2 = fmul(dx, dx), dy2 = fmul(dy, dy), dz2 = fmul(dz, dz);
    v[0] = dadd(v[0], f2d(fmul(dx2, m)));
    v[1] = dadd(v[1], f2d(fmul(fmul(dx, dy), m)));
    v[2] = dadd(v[2], f2d(fmul(fmul(dx, dz), m)));
    v[3] = dadd(v[3], f2d(fmul(dy2, m)));
    v[4] = dadd(v[4], f2d(fmul(fmul(dy, dz), m)));
    v[5] = dadd(v[5], f2d(fmul(dz2, m)));
    const float dr2 = __fdiv_rn(fadd(fadd(dx2, dy2), dz2), m);
    v[6] = dadd(v[6], f2d(__fdiv_rn(dx2, dr2)));
    v[7] = dadd(v[7], f2d(__fdiv_rn(fmul(dx, dy), dr2)));
    v[8] = dadd(v[8], f2d(__fdiv_rn(fmul(dx, dz), dr2)));
    v[9] = dadd(v[9], f2d(__fdiv_rn(dy2, dr2)));
    v[10] = dadd(v[10], f2d(__fdiv_rn(fmul(dy, dz), dr2)));
    v[11] = dadd(v[11], f2d(__fdiv_rn(dz2, dr2)));
  }
#pragma unroll
  for (int k = 0; k < 12; k++)
    for (int o = 16; o > 0; o >>= 1) v[k] = dadd(v[k], __shfl_xor_sync(0xffffffffu, v[k], o));
  if (lane < 12) {
    double t = v[0];
#pragma unroll
    for (int k = 1; k < 12; k++)
      if (lane == k) t = v[k];
    csum[(size_t)b * 12 + lane] = t;
  }
}

// One warp per subhalo: the chunk sums in order, then every property but
// R200CritComoving (a cube root, taken on the host).
__global__ void k_pr_final(const PropSeg *seg, int S, const double *csum, const float *rc,
                           const float *mc, const unsigned long long *vmax, const long long *so,
                           const float *quant, const float *last_max, const int *last_snap,
                           int snapshot_index, float velocity_unit, hbtu_props *out)
{
  HBTU_KERNEL_PROLOGUE();
  const int s = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (s >= S) return;
  const PropSeg g = seg[s];
  double part = 0.;
  if (g.nb > 1 && lane < 12)
    for (int c = g.chunk0; c < g.chunk0 + g.nchunk; c++)
      part = dadd(part, csum[(size_t)c * 12 + lane]);
  double I[12];
#pragma unroll
  for (int k = 0; k < 12; k++) I[k] = __shfl_sync(0xffffffffu, part, k);
  if (lane != 0) return;
  hbtu_props r;
  memset(&r, 0, sizeof(r));
  r.last_max_vmax_physical = last_max ? last_max[s] : 0.f;
  r.snapshot_of_last_max_vmax = last_snap ? last_snap[s] : -1;
  if (g.nb > 1) {
    const unsigned long long vm = vmax[s];
    const int64_t kmax = (int64_t)(0xffffffffu - (unsigned)(vm & 0xffffffffull));
    const float v = __uint_as_float((unsigned)(vm >> 32));
    r.rmax_comoving = rc[g.boff + kmax];
    r.vmax_physical = __fsqrt_rn(fmul(v, velocity_unit));
    r.rhalf_comoving = quant[2 * s];
    r.r2sigma_comoving = quant[2 * s + 1];
    if (so[s] >= 0) r.m200crit = mc[g.boff + so[s]];
    if (r.vmax_physical >= r.last_max_vmax_physical) {  // subhalo.cpp:320-324
      r.snapshot_of_last_max_vmax = snapshot_index;
      r.last_max_vmax_physical = r.vmax_physical;
    }
    // InertialTensor = {Ixx, Ixy, Ixz, Iyy, Iyz, Izz}: the double sums as float, over Mbound
    for (int k = 0; k < 6; k++) {
      r.inertial_tensor[k] = __fdiv_rn(d2f(I[k]), g.mbound);
      r.inertial_tensor_weighted[k] = __fdiv_rn(d2f(I[6 + k]), g.mbound);
    }
  }
  out[s] = r;
}

inline unsigned pblk(int64_t n) { return (unsigned)((n + kPB - 1) / kPB); }
inline size_t a256(size_t b) { return (b + 255) / 256 * 256; }

}  // namespace
}  // namespace hbtu

using namespace hbtu;

extern "C" hbtu_status hbtu_subhalo_properties(hbtu_handle *h, const hbtu_particles *p,
                                               int64_t nsub, const int64_t *offsets,
                                               const int64_t *order, const hbtu_result *res,
                                               const float *last_max_vmax,
                                               const int32_t *last_snap, int32_t snapshot_index,
                                               hbtu_props *out)
{
  if (!h) return HBTU_ERR_INVALID_ARGUMENT;
  if (nsub < 0 || (nsub > 0 && (!p || !offsets || !order || !res || !out || !p->pos ||
                                !p->mass))) {
    h->err = "subhalo properties: null argument";
    return HBTU_ERR_INVALID_ARGUMENT;
  }
  if (nsub == 0) return HBTU_OK;
  if (offsets[0] != 0) {
    h->err = "subhalo properties: offsets must start at 0";
    return HBTU_ERR_INVALID_ARGUMENT;
  }
  for (int64_t s = 0; s < nsub; s++)
    if (offsets[s + 1] < offsets[s]) {
      h->err = "subhalo properties: offsets must not decrease";
      return HBTU_ERR_INVALID_ARGUMENT;
    }
  const int64_t N = offsets[nsub];
  if (N >= HBTU_MAX_PARTICLES || nsub >= INT32_MAX) {
    h->err = "subhalo properties: batch too large";
    return HBTU_ERR_TOO_LARGE;
  }
  if (cudaSetDevice(h->device) != cudaSuccess) {
    cudaGetLastError();
    h->err = "subhalo properties: cudaSetDevice failed";
    return HBTU_ERR_CUDA;
  }
  cudaStream_t st = h->stream;
  const bool host = p->location == HBTU_HOST;
  char *mem = nullptr;
  const long long launches0 = g_launches;
  try {
    // results on the host for the plan
    std::vector<hbtu_result> hres;
    const hbtu_result *R = res;
    if (!host) {
      hres.resize(nsub);
      HBTU_CUDA(cudaMemcpyAsync(hres.data(), res, sizeof(hbtu_result) * nsub,
                                cudaMemcpyDeviceToHost, st));
      HBTU_CUDA(cudaStreamSynchronize(st));
      R = hres.data();
    }
    // host plan: bound ranges, centres, shape chunks
    std::vector<PropSeg> seg(nsub);
    std::vector<int64_t> boff(nsub + 1);
    std::vector<int> chunk_seg;
    int64_t T = 0;
    int nch = 0;
    for (int64_t s = 0; s < nsub; s++) {
      PropSeg &g = seg[s];
      g.off = offsets[s];
      const int64_t n = offsets[s + 1] - offsets[s];
      g.n = n;
      g.nb = R[s].nbound > 1 ? std::min<int64_t>(R[s].nbound, n) : 0;
      g.boff = T;
      boff[s] = T;
      T += g.nb;
      for (int j = 0; j < 3; j++) g.cen[j] = R[s].mostbound_pos[j];
      g.mbound = R[s].mbound;
      g.chunk0 = nch;
      g.nchunk = g.nb > 1 ? (int)((g.nb - 1 + kPChunk - 1) / kPChunk) : 0;
      for (int c = 0; c < g.nchunk; c++) chunk_seg.push_back((int)s);
      nch += g.nchunk;
    }
    boff[nsub] = T;
    const DevParams P = h->dp;
    const float velocity_unit = P.G / P.a;  // PhysicalConst::G / ScaleFactor (subhalo.cpp:282)
    // Snapshot_t::SphericalOverdensitySize with virialF_c200 = 200 (snapshot.cpp:259-281)
    const float rho_vir = (float)((double)(200.f * P.Hz * P.Hz) / 2.0 / (double)P.G *
                                  (double)P.a * (double)P.a * (double)P.a);
    // device buffers, one allocation
    const size_t nT = (size_t)std::max<int64_t>(T, 1), nC = (size_t)std::max(nch, 1);
    const size_t total =
        a256(sizeof(PropSeg) * nsub) + a256(8 * (nsub + 1)) +
        (host ? a256(12 * N) + a256(4 * N) + a256(8 * N) : 0) + 2 * a256(8 * nT) +
        4 * a256(4 * nT) + a256(4 * sort_status_words(T)) + 2 * a256(4 * 16 * 256) + 256 +
        2 * a256(8 * (nT + 1)) + 3 * a256(4 * nT) + 2 * a256(8 * nsub) + a256(8 * nsub) +
        a256(8 * 12 * nC) + a256(4 * nC) + 2 * a256(4 * nsub) + a256(sizeof(hbtu_props) * nsub) +
        a256(scan_tmp_bytes(T + 1)) + 256;
    // the handle's workspace (the unbinding's buffers are larger, so it is
    // normally in place already)
    const hbtu_status ws = grow_workspace(h, total);
    if (ws != HBTU_OK) return ws;
    mem = h->ws;
    size_t o = 0;
    auto take = [&](size_t bytes) {
      char *q = mem + o;
      o += a256(bytes);
      return q;
    };
    PropSeg *d_seg = (PropSeg *)take(sizeof(PropSeg) * nsub);
    int64_t *d_boff = (int64_t *)take(8 * (nsub + 1));
    const float *d_pos = p->pos, *d_mass = p->mass;
    const int64_t *d_ord = order;
    if (host) {
      float *tp = (float *)take(12 * N), *tm = (float *)take(4 * N);
      int64_t *to = (int64_t *)take(8 * N);
      HBTU_CUDA(cudaMemcpyAsync(tp, p->pos, 12 * N, cudaMemcpyHostToDevice, st));
      HBTU_CUDA(cudaMemcpyAsync(tm, p->mass, 4 * N, cudaMemcpyHostToDevice, st));
      HBTU_CUDA(cudaMemcpyAsync(to, order, 8 * N, cudaMemcpyHostToDevice, st));
      d_pos = tp;
      d_mass = tm;
      d_ord = to;
    }
    SortBuffers sb;
    sb.lo_a = (unsigned long long *)take(8 * nT);
    sb.lo_b = (unsigned long long *)take(8 * nT);
    sb.hi_a = (unsigned *)take(4 * nT);
    sb.hi_b = (unsigned *)take(4 * nT);
    sb.val_a = (int *)take(4 * nT);
    sb.val_b = (int *)take(4 * nT);
    sb.os_status = (unsigned *)take(4 * sort_status_words(T));
    sb.os_ghist = (unsigned *)take(4 * 16 * 256);
    sb.os_goff = (unsigned *)take(4 * 16 * 256);
    int *d_flags = (int *)take(4 * F_WORDS);
    sb.error = d_flags + F_SORT;
    long long *d_mfix = (long long *)take(8 * (nT + 1));
    long long *d_cum = (long long *)take(8 * (nT + 1));
    float *d_rc = (float *)take(4 * nT), *d_mc = (float *)take(4 * nT);
    float *d_ms = (float *)take(4 * nT);
    unsigned long long *d_vmax = (unsigned long long *)take(8 * nsub);
    long long *d_so = (long long *)take(8 * nsub);
    float *d_quant = (float *)take(8 * nsub);
    double *d_csum = (double *)take(8 * 12 * nC);
    int *d_cseg = (int *)take(4 * nC);
    float *d_last = last_max_vmax ? (float *)take(4 * nsub) : nullptr;
    int *d_lsnap = last_snap ? (int *)take(4 * nsub) : nullptr;
    hbtu_props *d_out = (hbtu_props *)take(sizeof(hbtu_props) * nsub);
    void *d_scan = take(scan_tmp_bytes(T + 1));
    HBTU_CUDA(cudaMemcpyAsync(d_seg, seg.data(), sizeof(PropSeg) * nsub, cudaMemcpyHostToDevice,
                              st));
    HBTU_CUDA(cudaMemcpyAsync(d_boff, boff.data(), 8 * (nsub + 1), cudaMemcpyHostToDevice, st));
    if (nch)
      HBTU_CUDA(cudaMemcpyAsync(d_cseg, chunk_seg.data(), 4 * nch, cudaMemcpyHostToDevice, st));
    if (d_last)
      HBTU_CUDA(cudaMemcpyAsync(d_last, last_max_vmax, 4 * nsub, cudaMemcpyHostToDevice, st));
    if (d_lsnap)
      HBTU_CUDA(cudaMemcpyAsync(d_lsnap, last_snap, 4 * nsub, cudaMemcpyHostToDevice, st));
    const int init_flags[F_WORDS] = {0, 0x7fffffff, -0x7fffffff, 0, 0};
    HBTU_CUDA(cudaMemcpyAsync(d_flags, init_flags, sizeof(init_flags), cudaMemcpyHostToDevice, st));
    HBTU_CUDA(cudaMemsetAsync(d_vmax, 0, 8 * nsub, st));
    HBTU_CUDA(cudaMemsetAsync(d_so, 0xff, 8 * nsub, st));  // -1: no radius qualifies
    HBTU_CUDA(cudaMemsetAsync(d_quant, 0, 8 * nsub, st));
    if (T > 0) {
      launch_k(k_pr_elem, pblk(T), kPB, 0, st, d_seg, d_boff, (int)nsub, T, d_pos, d_mass, d_ord,
               sb.lo_a, sb.hi_a, sb.val_a, d_flags, P);
      HBTU_LAUNCHED();
      // stable LSD passes: the distance's 32 bits, then the subhalo index
      int words[16], shifts[16], np = 0;
      for (int b = 0; b < 32; b += 8) {
        words[np] = 0;
        shifts[np++] = b;
      }
      for (int b = 0; b < 32 && (1ll << b) < nsub; b += 8) {
        words[np] = 1;
        shifts[np++] = b;
      }
      radix_sort(sb, T, words, shifts, np, st);
      launch_k(k_pr_fix, pblk(T + 1), kPB, 0, st, d_seg, d_boff, (int)nsub, T, sb.val_a, d_mass,
               d_ord, d_flags, d_ms, d_mfix);
      HBTU_LAUNCHED();
      exclusive_scan_i64(d_mfix, d_cum, T + 1, d_scan, st);
      launch_k(k_pr_seq, (unsigned)((nsub + 127) / 128), 128, 0, st, d_seg, (int)nsub, T, d_ms,
               d_flags, d_cum, d_mc);
      HBTU_LAUNCHED();
      launch_k(k_pr_prof, pblk(T), kPB, 0, st, d_seg, d_boff, (int)nsub, T, sb.lo_a, d_mfix, d_cum,
               d_flags, P.eps, rho_vir, d_rc, d_mc, d_vmax, d_so, d_quant);
      HBTU_LAUNCHED();
    }
    if (nch) {
      launch_k(k_pr_shape, (unsigned)((32 * (int64_t)nch + kPB - 1) / kPB), kPB, 0, st, d_seg,
               d_cseg, nch, d_pos, d_mass, d_ord, d_csum, P);
      HBTU_LAUNCHED();
    }
    launch_k(k_pr_final, (unsigned)((32 * nsub + 127) / 128), 128, 0, st, d_seg, (int)nsub, d_csum,
             d_rc, d_mc, d_vmax, d_so, d_quant, d_last, d_lsnap, snapshot_index, velocity_unit,
             d_out);
    HBTU_LAUNCHED();
    std::vector<long long> hso(nsub);
    int hflags[F_WORDS];
    HBTU_CUDA(cudaMemcpyAsync(out, d_out, sizeof(hbtu_props) * nsub, cudaMemcpyDeviceToHost, st));
    HBTU_CUDA(cudaMemcpyAsync(hso.data(), d_so, 8 * nsub, cudaMemcpyDeviceToHost, st));
    HBTU_CUDA(cudaMemcpyAsync(hflags, d_flags, sizeof(hflags), cudaMemcpyDeviceToHost, st));
    HBTU_CUDA(cudaStreamSynchronize(st));
    h->stats.kernel_launches += g_launches - launches0;
    if (hflags[F_SORT]) {
      h->err = "subhalo properties: radix sort look-back wait ran out";
      return HBTU_ERR_CUDA;
    }
    if (hflags[F_ORDER]) {
      h->err = "subhalo properties: an order entry lies outside its subhalo";
      return HBTU_ERR_INVALID_ARGUMENT;
    }
    // BoundR200CritComoving = pow(M200Crit / RhoVirial, 1/3) in double (snapshot.cpp:277)
    for (int64_t s = 0; s < nsub; s++)
      if (seg[s].nb > 1 && hso[s] >= 0)
        out[s].r200crit_comoving = (float)std::pow((double)(out[s].m200crit / rho_vir), 1.0 / 3);
    return HBTU_OK;
  } catch (const CudaError &e) {
    h->err = e.what;
    return HBTU_ERR_CUDA;
  }
}
