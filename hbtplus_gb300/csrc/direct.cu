// direct.cu -- exact pairwise potentials in FP64 (validation utility).
//
// phi(x_t) = G/a * sum_{j != t} m_j K(|NEAREST(x_j - x_t)|) with the reference's
// cubic-spline softening K (src/gravity_tree.cpp:144-160: -1/r beyond h = 2.8 eps,
// wp(u)/h inside, written here with the exact fractions that the reference
// rounds to 12 digits), over every particle of one set, for a chosen list of
// targets.  The self term is excluded, as the tree walk's targetMass/eps
// correction does (src/gravity_tree.cpp:98).  It is the accuracy check of the tree walk on sets too large for a
// CPU direct sum (e.g. a 1e4-particle subsample of a 2e7-particle host: 2e11
// pairs).  Targets in tiles of 128 threads, sources split across the grid's
// second dimension and staged through shared memory; the splits' partial sums
// are added in a fixed order.
#include "device_common.cuh"

namespace hbtu {
namespace {

constexpr int kDT = 128;
constexpr int kSrcTile = 256;

__global__ void __launch_bounds__(kDT) k_direct_fp64(const float4 *pm, int n, const int *tidx,
                                                     int nt, int nsplit, double *partial,
                                                     DevParams P)
{
  HBTU_KERNEL_PROLOGUE();
  __shared__ float4 src[kSrcTile];
  const int t = blockIdx.x * kDT + threadIdx.x;
  const int split = blockIdx.y;
  const int per = (n + nsplit - 1) / nsplit;
  const int j0 = split * per, j1 = min(n, j0 + per);
  const int me = t < nt ? tidx[t] : -1;
  double tx = 0., ty = 0., tz = 0.;
  if (me >= 0) {
    const float4 a = pm[me];
    tx = a.x;
    ty = a.y;
    tz = a.z;
  }
  double pot = 0.;
  for (int base = j0; base < j1; base += kSrcTile) {
    __syncthreads();
    for (int k = threadIdx.x; k < kSrcTile; k += kDT)
      src[k] = base + k < j1 ? pm[base + k] : make_float4(0.f, 0.f, 0.f, 0.f);
    __syncthreads();
    const int m = min(kSrcTile, j1 - base);
    if (me < 0) continue;
    for (int k = 0; k < m; k++) {
      if (base + k == me) continue;
      const float4 s = src[k];
      double dx = (double)s.x - tx, dy = (double)s.y - ty, dz = (double)s.z - tz;
      if (P.periodic) {
        dx = nearest_d(dx, P);
        dy = nearest_d(dy, P);
        dz = nearest_d(dz, P);
      }
      const double r = sqrt(dx * dx + dy * dy + dz * dz);
      if (r >= P.h) {
        pot -= (double)s.w / r;
      } else {
        const double u = r * P.h_inv;
        const double wp = u < 0.5 ? -2.8 + u * u * (16.0 / 3.0 + u * u * (6.4 * u - 9.6))
                                  : -3.2 + 1.0 / (15.0 * u) +
                                        u * u * (32.0 / 3.0 + u * (-16.0 + u * (9.6 - 32.0 / 15.0 * u)));
        pot += (double)s.w * P.h_inv * wp;
      }
    }
  }
  if (t < nt) partial[(size_t)split * nt + t] = pot;
}

__global__ void k_direct_reduce(const double *partial, int nt, int nsplit, double *out,
                                DevParams P)
{
  HBTU_KERNEL_PROLOGUE();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  double s = 0.;
  for (int k = 0; k < nsplit; k++) s += partial[(size_t)k * nt + t];
  out[t] = s * (double)P.G / (double)P.a;
}

}  // namespace

void direct_potential_fp64(const DevParams &P, const float4 *pm, int n, const int *tidx, int nt,
                           double *out, double *partial, int nsplit, cudaStream_t st)
{
  if (nt <= 0) return;
  dim3 grid((nt + kDT - 1) / kDT, nsplit);
  launch_k(k_direct_fp64, grid, kDT, 0, st, pm, n, tidx, nt, nsplit, partial, P);
  HBTU_LAUNCHED();
  launch_k(k_direct_reduce, (nt + 255) / 256, 256, 0, st, partial, nt, nsplit, out, P);
  HBTU_LAUNCHED();
}

}  // namespace hbtu
