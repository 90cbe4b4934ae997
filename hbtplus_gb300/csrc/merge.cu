// merge.cu -- trap detection of the merging step, for every subhalo at once.
//
// Reference: SubhaloSnapshot_t::MergeSubhalos (src/subhalo_merge.cpp:187-220)
// starts with FillCores and DetectTraps (:30-180):
//   core of a subhalo: mean position (around its first particle when the box
//     is periodic) and mean velocity of its first min(Nbound, 20) particles,
//     with the dispersions, summed in double in particle order (SubHelper_t::
//     BuildPosition / BuildVelocity);
//   trap: a subhalo not trapped yet walks up its chain of hosts; the first
//     host with Nbound > 1 whose core lies within DeltaCrit = 2 of the
//     subhalo's most-bound particle in the phase-space distance
//     |x - x_core| / sigma_r + |v - v_core| / sigma_v (SinkDistance, float)
//     becomes its sink, and a host that swallows a subhalo with Nbound > 1 is
//     marked for re-unbinding.
// One thread per subhalo for each: the cores read 20 particles, the chains
// are a few hosts deep.  The double sums keep the reference's order and are
// spelled with round-to-nearest intrinsics, so the cores are bit-exact; a
// host chain longer than the number of subhaloes (a cycle, which would make
// the reference loop forever) is reported instead of followed.
#include <algorithm>
#include <string>
#include <vector>

#include "device_common.cuh"
#include "handle.h"

namespace hbtu {
namespace {

constexpr int kCoreParticles = 20;  // NumPartCoreMax, subhalo_merge.cpp:11
constexpr float kDeltaCrit = 2.f;   // DeltaCrit, :12

struct MergeSeg {
  int64_t off, n, nbound, host;
};

// The mean and dispersion of x (positions: around origin when periodic) of
// the first np particles, as BuildPosition / BuildVelocity form them.
__device__ void core_moments(const float *x, const float *mass, int64_t np, bool wrap,
                             const double origin[3], const DevParams &P, float mean[3],
                             float *sigma)
{
  double s1[3] = {0., 0., 0.}, s2[3] = {0., 0., 0.}, msum = 0.;
  for (int64_t i = 0; i < np; i++) {
    const double m = f2d(mass[i]);
    msum = dadd(msum, m);
    for (int j = 0; j < 3; j++) {
      double d = f2d(x[3 * i + j]);
      if (wrap) d = nearest_d(dsub(d, origin[j]), P);
      s1[j] = dadd(s1[j], dmul(d, m));
      s2[j] = dadd(s2[j], dmul(dmul(d, d), m));
    }
  }
  for (int j = 0; j < 3; j++) {
    s1[j] = ddiv(s1[j], msum);
    s2[j] = ddiv(s2[j], msum);
    mean[j] = d2f(s1[j]);
    if (wrap) mean[j] = d2f(dadd(f2d(mean[j]), origin[j]));
    s2[j] = dsub(s2[j], dmul(s1[j], s1[j]));
  }
  *sigma = d2f(__dsqrt_rn(dadd(dadd(s2[0], s2[1]), s2[2])));
}

__global__ void k_cores(const MergeSeg *seg, int64_t S, const float *pos, const float *vel,
                        const float *mass, hbtu_core *cores, DevParams P)
{
  HBTU_KERNEL_PROLOGUE();
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= S) return;
  const MergeSeg g = seg[s];
  hbtu_core c;
  for (int j = 0; j < 3; j++) c.pos[j] = c.vel[j] = 0.f;
  c.sigma_r = c.sigma_v = 0.f;
  const int64_t nb = min(g.nbound, g.n);
  const float *x = pos + 3 * g.off, *v = vel + 3 * g.off, *m = mass + g.off;
  if (nb == 1) {  // subhalo_merge.cpp:37-42, :88-93
    for (int j = 0; j < 3; j++) {
      c.pos[j] = x[j];
      c.vel[j] = v[j];
    }
  } else if (nb > 1) {
    const int64_t np = min(nb, (int64_t)kCoreParticles);
    double origin[3] = {0., 0., 0.};
    if (P.periodic)
      for (int j = 0; j < 3; j++) origin[j] = f2d(x[j]);
    core_moments(x, m, np, P.periodic != 0, origin, P, c.pos, &c.sigma_r);
    core_moments(v, m, np, false, origin, P, c.vel, &c.sigma_v);
  }
  cores[s] = c;
}

// SinkDistance (subhalo_merge.cpp:128-133): PeriodicDistance
// (config_parser.h:143-156) and Distance (mymath.h:184-187) in float.
__device__ __forceinline__ float sink_distance(const float mbp[3], const float mbv[3],
                                               const hbtu_core &c, const DevParams &P)
{
  float dx[3], dv[3];
  for (int j = 0; j < 3; j++) {
    dx[j] = fsub(c.pos[j], mbp[j]);
    if (P.periodic) dx[j] = nearest_f(dx[j], P);
    dv[j] = fsub(c.vel[j], mbv[j]);
  }
  const float r = __fsqrt_rn(fadd(fadd(fmul(dx[0], dx[0]), fmul(dx[1], dx[1])), fmul(dx[2], dx[2])));
  const float v = __fsqrt_rn(fadd(fadd(fmul(dv[0], dv[0]), fmul(dv[1], dv[1])), fmul(dv[2], dv[2])));
  return fadd(__fdiv_rn(r, c.sigma_r), __fdiv_rn(v, c.sigma_v));
}

__global__ void k_traps(const MergeSeg *seg, int64_t S, const hbtu_core *cores,
                        const float *mb_pos, const float *mb_vel, int isnap, long long *sink,
                        int *sink_snap, int *merged, int *error, DevParams P)
{
  HBTU_KERNEL_PROLOGUE();
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= S || sink[s] >= 0) return;  // IsTrapped already
  const float mbp[3] = {mb_pos[3 * s], mb_pos[3 * s + 1], mb_pos[3 * s + 2]};
  const float mbv[3] = {mb_vel[3 * s], mb_vel[3 * s + 1], mb_vel[3 * s + 2]};
  int64_t h = seg[s].host, steps = 0;
  while (h >= 0 && h < S) {
    if (++steps > S) {  // a cycle in the host chain
      atomicOr(error, 1);
      return;
    }
    if (seg[h].nbound > 1 && sink_distance(mbp, mbv, cores[h], P) < kDeltaCrit) {
      sink[s] = h;
      sink_snap[s] = isnap;
      if (seg[s].nbound > 1) merged[h] = 1;
      return;
    }
    h = seg[h].host;
  }
}

inline size_t a256(size_t b) { return (b + 255) / 256 * 256; }

}  // namespace
}  // namespace hbtu

using namespace hbtu;

extern "C" hbtu_status hbtu_merge_detect(hbtu_handle *h, const hbtu_particles *p, int64_t nsub,
                                         const int64_t *list_off, const int64_t *nbound,
                                         const int64_t *host, const float *mostbound_pos,
                                         const float *mostbound_vel, int32_t snapshot_index,
                                         int64_t *sink, int32_t *sink_snap, int32_t *merged,
                                         hbtu_core *cores)
{
  if (!h) return HBTU_ERR_INVALID_ARGUMENT;
  if (nsub < 0 || (nsub > 0 && (!p || !p->pos || !p->vel || !p->mass || !list_off || !nbound ||
                                !host || !mostbound_pos || !mostbound_vel || !sink ||
                                !sink_snap || !merged))) {
    h->err = "merge detect: null argument";
    return HBTU_ERR_INVALID_ARGUMENT;
  }
  if (nsub == 0) return HBTU_OK;
  if (list_off[0] != 0) {
    h->err = "merge detect: list offsets must start at 0";
    return HBTU_ERR_INVALID_ARGUMENT;
  }
  std::vector<MergeSeg> seg(nsub);
  for (int64_t s = 0; s < nsub; s++) {
    if (list_off[s + 1] < list_off[s] || host[s] >= nsub) {
      h->err = "merge detect: decreasing list offsets or a host index out of range";
      return HBTU_ERR_INVALID_ARGUMENT;
    }
    seg[s] = MergeSeg{list_off[s], list_off[s + 1] - list_off[s], nbound[s], host[s]};
  }
  const int64_t N = list_off[nsub];
  if (N >= HBTU_MAX_PARTICLES) {
    h->err = "merge detect: too many particles";
    return HBTU_ERR_TOO_LARGE;
  }
  if (cudaSetDevice(h->device) != cudaSuccess) {
    cudaGetLastError();
    h->err = "merge detect: cudaSetDevice failed";
    return HBTU_ERR_CUDA;
  }
  cudaStream_t st = h->stream;
  const bool hostmem = p->location == HBTU_HOST;
  const size_t total = a256(sizeof(MergeSeg) * nsub) + a256(sizeof(hbtu_core) * nsub) +
                       2 * a256(12 * nsub) + a256(8 * nsub) + 2 * a256(4 * nsub) + 256 +
                       (hostmem ? 2 * a256(12 * N) + a256(4 * N) : 0);
  const hbtu_status ws = grow_workspace(h, total);
  if (ws != HBTU_OK) return ws;
  char *mem = h->ws;
  size_t o = 0;
  auto take = [&](size_t bytes) {
    char *q = mem + o;
    o += a256(bytes);
    return q;
  };
  const long long launches0 = g_launches;
  try {
    MergeSeg *d_seg = (MergeSeg *)take(sizeof(MergeSeg) * nsub);
    hbtu_core *d_core = (hbtu_core *)take(sizeof(hbtu_core) * nsub);
    float *d_mbp = (float *)take(12 * nsub), *d_mbv = (float *)take(12 * nsub);
    long long *d_sink = (long long *)take(8 * nsub);
    int *d_snap = (int *)take(4 * nsub), *d_merged = (int *)take(4 * nsub);
    int *d_err = (int *)take(4);
    const float *d_pos = p->pos, *d_vel = p->vel, *d_mass = p->mass;
    if (hostmem) {
      float *tp = (float *)take(12 * N), *tv = (float *)take(12 * N), *tm = (float *)take(4 * N);
      HBTU_CUDA(cudaMemcpyAsync(tp, p->pos, 12 * N, cudaMemcpyHostToDevice, st));
      HBTU_CUDA(cudaMemcpyAsync(tv, p->vel, 12 * N, cudaMemcpyHostToDevice, st));
      HBTU_CUDA(cudaMemcpyAsync(tm, p->mass, 4 * N, cudaMemcpyHostToDevice, st));
      d_pos = tp;
      d_vel = tv;
      d_mass = tm;
    }
    HBTU_CUDA(cudaMemcpyAsync(d_seg, seg.data(), sizeof(MergeSeg) * nsub, cudaMemcpyHostToDevice,
                              st));
    HBTU_CUDA(cudaMemcpyAsync(d_mbp, mostbound_pos, 12 * nsub, cudaMemcpyHostToDevice, st));
    HBTU_CUDA(cudaMemcpyAsync(d_mbv, mostbound_vel, 12 * nsub, cudaMemcpyHostToDevice, st));
    HBTU_CUDA(cudaMemcpyAsync(d_sink, sink, 8 * nsub, cudaMemcpyHostToDevice, st));
    HBTU_CUDA(cudaMemcpyAsync(d_snap, sink_snap, 4 * nsub, cudaMemcpyHostToDevice, st));
    HBTU_CUDA(cudaMemsetAsync(d_merged, 0, 4 * nsub, st));
    HBTU_CUDA(cudaMemsetAsync(d_err, 0, 4, st));
    const unsigned blocks = (unsigned)((nsub + 127) / 128);
    launch_k(k_cores, blocks, 128, 0, st, d_seg, nsub, d_pos, d_vel, d_mass, d_core, h->dp);
    HBTU_LAUNCHED();
    launch_k(k_traps, blocks, 128, 0, st, d_seg, nsub, d_core, d_mbp, d_mbv, snapshot_index, d_sink,
             d_snap, d_merged, d_err, h->dp);
    HBTU_LAUNCHED();
    int err = 0;
    HBTU_CUDA(cudaMemcpyAsync(sink, d_sink, 8 * nsub, cudaMemcpyDeviceToHost, st));
    HBTU_CUDA(cudaMemcpyAsync(sink_snap, d_snap, 4 * nsub, cudaMemcpyDeviceToHost, st));
    HBTU_CUDA(cudaMemcpyAsync(merged, d_merged, 4 * nsub, cudaMemcpyDeviceToHost, st));
    if (cores)
      HBTU_CUDA(cudaMemcpyAsync(cores, d_core, sizeof(hbtu_core) * nsub, cudaMemcpyDeviceToHost,
                                st));
    HBTU_CUDA(cudaMemcpyAsync(&err, d_err, 4, cudaMemcpyDeviceToHost, st));
    HBTU_CUDA(cudaStreamSynchronize(st));
    h->stats.kernel_launches += g_launches - launches0;
    if (err) {
      h->err = "merge detect: a host chain has a cycle";
      return HBTU_ERR_INVALID_ARGUMENT;
    }
    return HBTU_OK;
  } catch (const CudaError &e) {
    h->err = e.what;
    return HBTU_ERR_CUDA;
  }
}
