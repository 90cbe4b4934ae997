// prims.cu -- device-wide scan and stable LSD radix sort used by the tree
// build (Morton-key sort) and by the energy-ordering sorts of the unbinding
// loop (src/subhalo_unbind.cpp:382, :405).  Both are HBM-bound integer work:
// one read and one write of each record per pass, tiles of 2048 records per
// 256-thread block.
#include "hbtu_internal.h"

#include <cstdio>
#include <utility>

namespace hbtu {

thread_local long long g_launches = 0;

CudaError::CudaError(cudaError_t e, const char *expr, const char *file, int line) : err(e)
{
  char buf[512];
  snprintf(buf, sizeof(buf), "%s failed: %s (%s:%d)", expr, cudaGetErrorString(e), file, line);
  what = buf;
}

namespace {
constexpr int kBlock = 256;
constexpr int kItems = 8;
constexpr int kTile = kBlock * kItems;

__device__ __forceinline__ long long block_exclusive_sum(long long v, long long *total)
{
  __shared__ long long warp_sums[kBlock / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  long long x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    long long w = lane < kBlock / 32 ? warp_sums[lane] : 0;
#pragma unroll
    for (int o = 1; o < kBlock / 32; o <<= 1) {
      long long y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < kBlock / 32) warp_sums[lane] = w;
  }
  __syncthreads();
  long long pre = (warp > 0 ? warp_sums[warp - 1] : 0) + x - v;
  if (total) *total = warp_sums[kBlock / 32 - 1];
  __syncthreads();
  return pre;
}

__global__ void __launch_bounds__(kBlock) k_scan_reduce(const long long *in, long long n,
                                                        long long *sums)
{
  const long long base = (long long)blockIdx.x * kTile + (long long)threadIdx.x * kItems;
  long long s = 0;
#pragma unroll
  for (int k = 0; k < kItems; k++)
    if (base + k < n) s += in[base + k];
  long long total;
  block_exclusive_sum(s, &total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kBlock) k_scan_apply(const long long *in, long long *out,
                                                       long long n, const long long *offs)
{
  const long long base = (long long)blockIdx.x * kTile + (long long)threadIdx.x * kItems;
  long long v[kItems], s = 0;
#pragma unroll
  for (int k = 0; k < kItems; k++) {
    v[k] = (base + k < n) ? in[base + k] : 0;
    s += v[k];
  }
  long long pre = block_exclusive_sum(s, nullptr) + (offs ? offs[blockIdx.x] : 0);
#pragma unroll
  for (int k = 0; k < kItems; k++) {
    if (base + k < n) out[base + k] = pre;
    pre += v[k];
  }
}

__device__ __forceinline__ unsigned rs_digit(unsigned hi, unsigned long long lo, int word,
                                             int shift)
{
  return word ? (hi >> shift) & 255u : (unsigned)(lo >> shift) & 255u;
}

__global__ void __launch_bounds__(kBlock) k_rs_hist(const unsigned *hi,
                                                    const unsigned long long *lo, long long n,
                                                    int word, int shift, long long *counts,
                                                    int nblocks)
{
  __shared__ unsigned hist[256];
  hist[threadIdx.x] = 0;
  __syncthreads();
  const long long tile = (long long)blockIdx.x * kTile;
#pragma unroll
  for (int r = 0; r < kItems; r++) {
    long long e = tile + r * kBlock + threadIdx.x;
    if (e < n) atomicAdd(&hist[rs_digit(word ? hi[e] : 0u, word ? 0ull : lo[e], word, shift)], 1u);
  }
  __syncthreads();
  counts[(long long)threadIdx.x * nblocks + blockIdx.x] = hist[threadIdx.x];
}

__global__ void __launch_bounds__(kBlock) k_rs_scatter(
    const unsigned *hi_in, const unsigned long long *lo_in, const int *val_in, unsigned *hi_out,
    unsigned long long *lo_out, int *val_out, long long n, int word, int shift,
    const long long *offsets, int nblocks)
{
  __shared__ unsigned wcnt[kBlock / 32][256];
  __shared__ unsigned run_base[256];
  __shared__ long long goff[256];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  goff[tid] = offsets[(long long)tid * nblocks + blockIdx.x];
  run_base[tid] = 0;
#pragma unroll
  for (int w = 0; w < kBlock / 32; w++) wcnt[w][tid] = 0;
  __syncthreads();
  const unsigned lt = (1u << lane) - 1u;
  const long long tile = (long long)blockIdx.x * kTile;
  for (int r = 0; r < kItems; r++) {
    const long long e = tile + r * kBlock + tid;
    const bool valid = e < n;
    unsigned h = 0, d = 256u + lane;  // unique sentinel for invalid lanes
    unsigned long long l = 0;
    int v = 0;
    if (valid) {
      h = hi_in[e];
      l = lo_in[e];
      v = val_in[e];
      d = rs_digit(h, l, word, shift);
    }
    const unsigned mask = __match_any_sync(0xffffffffu, d);
    const unsigned rank = __popc(mask & lt);
    if (valid && rank == 0) wcnt[warp][d] = __popc(mask);
    __syncthreads();
    {
      unsigned run = run_base[tid];
#pragma unroll
      for (int w = 0; w < kBlock / 32; w++) {
        unsigned t = wcnt[w][tid];
        wcnt[w][tid] = run;
        run += t;
      }
      run_base[tid] = run;
    }
    __syncthreads();
    if (valid) {
      const long long dst = goff[d] + wcnt[warp][d] + rank;
      hi_out[dst] = h;
      lo_out[dst] = l;
      val_out[dst] = v;
    }
    __syncthreads();
#pragma unroll
    for (int w = 0; w < kBlock / 32; w++) wcnt[w][tid] = 0;
    __syncthreads();
  }
}

}  // namespace

size_t scan_tmp_bytes(long long n)
{
  size_t bytes = 0;
  while (n > kTile) {
    n = (n + kTile - 1) / kTile;
    bytes += (size_t)n * sizeof(long long) + 256;
  }
  return bytes + 256;
}

void exclusive_scan_i64(const long long *in, long long *out, long long n, void *tmp,
                        cudaStream_t st)
{
  if (n <= 0) return;
  const long long nb = (n + kTile - 1) / kTile;
  if (nb == 1) {
    k_scan_apply<<<1, kBlock, 0, st>>>(in, out, n, nullptr);
    HBTU_LAUNCHED();
    return;
  }
  long long *sums = (long long *)tmp;
  char *rest = (char *)tmp + (((size_t)nb * sizeof(long long) + 255) / 256) * 256;
  k_scan_reduce<<<(unsigned)nb, kBlock, 0, st>>>(in, n, sums);
  HBTU_LAUNCHED();
  exclusive_scan_i64(sums, sums, nb, rest, st);
  k_scan_apply<<<(unsigned)nb, kBlock, 0, st>>>(in, out, n, sums);
  HBTU_LAUNCHED();
}

size_t sort_count_entries(long long n)
{
  long long nb = (n + kTile - 1) / kTile;
  if (nb < 1) nb = 1;
  return (size_t)nb * 256;
}

void radix_sort(SortBuffers &b, long long n, const int *words, const int *shifts, int npasses,
                cudaStream_t st)
{
  if (n <= 1 || npasses <= 0) return;
  const int nblocks = (int)((n + kTile - 1) / kTile);
  const long long ncount = (long long)nblocks * 256;
  for (int p = 0; p < npasses; p++) {
    k_rs_hist<<<nblocks, kBlock, 0, st>>>(b.hi_a, b.lo_a, n, words[p], shifts[p], b.counts64,
                                           nblocks);
    HBTU_LAUNCHED();
    exclusive_scan_i64(b.counts64, b.counts64, ncount, b.scan_tmp, st);
    k_rs_scatter<<<nblocks, kBlock, 0, st>>>(b.hi_a, b.lo_a, b.val_a, b.hi_b, b.lo_b, b.val_b, n,
                                              words[p], shifts[p], b.counts64, nblocks);
    HBTU_LAUNCHED();
    std::swap(b.hi_a, b.hi_b);
    std::swap(b.lo_a, b.lo_b);
    std::swap(b.val_a, b.val_b);
  }
}

}  // namespace hbtu
