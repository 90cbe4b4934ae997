// prims.cu -- device-wide scan and stable LSD radix sort used by the tree
// build (Morton-key sort) and by the energy-ordering sorts of the unbinding
// loop (src/subhalo_unbind.cpp:382, :405).  Both are HBM-bound integer work:
// one read and one write of each record per pass, tiles of 2048 records per
// 256-thread block; up to 4096 records sort in one block in shared memory.
#include "hbtu_internal.h"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <utility>

namespace hbtu {

thread_local long long g_launches = 0;

bool launch_overlap()
{
  static const bool on = [] {
    const char *v = getenv("HBTU_LAUNCH_OVERLAP");
    return !(v && strcmp(v, "0") == 0);
  }();
  return on;
}

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
  HBTU_KERNEL_PROLOGUE();
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
  HBTU_KERNEL_PROLOGUE();
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

// Stable ranking of a block's records by digit, each warp owning a run of
// consecutive records (round r of warp w holds its records r*32 .. r*32+31):
// within a round __match_any_sync groups the lanes of one digit, and a
// per-warp count per digit carries the rank across rounds, so the records of
// a warp are ranked without block barriers.  rk[r] is the record's rank among
// the warp's records of its digit; wcnt[w][d] ends as the warp's count of d.
// Lanes without a record pass a unique sentinel digit (256 + lane).
template <int kRounds>
__device__ __forceinline__ void warp_rank(const unsigned (&dg)[kRounds], unsigned (&rk)[kRounds],
                                          unsigned (*wcnt)[256])
{
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
#pragma unroll
  for (int r = 0; r < kRounds; r++) {
    const unsigned d = dg[r];
    const unsigned mask = __match_any_sync(0xffffffffu, d);
    const unsigned before = __popc(mask & lt);
    const bool real = d < 256u;
    const unsigned base = real ? wcnt[warp][d] : 0u;
    __syncwarp();
    if (real && before == 0) wcnt[warp][d] = base + __popc(mask);
    __syncwarp();
    rk[r] = base + before;
  }
}

// After warp_rank: the warps' counts become the warps' offsets within each
// digit (wcnt[w][d] = records of digit d in warps before w), and the return
// value is the block's count of digit threadIdx.x (kBlock == 256 threads,
// one digit each).
__device__ __forceinline__ unsigned warp_offsets(unsigned (*wcnt)[256])
{
  const int t = threadIdx.x;
  unsigned run = 0;
#pragma unroll
  for (int w = 0; w < kBlock / 32; w++) {
    const unsigned c = wcnt[w][t];
    wcnt[w][t] = run;
    run += c;
  }
  return run;
}

// Exclusive scan over the block of one value per thread (kBlock threads).
__device__ __forceinline__ unsigned block_excl_scan_u32(unsigned v, unsigned *wsum)
{
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[warp] = x;
  __syncthreads();
  unsigned before = 0;
  for (int w = 0; w < warp; w++) before += wsum[w];
  __syncthreads();
  return before + x - v;
}

// Sorts of at most kSmallN records go by rank counting, over many blocks
// (one launch, instead of a kernel per digit): a record's composite key
// packs its digits with the last digit most significant (the order the LSD
// passes produce), and its place is the number of records with a smaller key,
// or an equal key and a smaller index (so the sort is stable).  Each block
// holds every record's key in shared memory; kRankSplit threads share one
// record's count.
constexpr int kSmallN = 2 * kTile;  // 4096 records
constexpr int kRankSplit = 8;

struct SmallSortPasses {
  int words[16], shifts[16], n;
};

constexpr size_t kRankSmem = (size_t)kSmallN * 2 * sizeof(unsigned long long);

__global__ void __launch_bounds__(kBlock) k_rank_small(const unsigned *hi, const unsigned long long *lo,
                                                       const int *val, unsigned *hi_o,
                                                       unsigned long long *lo_o, int *val_o, int n,
                                                       SmallSortPasses ps)
{
  HBTU_KERNEL_PROLOGUE();
  extern __shared__ __align__(16) unsigned char smem[];
  unsigned long long *const kh = (unsigned long long *)smem;  // digits 8..15
  unsigned long long *const kl = kh + kSmallN;                // digits 0..7
  for (int e = threadIdx.x; e < n; e += kBlock) {
    const unsigned h = hi[e];
    const unsigned long long l = lo[e];
    unsigned long long a = 0, b = 0;
    for (int p = 0; p < ps.n; p++) {
      const unsigned long long d = rs_digit(h, l, ps.words[p], ps.shifts[p]);
      if (p < 8)
        a |= d << (8 * p);
      else
        b |= d << (8 * (p - 8));
    }
    kl[e] = a;
    kh[e] = b;
  }
  __syncthreads();
  const int rec = blockIdx.x * (kBlock / kRankSplit) + threadIdx.x / kRankSplit;
  const int part = threadIdx.x % kRankSplit;
  unsigned cnt = 0;
  unsigned long long mh = 0, ml = 0;
  if (rec < n) {
    mh = kh[rec];
    ml = kl[rec];
    for (int j = part; j < n; j += kRankSplit) {
      const unsigned long long h = kh[j], l = kl[j];
      cnt += (h < mh) || (h == mh && (l < ml || (l == ml && j < rec)));
    }
  }
#pragma unroll
  for (int o = kRankSplit / 2; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  if (rec < n && part == 0) {
    hi_o[cnt] = hi[rec];
    lo_o[cnt] = lo[rec];
    val_o[cnt] = val[rec];
  }
}

// ---------------------------------------------------------------- onesweep
// Larger sorts: one kernel per digit (Adinets & Merrill 2022, "Onesweep").
// The global offset of every digit value is known up front (one histogram
// pass over all digits); each tile then finds how many earlier elements
// share its digit values by decoupled look-back over the tiles before it
// (tile indices come from an atomic counter, so a tile only waits on tiles
// that have started).  The tile is first sorted stably in shared memory,
// with the same ranks as above, so each digit's run is written out to
// consecutive addresses.
// Status words: bits 30-31 flag (1 = tile count, 2 = inclusive prefix),
// bits 0-29 the count.  Every wait is bounded; a wait that runs out sets
// *err and the pass continues (results are then wrong and the call fails).
constexpr unsigned kFlagAgg = 1u << 30, kFlagPre = 2u << 30, kCountMask = (1u << 30) - 1u;
constexpr int kMaxPasses = 16;
constexpr long long kSpinLimit = 1ll << 24;

struct Passes {
  int words[kMaxPasses], shifts[kMaxPasses], n;
};

// Also clears the first pass's look-back words (nstatus) and tile counter.
__global__ void __launch_bounds__(kBlock) k_os_hist(const unsigned *hi,
                                                    const unsigned long long *lo, long long n,
                                                    Passes ps, unsigned *ghist, unsigned *status,
                                                    long long nstatus, int *counter)
{
  HBTU_KERNEL_PROLOGUE();
  for (long long i = (long long)blockIdx.x * kBlock + threadIdx.x; i < nstatus;
       i += (long long)gridDim.x * kBlock)
    status[i] = 0u;
  if (blockIdx.x == 0 && threadIdx.x == 0) *counter = 0;
  __shared__ unsigned h[kMaxPasses][256];
  for (int p = 0; p < ps.n; p++) h[p][threadIdx.x] = 0;
  __syncthreads();
  for (long long e = (long long)blockIdx.x * kBlock + threadIdx.x; e < n;
       e += (long long)gridDim.x * kBlock) {
    const unsigned hv = hi[e];
    const unsigned long long lv = lo[e];
    for (int p = 0; p < ps.n; p++)
      atomicAdd(&h[p][rs_digit(hv, lv, ps.words[p], ps.shifts[p])], 1u);
  }
  __syncthreads();
  for (int p = 0; p < ps.n; p++)
    if (h[p][threadIdx.x]) atomicAdd(&ghist[p * 256 + threadIdx.x], h[p][threadIdx.x]);
}

// Exclusive scan of each digit's 256 counts (one block, thread = digit value).
__global__ void __launch_bounds__(kBlock) k_os_offsets(const unsigned *ghist, int npasses,
                                                       unsigned *goff)
{
  HBTU_KERNEL_PROLOGUE();
  __shared__ unsigned wsum[kBlock / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int p = 0; p < npasses; p++) {
    const unsigned v = ghist[p * 256 + threadIdx.x];
    unsigned x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    unsigned before = 0;
    for (int w = 0; w < warp; w++) before += wsum[w];
    goff[p * 256 + threadIdx.x] = before + x - v;
    __syncthreads();
  }
}

// status / tile_counter: this pass's look-back words and tile counter (zero
// when it starts); next_status / next_counter: the next pass's, cleared here
// (each tile its own words) so that no memset runs between passes.
__global__ void __launch_bounds__(kBlock) k_os_pass(
    const unsigned *hi_in, const unsigned long long *lo_in, const int *val_in, unsigned *hi_out,
    unsigned long long *lo_out, int *val_out, long long n, int word, int shift,
    const unsigned *goff, unsigned *status, int *tile_counter, unsigned *next_status,
    int *next_counter, int *err)
{
  HBTU_KERNEL_PROLOGUE();
  __shared__ unsigned wcnt[kBlock / 32][256];
  __shared__ unsigned toff[256];  // first slot of each digit in the tile's sorted order
  __shared__ unsigned base[256];
  __shared__ unsigned wsum[kBlock / 32];
  __shared__ unsigned long long s_lo[kTile];
  __shared__ unsigned s_hi[kTile];
  __shared__ int s_val[kTile];
  __shared__ int tile_s;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) tile_s = atomicAdd(tile_counter, 1);
#pragma unroll
  for (int w = 0; w < kBlock / 32; w++) wcnt[w][tid] = 0;
  __syncthreads();
  const int tile = tile_s;
  const long long t0 = (long long)tile * kTile;
  next_status[(long long)tile * 256 + tid] = 0u;
  if (tile == 0 && tid == 0) *next_counter = 0;
  // this tile's records: warp w holds tile positions w*256 .. w*256+255, lane-contiguous
  unsigned dg[kItems], rk[kItems], hv[kItems];
  unsigned long long lv[kItems];
  int vv[kItems];
#pragma unroll
  for (int r = 0; r < kItems; r++) {
    const long long e = t0 + warp * 32 * kItems + r * 32 + lane;
    dg[r] = 256u + lane;  // unique sentinel for lanes past the end
    hv[r] = 0;
    lv[r] = 0;
    vv[r] = 0;
    if (e < n) {
      hv[r] = hi_in[e];
      lv[r] = lo_in[e];
      vv[r] = val_in[e];
      dg[r] = rs_digit(hv[r], lv[r], word, shift);
    }
  }
  warp_rank<kItems>(dg, rk, wcnt);
  __syncthreads();
  const unsigned cnt = warp_offsets(wcnt);
  // publish this tile's counts at once, so later tiles can look back past it
  volatile unsigned *st = status;
  st[(long long)tile * 256 + tid] = (tile == 0 ? kFlagPre : kFlagAgg) | cnt;
  toff[tid] = block_excl_scan_u32(cnt, wsum);  // tile-local start of each digit
  __syncthreads();
  // stable local sort of the tile into shared memory
#pragma unroll
  for (int r = 0; r < kItems; r++) {
    if (dg[r] >= 256u) continue;
    const unsigned slot = toff[dg[r]] + wcnt[warp][dg[r]] + rk[r];
    s_hi[slot] = hv[r];
    s_lo[slot] = lv[r];
    s_val[slot] = vv[r];
  }
  __syncthreads();
  // look back for the earlier tiles' total of each digit
  unsigned prefix = 0;
  for (int k = tile - 1; k >= 0;) {
    const unsigned v = st[(long long)k * 256 + tid];
    const unsigned flag = v & ~kCountMask;
    if (flag == 0u) {
      long long spins = 0;
      unsigned w = 0;
      while ((w = st[(long long)k * 256 + tid]) == 0u && ++spins < kSpinLimit) {
      }
      if (w == 0u) {  // the earlier tile never published: give up on this pass
        atomicExch(err, 1);
        break;
      }
      continue;
    }
    prefix += v & kCountMask;
    if (flag == kFlagPre) break;
    k--;
  }
  if (tile > 0) st[(long long)tile * 256 + tid] = kFlagPre | ((prefix + cnt) & kCountMask);
  base[tid] = goff[tid] + prefix;
  __syncthreads();
  // write out in sorted order: each digit's run lands contiguously
  const int tn = (int)min((long long)kTile, n - t0);
  for (int i = tid; i < tn; i += kBlock) {
    const unsigned h = s_hi[i];
    const unsigned long long l = s_lo[i];
    const unsigned d = rs_digit(h, l, word, shift);
    const long long dst = (long long)base[d] + (i - (int)toff[d]);
    hi_out[dst] = h;
    lo_out[dst] = l;
    val_out[dst] = s_val[i];
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
    launch_k(k_scan_apply, 1, kBlock, 0, st, in, out, n, nullptr);
    HBTU_LAUNCHED();
    return;
  }
  long long *sums = (long long *)tmp;
  char *rest = (char *)tmp + (((size_t)nb * sizeof(long long) + 255) / 256) * 256;
  launch_k(k_scan_reduce, (unsigned)nb, kBlock, 0, st, in, n, sums);
  HBTU_LAUNCHED();
  exclusive_scan_i64(sums, sums, nb, rest, st);
  launch_k(k_scan_apply, (unsigned)nb, kBlock, 0, st, in, out, n, sums);
  HBTU_LAUNCHED();
}

size_t sort_status_words(long long n)
{
  long long nb = (n + kTile - 1) / kTile;
  if (nb < 1) nb = 1;
  return 2 * (size_t)nb * 256 + 16;  // two passes' look-back words + their tile counters
}

void radix_sort(SortBuffers &b, long long n, const int *words, const int *shifts, int npasses,
                cudaStream_t st)
{
  if (n <= 1 || npasses <= 0) return;
  if (n <= kSmallN && npasses <= 16) {
    // more than 48 KB of shared memory needs an opt-in (per device, so every time)
    HBTU_CUDA(cudaFuncSetAttribute(k_rank_small, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)kRankSmem));
    SmallSortPasses ps;
    ps.n = npasses;
    for (int p = 0; p < npasses; p++) {
      ps.words[p] = words[p];
      ps.shifts[p] = shifts[p];
    }
    const int per_block = kBlock / kRankSplit;
    launch_k(k_rank_small, (unsigned)((n + per_block - 1) / per_block), kBlock, kRankSmem, st,
             b.hi_a, b.lo_a, b.val_a, b.hi_b, b.lo_b, b.val_b, (int)n, ps);
    HBTU_LAUNCHED();
    std::swap(b.hi_a, b.hi_b);  // the result lands in *_a
    std::swap(b.lo_a, b.lo_b);
    std::swap(b.val_a, b.val_b);
    return;
  }
  if (npasses > kMaxPasses)
    throw CudaError(cudaErrorInvalidValue, "radix sort: too many digit passes", __FILE__, __LINE__);
  const long long ntiles = (n + kTile - 1) / kTile;
  Passes ps;
  ps.n = npasses;
  for (int p = 0; p < npasses; p++) {
    ps.words[p] = words[p];
    ps.shifts[p] = shifts[p];
  }
  // global digit counts of every pass, their offsets, then one kernel per pass
  // pass p uses status half p & 1 and clears the other half for pass p + 1;
  // the histogram kernel clears the first pass's half
  unsigned *half[2] = {b.os_status, b.os_status + 256 * ntiles};
  int *counter[2] = {reinterpret_cast<int *>(b.os_status + 512 * ntiles),
                     reinterpret_cast<int *>(b.os_status + 512 * ntiles) + 1};
  HBTU_CUDA(cudaMemsetAsync(b.os_ghist, 0, sizeof(unsigned) * 256 * kMaxPasses, st));
  const unsigned hblocks = (unsigned)std::min<long long>(ntiles, 152 * 4);
  launch_k(k_os_hist, hblocks, kBlock, 0, st, b.hi_a, b.lo_a, n, ps, b.os_ghist, half[0],
           256 * ntiles, counter[0]);
  HBTU_LAUNCHED();
  launch_k(k_os_offsets, 1, kBlock, 0, st, b.os_ghist, npasses, b.os_goff);
  HBTU_LAUNCHED();
  for (int p = 0; p < npasses; p++) {
    launch_k(k_os_pass, (unsigned)ntiles, kBlock, 0, st, b.hi_a, b.lo_a, b.val_a, b.hi_b, b.lo_b,
             b.val_b, n, words[p], shifts[p], b.os_goff + 256 * p, half[p & 1], counter[p & 1],
             half[(p + 1) & 1], counter[(p + 1) & 1], b.error);
    HBTU_LAUNCHED();
    std::swap(b.hi_a, b.hi_b);
    std::swap(b.lo_a, b.lo_b);
    std::swap(b.val_a, b.val_b);
  }
}

}  // namespace hbtu
