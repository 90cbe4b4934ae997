// index.cu -- particle-ID -> index tables on the GPU.
//
// Reference: IndexTable_t and its two forms (src/hash.h:47-112,
// src/hash.tpp, src/hash_remote.tpp), which ParticleSnapshot_t uses to turn
// particle IDs back into snapshot positions (src/snapshot.h:191-224).
//   mapped (MappedIndexTable_t): the (key, index) pairs sorted by key, then a
//     binary search per query; a negative key is absent (hash.tpp:18-55).
//     Here: a stable radix sort of key - KeyMin (only the digits the key span
//     needs) and a lower-bound search per query, one thread per query.
//   flat (FlatIndexTable_t): a dense array over [KeyMin, KeyMax]
//     (hash.tpp:59-109).  Here: the position of each pair scattered into the
//     dense array, one thread per pair.
// Duplicate keys: the reference leaves them undefined (std::sort is not
// stable; the flat fill writes in parallel).  Here the first pair in input
// order wins for the mapped table and the last for the flat table, as a
// serial fill would do.
#include <algorithm>
#include <cstring>

#include "handle.h"

struct hbtu_index_table {
  hbtu_handle *h = nullptr;
  int flat = 0;
  int64_t n = 0, null_index = -1, kmin = 0, kmax = -1;
  // device memory is kept from fill to fill and only grows, so refilling a
  // table every snapshot allocates nothing once it has reached its size
  char *mem = nullptr;  // the table: everything below but aux
  size_t cap = 0;
  char *stage = nullptr;  // host-memory calls: staging of keys, values, queries
  size_t stage_cap = 0;
  unsigned long long *aux = nullptr;  // key min / max (biased), sort error flag
  int64_t *values = nullptr;
  unsigned long long *skeys = nullptr;  // mapped: sorted key - kmin
  int *spos = nullptr;                  // mapped: input position of each sorted key
  int *dense = nullptr;                 // flat: input position per key - kmin, -1 if none
};

namespace hbtu {
namespace {

constexpr int kIB = 256;
constexpr unsigned long long kSign = 0x8000000000000000ull;  // signed -> unsigned order

__global__ void __launch_bounds__(kIB) k_ix_minmax(const int64_t *keys, int64_t n,
                                                   unsigned long long *mm)
{
  unsigned long long lo = ~0ull, hi = 0ull;
  for (int64_t i = (int64_t)blockIdx.x * kIB + threadIdx.x; i < n; i += (int64_t)gridDim.x * kIB) {
    const unsigned long long b = (unsigned long long)keys[i] ^ kSign;
    lo = min(lo, b);
    hi = max(hi, b);
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&mm[0], lo);
    atomicMax(&mm[1], hi);
  }
}

__global__ void __launch_bounds__(kIB) k_ix_prepare(const int64_t *keys, int64_t n, int64_t kmin,
                                                    unsigned long long *lo, unsigned *hi, int *pos)
{
  const int64_t i = (int64_t)blockIdx.x * kIB + threadIdx.x;
  if (i >= n) return;
  lo[i] = (unsigned long long)keys[i] - (unsigned long long)kmin;
  hi[i] = 0u;
  pos[i] = (int)i;
}

__global__ void __launch_bounds__(kIB) k_ix_flat_clear(int *dense, int64_t span)
{
  for (int64_t i = (int64_t)blockIdx.x * kIB + threadIdx.x; i < span;
       i += (int64_t)gridDim.x * kIB)
    dense[i] = -1;
}

__global__ void __launch_bounds__(kIB) k_ix_flat_fill(const int64_t *keys, int64_t n, int64_t kmin,
                                                      int *dense)
{
  const int64_t i = (int64_t)blockIdx.x * kIB + threadIdx.x;
  if (i >= n) return;
  atomicMax(&dense[(unsigned long long)keys[i] - (unsigned long long)kmin], (int)i);
}

__global__ void __launch_bounds__(kIB) k_ix_lookup_mapped(const unsigned long long *skeys,
                                                          const int *spos, const int64_t *values,
                                                          int64_t n, int64_t kmin, int64_t kmax,
                                                          int64_t null_index, const int64_t *q,
                                                          int64_t m, int64_t *out)
{
  const int64_t j = (int64_t)blockIdx.x * kIB + threadIdx.x;
  if (j >= m) return;
  const int64_t key = q[j];
  int64_t r = null_index;
  if (key >= 0 && n > 0 && key >= kmin && key <= kmax) {
    const unsigned long long k = (unsigned long long)key - (unsigned long long)kmin;
    int64_t lo = 0, hi = n;  // lower bound
    while (lo < hi) {
      const int64_t mid = lo + ((hi - lo) >> 1);
      if (skeys[mid] < k)
        lo = mid + 1;
      else
        hi = mid;
    }
    if (lo < n && skeys[lo] == k) r = values[spos[lo]];
  }
  out[j] = r;
}

__global__ void __launch_bounds__(kIB) k_ix_lookup_flat(const int *dense, const int64_t *values,
                                                        int64_t n, int64_t kmin, int64_t kmax,
                                                        int64_t null_index, const int64_t *q,
                                                        int64_t m, int64_t *out)
{
  const int64_t j = (int64_t)blockIdx.x * kIB + threadIdx.x;
  if (j >= m) return;
  const int64_t key = q[j];
  int64_t r = null_index;
  if (n > 0 && key >= kmin && key <= kmax) {
    const int p = dense[(unsigned long long)key - (unsigned long long)kmin];
    if (p >= 0) r = values[p];
  }
  out[j] = r;
}

inline unsigned iblk(int64_t n) { return (unsigned)((n + kIB - 1) / kIB); }

hbtu_status ix_fail(hbtu_index_table *t, hbtu_status st, const char *msg)
{
  if (t && t->h) t->h->err = msg;
  return st;
}

// Forget the table's content (its memory stays for the next fill).
void ix_release(hbtu_index_table *t)
{
  t->values = nullptr;
  t->skeys = nullptr;
  t->spos = nullptr;
  t->dense = nullptr;
  t->n = 0;
  t->kmin = 0;
  t->kmax = -1;
}

void ix_free(hbtu_index_table *t)
{
  ix_release(t);
  if (t->mem) cudaFree(t->mem);
  if (t->stage) cudaFree(t->stage);
  if (t->aux) cudaFree(t->aux);
  t->mem = t->stage = nullptr;
  t->aux = nullptr;
  t->cap = t->stage_cap = 0;
}

// Grow *buf to at least `bytes` (with headroom); false if that fails.
bool ix_grow(hbtu_index_table *t, char **buf, size_t *cap, size_t bytes)
{
  if (bytes <= *cap) return true;
  if (*buf) {
    cudaStreamSynchronize(t->h->stream);
    cudaFree(*buf);
    *buf = nullptr;
    *cap = 0;
  }
  const size_t want = bytes + bytes / 8;
  if (cudaMalloc(buf, want) != cudaSuccess) {
    cudaGetLastError();
    *buf = nullptr;
    return false;
  }
  *cap = want;
  return true;
}

size_t align256(size_t b) { return (b + 255) / 256 * 256; }

}  // namespace
}  // namespace hbtu

using namespace hbtu;

extern "C" {

hbtu_status hbtu_index_create(hbtu_handle *h, int32_t flat, hbtu_index_table **out)
{
  if (!h || !out) return HBTU_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  hbtu_index_table *t = new (std::nothrow) hbtu_index_table;
  if (!t) return HBTU_ERR_OUT_OF_MEMORY;
  t->h = h;
  t->flat = flat != 0;
  *out = t;
  return HBTU_OK;
}

hbtu_status hbtu_index_destroy(hbtu_index_table *t)
{
  if (!t) return HBTU_OK;
  if (t->h) cudaSetDevice(t->h->device);
  ix_free(t);
  delete t;
  return HBTU_OK;
}

hbtu_status hbtu_index_fill(hbtu_index_table *t, const int64_t *keys, const int64_t *values,
                            int64_t n, int64_t null_index, int32_t location)
{
  if (!t || !t->h) return HBTU_ERR_INVALID_ARGUMENT;
  if (n < 0 || (n > 0 && (!keys || !values)))
    return ix_fail(t, HBTU_ERR_INVALID_ARGUMENT, "index fill: bad count or null arrays");
  if (n >= HBTU_MAX_PARTICLES) return ix_fail(t, HBTU_ERR_TOO_LARGE, "index fill: too many keys");
  hbtu_handle *h = t->h;
  cudaSetDevice(h->device);
  cudaStream_t st = h->stream;
  ix_release(t);
  t->null_index = null_index;
  if (n == 0) return HBTU_OK;
  const bool host = location == HBTU_HOST;
  try {
    if (!t->aux) {
      if (cudaMalloc(&t->aux, 256) != cudaSuccess) {
        cudaGetLastError();
        t->aux = nullptr;
        return ix_fail(t, HBTU_ERR_OUT_OF_MEMORY, "index fill: small buffer");
      }
    }
    unsigned long long *mm = t->aux;
    int *err = reinterpret_cast<int *>(t->aux + 2);
    const size_t bkeys = align256(sizeof(int64_t) * n), bvals = align256(sizeof(int64_t) * n);
    const int64_t *ksrc = keys, *vsrc = values;
    if (host) {  // stage the host arrays on the device
      if (!ix_grow(t, &t->stage, &t->stage_cap, bkeys + bvals))
        return ix_fail(t, HBTU_ERR_OUT_OF_MEMORY, "index fill: staging");
      int64_t *dkeys = reinterpret_cast<int64_t *>(t->stage);
      int64_t *dvals = reinterpret_cast<int64_t *>(t->stage + bkeys);
      HBTU_CUDA(cudaMemcpyAsync(dkeys, keys, sizeof(int64_t) * n, cudaMemcpyHostToDevice, st));
      HBTU_CUDA(cudaMemcpyAsync(dvals, values, sizeof(int64_t) * n, cudaMemcpyHostToDevice, st));
      ksrc = dkeys;
      vsrc = dvals;
    }
    // pass 1: key range (one small read back)
    const unsigned long long init[2] = {~0ull, 0ull};
    HBTU_CUDA(cudaMemcpyAsync(mm, init, sizeof(init), cudaMemcpyHostToDevice, st));
    k_ix_minmax<<<std::min<int64_t>(iblk(n), 152 * 8), kIB, 0, st>>>(ksrc, n, mm);
    HBTU_LAUNCHED();
    unsigned long long hmm[2];
    HBTU_CUDA(cudaMemcpyAsync(hmm, mm, sizeof(hmm), cudaMemcpyDeviceToHost, st));
    HBTU_CUDA(cudaStreamSynchronize(st));
    t->kmin = (int64_t)(hmm[0] ^ kSign);
    t->kmax = (int64_t)(hmm[1] ^ kSign);
    const unsigned long long span = (unsigned long long)t->kmax - (unsigned long long)t->kmin + 1ull;
    if (t->flat) {
      if (span == 0ull || span > (1ull << 32)) {
        ix_release(t);
        return ix_fail(t, HBTU_ERR_TOO_LARGE, "flat index: key span above 2^32");
      }
      if (!ix_grow(t, &t->mem, &t->cap, bvals + align256(sizeof(int) * span))) {
        ix_release(t);
        return ix_fail(t, HBTU_ERR_OUT_OF_MEMORY, "flat index: dense array");
      }
      t->values = reinterpret_cast<int64_t *>(t->mem);
      t->dense = reinterpret_cast<int *>(t->mem + bvals);
      HBTU_CUDA(cudaMemcpyAsync(t->values, vsrc, sizeof(int64_t) * n, cudaMemcpyDeviceToDevice, st));
      k_ix_flat_clear<<<(unsigned)std::min<unsigned long long>((span + kIB - 1) / kIB, 152 * 16),
                        kIB, 0, st>>>(t->dense, (int64_t)span);
      HBTU_LAUNCHED();
      k_ix_flat_fill<<<iblk(n), kIB, 0, st>>>(ksrc, n, t->kmin, t->dense);
      HBTU_LAUNCHED();
    } else {
      // sort buffers (two copies of key / subhalo word / payload) + onesweep state
      const size_t b8 = align256(sizeof(unsigned long long) * n), b4 = align256(sizeof(int) * n);
      const size_t bstat = align256(sizeof(unsigned) * sort_status_words(n));
      const size_t bhist = align256(sizeof(unsigned) * 16 * 256);
      if (!ix_grow(t, &t->mem, &t->cap, bvals + 2 * b8 + 4 * b4 + bstat + 2 * bhist)) {
        ix_release(t);
        return ix_fail(t, HBTU_ERR_OUT_OF_MEMORY, "mapped index: sort buffers");
      }
      char *q = t->mem;
      t->values = reinterpret_cast<int64_t *>(q);
      q += bvals;
      SortBuffers sb;
      sb.lo_a = reinterpret_cast<unsigned long long *>(q);
      q += b8;
      sb.lo_b = reinterpret_cast<unsigned long long *>(q);
      q += b8;
      sb.hi_a = reinterpret_cast<unsigned *>(q);
      q += b4;
      sb.hi_b = reinterpret_cast<unsigned *>(q);
      q += b4;
      sb.val_a = reinterpret_cast<int *>(q);
      q += b4;
      sb.val_b = reinterpret_cast<int *>(q);
      q += b4;
      sb.os_status = reinterpret_cast<unsigned *>(q);
      q += bstat;
      sb.os_ghist = reinterpret_cast<unsigned *>(q);
      q += bhist;
      sb.os_goff = reinterpret_cast<unsigned *>(q);
      sb.error = err;
      HBTU_CUDA(cudaMemsetAsync(sb.error, 0, sizeof(int), st));
      HBTU_CUDA(cudaMemcpyAsync(t->values, vsrc, sizeof(int64_t) * n, cudaMemcpyDeviceToDevice, st));
      k_ix_prepare<<<iblk(n), kIB, 0, st>>>(ksrc, n, t->kmin, sb.lo_a, sb.hi_a, sb.val_a);
      HBTU_LAUNCHED();
      // only the digits the key span needs
      int bits = 0;
      while (bits < 64 && ((span - 1ull) >> bits) != 0ull) bits++;
      int words[8], shifts[8], np = 0;
      for (int b = 0; b < bits; b += 8) {
        words[np] = 0;
        shifts[np++] = b;
      }
      radix_sort(sb, n, words, shifts, np, st);
      t->skeys = sb.lo_a;
      t->spos = sb.val_a;
      int herr = 0;
      HBTU_CUDA(cudaMemcpyAsync(&herr, sb.error, sizeof(int), cudaMemcpyDeviceToHost, st));
      HBTU_CUDA(cudaStreamSynchronize(st));
      if (herr) {
        ix_release(t);
        return ix_fail(t, HBTU_ERR_CUDA, "mapped index: radix sort look-back");
      }
    }
    t->n = n;
    return HBTU_OK;
  } catch (const CudaError &e) {
    ix_release(t);
    return ix_fail(t, HBTU_ERR_CUDA, e.what.c_str());
  }
}

hbtu_status hbtu_index_lookup(hbtu_index_table *t, const int64_t *keys, int64_t m, int64_t *out,
                              int32_t location)
{
  if (!t || !t->h) return HBTU_ERR_INVALID_ARGUMENT;
  if (m < 0 || (m > 0 && (!keys || !out)))
    return ix_fail(t, HBTU_ERR_INVALID_ARGUMENT, "index lookup: bad count or null arrays");
  if (m == 0) return HBTU_OK;
  hbtu_handle *h = t->h;
  cudaSetDevice(h->device);
  cudaStream_t st = h->stream;
  const bool host = location == HBTU_HOST;
  try {
    const int64_t *dq = keys;
    int64_t *dout = out;
    if (host) {
      if (!ix_grow(t, &t->stage, &t->stage_cap, 2 * align256(sizeof(int64_t) * m)))
        return ix_fail(t, HBTU_ERR_OUT_OF_MEMORY, "index lookup: staging");
      int64_t *sq = reinterpret_cast<int64_t *>(t->stage);
      dout = reinterpret_cast<int64_t *>(t->stage + align256(sizeof(int64_t) * m));
      HBTU_CUDA(cudaMemcpyAsync(sq, keys, sizeof(int64_t) * m, cudaMemcpyHostToDevice, st));
      dq = sq;
    }
    if (t->flat)
      k_ix_lookup_flat<<<iblk(m), kIB, 0, st>>>(t->dense, t->values, t->n, t->kmin, t->kmax,
                                                t->null_index, dq, m, dout);
    else
      k_ix_lookup_mapped<<<iblk(m), kIB, 0, st>>>(t->skeys, t->spos, t->values, t->n, t->kmin,
                                                  t->kmax, t->null_index, dq, m, dout);
    HBTU_LAUNCHED();
    if (host) {
      HBTU_CUDA(cudaMemcpyAsync(out, dout, sizeof(int64_t) * m, cudaMemcpyDeviceToHost, st));
      HBTU_CUDA(cudaStreamSynchronize(st));
    }
    return HBTU_OK;
  } catch (const CudaError &e) {
    return ix_fail(t, HBTU_ERR_CUDA, e.what.c_str());
  }
}

hbtu_status hbtu_index_key_range(const hbtu_index_table *t, int64_t *key_min, int64_t *key_max)
{
  if (!t || !key_min || !key_max) return HBTU_ERR_INVALID_ARGUMENT;
  *key_min = t->kmin;
  *key_max = t->kmax;
  return HBTU_OK;
}

}  // extern "C"
