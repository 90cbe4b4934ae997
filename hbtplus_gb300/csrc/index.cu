// index.cu -- particle-ID -> index tables on the GPU.
//
// Reference: IndexTable_t and its two forms (src/hash.h:47-112,
// src/hash.tpp, src/hash_remote.tpp), which ParticleSnapshot_t uses to turn
// particle IDs back into snapshot positions (src/snapshot.h:191-224).
//   mapped (MappedIndexTable_t): the (key, index) pairs sorted by key, then a
//     binary search per query; a negative key is absent (hash.tpp:18-55).
//     Here: an open-addressing hash table in HBM (linear probing, at most half
//     full, splitmix64 finalizer as the hash) whose slots hold input
//     positions; one thread per pair claims a slot with a 32-bit atomicCAS
//     (a duplicate key keeps the smallest position, atomicMin), one thread per
//     query probes; no sort.  The answers are the sorted table's.
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
  unsigned long long *aux = nullptr;  // key min / max (biased)
  int64_t *values = nullptr;
  int64_t *keys = nullptr;   // mapped: the keys, by input position
  int *hslot = nullptr;      // mapped: input position held by each slot (-1: free)
  unsigned long long hmask = 0;  // mapped: slots - 1 (a power of two)
  int *dense = nullptr;                 // flat: input position per key - kmin, -1 if none
};

namespace hbtu {
namespace {

constexpr int kIB = 256;
constexpr unsigned long long kSign = 0x8000000000000000ull;  // signed -> unsigned order

__global__ void __launch_bounds__(kIB) k_ix_minmax(const int64_t *keys, int64_t n,
                                                   unsigned long long *mm)
{
  HBTU_KERNEL_PROLOGUE();
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

__device__ __forceinline__ unsigned long long ix_hash(unsigned long long x)
{  // splitmix64 finalizer (Steele, Lea & Flood 2014)
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebull;
  x ^= x >> 31;
  return x;
}

// One thread per pair: claim a free slot for the key's position, or, when
// the key holds a slot already, keep the smaller position there.  Negative
// keys are absent in the reference's table.
__global__ void __launch_bounds__(kIB) k_ix_hash_fill(const int64_t *keys, int64_t n, int *hslot,
                                                      unsigned long long mask)
{
  HBTU_KERNEL_PROLOGUE();
  const int64_t i = (int64_t)blockIdx.x * kIB + threadIdx.x;
  if (i >= n) return;
  const long long k = keys[i];
  if (k < 0) return;
  unsigned long long slot = ix_hash((unsigned long long)k) & mask;
  for (unsigned long long probe = 0; probe <= mask; probe++) {  // the table is at most half full
    const int prev = atomicCAS(&hslot[slot], -1, (int)i);
    if (prev < 0) return;
    if (keys[prev] == k) {
      atomicMin(&hslot[slot], (int)i);
      return;
    }
    slot = (slot + 1) & mask;
  }
}

__global__ void __launch_bounds__(kIB) k_ix_flat_clear(int *dense, int64_t span)
{
  HBTU_KERNEL_PROLOGUE();
  for (int64_t i = (int64_t)blockIdx.x * kIB + threadIdx.x; i < span;
       i += (int64_t)gridDim.x * kIB)
    dense[i] = -1;
}

__global__ void __launch_bounds__(kIB) k_ix_flat_fill(const int64_t *keys, int64_t n, int64_t kmin,
                                                      int *dense)
{
  HBTU_KERNEL_PROLOGUE();
  const int64_t i = (int64_t)blockIdx.x * kIB + threadIdx.x;
  if (i >= n) return;
  atomicMax(&dense[(unsigned long long)keys[i] - (unsigned long long)kmin], (int)i);
}

__global__ void __launch_bounds__(kIB) k_ix_lookup_mapped(const int64_t *keys, const int *hslot,
                                                          const int64_t *values,
                                                          unsigned long long mask, int64_t n,
                                                          int64_t kmin, int64_t kmax,
                                                          int64_t null_index, const int64_t *q,
                                                          int64_t m, int64_t *out)
{
  HBTU_KERNEL_PROLOGUE();
  const int64_t j = (int64_t)blockIdx.x * kIB + threadIdx.x;
  if (j >= m) return;
  const int64_t key = q[j];
  int64_t r = null_index;
  if (key >= 0 && n > 0 && key >= kmin && key <= kmax) {
    unsigned long long slot = ix_hash((unsigned long long)key) & mask;
    for (unsigned long long probe = 0; probe <= mask; probe++) {
      const int p = hslot[slot];
      if (p < 0) break;
      if (keys[p] == key) {
        r = values[p];
        break;
      }
      slot = (slot + 1) & mask;
    }
  }
  out[j] = r;
}

__global__ void __launch_bounds__(kIB) k_ix_lookup_flat(const int *dense, const int64_t *values,
                                                        int64_t n, int64_t kmin, int64_t kmax,
                                                        int64_t null_index, const int64_t *q,
                                                        int64_t m, int64_t *out)
{
  HBTU_KERNEL_PROLOGUE();
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
  t->keys = nullptr;
  t->hslot = nullptr;
  t->hmask = 0;
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
    launch_k(k_ix_minmax, (unsigned)std::min<int64_t>(iblk(n), 152 * 8), kIB, 0, st, ksrc, n, mm);
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
      launch_k(k_ix_flat_clear,
               (unsigned)std::min<unsigned long long>((span + kIB - 1) / kIB, 152 * 16), kIB, 0, st,
               t->dense, (int64_t)span);
      HBTU_LAUNCHED();
      launch_k(k_ix_flat_fill, iblk(n), kIB, 0, st, ksrc, n, t->kmin, t->dense);
      HBTU_LAUNCHED();
    } else {
      // hash slots: a power of two at least twice the pairs
      unsigned long long slots = 1024;
      while (slots < 2ull * (unsigned long long)n) slots <<= 1;
      const size_t bs = align256(sizeof(int) * slots);
      if (!ix_grow(t, &t->mem, &t->cap, bvals + bkeys + bs)) {
        ix_release(t);
        return ix_fail(t, HBTU_ERR_OUT_OF_MEMORY, "mapped index: hash slots");
      }
      t->values = reinterpret_cast<int64_t *>(t->mem);
      t->keys = reinterpret_cast<int64_t *>(t->mem + bvals);
      t->hslot = reinterpret_cast<int *>(t->mem + bvals + bkeys);
      t->hmask = slots - 1;
      HBTU_CUDA(cudaMemcpyAsync(t->values, vsrc, sizeof(int64_t) * n, cudaMemcpyDeviceToDevice, st));
      HBTU_CUDA(cudaMemcpyAsync(t->keys, ksrc, sizeof(int64_t) * n, cudaMemcpyDeviceToDevice, st));
      HBTU_CUDA(cudaMemsetAsync(t->hslot, 0xff, sizeof(int) * slots, st));  // -1: free
      launch_k(k_ix_hash_fill, iblk(n), kIB, 0, st, t->keys, n, t->hslot, t->hmask);
      HBTU_LAUNCHED();
      HBTU_CUDA(cudaStreamSynchronize(st));
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
      launch_k(k_ix_lookup_flat, iblk(m), kIB, 0, st, t->dense, t->values, t->n, t->kmin, t->kmax,
               t->null_index, dq, m, dout);
    else
      launch_k(k_ix_lookup_mapped, iblk(m), kIB, 0, st,
               t->keys, t->hslot, t->values, t->hmask, t->n,
               t->kmin, t->kmax, t->null_index, dq, m, dout);
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
