// Kernels of the device value cache of a caller-supplied f (fcache.h): probe a
// product of row and column keys against the table and compact the misses,
// insert new values, and rehash into a larger table.  All HBM-bound integer
// work: one 32-byte slot per probe step, load factor at most 1/2.
#include <cuda_runtime.h>
#include <stdint.h>

#include "fc_slot.h"
#include "fcache.h"

namespace tci {
namespace {

constexpr int FC_THREADS = 256;

int fc_grid(int64_t n) {
  int64_t g = (n + FC_THREADS - 1) / FC_THREADS;
  if (g > 152 * 16) g = 152 * 16;
  return (int)(g < 1 ? 1 : g);
}

__device__ __forceinline__ bool fc_find(const tci_fc_entry* tab, uint64_t mask, uint64_t k0, uint64_t k1) {
  uint64_t h = tci_fc_hash(k0, k1) & mask;
  for (uint64_t q = 0; q <= mask; ++q) {
    const uint64_t e0 = tab[h].k0;
    if (e0 == k0 && tab[h].k1 == k1) return true;
    if (e0 == TCI_FC_EMPTY) return false;
    h = (h + 1) & mask;
  }
  return false;
}

// Element e = i + nr * j of the product rows x columns: key = rk[i] + ck[j]
// (word by word; the halves of a row and a column cover disjoint sites).  A miss
// appends (j << 32 | i) to miss[].
__global__ void __launch_bounds__(FC_THREADS)
    fc_probe_kernel(const tci_fc_entry* __restrict__ tab, uint64_t mask, const int64_t* __restrict__ rk, int64_t nr,
                    const int64_t* __restrict__ ck, int64_t nc, unsigned long long* count,
                    uint64_t* __restrict__ miss) {
  const int64_t n = nr * nc;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e % nr, j = e / nr;
    const uint64_t k0 = (uint64_t)(rk[2 * i] + ck[2 * j]);
    const uint64_t k1 = (uint64_t)(rk[2 * i + 1] + ck[2 * j + 1]);
    if (!fc_find(tab, mask, k0, k1)) {
      const unsigned long long at = atomicAdd(count, 1ull);
      miss[at] = ((uint64_t)j << 32) | (uint64_t)i;
    }
  }
}

// Keys in `in` are distinct and absent from the table, so a slot whose word 0
// is taken (even by an equal word 0) belongs to another key: claim the first
// free slot on the probe path.
__device__ __forceinline__ void fc_put(tci_fc_entry* tab, uint64_t mask, const tci_fc_entry& x) {
  uint64_t h = tci_fc_hash(x.k0, x.k1) & mask;
  for (uint64_t q = 0; q <= mask; ++q) {
    const unsigned long long prev =
        atomicCAS((unsigned long long*)&tab[h].k0, (unsigned long long)TCI_FC_EMPTY, (unsigned long long)x.k0);
    if (prev == TCI_FC_EMPTY) {
      tab[h].k1 = x.k1;
      tab[h].v = x.v;
      return;
    }
    h = (h + 1) & mask;
  }
}

__global__ void __launch_bounds__(FC_THREADS)
    fc_insert_kernel(tci_fc_entry* tab, uint64_t mask, const tci_fc_entry* __restrict__ in, int64_t n) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    fc_put(tab, mask, in[e]);
}

__global__ void __launch_bounds__(FC_THREADS)
    fc_rehash_kernel(tci_fc_entry* dst, uint64_t dmask, const tci_fc_entry* __restrict__ src, uint64_t scap) {
  for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < scap; e += (uint64_t)gridDim.x * blockDim.x)
    if (src[e].k0 != TCI_FC_EMPTY) fc_put(dst, dmask, src[e]);
}

}  // namespace

void fc_probe_launch(const tci_fc_entry* tab, uint64_t mask, const int64_t* rk, int64_t nr, const int64_t* ck,
                     int64_t nc, unsigned long long* count, uint64_t* miss, cudaStream_t s) {
  if (nr <= 0 || nc <= 0) return;
  fc_probe_kernel<<<fc_grid(nr * nc), FC_THREADS, 0, s>>>(tab, mask, rk, nr, ck, nc, count, miss);
}

void fc_insert_launch(tci_fc_entry* tab, uint64_t mask, const tci_fc_entry* in, int64_t n, cudaStream_t s) {
  if (n <= 0) return;
  fc_insert_kernel<<<fc_grid(n), FC_THREADS, 0, s>>>(tab, mask, in, n);
}

void fc_rehash_launch(tci_fc_entry* dst, uint64_t dmask, const tci_fc_entry* src, uint64_t scap, cudaStream_t s) {
  if (scap == 0) return;
  fc_rehash_kernel<<<fc_grid((int64_t)scap), FC_THREADS, 0, s>>>(dst, dmask, src, scap);
}

}  // namespace tci
