// Slot layout and hash of the device value cache of a caller-supplied f, shared
// by the step kernel's lookup (tci_functions.h), the cache kernels (fcache.cu)
// and the host (fcache.cpp).
#pragma once

#if defined(__CUDACC__)
#define TCI_FC_HD __host__ __device__ __forceinline__
#else
#define TCI_FC_HD static inline
#endif

// Function id of solves whose f is caller-supplied (values from the cache).
#define TCI_FID_CACHE 7

// k0 == TCI_FC_EMPTY marks a free slot.
struct tci_fc_entry {
  unsigned long long k0, k1;
  double v;
  unsigned long long unused;
};
#define TCI_FC_EMPTY 0xffffffffffffffffull

TCI_FC_HD unsigned long long tci_fc_hash(unsigned long long k0, unsigned long long k1) {
  unsigned long long h = k0 * 0x9e3779b97f4a7c15ull ^ (k1 + 0x632be59bd9b4e019ull) * 0xc2b2ae3d27d4eb4full;
  h ^= h >> 31;
  h *= 0xd6e8feb86659fd93ull;
  h ^= h >> 32;
  return h;
}
