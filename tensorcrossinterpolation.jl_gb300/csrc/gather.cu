// Gather of many device arrays (site tensors of many solves) into one
// contiguous buffer, so results leave the device in a single copy.
#include <cuda_runtime.h>
#include <stdint.h>

namespace {

__global__ void __launch_bounds__(256) gather_kernel(const double* const* __restrict__ src,
                                                     const int64_t* __restrict__ len,
                                                     const int64_t* __restrict__ dst_off,
                                                     double* __restrict__ dst, int n) {
  for (int s = blockIdx.x; s < n; s += gridDim.x) {
    const double* p = src[s];
    double* d = dst + dst_off[s];
    const int64_t L = len[s];
    for (int64_t i = threadIdx.x; i < L; i += blockDim.x) d[i] = p[i];
  }
}

}  // namespace

// table: n source pointers, then n lengths, then n destination offsets (device memory).
cudaError_t tci_gather_launch(const void* table_dev, int n, double* dst_dev, int grid, cudaStream_t stream) {
  const double* const* src = (const double* const*)table_dev;
  const int64_t* len = (const int64_t*)((const char*)table_dev + (size_t)n * sizeof(void*));
  const int64_t* off = len + n;
  gather_kernel<<<grid, 256, 0, stream>>>(src, len, off, dst_dev, n);
  return cudaGetLastError();
}
