// FP64 pipe throughput probe, used as the roofline denominator of the
// FP64-bound step kernel.  Each thread runs 8 independent chains of
// x = x * y - z issued as a separate multiply and subtract (the instruction mix
// of the rank-1 Schur update), or as a fused multiply-add.  The result is in
// FP64 operations per second (a fused multiply-add counts as two).
#include <cuda_runtime.h>
#include <stdint.h>

namespace {

template <bool FUSED>
__global__ void fp64_probe(double* out, int iters, double y, double z) {
  double x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = 1.0 + 1e-3 * (threadIdx.x + k);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      if (FUSED)
        x[k] = __fma_rn(x[k], y, -z);
      else
        x[k] = __dsub_rn(__dmul_rn(x[k], y), z);
    }
  }
  double s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  if (s == 12345.678) out[blockIdx.x] = s;  // keep the work live
}

}  // namespace

// Returns FP64 operations per second (separate mul+sub, and fused) measured on
// the given stream with CUDA events.
extern "C" int tci_fp64_peak(uintptr_t stream_u, double* ops_separate, double* ops_fused) {
  cudaStream_t stream = (cudaStream_t)stream_u;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  double* out = nullptr;
  if (cudaMalloc(&out, 65536 * sizeof(double)) != cudaSuccess) return 6;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  const int blocks = sms * 8, threads = 256, iters = 4096;
  const double y = 0.999999, z = 1e-7;
  float ms = 0;
  double ops = (double)blocks * threads * iters * 8 * 2;
  // warm-up
  fp64_probe<false><<<blocks, threads, 0, stream>>>(out, 64, y, z);
  cudaEventRecord(a, stream);
  fp64_probe<false><<<blocks, threads, 0, stream>>>(out, iters, y, z);
  cudaEventRecord(b, stream);
  cudaEventSynchronize(b);
  cudaEventElapsedTime(&ms, a, b);
  if (ops_separate) *ops_separate = ops / (ms * 1e-3);
  fp64_probe<true><<<blocks, threads, 0, stream>>>(out, 64, y, z);
  cudaEventRecord(a, stream);
  fp64_probe<true><<<blocks, threads, 0, stream>>>(out, iters, y, z);
  cudaEventRecord(b, stream);
  cudaEventSynchronize(b);
  cudaEventElapsedTime(&ms, a, b);
  if (ops_fused) *ops_fused = ops / (ms * 1e-3);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(out);
  return cudaGetLastError() == cudaSuccess ? 0 : 6;
}
