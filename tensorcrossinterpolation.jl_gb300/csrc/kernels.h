// The step-kernel family is compiled twice from step_kernel.cu:
//   tci_k256: two 256-thread task CTAs per SM (throughput: batched and served
//             solves, batched rrLU).  While one task waits on a pivot's latency
//             chain, the other's rank-1 update keeps the FP64 pipe busy.
//   tci_k512: one 512-thread task CTA per SM (latency: a single solve, whose
//             tasks run one at a time).
// Both share the task records, the resident ring and the results; the engine
// picks the set per launch.  The multi-CTA rrLU (one 512-thread CTA per SM in
// either) is taken from tci_k256.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "tci_tasks.h"

struct tci_kernel_set {
  int threads;      // threads of one task CTA
  int ctas_per_sm;  // task CTAs resident per SM
  size_t (*step_smem_bytes)();      // dynamic shared memory of one task CTA
  size_t (*resident_smem_bytes)();  // the same for the resident kernel
  cudaError_t (*configure)();
  cudaError_t (*step_launch)(const char* blob_dev, char* res_dev, const int* order_dev, int ntasks,
                             int* counter_dev, int grid, double* cta_area, size_t cta_stride,
                             cudaStream_t stream);
  cudaError_t (*resident_launch)(tci_queue_slot* slots, uint32_t mask, tci_resident_state* st,
                                 tci_queue_ctl* qc, int grid, unsigned long long wait_ns, cudaStream_t stream);
};

namespace tci_k256 {
extern const tci_kernel_set kernels;
size_t tci_rrlu_big_smem(int64_t m, int64_t n, int G);
bool tci_rrlu_big_fits(int64_t m, int64_t n, int G);
size_t tci_rrlu_big_scratch_bytes(int grid, int kmax);
cudaError_t tci_rrlu_big_launch(const double* ain, double* work, double* fact, char* res, void* scratch, int m,
                                int n, int kmax, int kcap, int leftorth, double reltol, double abstol, int grid,
                                cudaStream_t stream);
}  // namespace tci_k256
namespace tci_k512 {
extern const tci_kernel_set kernels;
}
