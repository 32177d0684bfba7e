// Split-precision tensor-core GEMM for the tensor-train contractions
// (contraction.jl:71-93 `_contract`, :442-486 `contract_zipup`): FP64 operands
// are split into TF32 hi/lo pairs and multiplied on the 5th-generation tensor
// cores (tcgen05.mma kind::tf32) as hi*hi + hi*lo + lo*hi, accumulated in FP32
// in tensor memory, and written back as FP64.
//
//   C[m, n] = sum_k A[m, k] * B[n, k]
//
// Operands and result are addressed through `tci_map3` index maps
// (off(i) = (i % d0) s0 + ((i / d0) % d1) s1 + (i / (d0 d1)) s2 elements), so the
// permuted/fused tensor legs of a contraction are read and written in place.
//
// Two kernels per product:
//   pack  : FP64 -> TF32 hi/lo rows, K-major, K padded to 32, rows padded to
//           the tile; hi rows [0, Mp), lo rows [Mp, 2 Mp) of one array;
//   gemm  : one 128 x BN output tile per CTA.  Warp 0 issues TMA tile loads
//           (cp.async.bulk.tensor, 128-byte swizzle) into a STAGES-deep ring of
//           shared-memory stages guarded by mbarriers; warp 1 issues the MMAs
//           (one thread), 3 per 8-deep K slice, into a 128 x BN FP32
//           accumulator in tensor memory and releases each stage with
//           tcgen05.commit; all four warps then read the accumulator rows
//           (tcgen05.ld, warp w owns TMEM lanes 32w..32w+31) and store FP64.
//
// Error: |hi + lo - x| <= 2^-22 |x| per operand and the dropped lo*lo term is
// below 2^-22 |a b|, so each product carries ~2^-21 relative error; the FP32
// accumulation adds ~2^-24 per addition.  Operands must lie inside the FP32
// range.  Every wait on an mbarrier is bounded (TC_WAIT_NS); a wait that runs
// out sets the error word, and the CTA still releases its tensor memory.
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "tc_gemm.h"

namespace {

constexpr int TC_THREADS = 128;
constexpr int BM = 128;     // tile rows (MMA M)
constexpr int BK = 32;      // fp32 elements per 128-byte swizzle row
constexpr int KSUB = 8;     // MMA K for kind::tf32
constexpr unsigned long long TC_WAIT_NS = 2000000000ULL;  // 2 s bound on any wait

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for the phase of `parity` to complete; false (and the error word
// set) if it did not within TC_WAIT_NS.
__device__ bool mbar_wait(uint32_t bar, uint32_t parity, int* err, int code) {
  if (mbar_try(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  for (;;) {
    if (mbar_try(bar, parity)) return true;
    if (global_ns() - t0 > TC_WAIT_NS) {
      atomicExch(err, code);
      return false;
    }
  }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"((uint64_t)map), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

// Shared-memory matrix descriptor of a K-major tile with 128-byte swizzle: rows
// of 128 bytes, 8-row groups 1024 bytes apart (SBO), descriptor version 1.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  // leading byte offset 0: one swizzle atom spans the tile's whole K extent
  d |= (uint64_t)(1024 >> 4) << 32;    // stride byte offset
  d |= (uint64_t)1 << 46;              // version
  d |= (uint64_t)2 << 61;              // SWIZZLE_128B
  return d;
}

// Instruction descriptor: D f32, A and B tf32, both K-major, M x N.
__host__ __device__ constexpr uint32_t tf32_idesc(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ int64_t map_off(const tci_map3& m, int64_t i) {
  const int64_t a = i % m.d0, q = i / m.d0;
  return a * m.s0 + (q % m.d1) * m.s1 + (q / m.d1) * m.s2;
}

// x = hi + lo + O(2^-22 |x|) with hi, lo TF32 values (FP32 with the low 13
// mantissa bits zero), each rounded to nearest.
__device__ __forceinline__ void split_tf32(double x, float& hi, float& lo) {
  uint32_t h, l;
  const float xf = __double2float_rn(x);
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(xf));
  hi = __uint_as_float(h);
  const float rf = __double2float_rn(x - (double)hi);
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(l) : "f"(rf));
  lo = __uint_as_float(l);
}

// Packs rows [0, rows) x k [0, K) of a mapped FP64 operand into out (2 * rows_p
// rows of kp floats: hi rows then lo rows), zero padding.  32 x 32 tiles through
// shared memory; `k_fast` reads along k (the operand's unit stride) instead of
// along the rows.
__global__ void __launch_bounds__(256) pack_split_kernel(const double* __restrict__ src, tci_map3 rmap, tci_map3 kmap,
                                                         int rows, int K, int rows_p, int kp, int k_fast,
                                                         float* __restrict__ out) {
  __shared__ double tile[32][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  const int k0 = blockIdx.x * 32;
  for (int r0 = blockIdx.y * 32; r0 < rows_p; r0 += gridDim.y * 32) {
  for (int yy = ty; yy < 32; yy += 8) {
    int r, k;
    if (k_fast) {
      r = r0 + yy;
      k = k0 + tx;
    } else {
      r = r0 + tx;
      k = k0 + yy;
    }
    double v = 0.0;
    if (r < rows && k < K) v = src[map_off(rmap, r) + map_off(kmap, k)];
    if (k_fast)
      tile[yy][tx] = v;  // [row][k]
    else
      tile[tx][yy] = v;
  }
  __syncthreads();
  for (int yy = ty; yy < 32; yy += 8) {
    const int r = r0 + yy, k = k0 + tx;
    if (r < rows_p && k < kp) {
      float hi, lo;
      split_tf32(tile[yy][tx], hi, lo);
      out[(size_t)r * kp + k] = hi;
      out[((size_t)rows_p + r) * kp + k] = lo;
    }
  }
  __syncthreads();
  }
}

template <int BN, int STAGES>
struct TcSmem {
  static constexpr int A_BYTES = BM * BK * 4;  // 16 KB
  static constexpr int B_BYTES = BN * BK * 4;
  static constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;
  static constexpr int TOTAL = 1024 + STAGES * STAGE_BYTES + 256;  // alignment slack + barriers
};

template <int BN, int STAGES>
__global__ void __launch_bounds__(TC_THREADS, 1)
    tc_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int M, int N,
                   int Mp, int Np, int kiters, double* __restrict__ C, tci_map3 crow, tci_map3 ccol, int* err) {
  using S = TcSmem<BN, STAGES>;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* base = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* bars = (uint64_t*)(base + STAGES * S::STAGE_BYTES);  // full[STAGES], empty[STAGES], done
  uint32_t* tmem_slot = (uint32_t*)(bars + 2 * STAGES + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // N tiles run fastest: the CTAs that share an A tile run together and read it from L2
  const int n0 = blockIdx.x * BN, m0 = blockIdx.y * BM;
  constexpr int TMEM_COLS = BN <= 32 ? 32 : (BN <= 64 ? 64 : (BN <= 128 ? 128 : 256));

  if (threadIdx.x == 0) {
    for (int s = 0; s < 2 * STAGES + 1; ++s) mbar_init(smem_u32(bars + s), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmA) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmB) : "memory");
  }
  if (warp == 2) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + STAGES), done = smem_u32(bars + 2 * STAGES);
  bool ok = true;

  if (warp == 0 && lane == 0) {
    // producer: four tile loads per stage (A hi, A lo, B hi, B lo)
    int it = 0;
    for (; it < kiters; ++it) {
      const int s = it % STAGES;
      const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
      if (!mbar_wait(empty0 + 8 * s, ph ^ 1u, err, 1)) {
        ok = false;
        break;
      }
      uint8_t* st = base + s * S::STAGE_BYTES;
      const uint32_t fb = full0 + 8 * s;
      mbar_expect_tx(fb, S::STAGE_BYTES);
      tma_load_2d(smem_u32(st), &tmA, it * BK, m0, fb);
      tma_load_2d(smem_u32(st + S::A_BYTES), &tmA, it * BK, Mp + m0, fb);
      tma_load_2d(smem_u32(st + 2 * S::A_BYTES), &tmB, it * BK, n0, fb);
      tma_load_2d(smem_u32(st + 2 * S::A_BYTES + S::B_BYTES), &tmB, it * BK, Np + n0, fb);
    }
    // the loads of the last stages must land before the CTA can leave
    for (int j = it - STAGES; j < it; ++j)
      if (j >= 0) mbar_wait(full0 + 8 * (j % STAGES), (uint32_t)(j / STAGES) & 1u, err, 2);
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    constexpr uint32_t idesc = tf32_idesc(BM, BN);
    for (int it = 0; it < kiters; ++it) {
      const int s = it % STAGES;
      const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
      if (!mbar_wait(full0 + 8 * s, ph, err, 3)) {
        ok = false;
        break;
      }
      tc_fence_after();
      const uint32_t st = smem_u32(base + s * S::STAGE_BYTES);
      const uint32_t ahi = st, alo = st + S::A_BYTES, bhi = st + 2 * S::A_BYTES, blo = bhi + S::B_BYTES;
#pragma unroll
      for (int kk = 0; kk < BK / KSUB; ++kk) {
        const uint32_t koff = kk * KSUB * 4;  // bytes along the 128-byte swizzle row
        const uint32_t acc0 = (it > 0 || kk > 0) ? 1u : 0u;
        mma_tf32(tmem, sw128_desc(alo + koff), sw128_desc(bhi + koff), idesc, acc0);
        mma_tf32(tmem, sw128_desc(ahi + koff), sw128_desc(blo + koff), idesc, 1u);
        mma_tf32(tmem, sw128_desc(ahi + koff), sw128_desc(bhi + koff), idesc, 1u);
      }
      mma_commit(empty0 + 8 * s);  // the stage is free once these MMAs have read it
    }
    mma_commit(done);  // accumulator complete (also after an early stop: epilogue must not hang)
  }
  __syncwarp();

  // epilogue: warp w reads TMEM lanes 32w..32w+31 = tile rows
  const bool have = mbar_wait(done, 0, err, 4);
  tc_fence_after();
  // tcgen05.ld is warp-collective: the whole warp reads or none of it
  if (__all_sync(0xffffffffu, have && ok)) {
    const int row = m0 + warp * 32 + lane;
    const int64_t roff = row < M ? map_off(crow, row) : 0;
#pragma unroll 1
    for (int c = 0; c < BN; c += 32) {
      float v[32];
      tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
      if (row < M) {
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int col = n0 + c + j;
          if (col < N) C[roff + map_off(ccol, col)] = (double)v[j];
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 2) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
  (void)Np;
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  }
  return fn;
}

// 2-D map over a (2 * rows_p) x kp FP32 array, box 32 x box_rows, 128-byte swizzle.
bool make_map(CUtensorMap* map, const float* p, int64_t rows2, int64_t kp, int box_rows) {
  EncodeTiledFn enc = encode_fn();
  if (!enc) return false;
  cuuint64_t dims[2] = {(cuuint64_t)kp, (cuuint64_t)rows2};
  cuuint64_t strides[1] = {(cuuint64_t)kp * 4};
  cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
  cuuint32_t es[2] = {1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)p, dims, strides, box, es,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int BN, int STAGES>
cudaError_t launch_bn(const CUtensorMap& ta, const CUtensorMap& tb, int M, int N, int Mp, int Np, int kiters,
                      double* C, tci_map3 crow, tci_map3 ccol, int* err, cudaStream_t st) {
  using S = TcSmem<BN, STAGES>;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(tc_gemm_kernel<BN, STAGES>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         S::TOTAL);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  if (Mp / BM > 65535) return cudaErrorInvalidValue;
  dim3 grid((unsigned)(Np / BN), (unsigned)(Mp / BM));
  tc_gemm_kernel<BN, STAGES><<<grid, TC_THREADS, S::TOTAL, st>>>(ta, tb, M, N, Mp, Np, kiters, C, crow, ccol, err);
  return cudaGetLastError();
}

int64_t round_up(int64_t x, int64_t a) { return (x + a - 1) / a * a; }

int pick_bn(int64_t N) { return N <= 64 ? 64 : (N <= 128 ? 128 : 256); }

// FP64 check of a computed product at `ns` sampled entries (a splitmix64 hash
// of the sample number picks (m, n)): out[0] = max |C - exact|, out[1] = max
// |exact|, as bit patterns of non-negative doubles (atomicMax on the bits).
__global__ void sample_err_kernel(int64_t M, int64_t N, int64_t K, const double* __restrict__ A, tci_map3 a_row,
                                  tci_map3 a_k, const double* __restrict__ B, tci_map3 b_row, tci_map3 b_k,
                                  const double* __restrict__ C, tci_map3 c_row, tci_map3 c_col, int ns,
                                  uint64_t seed, unsigned long long* out) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= ns) return;
  uint64_t z = seed + 0x9E3779B97F4A7C15ULL * (uint64_t)(s + 1);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  z ^= z >> 31;
  const int64_t m = (int64_t)((z & 0xffffffffULL) % (uint64_t)M), n = (int64_t)((z >> 32) % (uint64_t)N);
  const int64_t ra = map_off(a_row, m), rb = map_off(b_row, n);
  double acc = 0.0;
  for (int64_t k = 0; k < K; ++k) acc += A[ra + map_off(a_k, k)] * B[rb + map_off(b_k, k)];
  const double d = fabs(C[map_off(c_row, m) + map_off(c_col, n)] - acc);
  atomicMax(out, (unsigned long long)__double_as_longlong(d));
  atomicMax(out + 1, (unsigned long long)__double_as_longlong(fabs(acc)));
}

}  // namespace

cudaError_t tci_tc_gemm_sample_error(int64_t M, int64_t N, int64_t K, const double* A, tci_map3 a_row,
                                     tci_map3 a_k, const double* B, tci_map3 b_row, tci_map3 b_k, const double* C,
                                     tci_map3 c_row, tci_map3 c_col, int nsample, uint64_t seed,
                                     unsigned long long* out2, cudaStream_t st) {
  if (M <= 0 || N <= 0 || nsample <= 0) return cudaSuccess;
  sample_err_kernel<<<(nsample + 127) / 128, 128, 0, st>>>(M, N, K, A, a_row, a_k, B, b_row, b_k, C, c_row, c_col,
                                                            nsample, seed, out2);
  return cudaGetLastError();
}

size_t tci_tc_gemm_workspace(int64_t M, int64_t N, int64_t K) {
  const int bn = pick_bn(N);
  const int64_t kp = round_up(K < 1 ? 1 : K, BK), mp = round_up(M, BM), np = round_up(N, bn);
  return (size_t)(2 * mp * kp + 2 * np * kp) * sizeof(float) + 256;
}

cudaError_t tci_tc_gemm_split(int64_t M, int64_t N, int64_t K, const double* A, tci_map3 a_row, tci_map3 a_k,
                              int a_kfast, const double* B, tci_map3 b_row, tci_map3 b_k, int b_kfast, double* C,
                              tci_map3 c_row, tci_map3 c_col, void* workspace, int* err_dev, cudaStream_t st) {
  if (M <= 0 || N <= 0) return cudaSuccess;
  const int bn = pick_bn(N);
  const int64_t kp = round_up(K < 1 ? 1 : K, BK), mp = round_up(M, BM), np = round_up(N, bn);
  if (mp > (1LL << 30) || np > (1LL << 30) || kp > (1LL << 30)) return cudaErrorInvalidValue;
  float* pa = (float*)(((uintptr_t)workspace + 255) & ~(uintptr_t)255);
  float* pb = pa + 2 * mp * kp;
  {
    dim3 g((unsigned)(kp / 32), (unsigned)(mp / 32 < 32768 ? mp / 32 : 32768));
    pack_split_kernel<<<g, 256, 0, st>>>(A, a_row, a_k, (int)M, (int)K, (int)mp, (int)kp, a_kfast, pa);
    dim3 h((unsigned)(kp / 32), (unsigned)(np / 32 < 32768 ? np / 32 : 32768));
    pack_split_kernel<<<h, 256, 0, st>>>(B, b_row, b_k, (int)N, (int)K, (int)np, (int)kp, b_kfast, pb);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  CUtensorMap ta, tb;
  if (!make_map(&ta, pa, 2 * mp, kp, BM) || !make_map(&tb, pb, 2 * np, kp, bn)) return cudaErrorInvalidValue;
  const int kiters = (int)(kp / BK);
  switch (bn) {
    case 64: return launch_bn<64, 4>(ta, tb, (int)M, (int)N, (int)mp, (int)np, kiters, C, c_row, c_col, err_dev, st);
    case 128: return launch_bn<128, 3>(ta, tb, (int)M, (int)N, (int)mp, (int)np, kiters, C, c_row, c_col, err_dev, st);
    default: return launch_bn<256, 2>(ta, tb, (int)M, (int)N, (int)mp, (int)np, kiters, C, c_row, c_col, err_dev, st);
  }
}

// ============================================================================
// Split-precision evaluation of a tensor train at many points
// (abstracttensortrain.jl:124-132: evaluate(tt, indexset) = only(prod of
// T_b[:, i_b, :])) on the tensor cores.
//
// One CTA runs 128-point tiles (persistent over tiles).  The running row
// vectors of its 128 points are a 128 x r tile V kept in shared memory as TF32
// hi/lo, K-major with the 128-byte swizzle.  For site b and every local value
// i the tensor cores form D_i = V * T_b[:, i, :] (3 split products per 8-deep
// K slice) into tensor-memory columns [i r1p, (i+1) r1p); each point then takes
// the block of its own local index i_b, and the epilogue writes it back into V
// (split again) for the next site.  The core slices T_b[:, i, :]^T come from a
// once-packed buffer of pre-swizzled TF32 hi/lo images, one per (b, i, 32-deep
// K chunk), copied whole into a two-stage shared-memory ring by bulk async
// copies (cp.async.bulk) that a producer warp issues ahead of the MMA warp.
//   warps 0-3: epilogue (warp w owns tensor-memory lanes / tile rows 32w..)
//   warp 4   : producer (one thread)
//   warp 5   : MMA issuer (one thread)
// Synchronisation is by mbarriers only: full/empty per stage, d_full (the MMAs
// of a site are complete), v_ready (128 arrivals: V holds the next site's rows).
// Limits: bonds <= 128, d * roundup(r_b, 16) <= 512 tensor-memory columns.
// ============================================================================

namespace {

constexpr int EV_EPI_THREADS = 128;
constexpr int EV_THREADS = 192;
constexpr int EV_RMAX = 128;                       // bond limit
constexpr int EV_KC_MAX = EV_RMAX / BK;            // 4 chunks of 32
constexpr int EV_CHUNK_BYTES = BM * 128;           // 16 KB: 128 rows x 128 B
constexpr int EV_STAGES = 2;
constexpr int EV_IMG_MAX = EV_RMAX * 128;          // one image: r1p rows x 128 B
constexpr int EV_STAGE_BYTES = 2 * EV_IMG_MAX;     // hi + lo
constexpr int EV_V_BYTES = 2 * EV_KC_MAX * EV_CHUNK_BYTES;  // hi chunks then lo chunks
constexpr int EV_SMEM = 1024 + EV_V_BYTES + EV_STAGES * EV_STAGE_BYTES + 256;

__device__ __forceinline__ void bulk_copy(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"((uint64_t)src), "r"(bytes), "r"(bar)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane (warp-collective).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Byte offset of element (row, k) inside a 128-row image of 128-byte rows with
// the 128-byte swizzle (16-byte granule index XOR row % 8), k < 32.
__device__ __forceinline__ uint32_t sw128_off(int row, int k) {
  return (uint32_t)row * 128u + ((((uint32_t)k >> 2) ^ ((uint32_t)row & 7u)) << 4) + (((uint32_t)k & 3u) << 2);
}

__device__ __forceinline__ void split_tf32f(float x, float& hi, float& lo) {
  uint32_t h, l;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(x));
  hi = __uint_as_float(h);
  const float r = x - hi;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(l) : "f"(r));
  lo = __uint_as_float(l);
}

// Packs core b (r0 x d x r1, column-major FP64) into its images: for each local
// value i and 32-deep chunk kc of the input bond, the hi image then the lo image
// of T_b[kc*32 .. +32, i, 0 .. r1p)^T (rows = output bond index, zero padded).
__global__ void ev_pack_kernel(const double* __restrict__ core, int r0, int d, int r1, int r1p, int nkc,
                               uint8_t* __restrict__ img) {
  const int64_t total = (int64_t)d * nkc * r1p * 32;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(e % 32);
    int64_t q = e / 32;
    const int n = (int)(q % r1p);
    q /= r1p;
    const int kc = (int)(q % nkc);
    const int i = (int)(q / nkc);
    const int a = kc * 32 + k;
    const double v = (a < r0 && n < r1) ? core[a + (int64_t)r0 * (i + (int64_t)d * n)] : 0.0;
    float hi, lo;
    split_tf32(v, hi, lo);
    uint8_t* base = img + ((int64_t)(i * nkc + kc) * 2) * r1p * 128;
    *(float*)(base + sw128_off(n, k)) = hi;
    *(float*)(base + (int64_t)r1p * 128 + sw128_off(n, k)) = lo;
  }
}

struct EvSite {
  const double* core;  // FP64 core (site 0 only)
  const uint8_t* img;  // packed images (sites >= 1)
  int r0, d, r1, r1p, nkc;
};

__global__ void __launch_bounds__(EV_THREADS, 1)
    tc_eval_kernel(const EvSite* __restrict__ sites, int L, const uint8_t* __restrict__ pts, int64_t np,
                   double* __restrict__ out, int* err) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* base = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint8_t* V = base;                               // hi chunks [0, 4), lo chunks [4, 8)
  uint8_t* stages = base + EV_V_BYTES;
  // full[2], empty[2], d_full, v_ready, mma_end
  uint64_t* bars = (uint64_t*)(stages + EV_STAGES * EV_STAGE_BYTES);
  uint32_t* tmem_slot = (uint32_t*)(bars + 2 * EV_STAGES + 3);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + EV_STAGES);
  const uint32_t d_full = smem_u32(bars + 2 * EV_STAGES), v_ready = smem_u32(bars + 2 * EV_STAGES + 1);
  const uint32_t mma_end = smem_u32(bars + 2 * EV_STAGES + 2);
  const int64_t ntiles = (np + BM - 1) / BM;

  if (threadIdx.x == 0) {
    for (int s = 0; s < 2 * EV_STAGES; ++s) mbar_init(smem_u32(bars + s), 1);
    mbar_init(d_full, 1);
    mbar_init(v_ready, EV_EPI_THREADS);
    mbar_init(mma_end, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(512)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 4) {
    if (lane == 0) {  // producer
      int it = 0;
      bool ok = true;
      for (int64_t t = blockIdx.x; t < ntiles && ok; t += gridDim.x)
        for (int b = 1; b < L && ok; ++b) {
          const EvSite S = sites[b];
          const uint32_t img_bytes = (uint32_t)S.r1p * 128u;
          for (int i = 0; i < S.d && ok; ++i)
            for (int kc = 0; kc < S.nkc; ++kc, ++it) {
              const int s = it % EV_STAGES;
              if (!mbar_wait(empty0 + 8 * s, ((uint32_t)(it / EV_STAGES) & 1u) ^ 1u, err, 11)) {
                ok = false;
                break;
              }
              const uint32_t fb = full0 + 8 * s;
              const uint8_t* src = S.img + (int64_t)((i * S.nkc + kc) * 2) * img_bytes;
              const uint32_t dst = smem_u32(stages + s * EV_STAGE_BYTES);
              mbar_expect_tx(fb, 2 * img_bytes);
              bulk_copy(dst, src, img_bytes, fb);
              bulk_copy(dst + EV_IMG_MAX, src + img_bytes, img_bytes, fb);
            }
        }
      for (int j = it - EV_STAGES; j < it; ++j)  // in-flight copies land before the CTA leaves
        if (j >= 0) mbar_wait(full0 + 8 * (j % EV_STAGES), (uint32_t)(j / EV_STAGES) & 1u, err, 12);
    }
  } else if (warp == 5) {
    if (lane == 0) {  // MMA issuer
      int it = 0, site_it = 0;
      bool ok = true;
      for (int64_t t = blockIdx.x; t < ntiles && ok; t += gridDim.x)
        for (int b = 1; b < L && ok; ++b, ++site_it) {
          const EvSite S = sites[b];
          if (!mbar_wait(v_ready, (uint32_t)site_it & 1u, err, 13)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t idesc = tf32_idesc(BM, S.r1p);
          const uint32_t vh = smem_u32(V), vl = smem_u32(V + EV_KC_MAX * EV_CHUNK_BYTES);
          for (int i = 0; i < S.d && ok; ++i) {
            const uint32_t dcol = tmem + (uint32_t)(i * S.r1p);
            for (int kc = 0; kc < S.nkc; ++kc, ++it) {
              const int s = it % EV_STAGES;
              if (!mbar_wait(full0 + 8 * s, (uint32_t)(it / EV_STAGES) & 1u, err, 14)) {
                ok = false;
                break;
              }
              tc_fence_after();
              const uint32_t bh = smem_u32(stages + s * EV_STAGE_BYTES), bl = bh + EV_IMG_MAX;
              const uint32_t ah = vh + kc * EV_CHUNK_BYTES, al = vl + kc * EV_CHUNK_BYTES;
#pragma unroll
              for (int kk = 0; kk < BK / KSUB; ++kk) {
                const uint32_t ko = kk * KSUB * 4;
                mma_tf32(dcol, sw128_desc(al + ko), sw128_desc(bh + ko), idesc, (kc > 0 || kk > 0) ? 1u : 0u);
                mma_tf32(dcol, sw128_desc(ah + ko), sw128_desc(bl + ko), idesc, 1u);
                mma_tf32(dcol, sw128_desc(ah + ko), sw128_desc(bh + ko), idesc, 1u);
              }
              mma_commit(empty0 + 8 * s);
            }
          }
          mma_commit(d_full);
        }
      // every MMA of this thread has completed before tensor memory is released
      mma_commit(mma_end);
      mbar_wait(mma_end, 0, err, 16);
    }
  } else {
    // epilogue warps 0-3: row = threadIdx.x
    const int row = threadIdx.x;
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    uint8_t* Vh = V;
    uint8_t* Vl = V + EV_KC_MAX * EV_CHUNK_BYTES;
    int site_it = 0;
    bool ok = true;
    for (int64_t t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
      const int64_t p = t * BM + row;
      const bool live = p < np;
      const uint8_t* ip = pts + (live ? p : 0) * L;
      // site 0: V[row, :] = T_0[0, i_0, :]
      {
        const EvSite S = sites[0];
        const int i0 = live ? ip[0] : 0;
        const int r1 = S.r1;
        if (L == 1) {
          if (live) out[p] = S.core[i0];
        } else {
          const int kp = sites[1].nkc * 32;
          for (int c = 0; c < kp; ++c) {
            const double v = (live && c < r1) ? S.core[i0 + (int64_t)S.d * c] : 0.0;
            float hi, lo;
            split_tf32(v, hi, lo);
            const uint32_t o = (uint32_t)(c >> 5) * EV_CHUNK_BYTES + sw128_off(row, c & 31);
            *(float*)(Vh + o) = hi;
            *(float*)(Vl + o) = lo;
          }
          tc_fence_before();
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          mbar_arrive(v_ready);
        }
      }
      for (int b = 1; b < L; ++b, ++site_it) {
        const EvSite S = sites[b];
        const bool have = mbar_wait(d_full, (uint32_t)site_it & 1u, err, 15);
        if (!__all_sync(0xffffffffu, have)) {
          ok = false;  // a wait ran out: stop this warp (the others time out too)
          break;
        }
        tc_fence_after();
        const int ib = live ? ip[b] : 0;
        if (b == L - 1) {
          // r1 = 1: column 0 of the point's block
          float acc = 0.f;
          if (ok)
            for (int i = 0; i < S.d; ++i) {
              float v[16];
              tmem_ld16(lane_base + (uint32_t)(i * S.r1p), v);
              if (i == ib) acc = v[0];
            }
          if (live) out[p] = (double)acc;
        } else {
          const int kp = sites[b + 1].nkc * 32;  // next site's padded input bond
          for (int c = 0; c < S.r1p; c += 16) {
            float sel[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) sel[j] = 0.f;
            if (ok)
              for (int i = 0; i < S.d; ++i) {
                float v[16];
                tmem_ld16(lane_base + (uint32_t)(i * S.r1p + c), v);
                if (i == ib) {
#pragma unroll
                  for (int j = 0; j < 16; ++j) sel[j] = v[j];
                }
              }
#pragma unroll
            for (int j = 0; j < 16; ++j) {
              const int col = c + j;
              if (col < kp) {
                float hi, lo;
                split_tf32f(col < S.r1 ? sel[j] : 0.f, hi, lo);
                const uint32_t o = (uint32_t)(col >> 5) * EV_CHUNK_BYTES + sw128_off(row, col & 31);
                *(float*)(Vh + o) = hi;
                *(float*)(Vl + o) = lo;
              }
            }
          }
          for (int col = S.r1p; col < kp; ++col) {  // zero padding up to the next chunk edge
            const uint32_t o = (uint32_t)(col >> 5) * EV_CHUNK_BYTES + sw128_off(row, col & 31);
            *(float*)(Vh + o) = 0.f;
            *(float*)(Vl + o) = 0.f;
          }
          tc_fence_before();
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          mbar_arrive(v_ready);
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512) : "memory");
  }
}

// FP64 evaluation of the train at the first `ns` points (one thread per point,
// left to right, as abstracttensortrain.jl:124-132), for the error estimate.
__global__ void ev_fp64_kernel(const EvSite* __restrict__ sites, const double* const* __restrict__ cores, int L,
                               const uint8_t* __restrict__ pts, int ns, double* __restrict__ out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= ns) return;
  double v[EV_RMAX], w[EV_RMAX];
  v[0] = 1.0;
  int r0 = 1;
  for (int b = 0; b < L; ++b) {
    const EvSite S = sites[b];
    const double* T = cores[b];
    const int i = pts[(int64_t)p * L + b];
    for (int c = 0; c < S.r1; ++c) {
      double acc = 0.0;
      for (int a = 0; a < r0; ++a) acc += v[a] * T[a + (int64_t)r0 * (i + (int64_t)S.d * c)];
      w[c] = acc;
    }
    for (int c = 0; c < S.r1; ++c) v[c] = w[c];
    r0 = S.r1;
  }
  out[p] = v[0];
}

}  // namespace

bool tci_tc_eval_supported(int L, const int64_t* dims) {
  for (int b = 0; b < L; ++b) {
    const int64_t r0 = dims[3 * b], d = dims[3 * b + 1], r1 = dims[3 * b + 2];
    if (r0 > EV_RMAX || r1 > EV_RMAX || d < 1 || d > 256) return false;
    if (b > 0 && d * round_up(r1, 16) > 512) return false;
  }
  return dims[0] == 1 && dims[3 * (L - 1) + 2] == 1;
}

size_t tci_tc_eval_workspace(int L, const int64_t* dims) {
  size_t bytes = 256 + (size_t)L * sizeof(EvSite) + (size_t)L * sizeof(double*);
  for (int b = 1; b < L; ++b) {
    const int64_t r0 = dims[3 * b], d = dims[3 * b + 1], r1 = dims[3 * b + 2];
    const int64_t nkc = round_up(r0, 32) / 32, r1p = round_up(r1, 16);
    bytes += (size_t)(d * nkc * 2 * r1p * 128) + 1024;
  }
  return bytes;
}

cudaError_t tci_tc_evaluate_split(int L, const int64_t* dims, const double* const* cores_dev, const uint8_t* pts_dev,
                                  int64_t np, double* out_dev, int nsample, double* sample_out_dev, void* workspace,
                                  int* err_dev, int nsm, cudaStream_t st) {
  // workspace: [site table][core pointer table][images...]
  uint8_t* ws = (uint8_t*)(((uintptr_t)workspace + 255) & ~(uintptr_t)255);
  EvSite* sites_dev = (EvSite*)ws;
  const double** cptr_dev = (const double**)(ws + (size_t)L * sizeof(EvSite));
  uint8_t* img = (uint8_t*)(((uintptr_t)(cptr_dev + L) + 1023) & ~(uintptr_t)1023);
  EvSite host[64];
  if (L > 64) return cudaErrorInvalidValue;
  for (int b = 0; b < L; ++b) {
    EvSite& S = host[b];
    S.core = cores_dev[b];
    S.r0 = (int)dims[3 * b];
    S.d = (int)dims[3 * b + 1];
    S.r1 = (int)dims[3 * b + 2];
    S.r1p = (int)round_up(S.r1, 16);
    S.nkc = (int)(round_up(S.r0, 32) / 32);
    S.img = nullptr;
    if (b > 0) {
      S.img = img;
      const int64_t total = (int64_t)S.d * S.nkc * S.r1p * 32;
      ev_pack_kernel<<<(unsigned)std::min<int64_t>((total + 255) / 256, 4096), 256, 0, st>>>(
          cores_dev[b], S.r0, S.d, S.r1, S.r1p, S.nkc, img);
      img += (size_t)(S.d * S.nkc * 2 * S.r1p * 128);
      img = (uint8_t*)(((uintptr_t)img + 1023) & ~(uintptr_t)1023);
    }
  }
  cudaError_t e = cudaMemcpyAsync(sites_dev, host, (size_t)L * sizeof(EvSite), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(cptr_dev, cores_dev, (size_t)L * sizeof(double*), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  static bool attr = false;
  if (!attr) {
    e = cudaFuncSetAttribute(tc_eval_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, EV_SMEM);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  const int64_t ntiles = (np + BM - 1) / BM;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(ntiles, nsm));
  if (np > 0) tc_eval_kernel<<<grid, EV_THREADS, EV_SMEM, st>>>(sites_dev, L, pts_dev, np, out_dev, err_dev);
  if (nsample > 0)
    ev_fp64_kernel<<<(nsample + 63) / 64, 64, 0, st>>>(sites_dev, cptr_dev, L, pts_dev, nsample, sample_out_dev);
  return cudaGetLastError();
}
