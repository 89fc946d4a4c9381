// mlp.cu -- BF16 tensor-core kernels of the learned focusing + scattering
// surrogate (no counterpart in the reference).
//
// k_gemm_bf16: C[M x N] = A[M x K] * Bt[N x K]^T (+ bias[N]), A and Bt bf16
// with K contiguous, C fp32, on the 5th-generation tensor cores:
//   * a CTA owns a 128-row x NT-column tile of C; its accumulator lives in
//     tensor memory (TMEM, NT fp32 columns of 128 lanes: row i = lane i);
//   * K is walked in chunks of 64: the 128 threads copy the A and Bt chunks
//     from global memory into shared memory in the no-swizzle K-major
//     "core matrix" layout (8 rows x 16 bytes per 128-byte core matrix; core
//     (row group g, k group h) at g * 1024 + h * 128 bytes), then one thread
//     issues four tcgen05.mma (K = 16 each) and commits them to an mbarrier
//     that every thread waits on before the next chunk overwrites the tiles;
//   * the epilogue: warp w reads TMEM lanes 32w..32w+31 (its rows) with
//     tcgen05.ld, adds the bias and stores fp32.
// Every wait is bounded: on time-out the kernel records an error code,
// frees its TMEM and returns.  Shapes: M any, N any (tiles of up to 256
// columns), K a multiple of 8 with lda, ldb multiples of 8 (16-byte rows).
#include <cuda_bf16.h>

#include "common.cuh"
#include "kernels.h"

namespace eprem {

constexpr int kGemmThreads = 128;
constexpr int kTileM = 128;
constexpr int kTileK = 64;
constexpr uint32_t kLbo = 128;    // bytes between core matrices adjacent in K
constexpr uint32_t kSbo = 1024;   // bytes between 8-row groups (kTileK / 8 cores)
constexpr int kWaitLimit = 1 << 22;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint32_t core_offset(int row, int k) {
  return (uint32_t)((row >> 3) * kSbo + (k >> 3) * kLbo + (row & 7) * 16 + (k & 7) * 2);
}

// Shared-memory matrix descriptor: start, leading (K) and stride (row-group)
// byte offsets in 16-byte units, descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((kLbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((kSbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1u << 46;
  return d;
}

// Instruction descriptor of kind::f16: fp32 D, bf16 A and B, both K-major,
// N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t phase) {
  for (int i = 0; i < kWaitLimit; i++) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(mbar), "r"(phase)
        : "memory");
    if (done) return true;
    if (i > 64) __nanosleep(64);
  }
  return false;
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

template <int NT>
__global__ void __launch_bounds__(kGemmThreads)
    k_gemm_bf16(const __nv_bfloat16 *__restrict__ A, int lda, const __nv_bfloat16 *__restrict__ Bt,
                int ldb, const float *__restrict__ bias, float *__restrict__ C, int ldc, int M,
                int N, int K, int *err) {
  static_assert(NT % 16 == 0 && NT >= 16 && NT <= 256, "N tile");
  constexpr uint32_t TCOLS = NT <= 32 ? 32 : NT <= 64 ? 64 : NT <= 128 ? 128 : 256;
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_base;
  uint8_t *sA = smem;
  uint8_t *sB = smem + kTileM * kTileK * 2;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * kTileM, n0 = blockIdx.y * NT;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base)),
                 "r"(TCOLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;
  const uint32_t mb = smem_u32(&mbar);
  const uint32_t idesc = idesc_bf16(kTileM, NT);
  uint32_t phase = 0;
  bool ok = true;

  for (int k0 = 0; k0 < K && ok; k0 += kTileK) {
    // A chunk: 128 rows x 8 vectors of 8 bf16
    for (int v = tid; v < kTileM * (kTileK / 8); v += kGemmThreads) {
      const int row = v >> 3, kg = v & 7, k = k0 + kg * 8, gr = m0 + row;
      uint4 val = make_uint4(0u, 0u, 0u, 0u);
      if (gr < M && k < K) val = *reinterpret_cast<const uint4 *>(A + (size_t)gr * lda + k);
      *reinterpret_cast<uint4 *>(sA + core_offset(row, kg * 8)) = val;
    }
    for (int v = tid; v < NT * (kTileK / 8); v += kGemmThreads) {
      const int row = v >> 3, kg = v & 7, k = k0 + kg * 8, gn = n0 + row;
      uint4 val = make_uint4(0u, 0u, 0u, 0u);
      if (gn < N && k < K) val = *reinterpret_cast<const uint4 *>(Bt + (size_t)gn * ldb + k);
      *reinterpret_cast<uint4 *>(sB + core_offset(row, kg * 8)) = val;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
      const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
#pragma unroll
      for (int kk = 0; kk < kTileK / 16; kk++) {
        const uint64_t ad = smem_desc(a0 + kk * 2 * kLbo);
        const uint64_t bd = smem_desc(b0 + kk * 2 * kLbo);
        const uint32_t acc = (k0 > 0 || kk > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
            : "memory");
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mb)
          : "memory");
    }
    // block-uniform outcome: every thread leaves the loop together
    ok = __syncthreads_and(mbar_wait(mb, phase) ? 1 : 0) != 0;
    if (!ok) {
      if (tid == 0) atomicCAS(err, 0, 1);
      // the MMAs already committed still write TMEM: wait for them once
      // more (bounded) before the allocation is released below
      mbar_wait(mb, phase);
    }
    phase ^= 1u;
    tc_fence_after();
    __syncthreads();
  }

  if (ok) {
    const int row = m0 + warp * 32 + lane;
#pragma unroll 1
    for (int c = 0; c < NT; c += 8) {
      uint32_t r[8];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
            "=r"(r[7])
          : "r"(taddr)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (row < M) {
#pragma unroll
        for (int j = 0; j < 8; j++) {
          const int col = n0 + c + j;
          if (col < N) C[(size_t)row * ldc + col] = __uint_as_float(r[j]) + (bias ? bias[col] : 0.f);
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TCOLS)
                 : "memory");
}

template <int NT>
static cudaError_t launch_gemm_t(const void *A, int lda, const void *Bt, int ldb,
                                 const float *bias, float *C, int ldc, int M, int N, int K,
                                 int *err, cudaStream_t st) {
  const size_t smem = (size_t)(kTileM + NT) * kTileK * 2;
  auto kern = k_gemm_bf16<NT>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  dim3 grid((M + kTileM - 1) / kTileM, (N + NT - 1) / NT);
  kern<<<grid, kGemmThreads, smem, st>>>(static_cast<const __nv_bfloat16 *>(A), lda,
                                         static_cast<const __nv_bfloat16 *>(Bt), ldb, bias, C,
                                         ldc, M, N, K, err);
  return cudaGetLastError();
}

int launch_gemm_bf16(const void *A, int lda, const void *Bt, int ldb, const float *bias,
                     float *C, int ldc, int M, int N, int K, int *err, cudaStream_t st) {
  if (M <= 0 || N <= 0 || K <= 0 || K % 8 || lda % 8 || ldb % 8 || lda < K || ldb < K ||
      ldc < N)
    return EPREM_GPU_ERR_ARG;
  cudaError_t e;
  if (N <= 16)
    e = launch_gemm_t<16>(A, lda, Bt, ldb, bias, C, ldc, M, N, K, err, st);
  else if (N <= 32)
    e = launch_gemm_t<32>(A, lda, Bt, ldb, bias, C, ldc, M, N, K, err, st);
  else if (N <= 64)
    e = launch_gemm_t<64>(A, lda, Bt, ldb, bias, C, ldc, M, N, K, err, st);
  else if (N <= 128)
    e = launch_gemm_t<128>(A, lda, Bt, ldb, bias, C, ldc, M, N, K, err, st);
  else
    e = launch_gemm_t<256>(A, lda, Bt, ldb, bias, C, ldc, M, N, K, err, st);
  return e == cudaSuccess ? 0 : EPREM_GPU_ERR_CUDA;
}

}  // namespace eprem
