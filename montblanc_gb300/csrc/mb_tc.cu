// Tensor-core diagnostics: a one-CTA split-precision GEMM that exercises
// exactly the operand staging (no-swizzle K-major core-matrix layout),
// descriptors, tcgen05.mma, commit and TMEM readout used by the fused
// split-precision coherency kernel in mb_fused.cu.
#include "mb_fused.h"
#include "mb_tc_layout.cuh"
#include "mb_tcgen05.cuh"

namespace mb {

namespace {

// D (128 x 128) = A (128 x K) . B (128 x K)^T, both row-major FP32, K a
// multiple of 32; split into hi + lo parts, 3 products, FP32 accumulation.
// Threads 0..127 stage operands and read TMEM; warp 4 issues the MMAs.
template <int MODE>
__global__ void __launch_bounds__(160) tc_selftest_kernel(const float* __restrict__ A, const float* __restrict__ B,
                                                          int K, float* __restrict__ D, int* __restrict__ status) {
  extern __shared__ __align__(1024) unsigned char smem[];
  using L = StageLayout<MODE, 128>;
  unsigned char* sA_hi = smem;
  unsigned char* sA_lo = smem + L::kMatBytes;
  unsigned char* sB_hi = smem + 2 * L::kMatBytes;
  unsigned char* sB_lo = smem + 3 * L::kMatBytes;
  __shared__ uint64_t bar_mma;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar_mma, 1);
    abort_flag = 0;
  }
  if (warp == 4) tc::tmem_alloc(&tmem_base, 128);
  tc::fence_before_thread_sync();
  __syncthreads();
  tc::fence_after_thread_sync();
  const uint32_t tmem = tmem_base;
  const uint32_t idesc = L::instr(128, 128);
  int phase = 0;
  for (int k0 = 0; k0 < K; k0 += L::kKT) {
    if (threadIdx.x < 128) {
      const int r = threadIdx.x;
      for (int k = 0; k < L::kKT; ++k) {
        L::put(sA_hi, sA_lo, r, k, A[size_t(r) * K + k0 + k]);
        L::put(sB_hi, sB_lo, r, k, B[size_t(r) * K + k0 + k]);
      }
      tc::fence_proxy_async_smem();
    }
    __syncthreads();
    if (warp == 4 && lane == 0) {
      tc::fence_after_thread_sync();
      for (int kk = 0; kk < L::kKSteps; ++kk) {
        const uint32_t off = kk * L::kKStepBytes;
        uint64_t ah = L::desc(tc::smem_addr(sA_hi) + off), al = L::desc(tc::smem_addr(sA_lo) + off);
        uint64_t bh = L::desc(tc::smem_addr(sB_hi) + off), bl = L::desc(tc::smem_addr(sB_lo) + off);
        L::mma(tmem, ah, bh, idesc, (k0 > 0 || kk > 0) ? 1u : 0u);
        L::mma(tmem, ah, bl, idesc, 1u);
        L::mma(tmem, al, bh, idesc, 1u);
      }
      tc::mma_commit(&bar_mma);
      if (!tc::mbar_wait(&bar_mma, phase)) atomicExch(&abort_flag, 1);
    }
    phase ^= 1;
    __syncthreads();  // operands may be overwritten only after the MMAs finished
  }
  tc::fence_after_thread_sync();
  if (warp < 4) {
    const int r = warp * 32 + lane;
    for (int c0 = 0; c0 < 128; c0 += 32) {
      float v[32];
      tc::tmem_ld32(tmem + (uint32_t(warp * 32) << 16) + c0, v);
      for (int i = 0; i < 32; ++i) D[size_t(r) * 128 + c0 + i] = v[i];
    }
  }
  tc::fence_before_thread_sync();
  __syncthreads();
  if (warp == 4) tc::tmem_dealloc(tmem, 128);
  if (threadIdx.x == 0 && abort_flag) *status = 1;
}

// The BF16 product with the A operand (hi and lo parts) in TMEM: each row's
// lane stores its K values as bf16 pairs (even K index in the low half of a
// 32-bit column); B is staged in shared memory as above.  Same roles: threads
// 0..127 stage and read TMEM, warp 4 issues the MMAs.
__global__ void __launch_bounds__(160) tc_selftest_ta_kernel(const float* __restrict__ A, const float* __restrict__ B,
                                                             int K, float* __restrict__ D, int* __restrict__ status) {
  extern __shared__ __align__(1024) unsigned char smem[];
  using L = StageLayout<MB_MODE_SPLIT_BF16, 128>;
  unsigned char* sB_hi = smem;
  unsigned char* sB_lo = smem + L::kMatBytes;
  __shared__ uint64_t bar_mma;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar_mma, 1);
    abort_flag = 0;
  }
  if (warp == 4) tc::tmem_alloc(&tmem_base, 256);
  tc::fence_before_thread_sync();
  __syncthreads();
  tc::fence_after_thread_sync();
  const uint32_t tmem = tmem_base;
  const uint32_t tD = tmem, tAh = tmem + 128, tAl = tmem + 160;  // A: 64 K values = 32 columns each
  const uint32_t idesc = L::instr(128, 128);
  int phase = 0;
  for (int k0 = 0; k0 < K; k0 += L::kKT) {
    if (threadIdx.x < 128) {
      const int r = threadIdx.x;
      for (int k = 0; k < L::kKT; ++k) L::put(sB_hi, sB_lo, r, k, B[size_t(r) * K + k0 + k]);
      uint32_t hw[32], lw[32];
#pragma unroll
      for (int c = 0; c < 32; ++c) {
        __nv_bfloat16 h0, l0, h1, l1;
        tc::split_bf16(A[size_t(r) * K + k0 + 2 * c], h0, l0);
        tc::split_bf16(A[size_t(r) * K + k0 + 2 * c + 1], h1, l1);
        hw[c] = uint32_t(__bfloat16_as_ushort(h0)) | (uint32_t(__bfloat16_as_ushort(h1)) << 16);
        lw[c] = uint32_t(__bfloat16_as_ushort(l0)) | (uint32_t(__bfloat16_as_ushort(l1)) << 16);
      }
      const uint32_t lanes = uint32_t(32 * warp) << 16;
      tc::tmem_st32(tAh + lanes, hw);
      tc::tmem_st32(tAl + lanes, lw);
      tc::tmem_wait_st();
      tc::fence_proxy_async_smem();
    }
    tc::fence_before_thread_sync();
    __syncthreads();
    if (warp == 4 && lane == 0) {
      tc::fence_after_thread_sync();
      for (int kk = 0; kk < L::kKSteps; ++kk) {
        const uint32_t off = kk * L::kKStepBytes;
        const uint64_t bh = L::desc(tc::smem_addr(sB_hi) + off), bl = L::desc(tc::smem_addr(sB_lo) + off);
        tc::mma_f16_ta(tD, tAh + 8 * kk, bh, idesc, (k0 > 0 || kk > 0) ? 1u : 0u);
        tc::mma_f16_ta(tD, tAh + 8 * kk, bl, idesc, 1u);
        tc::mma_f16_ta(tD, tAl + 8 * kk, bh, idesc, 1u);
      }
      tc::mma_commit(&bar_mma);
      if (!tc::mbar_wait(&bar_mma, phase)) atomicExch(&abort_flag, 1);
    }
    phase ^= 1;
    tc::fence_before_thread_sync();
    __syncthreads();  // A and B may be overwritten only after the MMAs finished
    tc::fence_after_thread_sync();
  }
  if (warp < 4) {
    const int r = warp * 32 + lane;
    for (int c0 = 0; c0 < 128; c0 += 32) {
      float v[32];
      tc::tmem_ld32(tD + (uint32_t(warp * 32) << 16) + c0, v);
      for (int i = 0; i < 32; ++i) D[size_t(r) * 128 + c0 + i] = v[i];
    }
  }
  tc::fence_before_thread_sync();
  __syncthreads();
  if (warp == 4) tc::tmem_dealloc(tmem, 256);
  if (threadIdx.x == 0 && abort_flag) *status = 1;
}

// A wait that cannot complete: the mbarrier's phase 0 needs one arrival and
// none comes, so the bounded wait gives up after `limit` polls; the kernel
// records it and frees its TMEM like the fused kernels' abort path.
__global__ void wait_selftest_kernel(uint32_t limit, int* status) {
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_slot;
  const int warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) tc::mbar_init(&bar, 1);
  tc::fence_proxy_async_smem();
  if (warp == 0) tc::tmem_alloc(&tmem_slot, 32);
  tc::fence_before_thread_sync();
  __syncthreads();
  tc::fence_after_thread_sync();
  const bool ok = warp == 0 ? tc::mbar_wait(&bar, 0, limit) : true;
  if (!ok && threadIdx.x == 0) *status = 1;
  tc::fence_before_thread_sync();
  __syncthreads();
  tc::fence_after_thread_sync();
  if (warp == 0) tc::tmem_dealloc(tmem_slot, 32);
}

}  // namespace

}  // namespace mb

using namespace mb;

extern "C" {

mb_status mb_tc_selftest(const float* A, const float* B, int K, int mode, float* D, int* status, void* stream) {
  MB_REQUIRE(A, "A"); MB_REQUIRE(B, "B"); MB_REQUIRE(D, "D"); MB_REQUIRE(status, "status");
  const int kt = (mode & ~MB_TC_SELFTEST_A_IN_TMEM) == MB_MODE_SPLIT_BF16 ? 64 : 32;
  if (K <= 0 || K % kt != 0) return fail(MB_ERR_INVALID_ARG, "K must be a positive multiple of %d (got %d)", kt, K);
  cudaStream_t s = as_stream(stream);
  if (mode == MB_MODE_SPLIT_TF32) {
    const size_t smem = 4 * StageLayout<MB_MODE_SPLIT_TF32, 128>::kMatBytes;
    MB_CUDA(cudaFuncSetAttribute(tc_selftest_kernel<MB_MODE_SPLIT_TF32>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    {
      KernelScope ks_("tc_selftest_kernel", s);
      tc_selftest_kernel<MB_MODE_SPLIT_TF32><<<1, 160, smem, s>>>(A, B, K, D, status);
    }
  } else if (mode == (MB_MODE_SPLIT_BF16 | MB_TC_SELFTEST_A_IN_TMEM)) {
    const size_t smem = 2 * StageLayout<MB_MODE_SPLIT_BF16, 128>::kMatBytes;
    MB_CUDA(cudaFuncSetAttribute(tc_selftest_ta_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    {
      KernelScope ks_("tc_selftest_kernel", s);
      tc_selftest_ta_kernel<<<1, 160, smem, s>>>(A, B, K, D, status);
    }
  } else if (mode == MB_MODE_SPLIT_BF16) {
    const size_t smem = 4 * StageLayout<MB_MODE_SPLIT_BF16, 128>::kMatBytes;
    MB_CUDA(cudaFuncSetAttribute(tc_selftest_kernel<MB_MODE_SPLIT_BF16>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    {
      KernelScope ks_("tc_selftest_kernel", s);
      tc_selftest_kernel<MB_MODE_SPLIT_BF16><<<1, 160, smem, s>>>(A, B, K, D, status);
    }
  } else {
    return fail(MB_ERR_INVALID_ARG, "mode must be a split-precision mode");
  }
  return check_launch("tc_selftest_kernel");
}

mb_status mb_wait_selftest(uint32_t poll_limit, int* status, void* stream) {
  MB_REQUIRE(status, "status");
  cudaStream_t s = as_stream(stream);
  {
    KernelScope ks_("wait_selftest_kernel", s);
    wait_selftest_kernel<<<1, 64, 0, s>>>(poll_limit, status);
  }
  return check_launch("wait_selftest_kernel");
}

}  // extern "C"
