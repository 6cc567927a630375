// Shared-memory operand layout of one split-precision stage.
//
// An operand matrix has 128 rows (M or N) and ROWB bytes of K per row
// (ROWB / 4 TF32 or ROWB / 2 BF16 values), stored in the tensor core's
// no-swizzle K-major canonical layout: 8-row x 16-byte core matrices, core
// matrices adjacent in K 128 bytes apart (LBO), 8-row groups
// (ROWB / 16) * 128 bytes apart (SBO).  One MMA consumes 32 bytes of K
// (8 TF32 / 16 BF16), i.e. 2 core matrices, so k-step kk starts kk * 256
// bytes into the matrix.  A value x is stored as hi + lo in two such
// matrices.
#pragma once

#include "mb_tcgen05.cuh"

namespace mb {

// LBO and SBO may be padded beyond the dense 128 and (ROWB / 16) * 128 bytes
// (multiples of 16 bytes), which moves K-adjacent core matrices and 8-row
// groups onto other shared-memory banks.
template <int MODE, int ROWB = 128, int LBO = 128, int SBO = (ROWB / 16) * 128> struct StageLayout;

template <int ROWB, int LBO = 128, int SBO = (ROWB / 16) * 128>
struct StageGeometry {
  static_assert(ROWB % 32 == 0, "a stage row holds whole MMA k-steps");
  static_assert(LBO % 16 == 0 && LBO >= 128, "core matrices of 8 rows x 16 bytes");
  static_assert(SBO % 16 == 0 && SBO >= (ROWB / 16) * LBO, "8-row groups must not overlap");
  static constexpr int kRowBytes = ROWB;
  static constexpr int kMatBytes = 16 * SBO;  // 128 rows
  static constexpr uint32_t kLBO = LBO, kSBO = SBO;
  static constexpr int kKStepBytes = 2 * LBO;  // one MMA k-step: 2 core matrices along K
  static constexpr int kKSteps = kRowBytes / 32;
  __device__ __forceinline__ static uint32_t offset(int row, int kbyte) {
    return uint32_t((row >> 3) * kSBO + (kbyte >> 4) * kLBO + (row & 7) * 16 + (kbyte & 15));
  }
  __device__ __forceinline__ static uint64_t desc(uint32_t saddr) { return tc::smem_desc(saddr, kLBO, kSBO); }
};

template <int ROWB, int LBO, int SBO>
struct StageLayout<MB_MODE_SPLIT_TF32, ROWB, LBO, SBO> : StageGeometry<ROWB, LBO, SBO> {
  using G = StageGeometry<ROWB, LBO, SBO>;
  static constexpr int kElem = 4;
  static constexpr int kKT = ROWB / kElem;  // values of K per stage
  __host__ __device__ static constexpr uint32_t instr(uint32_t M, uint32_t N) { return tc::instr_desc(2, M, N); }
  __device__ __forceinline__ static void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
    tc::mma_tf32(d, a, b, id, acc);
  }
  __device__ __forceinline__ static void put(unsigned char* hi, unsigned char* lo, int row, int k, float x) {
    float h, l;
    tc::split_tf32(x, h, l);
    const uint32_t o = G::offset(row, k * kElem);
    *reinterpret_cast<float*>(hi + o) = h;
    *reinterpret_cast<float*>(lo + o) = l;
  }
  // Two consecutive values (k even).
  __device__ __forceinline__ static void put2(unsigned char* hi, unsigned char* lo, int row, int k, float x0,
                                              float x1) {
    float2 h, l;
    tc::split_tf32x2(x0, x1, h, l);
    const uint32_t o = G::offset(row, k * kElem);
    *reinterpret_cast<float2*>(hi + o) = h;
    *reinterpret_cast<float2*>(lo + o) = l;
  }
};

template <int ROWB, int LBO, int SBO>
struct StageLayout<MB_MODE_SPLIT_BF16, ROWB, LBO, SBO> : StageGeometry<ROWB, LBO, SBO> {
  using G = StageGeometry<ROWB, LBO, SBO>;
  static constexpr int kElem = 2;
  static constexpr int kKT = ROWB / kElem;  // values of K per stage
  __host__ __device__ static constexpr uint32_t instr(uint32_t M, uint32_t N) { return tc::instr_desc(1, M, N); }
  __device__ __forceinline__ static void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
    tc::mma_f16(d, a, b, id, acc);
  }
  __device__ __forceinline__ static void put(unsigned char* hi, unsigned char* lo, int row, int k, float x) {
    __nv_bfloat16 h, l;
    tc::split_bf16(x, h, l);
    const uint32_t o = G::offset(row, k * kElem);
    *reinterpret_cast<__nv_bfloat16*>(hi + o) = h;
    *reinterpret_cast<__nv_bfloat16*>(lo + o) = l;
  }
  __device__ __forceinline__ static void put2(unsigned char* hi, unsigned char* lo, int row, int k, float x0,
                                              float x1) {
    __nv_bfloat162 hh, ll;
    tc::split_bf16x2(x0, x1, hh, ll);
    const uint32_t o = G::offset(row, k * kElem);
    *reinterpret_cast<__nv_bfloat162*>(hi + o) = hh;
    *reinterpret_cast<__nv_bfloat162*>(lo + o) = ll;
  }
};

}  // namespace mb
