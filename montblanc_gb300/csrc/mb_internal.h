// Host-side helpers shared by the C-ABI translation units: error state,
// argument validation and launch checks.
#pragma once

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cuda_runtime.h>

#include "../../include/montblanc_gb300.h"

namespace mb {

// Record a message in the calling thread's error slot and return status.
mb_status fail(mb_status s, const char* fmt, ...);
void clear_error();

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

inline uint32_t ext(const mb_dim& d) { return d.upper_extent - d.lower_extent; }

// Check one dimension: lower <= upper <= local <= global.
inline bool dim_ok(const mb_dim& d) {
  return d.lower_extent <= d.upper_extent && d.upper_extent - d.lower_extent <= d.local_size &&
         d.local_size <= d.global_size;
}

mb_status check_dims(const mb_dims* dims, bool need_beam);

inline mb_status check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(MB_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  return MB_OK;
}

#define MB_REQUIRE(ptr, name)                                              \
  do {                                                                     \
    if ((ptr) == nullptr) return ::mb::fail(MB_ERR_NULL_PTR, "%s is NULL", name); \
  } while (0)

#define MB_CHECK(expr)                          \
  do {                                          \
    mb_status _st = (expr);                     \
    if (_st != MB_OK) return _st;               \
  } while (0)

#define MB_CUDA(expr)                                                          \
  do {                                                                         \
    cudaError_t _e = (expr);                                                   \
    if (_e != cudaSuccess)                                                     \
      return ::mb::fail(MB_ERR_CUDA, "%s: %s", #expr, cudaGetErrorString(_e)); \
  } while (0)

// Launch accounting around one kernel launch: counts every launch of this
// library and, while per-kernel timing is switched on, records a CUDA event
// pair on the launch stream (read back by mb_kernel_time).
class KernelScope {
 public:
  KernelScope(const char* name, cudaStream_t stream);
  ~KernelScope();
  KernelScope(const KernelScope&) = delete;
  KernelScope& operator=(const KernelScope&) = delete;

 private:
  int slot_;
  cudaStream_t stream_;
};

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Arrays read with vector loads must be aligned: complex Jones arrays to
// 16 bytes, flags to 4 bytes.
inline bool aligned(const void* p, size_t a) { return (reinterpret_cast<uintptr_t>(p) & (a - 1)) == 0; }

#define MB_ALIGNED(ptr, a, name)                                                            \
  do {                                                                                      \
    if ((ptr) != nullptr && !::mb::aligned((ptr), (a)))                                     \
      return ::mb::fail(MB_ERR_INVALID_ARG, "%s must be %d-byte aligned", name, int(a));   \
  } while (0)

}  // namespace mb
