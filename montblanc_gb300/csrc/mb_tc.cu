// Tensor-core (tcgen05) point-source coherencies: placeholder until the
// split-precision GEMM lands.
#include "mb_fused.h"

namespace mb {

size_t tc_scratch_bytes(const mb_dims* d) {
  const size_t na = ext(d->na);
  return size_t(ext(d->ntime)) * ext(d->nchan) * na * na * 8 * sizeof(float);
}

mb_status tc_point_coherencies(const FusedArgs<float>& A, mb_mode mode, float* Vpoint, cudaStream_t stream) {
  (void)A; (void)mode; (void)Vpoint; (void)stream;
  return fail(MB_ERR_UNSUPPORTED, "split-precision tensor-core path not built");
}

}  // namespace mb
