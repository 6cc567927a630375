/*
 * montblanc_gb300: C ABI of the GB300 (sm_103a) RIME v4 hot path.
 *
 * Every entry point takes plain device pointers (C-order arrays with the
 * shapes of the reference's v4 array specification,
 * montblanc/impl/rime/v4/config.py:131-247), a dims record that mirrors the
 * reference's per-dimension constant data (global size, local size, lower
 * and upper extent; montblanc/util/const_data.py:58-86), and a CUDA stream
 * (cudaStream_t passed as void*; NULL = legacy default stream).  Complex
 * arrays are interleaved (re, im); Jones matrices are row-major
 * [00, 01, 10, 11].
 *
 * Nothing throws across the ABI: each call returns an mb_status and, on
 * failure, sets a thread-local message readable with mb_last_error_string().
 * No entry point allocates device memory; scratch space is reported by the
 * *_workspace_size functions and passed in by the caller.  Launches are
 * asynchronous on the given stream; only the status and timing queries
 * (mb_rime_status, mb_kernel_time) synchronise the host.
 */
#ifndef MONTBLANC_GB300_H
#define MONTBLANC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum mb_status {
  MB_OK = 0,
  MB_ERR_NULL_PTR = 1,          /* a required pointer is NULL */
  MB_ERR_BAD_SHAPE = 2,         /* inconsistent dimension sizes */
  MB_ERR_BAD_EXTENT = 3,        /* extents outside [0, local] or local > global */
  MB_ERR_UNSUPPORTED_DTYPE = 4, /* dtype is neither MB_FLOAT32 nor MB_FLOAT64 */
  MB_ERR_CUDA = 5,              /* a CUDA runtime call failed */
  MB_ERR_TIMEOUT = 6,           /* a bounded device-side wait gave up */
  MB_ERR_WORKSPACE = 7,         /* workspace NULL, misaligned or too small */
  MB_ERR_INVALID_ARG = 8,       /* any other invalid argument */
  MB_ERR_UNSUPPORTED = 9        /* valid request this build cannot serve */
} mb_status;

typedef enum mb_dtype { MB_FLOAT32 = 0, MB_FLOAT64 = 1 } mb_dtype;

/* Arithmetic form of the fused coherency sums.
 * MB_MODE_NATIVE: CUDA-core arithmetic in the array dtype.
 * MB_MODE_SPLIT_TF32 / MB_MODE_SPLIT_BF16: point sources as a per-(time,
 * channel) complex GEMM on the tensor cores, operands split into hi + lo
 * parts (3 products, FP32 accumulation); FLOAT32 data only.
 * In every mode the path length u l + v m + w (n - 1) is formed in FP64.
 * The FP64 mode forms the phase argument in FP64; the FP32 modes form it
 * and its reduction to [-1/2, 1/2] cycles from FP32 pairs (hi, lo) of the
 * path length and of nu / c (about 47 significant bits; an absolute error
 * near |cycles| 2^-47), then take an FP32 sincospi of the reduced value. */
typedef enum mb_mode {
  MB_MODE_NATIVE = 0,
  MB_MODE_SPLIT_TF32 = 1,
  MB_MODE_SPLIT_BF16 = 2
} mb_mode;

/* Option bits */
#define MB_APPLY_WEIGHTS 0x1u /* weight chi^2 terms by weight_vector */
#define MB_RESIDUALS 0x2u     /* write observed - model instead of model */
/* Source tile of the CUDA-core coherency kernels (the native forms and the
 * extended sources' adjoint of the split forms): sources per shared-memory
 * tile, a tuning hint that does not change results beyond rounding order.
 * 0 keeps the default (16 in FP32, 8 in FP64; 32 for the split forms'
 * extended-source adjoint); a tile whose shared memory does not fit is
 * halved until it does. */
#define MB_SOURCE_TILE_SHIFT 8
#define MB_SOURCE_TILE_MASK (0x3u << MB_SOURCE_TILE_SHIFT)
#define MB_SOURCE_TILE_8 (0x1u << MB_SOURCE_TILE_SHIFT)
#define MB_SOURCE_TILE_16 (0x2u << MB_SOURCE_TILE_SHIFT)
#define MB_SOURCE_TILE_32 (0x3u << MB_SOURCE_TILE_SHIFT)

typedef struct mb_dim {
  uint32_t global_size;
  uint32_t local_size;
  uint32_t lower_extent;
  uint32_t upper_extent;
} mb_dim;

/* Mirrors the reference's rime_const_data (montblanc/util/const_data.py).
 * Strides use local_size; loops run over [0, upper_extent - lower_extent).
 * For nsrc: lower_extent > 0 means "accumulate onto the partial sums held
 * in model_vis", upper_extent < global_size means "store partial sums in
 * model_vis and stop" (RimeSumCoherencies.py:185-190, 311-316). */
typedef struct mb_dims {
  mb_dim ntime, na, nbl, nchan, npol, npolchan;
  mb_dim nsrc, npsrc, ngsrc, nssrc;
  mb_dim beam_lw, beam_mh, beam_nud;
} mb_dims;

/* Scalar solver properties (montblanc/impl/rime/v4/config.py:54-69). */
typedef struct mb_props {
  double gauss_scale;
  double two_pi_over_c;
  double sigma_sqrd;
  double beam_ll, beam_lm, beam_lfreq;
  double beam_ul, beam_um, beam_ufreq;
} mb_props;

/* Library identification and error reporting. */
const char* mb_version(void);
const char* mb_last_error_string(void);
const char* mb_status_string(mb_status s);

/* ------------------------------------------------------------------------
 * Per-stage entry points: the kernels behind the reference's pipeline nodes.
 * ---------------------------------------------------------------------- */

/* B_sqrt(nsrc, ntime, nchan, 4) from stokes(nsrc, ntime, 4),
 * alpha(nsrc, ntime), frequency(nchan), ref_frequency(nchan).
 * Replaces rime_jones_B_sqrt_{float,double}
 * (montblanc/impl/rime/v4/gpu/RimeBSqrt.py:79-146) launched by
 * RimeBSqrt.execute (RimeBSqrt.py:210-225). */
mb_status mb_bsqrt(mb_dtype dtype, const mb_dims* dims, const void* stokes,
                   const void* alpha, const void* frequency,
                   const void* ref_frequency, void* B_sqrt, void* stream);

/* jones(nsrc, ntime, na, nchan, 4) <- E beam from lm(nsrc, 2),
 * parallactic_angles(ntime, na), point_errors(ntime, na, nchan, 2),
 * antenna_scaling(na, nchan, 2), frequency(nchan),
 * E_beam(beam_lw, beam_mh, beam_nud, 4).
 * Replaces rime_jones_E_beam_{float,double}
 * (montblanc/impl/rime/v4/gpu/RimeEBeam.py:138-368) launched by
 * RimeEBeam.execute (RimeEBeam.py:442-460). */
mb_status mb_ebeam(mb_dtype dtype, const mb_dims* dims, const mb_props* props,
                   const void* lm, const void* parallactic_angles,
                   const void* point_errors, const void* antenna_scaling,
                   const void* frequency, const void* E_beam, void* jones,
                   void* stream);

/* jones <- jones . (K * B_sqrt) in place, K from uvw(ntime, na, 3),
 * lm(nsrc, 2), frequency(nchan).
 * Replaces rime_jones_EKBSqrt_{float,double}
 * (montblanc/impl/rime/v4/gpu/RimeEKBSqrt.py:98-196) launched by
 * RimeEKBSqrt.execute (RimeEKBSqrt.py:258-273). */
mb_status mb_ekb_sqrt(mb_dtype dtype, const mb_dims* dims, const mb_props* props,
                      const void* uvw, const void* lm, const void* frequency,
                      const void* B_sqrt, void* jones, void* stream);

/* Coherency sum over sources per (time, baseline, channel) with shapes,
 * G-Jones, flags, model/residual output and chi^2 terms.
 * gauss_shape(3, ngsrc) / sersic_shape(3, nssrc) may be NULL when empty.
 * weight_vector may be NULL unless MB_APPLY_WEIGHTS is set.
 * Replaces rime_sum_coherencies
 * (montblanc/impl/rime/v4/gpu/RimeSumCoherencies.py:103-429) launched by
 * RimeSumCoherencies.execute (RimeSumCoherencies.py:499-529). */
mb_status mb_sum_coherencies(mb_dtype dtype, const mb_dims* dims,
                             const mb_props* props, uint32_t options,
                             const void* uvw, const void* gauss_shape,
                             const void* sersic_shape, const void* frequency,
                             const int32_t* antenna1, const int32_t* antenna2,
                             const void* jones, const uint8_t* flag,
                             const void* weight_vector,
                             const void* observed_vis, const void* G_term,
                             void* model_vis, void* chi_sqrd_result,
                             void* stream);

/* X2_out[0] = scale * sum of chi_sqrd_result over the active extents
 * [0:ntime, 0:nbl, 0:nchan], summed in FP64 in a fixed order.
 * Replaces pycuda.gpuarray.sum in RimeSumCoherencies.py:531-536 and
 * RimeReduction.execute (montblanc/impl/rime/v5/gpu/RimeReduction.py:46-61);
 * X2_out is a device pointer. */
size_t mb_reduce_chi2_workspace_size(const mb_dims* dims);
mb_status mb_reduce_chi2(mb_dtype dtype, const mb_dims* dims,
                         const void* chi_sqrd_result, double scale,
                         double* X2_out, void* workspace,
                         size_t workspace_bytes, void* stream);

/* ------------------------------------------------------------------------
 * Fused forward chi^2 and its adjoint (no per-antenna Jones array).
 * ---------------------------------------------------------------------- */

typedef struct mb_rime_inputs {
  const void* uvw;                /* (ntime, na, 3) */
  const int32_t* antenna1;        /* (ntime, nbl) */
  const int32_t* antenna2;        /* (ntime, nbl) */
  const void* frequency;          /* (nchan) */
  const void* ref_frequency;      /* (nchan) */
  const void* parallactic_angles; /* (ntime, na) */
  const void* point_errors;       /* (ntime, na, nchan, 2) */
  const void* antenna_scaling;    /* (na, nchan, 2) */
  const void* E_beam;             /* (beam_lw, beam_mh, beam_nud, 4) complex */
  const void* G_term;             /* (ntime, na, nchan, 4) complex */
  const void* lm;                 /* (nsrc, 2) */
  const void* stokes;             /* (nsrc, ntime, 4) */
  const void* alpha;              /* (nsrc, ntime) */
  const void* gauss_shape;        /* (3, ngsrc), NULL if ngsrc == 0 */
  const void* sersic_shape;       /* (3, nssrc), NULL if nssrc == 0 */
  const uint8_t* flag;            /* (ntime, nbl, nchan, 4) */
  const void* weight_vector;      /* (ntime, nbl, nchan, 4), NULL unless weights */
  const void* observed_vis;       /* (ntime, nbl, nchan, 4) complex */
} mb_rime_inputs;

/* Gradient outputs of mb_rime_adjoint, each in the input dtype and shape;
 * any may be NULL.  Complex gradients are d/dRe + i d/dIm. */
typedef struct mb_rime_grads {
  void* lm;           /* (nsrc, 2) */
  void* stokes;       /* (nsrc, ntime, 4) */
  void* alpha;        /* (nsrc, ntime) */
  void* gauss_shape;  /* (3, ngsrc) */
  void* sersic_shape; /* (3, nssrc) */
  void* G_term;       /* (ntime, na, nchan, 4) complex */
} mb_rime_grads;

/* Forward-only workspace (want_grad = 0) or forward + adjoint (1). */
size_t mb_rime_workspace_size(mb_dtype dtype, mb_mode mode, const mb_dims* dims,
                              int want_grad);

/* Forward: per-antenna E . K . sqrt(B) formed on the fly, coherency sums over
 * all source types, G-Jones, flags, model/residual output (model_vis may be
 * NULL), chi^2 terms (chi_sqrd_result may be NULL) and the chi^2 scalar
 * (X2, device double, already divided by sigma_sqrd when weights are off).
 * With want_grad = 1 it also leaves in the workspace what mb_rime_adjoint
 * needs.  Fuses RimeBSqrt, RimeEBeam, RimeEKBSqrt, RimeSumCoherencies and the
 * chi^2 reduction (montblanc/impl/rime/v4/RimeSolver.py:36-40). */
mb_status mb_rime_forward(mb_dtype dtype, mb_mode mode, const mb_dims* dims,
                          const mb_props* props, uint32_t options,
                          const mb_rime_inputs* in, void* model_vis,
                          void* chi_sqrd_result, double* X2, int want_grad,
                          void* workspace, size_t workspace_bytes,
                          void* stream);

/* Adjoint: grad_scale * d(chi^2)/d(parameters), using the state a preceding
 * mb_rime_forward(..., want_grad = 1, same workspace) left behind.  K and E
 * are recomputed, not stored.  No counterpart in the reference (it has no
 * gradient). */
mb_status mb_rime_adjoint(mb_dtype dtype, mb_mode mode, const mb_dims* dims,
                          const mb_props* props, uint32_t options,
                          const mb_rime_inputs* in, double grad_scale,
                          const mb_rime_grads* grads, void* workspace,
                          size_t workspace_bytes, void* stream);

/* Device-side status of the last mb_rime_forward (and the mb_rime_adjoint
 * calls after it) that used this workspace, with the same dtype, mode, dims
 * and want_grad as the forward.  The tensor-core kernels' waits are bounded:
 * a wait that gives up makes the kernel skip its remaining work and record
 * MB_ERR_TIMEOUT in the workspace; the chi^2 of such a call is NaN.  This
 * synchronises `stream`, reads that record and returns MB_ERR_TIMEOUT if it
 * is set, MB_OK otherwise.  (The launches themselves return before the
 * kernels run, so they cannot report it.)  Replaces the error surfacing of
 * the blocking .get() in RimeSumCoherencies.py:531-536. */
mb_status mb_rime_status(mb_dtype dtype, mb_mode mode, const mb_dims* dims,
                         int want_grad, const void* workspace,
                         size_t workspace_bytes, void* stream);

/* ------------------------------------------------------------------------
 * Batched likelihood.  No counterpart in the reference: it solves one
 * resident problem per solver; its closest caller is the v5 driver's
 * per-chunk enqueue (impl/rime/v5/CompositeRimeSolver.py:925-975).
 *
 * chi^2 and its gradient for nsets parameter sets (sampler proposals)
 * against one observation.  Every input of mb_rime_inputs except the source
 * arrays (lm, stokes, alpha, gauss_shape, sersic_shape, which are ignored)
 * is shared; each set brings its own source counts, source arrays (stokes
 * and alpha with the observation's local time size as row stride, shapes as
 * (3, n) with n its own count) and gradient outputs.  The source dimensions
 * of `dims` are ignored.  All sets of one kernel form (mode and source tile)
 * run as one forward launch and one adjoint launch whose CTAs are the sets'
 * (time, channel) units, largest sets first, so a call launches a fixed
 * handful of kernels however many sets it holds.
 * ---------------------------------------------------------------------- */
typedef struct mb_batch_set {
  uint32_t npsrc, ngsrc, nssrc;
  uint32_t mode;      /* mb_mode of this set's kernels (split modes: FLOAT32) */
  uint32_t options;   /* MB_SOURCE_TILE_* bits of this set's CUDA-core kernels, or 0 */
  uint32_t reserved;  /* 0 */
  const void* lm;           /* (nsrc, 2) */
  const void* stokes;       /* (nsrc, ntime, 4) */
  const void* alpha;        /* (nsrc, ntime) */
  const void* gauss_shape;  /* (3, ngsrc), NULL if ngsrc == 0 */
  const void* sersic_shape; /* (3, nssrc), NULL if nssrc == 0 */
  mb_rime_grads grads;      /* this set's gradient outputs, any may be NULL */
} mb_batch_set;

/* Workspace bytes of a batch (per set: FP64 path lengths, d chi^2 / dV,
 * d chi^2 / dG and accumulators), or 0 if the arguments are invalid. */
size_t mb_rime_batch_workspace_size(mb_dtype dtype, const mb_dims* dims,
                                    const mb_batch_set* sets, int nsets);

/* Writes the per-set table and the launches' (set, unit) lists into the
 * workspace; synchronises `stream`.  Call it again after changing any set's
 * counts, mode, options, arrays or outputs; not capturable in a CUDA graph. */
mb_status mb_rime_batch_prepare(mb_dtype dtype, const mb_dims* dims,
                                const mb_batch_set* sets, int nsets,
                                void* workspace, size_t workspace_bytes,
                                void* stream);

/* chi^2 of every set into X2[0 .. nsets) (device doubles, divided by
 * sigma_sqrd when weights are off) and grad_scale * d chi^2 / d(parameters)
 * into each set's outputs, from the tables mb_rime_batch_prepare wrote for
 * the same `sets`.  Stream-ordered, allocates nothing, capturable. */
mb_status mb_rime_batch(mb_dtype dtype, const mb_dims* dims,
                        const mb_props* props, uint32_t options,
                        const mb_rime_inputs* shared, const mb_batch_set* sets,
                        int nsets, double* X2, double grad_scale,
                        void* workspace, size_t workspace_bytes, void* stream);

/* Diagnostic, no counterpart in the reference: the poll limit of the
 * pipeline waits of the tensor-core kernels on the current device (default
 * mb_default_wait_limit() = 2^20).  0 makes every such wait give up at once,
 * which exercises the MB_ERR_TIMEOUT path without a fault: the kernels still
 * wait, with the default limit, for the MMAs they issued before freeing
 * tensor memory.  Synchronous. */
mb_status mb_set_wait_limit(uint32_t polls);
uint32_t mb_default_wait_limit(void);

/* Diagnostic, no counterpart in the reference: D (128 x 128, row-major) =
 * A (128 x K) . B (128 x K)^T for row-major FP32 device arrays, computed
 * with the split-precision tensor-core operand path of the fused kernels
 * (mode MB_MODE_SPLIT_TF32: K % 32 == 0; MB_MODE_SPLIT_BF16: K % 64 == 0).
 * With mode MB_MODE_SPLIT_BF16 | MB_TC_SELFTEST_A_IN_TMEM the A operand is
 * read from tensor memory (as the split-precision adjoint reads dchi^2/dV).
 * *status (device int) is set to 1 if a bounded wait gave up. */
#define MB_TC_SELFTEST_A_IN_TMEM 0x10
mb_status mb_tc_selftest(const float* A, const float* B, int K, int mode,
                         float* D, int* status, void* stream);

/* Diagnostic, no counterpart in the reference: the bounded-wait path of the
 * tensor-core kernels on a wait that cannot complete.  One CTA allocates
 * TMEM, waits at most poll_limit polls on an mbarrier that nothing arrives
 * on, sets *status (device int) to 1 when the wait gives up, frees TMEM and
 * returns.  Stream-ordered, no host synchronisation. */
mb_status mb_wait_selftest(uint32_t poll_limit, int* status, void* stream);

/* Diagnostics, no counterpart in the reference: launch accounting and
 * per-kernel CUDA-event timing of this library's kernels.
 * mb_kernel_launches: kernels launched by the library in this process.
 * mb_kernel_timing(1) starts recording a CUDA event pair on the launch
 * stream around every launch (0 stops; recorded events are kept).
 * mb_kernel_time: total milliseconds and launch count of the recorded
 * launches whose kernel name equals `name` (NULL: all); synchronises on
 * the recorded events.  mb_kernel_timing_reset drops the records. */
uint64_t mb_kernel_launches(void);
mb_status mb_kernel_timing(int enable);
mb_status mb_kernel_time(const char* name, double* total_ms, int64_t* launches);
mb_status mb_kernel_timing_reset(void);
/* Name of the i-th distinct kernel timed since the process started (NULL
 * past the end); the returned string stays valid for the process. */
const char* mb_kernel_timing_name(int i);

/* ------------------------------------------------------------------------
 * Allocation-free forward.  No counterpart in the reference.
 *
 * For callers that must not allocate device memory themselves: applications
 * that hand all device memory to their own pool or framework allocator at
 * start-up (so a foreign cudaMalloc fails or breaks their budget), and
 * latency-bound pipelines that cannot afford cudaMalloc/cudaFree, which may
 * synchronise the device.  Such callers cannot size and pass the workspace
 * mb_rime_forward needs.
 *
 * Same inputs and outputs as mb_rime_forward in MB_MODE_NATIVE with
 * want_grad = 0, and the same results up to rounding: in FP32 the beam is
 * interpolated from the cube and sqrt(B) formed in the kernel (no per-call
 * tables), so results differ from mb_rime_forward's in the last bits.  Its
 * only scratch (one FP64 partial sum per (time, channel) unit) is a static
 * device array inside the library: at most mb_rime_noalloc_max_units() =
 * 131072 units (ntime * nchan active extents); larger requests return
 * MB_ERR_UNSUPPORTED.  The array costs 1 MiB on every GPU that loads the
 * library, for the life of the process.  Each call outside stream capture
 * looks the array's device address up (cudaGetSymbolAddress, no
 * allocation); a call during capture uses the address the last uncaptured
 * call on that device found, so make one call on each device before
 * capturing, and one after a cudaDeviceReset before capturing again.
 * All calls share the array: calls whose kernels may run at the same time
 * (on unordered streams) race on it and must be serialised by the caller.
 * It allocates nothing: no cudaMalloc, cudaFree or allocating library call.
 * ---------------------------------------------------------------------- */
size_t mb_rime_noalloc_max_units(void);
mb_status mb_rime_forward_noalloc(mb_dtype dtype, const mb_dims* dims,
                                  const mb_props* props, uint32_t options,
                                  const mb_rime_inputs* in, void* model_vis,
                                  void* chi_sqrd_result, double* X2,
                                  void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MONTBLANC_GB300_H */
