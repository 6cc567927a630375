// Parameters and shared-memory plan of the fused per-(time, channel)
// kernels.  Shared between the CUDA-core kernels (mb_fused.cu) and the
// tensor-core point-source kernels (mb_tc.cu).
#pragma once

#include "mb_common.cuh"
#include "mb_internal.h"

namespace mb {

// One parameter set of a batched evaluation, as the kernels see it: the
// set's source counts and arrays, and its regions of the batch workspace.
template <typename T>
struct BatchSet {
  const T *lm, *stokes, *alpha, *gauss, *sersic;
  const double* phi;
  const T* bsq0;
  double* partial;
  T *gV, *dG;
  double *acc_lm, *acc_stokes, *acc_alpha, *acc_gauss, *acc_sersic;
  T *g_lm, *g_stokes, *g_alpha, *g_gauss, *g_sersic, *g_G;  // gradient outputs (any may be NULL)
  T* vis_ext;  // the extended sources' visibility sums of a split-form set, or NULL
  int npsrc, ngsrc, nssrc, pad;
};

template <typename T>
struct FusedArgs {
  // active extents and local strides
  int ntime, na, nbl, nchan, nsrc, npsrc, ngsrc, nssrc;
  int ltime, lna, lnbl, lchan, lgsrc, lssrc;
  int lw, mh, nud;
  int sbeg;     // first source handled by the CUDA-core adjoint (batched: < 0 for the set's npsrc)
  // Antenna sub-array of this launch (arrays above 64 antennas): na local
  // antennas, the first sub_n0 of them global sub_off0 + a, the others
  // global sub_off1 + (a - sub_n0); blocks of sub_blk antennas, this launch
  // owning the baselines between blocks sub_i and sub_j, and those within
  // sub_i (sub_diag bit 0) and within sub_j (bit 1).  sub_blk = 0: the
  // whole array (local = global).  na_glob: the call's active antennas.
  int na_glob, sub_blk, sub_i, sub_j, sub_n0, sub_off0, sub_off1, sub_diag;
  int src_tile; // requested sources per tile of the CUDA-core kernels (0: default)
  bool accumulate_in, partial_out, weights, residuals, want_grad;
  T ll, lmm, ul, um, lfreq, ufreq, lscale, mscale, gauss_scale, two_pi_over_c;
  double inv_sigma2;
  // inputs
  const T *uvw, *freq, *ref_freq, *pa, *pe, *sc, *E_beam, *G, *lm, *stokes, *alpha, *gauss, *sersic,
      *weight, *obs;
  const int32_t *ant1, *ant2;
  const uint8_t* flag;
  // outputs
  T* model_vis;
  T* chi2;
  // Partial sums added in with accumulate_in (the caller's model_vis, or the
  // split forms' extended-source sums in the workspace).
  const T* vis_in;
  // The tensor-core forward sums the extended sources itself (false: a
  // CUDA-core launch before it has left their sums in vis_in).
  bool tc_ext;
  // workspace
  const double* phi;  // (ntime, nsrc, na) path lengths: FP64, or FP32 (hi, lo) pairs in FP32 kernels
  const T* plane;     // (nchan, beam_lw, beam_mh, 12) frequency-blended beam, or NULL
  const T* bsq0;      // (nsrc, ntime, 8) sqrt(B) at nu = nu_ref and alpha / 2, or NULL
  double* partial;    // (ntime * nchan) chi^2 partial sums
  T* gV;              // (ntime, nbl, nchan, 4) complex d chi^2 / d V
  T* dG;              // (ntime, na, nchan, 4) complex d chi^2 / d G
  // adjoint accumulators (FP64)
  double *acc_lm, *acc_stokes, *acc_alpha, *acc_gauss, *acc_sersic;
  int* err;  // device error word (bounded waits that gave up), or NULL
  // Batched evaluation (mb_rime_batch): CTA b of a launch handles unit
  // bitems[b].y of parameter set bitems[b].x, whose source counts, source
  // arrays, tables, partials and accumulators bsets[set] gives; NULL for a
  // single problem.  Kernels of a launch over sets (grid.y = set) read
  // bsets[blockIdx.y].
  const BatchSet<T>* bsets;
  const int2* bitems;
};

// Per-antenna data for one (time, channel) unit.
template <typename T>
struct AntInfo {
  T sin_pa, cos_pa, pe_l, pe_m, sc_l, sc_m, u, v, w;
};

// Per-source data for one (time, channel) unit.
template <typename T>
struct SrcInfo {
  Jones<T> B;        // sqrt of the brightness matrix at this channel
  T l, m;            // direction cosines
  T s0, s1, s2;      // shape parameters (gaussian el, em, R / sersic e1, e2, R)
  T power, I, Q, U, V;
  T l_over_n, m_over_n;  // l / sqrt(1 - l^2 - m^2), m / sqrt(1 - l^2 - m^2)
  int type;
  int pad;
};

// Byte offsets of the dynamic shared-memory regions of one CTA.
struct SmemPlan {
  int nap;          // antennas padded to the register tile
  int st;           // sources per tile
  int npairs;       // na (na + 1) / 2
  int nitems;       // pair tiles
  int nthreads;     // threads per CTA
  int groups;       // source groups sharing each pair tile (forward)
  int jrow;         // bytes per source row of the Jones tiles (see jtile)
  size_t off_ant, off_antd, off_src, off_J, off_gJ, off_V, off_Vlo, off_items, off_acc, off_red, total;
};

constexpr int kFusedThreads = 256;
constexpr int kAdjThreads = 512;
constexpr int kFwdMaxThreads = 320;

size_t fused_workspace_size(mb_dtype dtype, mb_mode mode, const mb_dims* d, bool want_grad);

}  // namespace mb
