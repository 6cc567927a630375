// Per-stage kernels: the work behind the reference's four v4 pipeline nodes
// (RimeBSqrt, RimeEBeam, RimeEKBSqrt, RimeSumCoherencies) and the chi^2
// reduction (RimeReduction).  These operate on the reference's materialised
// intermediate arrays (B_sqrt, jones) so that each node stays a drop-in
// replacement; the fused path in mb_fused.cu avoids those arrays.
//
// Each thread owns one full 2x2 Jones (all four correlations) rather than
// one correlation per lane, so no warp shuffles are needed and every global
// access is a 16-byte vector load of contiguous correlations.
#include "mb_common.cuh"
#include "mb_internal.h"

namespace mb {
namespace {

constexpr int kThreads = 256;

inline unsigned grid_for(size_t n) {
  size_t b = (n + kThreads - 1) / kThreads;
  if (b > (1u << 30)) b = 1u << 30;
  return static_cast<unsigned>(b < 1 ? 1 : b);
}

struct StageDims {
  int nsrc, ntime, na, nbl, nchan;          // active extents
  int lsrc, ltime, lna, lnbl, lchan;        // local sizes (strides)
  int npsrc, ngsrc, nssrc;                  // active extents per type
  int lgsrc, lssrc;                         // local sizes of the shape arrays
  int lw, mh, nud;
  bool accumulate_in, partial_out;          // source-batch semantics
};

StageDims stage_dims(const mb_dims* d) {
  StageDims s;
  s.nsrc = ext(d->nsrc); s.ntime = ext(d->ntime); s.na = ext(d->na);
  s.nbl = ext(d->nbl); s.nchan = ext(d->nchan);
  s.lsrc = d->nsrc.local_size; s.ltime = d->ntime.local_size; s.lna = d->na.local_size;
  s.lnbl = d->nbl.local_size; s.lchan = d->nchan.local_size;
  s.npsrc = ext(d->npsrc); s.ngsrc = ext(d->ngsrc); s.nssrc = ext(d->nssrc);
  s.lgsrc = d->ngsrc.local_size; s.lssrc = d->nssrc.local_size;
  s.lw = d->beam_lw.local_size; s.mh = d->beam_mh.local_size; s.nud = d->beam_nud.local_size;
  s.accumulate_in = d->nsrc.lower_extent > 0;
  s.partial_out = d->nsrc.upper_extent < d->nsrc.global_size;
  return s;
}

// ---- B sqrt ----------------------------------------------------------------
template <typename T>
__global__ void bsqrt_kernel(StageDims D, const T* __restrict__ stokes, const T* __restrict__ alpha,
                             const T* __restrict__ freq, const T* __restrict__ ref_freq,
                             T* __restrict__ B_sqrt) {
  size_t total = size_t(D.nsrc) * D.ntime * D.nchan;
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < total; i += size_t(gridDim.x) * blockDim.x) {
    int ch = int(i % D.nchan);
    int t = int((i / D.nchan) % D.ntime);
    int s = int(i / (size_t(D.nchan) * D.ntime));
    size_t st = size_t(s) * D.ltime + t;
    T power = mb_pow(freq[ch] / ref_freq[ch], alpha[st]);
    const T* S = stokes + 4 * st;
    Jones<T> B = brightness_sqrt<T>(S[0], S[1], S[2], S[3], power);
    jstore(B_sqrt + 8 * (st * D.lchan + ch), B);
  }
}

// ---- E beam ----------------------------------------------------------------
template <typename T>
__global__ void ebeam_kernel(StageDims D, mb_props P, const T* __restrict__ lm, const T* __restrict__ pa,
                             const T* __restrict__ pe, const T* __restrict__ sc, const T* __restrict__ freq,
                             const T* __restrict__ E_beam, T* __restrict__ jones) {
  size_t total = size_t(D.ntime) * D.na * D.nchan;
  size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (i >= total) return;
  int ch = int(i % D.nchan);
  int a = int((i / D.nchan) % D.na);
  int t = int(i / (size_t(D.nchan) * D.na));
  BeamGeom G{D.lw, D.mh, D.nud};
  const T ll = T(P.beam_ll), lmm = T(P.beam_lm), ul = T(P.beam_ul), um = T(P.beam_um);
  const T lscale = T(D.lw - 1) / (ul - ll), mscale = T(D.mh - 1) / (um - lmm);
  ChanPos<T> cp = chan_pos<T>(freq[ch], T(P.beam_lfreq), T(P.beam_ufreq), D.nud);
  size_t ta = size_t(t) * D.lna + a;
  T sp, cpa;
  if (sizeof(T) == 8) { double s_, c_; sincos(double(pa[ta]), &s_, &c_); sp = T(s_); cpa = T(c_); }
  else { float s_, c_; sincosf(float(pa[ta]), &s_, &c_); sp = T(s_); cpa = T(c_); }
  size_t tac = ta * D.lchan + ch;
  T pel = pe[2 * tac], pem = pe[2 * tac + 1];
  size_t ac = size_t(a) * D.lchan + ch;
  T scl = sc[2 * ac], scm = sc[2 * ac + 1];
  for (int s = 0; s < D.nsrc; ++s) {
    T l, m;
    beam_lm<T>(lm[2 * s], lm[2 * s + 1], sp, cpa, pel, pem, scl, scm, l, m);
    GridPos<T> gl = grid_pos<T>(l, ll, ul, lscale, D.lw);
    GridPos<T> gm = grid_pos<T>(m, lmm, um, mscale, D.mh);
    Jones<T> E = beam_interp<T>(E_beam, G, gl, gm, cp);
    jstore(jones + 8 * (((size_t(s) * D.ltime + t) * D.lna + a) * D.lchan + ch), E);
  }
}

// ---- E K B_sqrt ------------------------------------------------------------
template <typename T>
__global__ void ekb_kernel(StageDims D, const T* __restrict__ uvw, const T* __restrict__ lm,
                           const T* __restrict__ freq, const T* __restrict__ B_sqrt, T* __restrict__ jones) {
  size_t total = size_t(D.ntime) * D.na * D.nchan;
  size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (i >= total) return;
  int ch = int(i % D.nchan);
  int a = int((i / D.nchan) % D.na);
  int t = int(i / (size_t(D.nchan) * D.na));
  size_t ta = size_t(t) * D.lna + a;
  double u = uvw[3 * ta], v = uvw[3 * ta + 1], w = uvw[3 * ta + 2];
  double f = freq[ch];
  for (int s = 0; s < D.nsrc; ++s) {
    double l = lm[2 * s], m = lm[2 * s + 1];
    double n = sqrt(1.0 - l * l - m * m) - 1.0;
    double phi = l * u + m * v + n * w;
    Cx<T> K = phase_from_phi<T>(phi, f);
    Jones<T> B = jldg<T>(B_sqrt + 8 * ((size_t(s) * D.ltime + t) * D.lchan + ch));
    Jones<T> KB = {cmul(K, B.a), cmul(K, B.b), cmul(K, B.c), cmul(K, B.d)};
    T* jp = jones + 8 * (((size_t(s) * D.ltime + t) * D.lna + a) * D.lchan + ch);
    Jones<T> E = jload<T>(jp);
    jstore(jp, jmul(E, KB));
  }
}

// ---- coherency sum ---------------------------------------------------------
template <typename T, bool WEIGHTS, bool RESIDUALS>
__global__ void sumcoh_kernel(StageDims D, mb_props P, const T* __restrict__ uvw,
                              const T* __restrict__ gauss, const T* __restrict__ sersic,
                              const T* __restrict__ freq, const int32_t* __restrict__ ant1,
                              const int32_t* __restrict__ ant2, const T* __restrict__ jones,
                              const uint8_t* __restrict__ flag, const T* __restrict__ weight,
                              const T* __restrict__ obs, const T* __restrict__ G,
                              T* __restrict__ vis, T* __restrict__ chi2) {
  size_t total = size_t(D.ntime) * D.nbl * D.nchan;
  size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (i >= total) return;
  int ch = int(i % D.nchan);
  int bl = int((i / D.nchan) % D.nbl);
  int t = int(i / (size_t(D.nchan) * D.nbl));
  size_t tbl = size_t(t) * D.lnbl + bl;
  int p = ant1[tbl], q = ant2[tbl];
  size_t vidx = tbl * D.lchan + ch;
  if (p < 0 || p >= D.lna || q < 0 || q >= D.lna) {  // invalid antenna index: NaN output
    const T nan = T(NAN);
    jstore(vis + 8 * vidx, Jones<T>{{nan, nan}, {nan, nan}, {nan, nan}, {nan, nan}});
    if (!D.partial_out) chi2[vidx] = nan;
    return;
  }

  Jones<T> V = jzero<T>();
  if (D.accumulate_in) V = jload<T>(vis + 8 * vidx);

  const T* up = uvw + 3 * (size_t(t) * D.lna + p);
  const T* uq = uvw + 3 * (size_t(t) * D.lna + q);
  T u = uq[0] - up[0], v = uq[1] - up[1];
  T f = freq[ch];
  const size_t sstride = size_t(D.ltime) * D.lna * D.lchan;
  const T* jp = jones + 8 * ((size_t(t) * D.lna + p) * D.lchan + ch);
  const T* jq = jones + 8 * ((size_t(t) * D.lna + q) * D.lchan + ch);

  int s = 0;
  for (; s < D.npsrc; ++s) {
    Jones<T> A = jldg<T>(jp + 8 * s * sstride);
    Jones<T> B = jldg<T>(jq + 8 * s * sstride);
    jmac_h(V, A, B);
  }
  const T kg = T(P.gauss_scale) * f;
  for (int g = 0; g < D.ngsrc; ++g, ++s) {
    T c = gauss_shape<T>(u, v, gauss[g], gauss[D.lgsrc + g], gauss[2 * D.lgsrc + g], kg);
    Jones<T> A = jscale(jldg<T>(jp + 8 * s * sstride), c);
    Jones<T> B = jldg<T>(jq + 8 * s * sstride);
    jmac_h(V, A, B);
  }
  const T ks = T(P.two_pi_over_c) * f;
  for (int x = 0; x < D.nssrc; ++x, ++s) {
    T c = sersic_shape<T>(u, v, sersic[x], sersic[D.lssrc + x], sersic[2 * D.lssrc + x], ks);
    Jones<T> A = jscale(jldg<T>(jp + 8 * s * sstride), c);
    Jones<T> B = jldg<T>(jq + 8 * s * sstride);
    jmac_h(V, A, B);
  }

  if (D.partial_out) {  // more source batches to come: store the partial sum
    jstore(vis + 8 * vidx, V);
    return;
  }

  Jones<T> Gp = jldg<T>(G + 8 * ((size_t(t) * D.lna + p) * D.lchan + ch));
  Jones<T> Gq = jldg<T>(G + 8 * ((size_t(t) * D.lna + q) * D.lchan + ch));
  Jones<T> M = jmulh(jmul(Gp, V), Gq);
  Jones<T> O = jldg<T>(obs + 8 * vidx);
  uchar4 fl = *reinterpret_cast<const uchar4*>(flag + 4 * vidx);
  Cx<T>* m4 = &M.a;
  Cx<T>* o4 = &O.a;
  const uint8_t fv[4] = {fl.x, fl.y, fl.z, fl.w};
  Jones<T> R;
  Cx<T>* r4 = &R.a;
  T term = T(0);
  T w4[4] = {T(1), T(1), T(1), T(1)};
  if (WEIGHTS) {
    for (int k = 0; k < 4; ++k) w4[k] = weight[4 * vidx + k];
  }
  for (int k = 0; k < 4; ++k) {
    if (fv[k] > 0) { m4[k] = Cx<T>{T(0), T(0)}; o4[k] = Cx<T>{T(0), T(0)}; }
    r4[k] = o4[k] - m4[k];
    T re2 = r4[k].r * r4[k].r, im2 = r4[k].i * r4[k].i;
    if (WEIGHTS) { re2 *= w4[k]; im2 *= w4[k]; }
    term += re2 + im2;
  }
  jstore(vis + 8 * vidx, RESIDUALS ? R : M);
  chi2[vidx] = term;
}

// ---- deterministic chi^2 reduction ------------------------------------------
template <typename T>
__global__ void chi2_partial_kernel(const T* __restrict__ chi2, int ntime, int nbl, int nchan, int lnbl,
                                    int lchan, double* __restrict__ partial) {
  __shared__ double red[kThreads / 32];
  size_t total = size_t(ntime) * nbl * nchan;
  double acc = 0.0;
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < total; i += size_t(gridDim.x) * blockDim.x) {
    int ch = int(i % nchan);
    int bl = int((i / nchan) % nbl);
    int t = int(i / (size_t(nchan) * nbl));
    acc += double(chi2[(size_t(t) * lnbl + bl) * lchan + ch]);
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    acc = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (threadIdx.x == 0) partial[blockIdx.x] = acc;
  }
}

}  // namespace

// Sums `n` doubles in a fixed order with one block; out = scale * sum.
__global__ void sum_partials_kernel(const double* __restrict__ partial, int n, double scale,
                                    double* __restrict__ out) {
  __shared__ double red[32];
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += partial[i];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    acc = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (threadIdx.x == 0) out[0] = acc * scale;
  }
}

constexpr int kReduceBlocks = 1024;

}  // namespace mb

using namespace mb;

extern "C" {

mb_status mb_bsqrt(mb_dtype dtype, const mb_dims* dims, const void* stokes, const void* alpha,
                   const void* frequency, const void* ref_frequency, void* B_sqrt, void* stream) {
  MB_CHECK(check_dims(dims, false));
  MB_REQUIRE(stokes, "stokes"); MB_REQUIRE(alpha, "alpha"); MB_REQUIRE(frequency, "frequency");
  MB_REQUIRE(ref_frequency, "ref_frequency"); MB_REQUIRE(B_sqrt, "B_sqrt");
  MB_ALIGNED(B_sqrt, 16, "B_sqrt");
  StageDims D = stage_dims(dims);
  size_t n = size_t(D.nsrc) * D.ntime * D.nchan;
  if (n == 0) return MB_OK;
  cudaStream_t s = as_stream(stream);
  if (dtype == MB_FLOAT32) {
    KernelScope ks_("bsqrt_kernel", s);
    bsqrt_kernel<float><<<grid_for(n), kThreads, 0, s>>>(D, (const float*)stokes, (const float*)alpha,
        (const float*)frequency, (const float*)ref_frequency, (float*)B_sqrt);
  } else if (dtype == MB_FLOAT64) {
    KernelScope ks_("bsqrt_kernel", s);
    bsqrt_kernel<double><<<grid_for(n), kThreads, 0, s>>>(D, (const double*)stokes, (const double*)alpha,
        (const double*)frequency, (const double*)ref_frequency, (double*)B_sqrt);
  } else return fail(MB_ERR_UNSUPPORTED_DTYPE, "dtype %d", int(dtype));
  return check_launch("mb_bsqrt");
}

mb_status mb_ebeam(mb_dtype dtype, const mb_dims* dims, const mb_props* props, const void* lm,
                   const void* parallactic_angles, const void* point_errors, const void* antenna_scaling,
                   const void* frequency, const void* E_beam, void* jones, void* stream) {
  MB_CHECK(check_dims(dims, true));
  MB_REQUIRE(props, "props"); MB_REQUIRE(lm, "lm"); MB_REQUIRE(parallactic_angles, "parallactic_angles");
  MB_REQUIRE(point_errors, "point_errors"); MB_REQUIRE(antenna_scaling, "antenna_scaling");
  MB_REQUIRE(frequency, "frequency"); MB_REQUIRE(E_beam, "E_beam"); MB_REQUIRE(jones, "jones");
  MB_ALIGNED(E_beam, 16, "E_beam"); MB_ALIGNED(jones, 16, "jones");
  StageDims D = stage_dims(dims);
  size_t n = size_t(D.ntime) * D.na * D.nchan;
  if (n == 0 || D.nsrc == 0) return MB_OK;
  cudaStream_t s = as_stream(stream);
  if (dtype == MB_FLOAT32) {
    KernelScope ks_("ebeam_kernel", s);
    ebeam_kernel<float><<<grid_for(n), kThreads, 0, s>>>(D, *props, (const float*)lm,
        (const float*)parallactic_angles, (const float*)point_errors, (const float*)antenna_scaling,
        (const float*)frequency, (const float*)E_beam, (float*)jones);
  } else if (dtype == MB_FLOAT64) {
    KernelScope ks_("ebeam_kernel", s);
    ebeam_kernel<double><<<grid_for(n), kThreads, 0, s>>>(D, *props, (const double*)lm,
        (const double*)parallactic_angles, (const double*)point_errors, (const double*)antenna_scaling,
        (const double*)frequency, (const double*)E_beam, (double*)jones);
  } else return fail(MB_ERR_UNSUPPORTED_DTYPE, "dtype %d", int(dtype));
  return check_launch("mb_ebeam");
}

mb_status mb_ekb_sqrt(mb_dtype dtype, const mb_dims* dims, const mb_props* props, const void* uvw,
                      const void* lm, const void* frequency, const void* B_sqrt, void* jones, void* stream) {
  MB_CHECK(check_dims(dims, false));
  MB_REQUIRE(props, "props"); MB_REQUIRE(uvw, "uvw"); MB_REQUIRE(lm, "lm");
  MB_REQUIRE(frequency, "frequency"); MB_REQUIRE(B_sqrt, "B_sqrt"); MB_REQUIRE(jones, "jones");
  MB_ALIGNED(B_sqrt, 16, "B_sqrt"); MB_ALIGNED(jones, 16, "jones");
  StageDims D = stage_dims(dims);
  size_t n = size_t(D.ntime) * D.na * D.nchan;
  if (n == 0 || D.nsrc == 0) return MB_OK;
  cudaStream_t s = as_stream(stream);
  if (dtype == MB_FLOAT32) {
    KernelScope ks_("ekb_kernel", s);
    ekb_kernel<float><<<grid_for(n), kThreads, 0, s>>>(D, (const float*)uvw, (const float*)lm,
        (const float*)frequency, (const float*)B_sqrt, (float*)jones);
  } else if (dtype == MB_FLOAT64) {
    KernelScope ks_("ekb_kernel", s);
    ekb_kernel<double><<<grid_for(n), kThreads, 0, s>>>(D, (const double*)uvw, (const double*)lm,
        (const double*)frequency, (const double*)B_sqrt, (double*)jones);
  } else return fail(MB_ERR_UNSUPPORTED_DTYPE, "dtype %d", int(dtype));
  return check_launch("mb_ekb_sqrt");
}

mb_status mb_sum_coherencies(mb_dtype dtype, const mb_dims* dims, const mb_props* props, uint32_t options,
                             const void* uvw, const void* gauss_shape, const void* sersic_shape,
                             const void* frequency, const int32_t* antenna1, const int32_t* antenna2,
                             const void* jones, const uint8_t* flag, const void* weight_vector,
                             const void* observed_vis, const void* G_term, void* model_vis,
                             void* chi_sqrd_result, void* stream) {
  MB_CHECK(check_dims(dims, false));
  MB_REQUIRE(props, "props"); MB_REQUIRE(uvw, "uvw"); MB_REQUIRE(frequency, "frequency");
  MB_REQUIRE(antenna1, "antenna1"); MB_REQUIRE(antenna2, "antenna2"); MB_REQUIRE(model_vis, "model_vis");
  StageDims D = stage_dims(dims);
  if (D.nsrc > 0) MB_REQUIRE(jones, "jones");
  if (D.ngsrc > 0) MB_REQUIRE(gauss_shape, "gauss_shape");
  if (D.nssrc > 0) MB_REQUIRE(sersic_shape, "sersic_shape");
  if (!D.partial_out) {
    MB_REQUIRE(flag, "flag"); MB_REQUIRE(observed_vis, "observed_vis"); MB_REQUIRE(G_term, "G_term");
    MB_REQUIRE(chi_sqrd_result, "chi_sqrd_result");
    if (options & MB_APPLY_WEIGHTS) MB_REQUIRE(weight_vector, "weight_vector");
  }
  if (options & ~(MB_APPLY_WEIGHTS | MB_RESIDUALS)) return fail(MB_ERR_INVALID_ARG, "unknown option bits 0x%x", options);
  MB_ALIGNED(jones, 16, "jones"); MB_ALIGNED(observed_vis, 16, "observed_vis"); MB_ALIGNED(G_term, 16, "G_term");
  MB_ALIGNED(model_vis, 16, "model_vis"); MB_ALIGNED(flag, 4, "flag");
  size_t n = size_t(D.ntime) * D.nbl * D.nchan;
  if (n == 0) return MB_OK;
  cudaStream_t s = as_stream(stream);
  const bool w = options & MB_APPLY_WEIGHTS, r = options & MB_RESIDUALS;
#define MB_SUMCOH(T, W, R)                                                                               \
  do {                                                                                                 \
    KernelScope ks_("sumcoh_kernel", s);                                                               \
    sumcoh_kernel<T, W, R><<<grid_for(n), kThreads, 0, s>>>(D, *props, (const T*)uvw,                  \
        (const T*)gauss_shape, (const T*)sersic_shape, (const T*)frequency, antenna1, antenna2,        \
        (const T*)jones, flag, (const T*)weight_vector, (const T*)observed_vis, (const T*)G_term,      \
        (T*)model_vis, (T*)chi_sqrd_result);                                                           \
  } while (0)
  if (dtype == MB_FLOAT32) {
    if (w && r) MB_SUMCOH(float, true, true); else if (w) MB_SUMCOH(float, true, false);
    else if (r) MB_SUMCOH(float, false, true); else MB_SUMCOH(float, false, false);
  } else if (dtype == MB_FLOAT64) {
    if (w && r) MB_SUMCOH(double, true, true); else if (w) MB_SUMCOH(double, true, false);
    else if (r) MB_SUMCOH(double, false, true); else MB_SUMCOH(double, false, false);
  } else return fail(MB_ERR_UNSUPPORTED_DTYPE, "dtype %d", int(dtype));
#undef MB_SUMCOH
  return check_launch("mb_sum_coherencies");
}

size_t mb_reduce_chi2_workspace_size(const mb_dims* dims) {
  (void)dims;
  return kReduceBlocks * sizeof(double);
}

mb_status mb_reduce_chi2(mb_dtype dtype, const mb_dims* dims, const void* chi_sqrd_result, double scale,
                         double* X2_out, void* workspace, size_t workspace_bytes, void* stream) {
  MB_CHECK(check_dims(dims, false));
  MB_REQUIRE(chi_sqrd_result, "chi_sqrd_result"); MB_REQUIRE(X2_out, "X2_out");
  if (workspace == nullptr || workspace_bytes < mb_reduce_chi2_workspace_size(dims) ||
      (reinterpret_cast<uintptr_t>(workspace) & 7))
    return fail(MB_ERR_WORKSPACE, "reduction workspace must be >= %zu bytes, 8-byte aligned",
                mb_reduce_chi2_workspace_size(dims));
  StageDims D = stage_dims(dims);
  cudaStream_t s = as_stream(stream);
  double* partial = static_cast<double*>(workspace);
  size_t n = size_t(D.ntime) * D.nbl * D.nchan;
  int blocks = int(std::min<size_t>(kReduceBlocks, std::max<size_t>(1, (n + kThreads - 1) / kThreads)));
  if (dtype == MB_FLOAT32) {
    KernelScope ks_("chi2_partial_kernel", s);
    chi2_partial_kernel<float><<<blocks, kThreads, 0, s>>>((const float*)chi_sqrd_result, D.ntime, D.nbl,
        D.nchan, D.lnbl, D.lchan, partial);
  } else if (dtype == MB_FLOAT64) {
    KernelScope ks_("chi2_partial_kernel", s);
    chi2_partial_kernel<double><<<blocks, kThreads, 0, s>>>((const double*)chi_sqrd_result, D.ntime, D.nbl,
        D.nchan, D.lnbl, D.lchan, partial);
  } else return fail(MB_ERR_UNSUPPORTED_DTYPE, "dtype %d", int(dtype));
  MB_CHECK(check_launch("mb_reduce_chi2 partials"));
  {
    KernelScope ks_("sum_partials_kernel", s);
    sum_partials_kernel<<<1, 1024, 0, s>>>(partial, blocks, scale, X2_out);
  }
  return check_launch("mb_reduce_chi2 final");
}

}  // extern "C"
