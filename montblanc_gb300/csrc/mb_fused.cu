// Fused RIME v4 forward chi^2 and adjoint, CUDA-core arithmetic.
//
// One CTA owns one (time, channel) unit.  For every tile of sources it
//   1. forms the per-antenna terms J(s, a) = E(s, a) . K(s, a) . sqrt(B)(s)
//      in shared memory (the "producer"; nothing is written to HBM),
//   2. accumulates the coherencies of all antenna pairs p <= q,
//      V_pq += shape * J_p J_q^H, from register tiles of RP x RQ antennas,
// and finally applies G, flags, weights and the residual per baseline and
// reduces chi^2 (the epilogue), optionally leaving d chi^2 / dV and
// d chi^2 / dG in the workspace for the adjoint.
//
// The adjoint CTA, per (time, channel), rebuilds the Hermitian matrix of
// d chi^2 / dV over antenna pairs, recomputes J per source tile, forms
// d chi^2 / dJ_a = sum_b shape_ab Y_ab J_b, then chains through E (beam
// interpolation), K (phase) and sqrt(B) (brightness) to the source
// parameters, reducing over antennas in shared memory and over time and
// channel with FP64 atomics.
//
// Reference behaviour: CPUSolver.py:59-737 (forward maths),
// RimeSumCoherencies.py:103-393 (epilogue, source-batch semantics).  The
// adjoint has no reference counterpart.
#include <algorithm>
#include <cstdlib>
#include <mutex>
#include <vector>

#include "mb_fused.h"
#include "mb_tc_layout.cuh"
#include "mb_tcgen05.cuh"

namespace mb {

// Poll limit of the pipeline waits (producer <-> MMA <-> drain) in the
// tensor-core kernels, per device.  A wait that runs out marks the CTA bad;
// the CTA then skips its remaining work, still waits (with the fixed limit
// of tc::mbar_wait) for every MMA it issued, frees its TMEM, and writes
// MB_ERR_TIMEOUT into the workspace's error word (read back by
// mb_rime_status).  mb_set_wait_limit changes it for tests of that path.
__device__ uint32_t g_pipe_wait_limit = 1u << 20;

__global__ void sum_partials_kernel(const double* __restrict__ partial, int n, double scale,
                                    double* __restrict__ out);

namespace {

template <typename T> struct FwdTile;
template <> struct FwdTile<float> { static constexpr int RP = 2, RQ = 4, ST = 32; };
template <> struct FwdTile<double> { static constexpr int RP = 1, RQ = 2, ST = 8; };
template <typename T> struct AdjTile;
// FULL_Y: the Hermitian matrix Y of d chi^2 / dV is kept complete (na x na
// Jones) in shared memory; otherwise only its packed upper triangle.  Full
// rows are padded by 16 bytes (y_row_vals), so that lanes reading the same
// column of consecutive rows hit distinct banks.
template <> struct AdjTile<float> {
  static constexpr int RA = 2, RS = 4, ST = 16, THREADS = 512;
  static constexpr bool FULL_Y = true;
};
template <> struct AdjTile<double> {
  static constexpr int RA = 1, RS = 2, ST = 8, THREADS = 256;
  static constexpr bool FULL_Y = false;
};

constexpr int kNAcc = 10;  // l, m, I, Q, U, V, alpha, shape0, shape1, shape2

// Values (T) per row of the full Y in shared memory: na Jones + 16 bytes.
template <typename T>
__host__ __device__ __forceinline__ int y_row_vals(int na) { return 8 * na + int(16 / sizeof(T)); }

template <typename T>
__device__ __forceinline__ T* y_full(T* sY, int a, int b, int na) { return sY + a * y_row_vals<T>(na) + 8 * b; }
// Values per (source, time) entry of the sqrt(B) table: sqrt(B) at nu_ref
// (a, d, Re b, Im b), alpha / 2, 0, l / n, m / n.
constexpr int kBsqVals = 8;

constexpr size_t kMaxDynamicSmem = 227 * 1024;  // per CTA on sm_100 / sm_103

int count_pair_tiles(int na, int RP, int RQ) {
  int npt = (na + RP - 1) / RP, nqt = (na + RQ - 1) / RQ, n = 0;
  for (int ip = 0; ip < npt; ++ip) n += nqt - (ip * RP) / RQ;
  return n;
}

// Bytes of npairs pair accumulators, dense or padded by 16 bytes after
// every 4 pairs (pair_acc).
inline size_t pair_acc_bytes(size_t jones_bytes, int npairs, bool pad) {
  return jones_bytes * size_t(npairs) + (pad ? size_t(npairs / 4 + 1) * 16 : 0);
}

// with_J = false leaves out the Jones tile (a caller that places it itself),
// with_gJ = false the adjoint's dchi^2/dJ tile (launches of extended sources
// only, which chain each item where it is formed).  tile > 0 asks for that
// many sources per tile; the tile is halved (down to 4) while the plan does
// not fit the shared memory of one CTA.
template <typename T>
SmemPlan make_plan_tile(int na, bool adjoint, bool with_J, int tile, bool with_gJ);

template <typename T>
SmemPlan make_plan(int na, bool adjoint, bool with_J = true, int tile = 0, bool with_gJ = true) {
  if (tile <= 0)
    return make_plan_tile<T>(na, adjoint, with_J, adjoint ? AdjTile<T>::ST : FwdTile<T>::ST, with_gJ);
  SmemPlan S = make_plan_tile<T>(na, adjoint, with_J, tile, with_gJ);
  while (S.total > kMaxDynamicSmem && S.st > 4) S = make_plan_tile<T>(na, adjoint, with_J, S.st / 2, with_gJ);
  return S;
}

template <typename T>
SmemPlan make_plan_tile(int na, bool adjoint, bool with_J, int tile, bool with_gJ) {
  SmemPlan S;
  S.nap = (na + 3) / 4 * 4;
  S.st = tile;
  S.jrow = (S.nap / 4) * (4 * int(sizeof(Jones<T>)) + 16);
  S.npairs = na * (na + 1) / 2;
  S.nitems = count_pair_tiles(na, FwdTile<T>::RP, FwdTile<T>::RQ);
  if (adjoint) {
    S.nthreads = AdjTile<T>::THREADS;
    S.groups = 1;
  } else if (S.nitems <= kFwdMaxThreads) {
    // one pair tile per thread; spare threads split each tile's sources
    S.nthreads = std::max(128, (S.nitems + 31) / 32 * 32);
    S.groups = std::min(8, std::max(1, S.nthreads / S.nitems));
  } else {
    S.nthreads = kFusedThreads;
    S.groups = 1;
  }
  size_t o = 0;
  auto take = [&o](size_t bytes) { size_t r = o; o = align_up(o + bytes, 16); return r; };
  S.off_ant = take(sizeof(AntInfo<T>) * na);
  S.off_antd = take(0);
  S.off_src = take(sizeof(SrcInfo<T>) * S.st);
  S.off_J = take(with_J ? size_t(S.jrow) * S.st : 0);
  S.off_gJ = take(adjoint && with_gJ ? size_t(S.jrow) * S.st : 0);
  S.off_V = take(adjoint && AdjTile<T>::FULL_Y ? sizeof(T) * size_t(na) * y_row_vals<T>(na)
                                                : pair_acc_bytes(sizeof(Jones<T>), S.npairs, !adjoint));
  // FP32 forward: low parts of float-float pair accumulators
  S.off_Vlo = take(!adjoint && sizeof(T) == 4 ? pair_acc_bytes(sizeof(Jones<T>), S.npairs, true) : 0);
  S.off_items = take(adjoint ? 0 : sizeof(int) * (S.nitems + 128));
  S.off_acc = take(adjoint ? sizeof(T) * S.st * kNAcc : 0);
  S.off_red = take(sizeof(double) * 32);
  S.total = o;
  return S;
}

// Jones tiles (J and dchi^2/dJ of a source tile) in shared memory: source si,
// antenna a at byte si * S.jrow + (a / 4) (4 Jones + 16) + (a % 4) Jones.
// The 16 bytes after every 4 antennas put the 4-antenna blocks that
// neighbouring lanes read at an odd number of 16-byte bank groups apart, so
// a quarter warp's 16-byte loads from 8 blocks meet no bank twice.
template <typename T>
__device__ __forceinline__ Jones<T>* jtile(Jones<T>* base, const SmemPlan& S, int si, int a) {
  return reinterpret_cast<Jones<T>*>(reinterpret_cast<unsigned char*>(base) + size_t(si) * S.jrow +
                                     (a >> 2) * (4 * sizeof(Jones<T>) + 16) + (a & 3) * sizeof(Jones<T>));
}
template <typename T>
__device__ __forceinline__ const Jones<T>* jtile(const Jones<T>* base, const SmemPlan& S, int si, int a) {
  return jtile(const_cast<Jones<T>*>(base), S, si, a);
}

// ---------------------------------------------------------------------------
// Shared set-up and producer
// ---------------------------------------------------------------------------
// Batched launches: the parameter set a CTA works on replaces the single
// problem's per-set fields of A (source counts and arrays, tables, partials,
// the forward's d chi^2 / dV and d chi^2 / dG, the FP64 accumulators).  A
// negative sbeg (the extended sources' adjoint of tensor-core sets) becomes
// the set's point-source count.
template <typename T>
__device__ __forceinline__ void use_set(FusedArgs<T>& A, const BatchSet<T>& b) {
  A.lm = b.lm; A.stokes = b.stokes; A.alpha = b.alpha; A.gauss = b.gauss; A.sersic = b.sersic;
  A.npsrc = b.npsrc; A.ngsrc = b.ngsrc; A.nssrc = b.nssrc; A.nsrc = b.npsrc + b.ngsrc + b.nssrc;
  A.lgsrc = b.ngsrc; A.lssrc = b.nssrc;
  A.phi = b.phi; A.bsq0 = b.bsq0; A.partial = b.partial; A.gV = b.gV; A.dG = b.dG;
  A.acc_lm = b.acc_lm; A.acc_stokes = b.acc_stokes; A.acc_alpha = b.acc_alpha;
  A.acc_gauss = b.acc_gauss; A.acc_sersic = b.acc_sersic;
  if (A.sbeg < 0) A.sbeg = b.npsrc;
  // the split forms' extended-source sums: written by the CUDA-core launch
  // (partial_out), added in by the tensor-core launch (accumulate_in)
  if (A.partial_out) A.model_vis = b.vis_ext;
  if (A.accumulate_in) {
    A.vis_in = b.vis_ext;
    A.accumulate_in = b.vis_ext != nullptr;
  }
}

// The (time, channel) unit of this CTA: blockIdx.x for a single problem;
// in a batched launch the CTA's (set, unit) item, whose set it selects.
template <typename T>
__device__ __forceinline__ int cta_unit(FusedArgs<T>& A) {
  if (A.bitems == nullptr) return blockIdx.x;
  const int2 it = A.bitems[blockIdx.x];
  use_set(A, A.bsets[it.x]);
  return it.y;
}

// Global index of local antenna a (identity unless the launch works on an
// antenna sub-array).
template <typename T>
__device__ __forceinline__ int gant(const FusedArgs<T>& A, int a) {
  return a < A.sub_n0 ? A.sub_off0 + a : A.sub_off1 + (a - A.sub_n0);
}

// Local index of global antenna p in this launch's sub-array, or -1.
template <typename T>
__device__ __forceinline__ int lant(const FusedArgs<T>& A, int p) {
  if (A.sub_blk == 0) return p;
  const int b = p / A.sub_blk;
  if (b == A.sub_i) return p - A.sub_off0;
  if (b == A.sub_j) return A.sub_n0 + (p - A.sub_off1);
  return -1;
}

// Does this launch own baseline (p, q) of valid global antennas?  Every
// baseline has exactly one owner among a call's sub-arrays.
template <typename T>
__device__ __forceinline__ bool owns(const FusedArgs<T>& A, int p, int q) {
  if (A.sub_blk == 0) return true;
  const int bp = p / A.sub_blk, bq = q / A.sub_blk;
  if (bp != bq) return min(bp, bq) == A.sub_i && max(bp, bq) == A.sub_j;
  return (bp == A.sub_i && (A.sub_diag & 1)) || (bp == A.sub_j && (A.sub_diag & 2));
}

// Baseline (p, q) of global antennas as local antennas of this launch:
// true if both are valid and the launch owns the baseline.
template <typename T>
__device__ __forceinline__ bool local_baseline(const FusedArgs<T>& A, int p, int q, int& pl, int& ql) {
  if (p < 0 || p >= A.na_glob || q < 0 || q >= A.na_glob || !owns(A, p, q)) return false;
  pl = lant(A, p);
  ql = lant(A, q);
  return true;
}

template <typename T>
__device__ void load_antennas(const FusedArgs<T>& A, int t, int ch, AntInfo<T>* sa) {
  for (int a = threadIdx.x; a < A.na; a += blockDim.x) {
    const int g = gant(A, a);
    size_t ta = size_t(t) * A.lna + g;
    AntInfo<T> ai;
    if (sizeof(T) == 8) {
      double s_, c_; sincos(double(A.pa[ta]), &s_, &c_); ai.sin_pa = T(s_); ai.cos_pa = T(c_);
    } else {
      float s_, c_; sincosf(float(A.pa[ta]), &s_, &c_); ai.sin_pa = T(s_); ai.cos_pa = T(c_);
    }
    size_t tac = ta * A.lchan + ch;
    ai.pe_l = A.pe[2 * tac]; ai.pe_m = A.pe[2 * tac + 1];
    size_t ac = size_t(g) * A.lchan + ch;
    ai.sc_l = A.sc[2 * ac]; ai.sc_m = A.sc[2 * ac + 1];
    ai.u = A.uvw[3 * ta]; ai.v = A.uvw[3 * ta + 1]; ai.w = A.uvw[3 * ta + 2];
    sa[a] = ai;
  }
}

template <typename T>
__device__ __forceinline__ int src_type(const FusedArgs<T>& A, int s) {
  return s < A.npsrc ? SRC_POINT : (s < A.npsrc + A.ngsrc ? SRC_GAUSS : SRC_SERSIC);
}

// Per-source information of global source s at time t, channel ch.
template <typename T>
__device__ __forceinline__ SrcInfo<T> load_source_one(const FusedArgs<T>& A, int t, int ch, int s) {
  const T f = A.freq[ch], rf = A.ref_freq[ch];
  SrcInfo<T> si;
  si.l = A.lm[2 * s]; si.m = A.lm[2 * s + 1];
  {
    const double l = si.l, m = si.m, nf = sqrt(1.0 - l * l - m * m);
    si.l_over_n = T(l / nf);
    si.m_over_n = T(m / nf);
  }
  size_t st = size_t(s) * A.ltime + t;
  si.I = A.stokes[4 * st]; si.Q = A.stokes[4 * st + 1];
  si.U = A.stokes[4 * st + 2]; si.V = A.stokes[4 * st + 3];
  si.power = mb_pow(f / rf, A.alpha[st]);
  si.B = brightness_sqrt<T>(si.I, si.Q, si.U, si.V, si.power);
  si.type = src_type(A, s);
  si.s0 = si.s1 = si.s2 = T(0);
  if (si.type == SRC_GAUSS) {
    int g = s - A.npsrc;
    si.s0 = A.gauss[g]; si.s1 = A.gauss[A.lgsrc + g]; si.s2 = A.gauss[2 * A.lgsrc + g];
  } else if (si.type == SRC_SERSIC) {
    int x = s - A.npsrc - A.ngsrc;
    si.s0 = A.sersic[x]; si.s1 = A.sersic[A.lssrc + x]; si.s2 = A.sersic[2 * A.lssrc + x];
  }
  return si;
}

// Per-source information of the tile [s0, s0 + ns) at time t, frequency f.
template <typename T>
__device__ void load_sources(const FusedArgs<T>& A, int t, int ch, int s0, int ns, SrcInfo<T>* ss) {
  for (int i = threadIdx.x; i < ns; i += blockDim.x) ss[i] = load_source_one(A, t, ch, s0 + i);
}

// K(s, a) at time t.  The path-length table (phi_kernel) holds FP64 values
// for the FP64 forms and, in the same 8 bytes per entry, the FP32 pair of
// the same FP64 value (split_f64) for the FP32 forms, whose phase is then
// formed on the FP32 pipe (frac_cycles_df).
template <typename T>
__device__ __forceinline__ Cx<T> phase_term(const FusedArgs<T>& A, int t, int s, int a, T f, const NuC& nu) {
  double phi;
  const size_t e = (size_t(t) * A.nsrc + s) * A.na_glob + gant(A, a);
  if constexpr (sizeof(T) == 4) {
    if (A.phi != nullptr) return phase_from_pair(__ldg(reinterpret_cast<const float2*>(A.phi) + e), nu.p);
  }
  if (A.phi != nullptr) {
    phi = A.phi[e];
  } else {  // no table: the same FP64 path length, formed in place
    double l = A.lm[2 * s], m = A.lm[2 * s + 1];
    double n = sqrt(1.0 - l * l - m * m) - 1.0;
    const T* p = A.uvw + 3 * (size_t(t) * A.lna + gant(A, a));
    phi = l * double(p[0]) + m * double(p[1]) + n * double(p[2]);
  }
  if (sizeof(T) == 8) return phase_from_phi<T>(phi, double(f));
  return phase_from_cycles<T>(phi, nu.d);
}

// J(s, a) = E(s, a) . (K(s, a) sqrt(B)(s)) for one source and antenna.
template <typename T>
__device__ __forceinline__ Jones<T> compute_jones(const FusedArgs<T>& A, int t, int s, int a, const SrcInfo<T>& src,
                                                  const AntInfo<T>& ai, T f, const NuC& nu,
                                                  const ChanPos<T>& cp, int plane_ch) {
  const BeamGeom G{A.lw, A.mh, A.nud};
  Cx<T> K = phase_term(A, t, s, a, f, nu);
  T l, m;
  beam_lm<T>(src.l, src.m, ai.sin_pa, ai.cos_pa, ai.pe_l, ai.pe_m, ai.sc_l, ai.sc_m, l, m);
  GridPos<T> gl = grid_pos<T>(l, A.ll, A.ul, A.lscale, A.lw);
  GridPos<T> gm = grid_pos<T>(m, A.lmm, A.um, A.mscale, A.mh);
  Jones<T> E = A.plane ? beam_interp_plane<T>(A.plane + size_t(plane_ch) * A.lw * A.mh * kPlaneVals, A.mh, gl, gm)
                       : beam_interp<T>(A.E_beam, G, gl, gm, cp);
  Jones<T> KB = {cmul(K, src.B.a), cmul(K, src.B.b), cmul(K, src.B.c), cmul(K, src.B.d)};
  return jmul(E, KB);
}

// J(s, a) for the tile into the Jones tile sJ; padded antennas get zeros.
// DF (the FP64 forward): each FP64 value is stored as the double-float pair
// (hi, lo) = (float(x), float(x - hi)) in the same 8 bytes, for the pair
// sums of consume_pairs.
template <typename T, bool DF = false>
__device__ void produce_jones(const FusedArgs<T>& A, const SmemPlan& S, int t, int ch, int s0, int ns,
                              const SrcInfo<T>* ss, const AntInfo<T>* sa, Jones<T>* sJ, const ChanPos<T>& cp) {
  const T f = A.freq[ch];
  const NuC nu = make_nuc(double(f) / kLightSpeed);
  for (int i = threadIdx.x; i < ns * S.nap; i += blockDim.x) {
    int si = i / S.nap, a = i - si * S.nap;
    const Jones<T> J = a < A.na ? compute_jones(A, t, s0 + si, a, ss[si], sa[a], f, nu, cp, ch)
                                : jzero<T>();
    if constexpr (DF && sizeof(T) == 8) {  // per entry (re hi, im hi, re lo, im lo)
      const double* v = reinterpret_cast<const double*>(&J);
      float4* o = reinterpret_cast<float4*>(jtile(sJ, S, si, a));
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const float hr = float(v[2 * k]), hi = float(v[2 * k + 1]);
        o[k] = make_float4(hr, hi, float(v[2 * k] - double(hr)), float(v[2 * k + 1] - double(hi)));
      }
    } else {
      *jtile(sJ, S, si, a) = J;
    }
  }
}

template <typename T>
__device__ __forceinline__ T shape_factor(int type, T u, T v, T s0, T s1, T s2, T kg, T ks) {
  return type == SRC_GAUSS ? gauss_shape<T>(u, v, s0, s1, s2, kg) : sersic_shape<T>(u, v, s0, s1, s2, ks);
}

template <typename T>
__device__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x < 32) {
    r = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
  }
  return r;
}

template <typename T>
__device__ __forceinline__ void atomic_add_jones(Jones<T>* dst, const Jones<T>& x) {
  T* d = reinterpret_cast<T*>(dst);
  atomicAdd(d + 0, x.a.r); atomicAdd(d + 1, x.a.i); atomicAdd(d + 2, x.b.r); atomicAdd(d + 3, x.b.i);
  atomicAdd(d + 4, x.c.r); atomicAdd(d + 5, x.c.i); atomicAdd(d + 6, x.d.r); atomicAdd(d + 7, x.d.i);
}

// Adds the NV values of every active lane to acc[key * stride + j].  When
// all active lanes of the warp share one key the warp sums first and one
// lane adds; otherwise each active lane adds its own.  Every lane of the
// warp calls it; key < 0 marks an inactive lane (its values must be 0).
template <typename T, int NV>
__device__ __forceinline__ void warp_keyed_add_stride(T* acc, int stride, int key, T (&v)[NV]) {
  const unsigned full = 0xffffffffu;
  const int k0 = __reduce_max_sync(full, key);
  if (__all_sync(full, key < 0 || key == k0)) {
    if (k0 < 0) return;
#pragma unroll
    for (int j = 0; j < NV; ++j)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v[j] += __shfl_xor_sync(full, v[j], o);
    if ((threadIdx.x & 31) == 0)
#pragma unroll
      for (int j = 0; j < NV; ++j) atomicAdd(acc + k0 * stride + j, v[j]);
  } else if (key >= 0) {
#pragma unroll
    for (int j = 0; j < NV; ++j) atomicAdd(acc + key * stride + j, v[j]);
  }
}

// Pair accumulator of packed pair index idx.  The CUDA-core forward (PAD)
// leaves 16 bytes after every 4 pairs: the lanes of a warp fold the pair
// tiles of one row, 4 pairs apart, which would otherwise sit a multiple of
// 128 bytes apart, on the same banks (one 16-byte access per lane and
// step: an 8-way conflict); with the pad they fall on 8 distinct 16-byte
// bank groups.  The tensor-core forward's drain writes the dense layout.
template <bool PAD, typename T>
__device__ __forceinline__ Jones<T>* pair_acc(Jones<T>* base, int idx) {
  if (!PAD) return base + idx;
  return reinterpret_cast<Jones<T>*>(reinterpret_cast<unsigned char*>(base) + size_t(idx) * sizeof(Jones<T>) +
                                     size_t(idx >> 2) * 16);
}
template <bool PAD, typename T>
__device__ __forceinline__ const Jones<T>* pair_acc(const Jones<T>* base, int idx) {
  return pair_acc<PAD>(const_cast<Jones<T>*>(base), idx);
}

// ---------------------------------------------------------------------------
// Epilogue (shared with the tensor-core path)
// ---------------------------------------------------------------------------
template <bool PAD, typename T>
__device__ void epilogue(const FusedArgs<T>& A, int t, int ch, int unit, const Jones<T>* sV, Jones<T>* scratch,
                         double* red) {
  Jones<T>* sG = scratch;
  Jones<T>* sdG = scratch + A.na;
  for (int a = threadIdx.x; a < A.na; a += blockDim.x) {
    sG[a] = jldg<T>(A.G + 8 * ((size_t(t) * A.lna + gant(A, a)) * A.lchan + ch));
    if (A.want_grad) sdG[a] = jzero<T>();
  }
  __syncthreads();
  double part = 0.0;
  // Whole rounds of blockDim baselines, so that every lane of a warp takes
  // part in the keyed warp sum of dchi^2/dG below.
  const int rounds = (A.nbl + blockDim.x - 1) / blockDim.x;
  for (int round = 0; round < rounds; ++round) {
    const int bl = round * blockDim.x + threadIdx.x;
    int key_p = -1;                  // antenna 1 of this lane's dchi^2/dG term (-1: none)
    Jones<T> gp = jzero<T>();        // the term itself
    if (bl < A.nbl) {
      size_t tbl = size_t(t) * A.lnbl + bl;
      int p = A.ant1[tbl], q = A.ant2[tbl];
      size_t vidx = tbl * A.lchan + ch;
      const bool valid = p >= 0 && p < A.na_glob && q >= 0 && q < A.na_glob;
      // with antenna sub-arrays, each baseline is written by the launch that
      // owns it (invalid ones by the first), in local antenna indices
      const bool mine = valid ? owns(A, p, q) : (A.sub_blk == 0 || (A.sub_i == 0 && A.sub_j == 1));
      if (mine && valid) {
        p = lant(A, p);
        q = lant(A, q);
      }
      if (!mine) {
      } else if (!valid) {  // invalid antenna index: NaN output
        const T nan = T(NAN);
        if (A.model_vis) jstore(A.model_vis + 8 * vidx, Jones<T>{{nan, nan}, {nan, nan}, {nan, nan}, {nan, nan}});
        if (A.chi2 && !A.partial_out) A.chi2[vidx] = nan;
        part += double(nan);
        if (A.want_grad) jstore(A.gV + 8 * ((size_t(t) * A.nbl + bl) * A.nchan + ch), jzero<T>());
      } else {
        Jones<T> V = p <= q ? *pair_acc<PAD>(sV, pair_index(p, q, A.na))
                            : jherm(*pair_acc<PAD>(sV, pair_index(q, p, A.na)));
        if (A.accumulate_in) V = jadd(V, jload<T>(A.vis_in + 8 * vidx));
        if (A.partial_out) {
          jstore(A.model_vis + 8 * vidx, V);
        } else {
          const Jones<T> Gp = sG[p], Gq = sG[q];
          Jones<T> M = jmulh(jmul(Gp, V), Gq);
          Jones<T> O = jldg<T>(A.obs + 8 * vidx);
          uchar4 fl = *reinterpret_cast<const uchar4*>(A.flag + 4 * vidx);
          const uint8_t fv[4] = {fl.x, fl.y, fl.z, fl.w};
          T w4[4] = {T(1), T(1), T(1), T(1)};
          if (A.weights) {
            for (int k = 0; k < 4; ++k) w4[k] = A.weight[4 * vidx + k];
          }
          Cx<T>* m4 = &M.a;
          Cx<T>* o4 = &O.a;
          Jones<T> R, gM;
          Cx<T>* r4 = &R.a;
          Cx<T>* g4 = &gM.a;
          T term = T(0);
          const T gscale = A.weights ? T(-2) : T(-2.0 * A.inv_sigma2);
          for (int k = 0; k < 4; ++k) {
            if (fv[k] > 0) { m4[k] = Cx<T>{T(0), T(0)}; o4[k] = Cx<T>{T(0), T(0)}; }
            r4[k] = o4[k] - m4[k];
            T re2 = r4[k].r * r4[k].r, im2 = r4[k].i * r4[k].i;
            if (A.weights) { re2 *= w4[k]; im2 *= w4[k]; }
            term += re2 + im2;
            g4[k] = fv[k] > 0 ? Cx<T>{T(0), T(0)} : r4[k] * (gscale * w4[k]);
          }
          if (A.model_vis) jstore(A.model_vis + 8 * vidx, A.residuals ? R : M);
          if (A.chi2) A.chi2[vidx] = term;
          part += double(term);
          if (A.want_grad) {
            Jones<T> gV = jmul(jhmul(Gp, gM), Gq);
            jstore(A.gV + 8 * ((size_t(t) * A.nbl + bl) * A.nchan + ch), gV);
            key_p = p;
            gp = jmul(gM, jmulh(Gq, V));
            // antenna 2 differs from lane to lane (consecutive baselines)
            atomic_add_jones(&sdG[q], jmul(jherm(gM), jmul(Gp, V)));
          }
        }
      }
    }
    // antenna 1 is mostly shared by the warp's consecutive baselines: sum
    // over the warp first, then one lane adds
    if (A.want_grad && !A.partial_out) {
      T* gv = reinterpret_cast<T*>(&gp);
      T v8[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) v8[k] = gv[k];
      warp_keyed_add_stride<T, 8>(reinterpret_cast<T*>(sdG), 8, key_p, v8);
    }
  }
  double tot = block_sum<T>(part, red);
  if (threadIdx.x == 0) A.partial[unit] = tot;
  if (A.want_grad) {
    __syncthreads();
    for (int a = threadIdx.x; a < A.na; a += blockDim.x) {
      T* dst = A.dG + 8 * ((size_t(t) * A.na_glob + gant(A, a)) * A.nchan + ch);
      if (A.sub_blk == 0) jstore(dst, sdG[a]);
      else atomic_add_jones(reinterpret_cast<Jones<T>*>(dst), sdG[a]);  // antenna in several sub-arrays
    }
  }
}

// ---------------------------------------------------------------------------
// Forward
// ---------------------------------------------------------------------------
// Pair accumulators: FP64 in FP64 mode; float-float (hi + lo, TwoSum) in
// FP32 mode, so that the sum over thousands of source tiles does not lose
// the precision of FP32 (the per-tile partial sums are plain FP32).
template <typename T>
__device__ __forceinline__ void fold_pair(Jones<T>* sV, Jones<T>* sVlo, const Jones<T>& x) {
  T* hi = reinterpret_cast<T*>(sV);
  const T* xv = reinterpret_cast<const T*>(&x);
  if (sVlo == nullptr) {
#pragma unroll
    for (int k = 0; k < 8; ++k) hi[k] += xv[k];
    return;
  }
  T* lo = reinterpret_cast<T*>(sVlo);
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    T a = hi[k], b = xv[k];
    T sum = a + b;
    T bp = sum - a;
    T err = (a - (sum - bp)) + (b - bp);
    hi[k] = sum;
    lo[k] += err;
  }
}

// Double-float arithmetic for the FP64 forward's pair sums.  GB300 runs FP32
// at 64 times its FP64 rate, so the O(na^2) pair sums of the FP64 forward
// use values held as hi + lo FP32 pairs (about 48 significant bits): an
// exact product by FMA (Dekker's product, with the cross terms of the low
// parts) added to the accumulator by TwoSum (Knuth), 11 FP32 operations per
// multiply-add against one FP64 FMA, and the real and imaginary parts of a
// complex value share packed FP32x2 instructions, so a complex multiply-add
// takes 24 of them; per tile the sums are converted to FP64 and folded into
// the FP64 pair accumulators.  The per-antenna terms J and the shape factors
// are formed in FP64.
//
// A complex double-float value: h = (re hi, im hi), l = (re lo, im lo).
struct CDf {
  float2 h, l;
};
struct JDf {
  CDf a, b, c, d;
};

// acc += x * (bh + bl): per lane, Dekker's product of x and the scalar
// double-float b (exact by FMA, with the cross terms of the low parts), added
// to acc by TwoSum.  12 packed instructions for the two lanes.
__device__ __forceinline__ void cdf_mac(CDf& acc, float2 xh, float2 xl, float bh, float bl) {
  const float2 bh2 = make_float2(bh, bh), bl2 = make_float2(bl, bl);
  const float2 p = __fmul2_rn(xh, bh2);
  float2 e = __ffma2_rn(xh, bh2, make_float2(-p.x, -p.y));
  e = __ffma2_rn(xh, bl2, e);
  e = __ffma2_rn(xl, bh2, e);
  const float2 s = __fadd2_rn(acc.h, p);
  const float2 v = __fadd2_rn(s, make_float2(-acc.h.x, -acc.h.y));
  const float2 sv = __fadd2_rn(s, make_float2(-v.x, -v.y));
  const float2 t = __fadd2_rn(__fadd2_rn(acc.h, make_float2(-sv.x, -sv.y)), __fadd2_rn(p, make_float2(-v.x, -v.y)));
  acc.h = s;
  acc.l = __fadd2_rn(acc.l, __fadd2_rn(t, e));
}
// acc += a * conj(b) = (a.r, a.i) b.r + (a.i, -a.r) b.i
__device__ __forceinline__ void cmacc_df(CDf& acc, const CDf& a, const CDf& b) {
  cdf_mac(acc, a.h, a.l, b.h.x, b.l.x);
  cdf_mac(acc, make_float2(a.h.y, -a.h.x), make_float2(a.l.y, -a.l.x), b.h.y, b.l.y);
}
// acc += X * Y^H
__device__ __forceinline__ void jmac_h_df(JDf& acc, const JDf& X, const JDf& Y) {
  cmacc_df(acc.a, X.a, Y.a); cmacc_df(acc.a, X.b, Y.b);
  cmacc_df(acc.b, X.a, Y.c); cmacc_df(acc.b, X.b, Y.d);
  cmacc_df(acc.c, X.c, Y.a); cmacc_df(acc.c, X.d, Y.b);
  cmacc_df(acc.d, X.c, Y.c); cmacc_df(acc.d, X.d, Y.d);
}
// A Jones tile entry written by produce_jones<double, true>.
__device__ __forceinline__ JDf jdf_load(const Jones<double>* p) {
  const float4* q = reinterpret_cast<const float4*>(p);
  JDf J;
  CDf* e = &J.a;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float4 x = q[k];
    e[k] = {make_float2(x.x, x.y), make_float2(x.z, x.w)};
  }
  return J;
}
__device__ __forceinline__ JDf jdf_zero() {
  JDf J;
  J.a = J.b = J.c = J.d = CDf{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
  return J;
}
// x * s, s an FP64 scalar, rounded back to double-float per lane (the
// product's low part kept)
__device__ __forceinline__ CDf cdf_scale(const CDf& x, float sh, float sl) {
  const float2 sh2 = make_float2(sh, sh), sl2 = make_float2(sl, sl);
  const float2 p = __fmul2_rn(x.h, sh2);
  float2 e = __ffma2_rn(x.h, sh2, make_float2(-p.x, -p.y));
  e = __ffma2_rn(x.h, sl2, e);
  e = __ffma2_rn(x.l, sh2, e);
  const float2 s = __fadd2_rn(p, e);
  const float2 d = __fadd2_rn(s, make_float2(-p.x, -p.y));
  return {s, __fadd2_rn(e, make_float2(-d.x, -d.y))};
}
__device__ __forceinline__ JDf jdf_scale(const JDf& X, double s) {
  const float sh = float(s), sl = float(s - double(sh));
  return {cdf_scale(X.a, sh, sl), cdf_scale(X.b, sh, sl), cdf_scale(X.c, sh, sl), cdf_scale(X.d, sh, sl)};
}
__device__ __forceinline__ Cx<double> cdf_value(const CDf& x) {
  return {double(x.h.x) + double(x.l.x), double(x.h.y) + double(x.l.y)};
}
__device__ __forceinline__ Jones<double> jdf_value(const JDf& X) {
  return {cdf_value(X.a), cdf_value(X.b), cdf_value(X.c), cdf_value(X.d)};
}

// consume_pairs for the FP64 forward on double-float Jones tiles (same work
// items, groups and fold as consume_pairs).
template <int RP, int RQ, bool PAD>
__device__ void consume_pairs_df(const FusedArgs<double>& A, const SmemPlan& S, int ns, const SrcInfo<double>* ss,
                                 const AntInfo<double>* sa, const Jones<double>* sJ, Jones<double>* sV,
                                 const int* items, bool extended, double kg, double ks) {
  const int total = S.nitems * S.groups;
  const int rounds = (total + blockDim.x - 1) / blockDim.x;
  for (int round = 0; round < rounds; ++round) {
    const int k = round * blockDim.x + threadIdx.x;
    const bool active = k < total;
    const int item = active ? k % S.nitems : 0, g = active ? k / S.nitems : 0;
    const int it = items[item];
    const int p0 = (it & 0xffff) * RP, q0 = (it >> 16) * RQ;
    JDf acc[RP][RQ];
    double u[RP][RQ], v[RP][RQ];
#pragma unroll
    for (int r = 0; r < RP; ++r)
#pragma unroll
      for (int c = 0; c < RQ; ++c) {
        acc[r][c] = jdf_zero();
        if (extended) {
          int pp = min(p0 + r, A.na - 1), qq = min(q0 + c, A.na - 1);
          u[r][c] = sa[qq].u - sa[pp].u;
          v[r][c] = sa[qq].v - sa[pp].v;
        }
      }
    if (active) {
      for (int si = g; si < ns; si += S.groups) {
        JDf Ja[RP], Jb[RQ];
#pragma unroll
        for (int r = 0; r < RP; ++r) Ja[r] = jdf_load(jtile(sJ, S, si, p0 + r));
#pragma unroll
        for (int c = 0; c < RQ; ++c) Jb[c] = jdf_load(jtile(sJ, S, si, q0 + c));
        if (!extended) {
#pragma unroll
          for (int r = 0; r < RP; ++r)
#pragma unroll
            for (int c = 0; c < RQ; ++c) jmac_h_df(acc[r][c], Ja[r], Jb[c]);
        } else {
          const SrcInfo<double>& src = ss[si];
#pragma unroll
          for (int r = 0; r < RP; ++r)
#pragma unroll
            for (int c = 0; c < RQ; ++c) {
              const double sh = shape_factor<double>(src.type, u[r][c], v[r][c], src.s0, src.s1, src.s2, kg, ks);
              jmac_h_df(acc[r][c], jdf_scale(Ja[r], sh), Jb[c]);
            }
        }
      }
    }
    for (int gg = 0; gg < S.groups; ++gg) {
      if (S.groups > 1) __syncthreads();
      if (active && g == gg) {
#pragma unroll
        for (int r = 0; r < RP; ++r)
#pragma unroll
          for (int c = 0; c < RQ; ++c) {
            int p = p0 + r, q = q0 + c;
            if (p <= q && q < A.na)
              fold_pair(pair_acc<PAD>(sV, pair_index(p, q, A.na)), static_cast<Jones<double>*>(nullptr),
                        jdf_value(acc[r][c]));
          }
      }
    }
  }
}

// Accumulate the tile's sources into the pair matrix.  Work item k covers
// pair tile (k mod nitems) for the sources si = g, g + G, ... of the tile,
// g = k / nitems, G = S.groups.  With G > 1 every thread owns at most one
// item and the groups fold their partial sums one after the other.
template <typename T, int RP, int RQ, bool PAD>
__device__ void consume_pairs(const FusedArgs<T>& A, const SmemPlan& S, int ns, const SrcInfo<T>* ss,
                              const AntInfo<T>* sa, const Jones<T>* sJ, Jones<T>* sV, Jones<T>* sVlo,
                              const int* items, bool extended, T kg, T ks) {
  const int total = S.nitems * S.groups;
  const int rounds = (total + blockDim.x - 1) / blockDim.x;
  for (int round = 0; round < rounds; ++round) {
    const int k = round * blockDim.x + threadIdx.x;
    const bool active = k < total;
    const int item = active ? k % S.nitems : 0, g = active ? k / S.nitems : 0;
    const int it = items[item];
    const int p0 = (it & 0xffff) * RP, q0 = (it >> 16) * RQ;
    Jones<T> acc[RP][RQ];
    T u[RP][RQ], v[RP][RQ];
#pragma unroll
    for (int r = 0; r < RP; ++r)
#pragma unroll
      for (int c = 0; c < RQ; ++c) {
        acc[r][c] = jzero<T>();
        if (extended) {
          int pp = min(p0 + r, A.na - 1), qq = min(q0 + c, A.na - 1);
          u[r][c] = sa[qq].u - sa[pp].u;
          v[r][c] = sa[qq].v - sa[pp].v;
        }
      }
    if (active) {
      for (int si = g; si < ns; si += S.groups) {
        Jones<T> Ja[RP], Jb[RQ];
#pragma unroll
        for (int r = 0; r < RP; ++r) Ja[r] = jload<T>(reinterpret_cast<const T*>(jtile(sJ, S, si, p0 + r)));
#pragma unroll
        for (int c = 0; c < RQ; ++c) Jb[c] = jload<T>(reinterpret_cast<const T*>(jtile(sJ, S, si, q0 + c)));
        if (!extended) {
#pragma unroll
          for (int r = 0; r < RP; ++r)
#pragma unroll
            for (int c = 0; c < RQ; ++c) jmac_h(acc[r][c], Ja[r], Jb[c]);
        } else {
          const SrcInfo<T>& src = ss[si];
#pragma unroll
          for (int r = 0; r < RP; ++r)
#pragma unroll
            for (int c = 0; c < RQ; ++c) {
              T sh = shape_factor<T>(src.type, u[r][c], v[r][c], src.s0, src.s1, src.s2, kg, ks);
              jmac_h(acc[r][c], jscale(Ja[r], sh), Jb[c]);
            }
        }
      }
    }
    for (int gg = 0; gg < S.groups; ++gg) {
      if (S.groups > 1) __syncthreads();
      if (active && g == gg) {
#pragma unroll
        for (int r = 0; r < RP; ++r)
#pragma unroll
          for (int c = 0; c < RQ; ++c) {
            int p = p0 + r, q = q0 + c;
            if (p <= q && q < A.na) {
              const int idx = pair_index(p, q, A.na);
              fold_pair(pair_acc<PAD>(sV, idx), sVlo ? pair_acc<PAD>(sVlo, idx) : nullptr, acc[r][c]);
            }
          }
      }
    }
  }
}

// BATCHED: CTAs are (set, unit) items of a batched launch (a separate
// instantiation, so that the single-problem kernel keeps the per-set fields
// in the parameter space instead of registers).
template <typename T, int RP, int RQ, bool BATCHED>
__global__ void __launch_bounds__(kFwdMaxThreads) coh_fwd_kernel(FusedArgs<T> A_in, SmemPlan S) {
  extern __shared__ __align__(16) unsigned char smem[];
  AntInfo<T>* sa = reinterpret_cast<AntInfo<T>*>(smem + S.off_ant);
  SrcInfo<T>* ss = reinterpret_cast<SrcInfo<T>*>(smem + S.off_src);
  Jones<T>* sJ = reinterpret_cast<Jones<T>*>(smem + S.off_J);
  Jones<T>* sV = reinterpret_cast<Jones<T>*>(smem + S.off_V);
  Jones<T>* sVlo = sizeof(T) == 4 ? reinterpret_cast<Jones<T>*>(smem + S.off_Vlo) : nullptr;
  int* items = reinterpret_cast<int*>(smem + S.off_items);
  double* red = reinterpret_cast<double*>(smem + S.off_red);

  FusedArgs<T> A = A_in;
  int unit = blockIdx.x;
  if constexpr (BATCHED) unit = cta_unit(A);
  const int t = unit / A.nchan, ch = unit - t * A.nchan;
  load_antennas(A, t, ch, sa);
  for (int i = threadIdx.x; i < S.npairs; i += blockDim.x) {
    *pair_acc<true>(sV, i) = jzero<T>();
    if (sVlo) *pair_acc<true>(sVlo, i) = jzero<T>();
  }
  if (threadIdx.x == 0) {
    const int npt = (A.na + RP - 1) / RP, nqt = (A.na + RQ - 1) / RQ;
    int k = 0;
    for (int ip = 0; ip < npt; ++ip)
      for (int jq = (ip * RP) / RQ; jq < nqt; ++jq) items[k++] = ip | (jq << 16);
  }
  __syncthreads();

  const T f = A.freq[ch];
  const ChanPos<T> cp = chan_pos<T>(f, A.lfreq, A.ufreq, A.nud);
  const T kg = A.gauss_scale * f, ks = A.two_pi_over_c * f;
  for (int s0 = A.sbeg; s0 < A.nsrc;) {
    int s1 = s0 < A.npsrc ? min(s0 + S.st, A.npsrc) : min(s0 + S.st, A.nsrc);
    int ns = s1 - s0;
    load_sources(A, t, ch, s0, ns, ss);
    __syncthreads();
    if constexpr (sizeof(T) == 8) {  // FP64: pair sums in double-float
      produce_jones<T, true>(A, S, t, ch, s0, ns, ss, sa, sJ, cp);
      __syncthreads();
      consume_pairs_df<RP, RQ, true>(A, S, ns, ss, sa, sJ, sV, items, s0 >= A.npsrc, kg, ks);
    } else {
      produce_jones(A, S, t, ch, s0, ns, ss, sa, sJ, cp);
      __syncthreads();
      consume_pairs<T, RP, RQ, true>(A, S, ns, ss, sa, sJ, sV, sVlo, items, s0 >= A.npsrc, kg, ks);
    }
    __syncthreads();
    s0 = s1;
  }
  if (sVlo) {  // collapse the float-float accumulators
    for (int i = threadIdx.x; i < S.npairs; i += blockDim.x)
      *pair_acc<true>(sV, i) = jadd(*pair_acc<true>(sV, i), *pair_acc<true>(sVlo, i));
    __syncthreads();
  }
  epilogue<true>(A, t, ch, unit, sV, sJ, red);
}

// ---------------------------------------------------------------------------
// Split-precision forward: point-source coherencies on the tensor cores
// ---------------------------------------------------------------------------
// Per (time, channel) unit, with A (128 x 4k) the per-stage operand whose row
// r = 2a + i holds, for the stage's k sources s and Jones columns c,
// Re J_s,a[i][c] (K index 2s + c) and Im J_s,a[i][c] (K index 2k + 2s + c):
//   D_re = A A^T                      = Re sum_s J_a J_b^H  (rows 2a+i, columns 2b+j)
//   D_im = A_im A_re^T - A_re A_im^T  = Im sum_s J_a J_b^H
// (the second product with the instruction's negate-A bit).  D_re is
// symmetric and D_im antisymmetric, so each antenna pair is drained once,
// from whichever of (a, b), (b, a) the cyclic rule in tc_drain picks.
// Each operand value is split into hi + lo parts: the large hi.hi products
// and the small hi.lo + lo.hi corrections accumulate in separate TMEM
// accumulators (FP32).  Every kTcGroup stages their sum is folded into FP32
// pair accumulators in shared memory, and the fold's rounding error goes
// back into the correction accumulator (tc_drain), so pair and correction
// accumulators together hold a float-float sum.  The tensor core's FP32
// accumulation rounds toward zero, so its error grows with the number of
// accumulations into one accumulator (about 2.5e-8 of the result per
// accumulation for a coherent sum).  Measured on 20 000 point sources, each
// stage of a group adds about 1.1e-7 to the relative visibility error
// against FP64 (4 stages: 5.9e-7, 5: 7.0e-7, 6: 8.1e-7, 7: 9.2e-7), while
// each drain costs a pass over the pair accumulators; 6 stages keep the
// error below 1e-6 with margin.
constexpr int kTcProducerWarps = 11;       // warps 0-10: operands (one source each), drain
constexpr int kTcProducers = 32 * kTcProducerWarps;
constexpr int kTcThreads = kTcProducers + 32;  // warp 11: MMA issue, drain
constexpr int kTcStages = 3;                // operand stages in flight
constexpr int kTcGroup = 6;                // stages per TMEM accumulation group (66 sources)
// TMEM columns: D_re 0-127, D_im 128-255 (hi.hi); their corrections 256-511.
constexpr uint32_t kTcCols = 512;

// Stage geometry: kSlots source slots per stage (the producer warps fill
// kTcProducerWarps of them, the rest stay zero), so that the K values of the
// real and of the imaginary parts (2 kSlots each) fill whole MMA K steps.
template <int MODE> struct TcGeom;
template <> struct TcGeom<MB_MODE_SPLIT_TF32> {
  static constexpr int kSlots = 12, kRowBytes = kSlots * 4 * 4;  // 6 K steps of 8
};
template <> struct TcGeom<MB_MODE_SPLIT_BF16> {
  static constexpr int kSlots = 16, kRowBytes = kSlots * 4 * 2;  // 4 K steps of 16
};
static_assert(TcGeom<MB_MODE_SPLIT_TF32>::kSlots >= kTcProducerWarps, "a slot per producer warp");
static_assert(TcGeom<MB_MODE_SPLIT_BF16>::kSlots >= kTcProducerWarps, "a slot per producer warp");

struct TcPlan {
  size_t off_stage, off_vlo32, off_bar, total;
  int group;
};

// Adds drained group sums x.x, x.y to the pair accumulators *h0, *h1 and
// returns the rounding errors of the additions (packed FP32x2 adds).
// Fast2Sum: x - ((h + x) - h) is exact when |h| >= |x|, the usual case (h
// is the sum over all earlier groups; also exact while h is 0); otherwise
// it is off by at most an ulp of the sum, the error of one plain FP32
// addition.
__device__ __forceinline__ float2 fold_carry2(float* h0, float* h1, float2 x) {
  const float2 a = make_float2(*h0, *h1);
  const float2 sum = __fadd2_rn(a, x);
  *h0 = sum.x;
  *h1 = sum.y;
  const float2 d = __fadd2_rn(sum, make_float2(-a.x, -a.y));
  return __fadd2_rn(x, make_float2(-d.x, -d.y));
}

// Drain TMEM into the FP32 pair accumulators (all 12 warps): a warp reads
// the 32 TMEM lanes of its quarter (rows 2a + i) and takes every third of the
// quarter's 8 tasks (D_re or D_im, one block of 16 column antennas).  Each
// unordered antenna pair is drained once, by the row whose cyclic distance
// to the other is below na / 2 (ties: the smaller index), so every row
// drains about na / 2 columns and the warps share the work evenly: row a
// drains the antennas b of the cyclic interval [a, a + dmax], b in
// [a, up_hi] from its own block of V_ab and the wrapped b in [0, wrap_end]
// as V_ba = (sum J_a J_b^H)^H (transposed, conjugated).
// Each drained value is main + correction accumulator; the rounding error
// of adding it to the pair accumulator is written back (carry) into the
// correction accumulator's entry, which the next group's hi.lo + lo.hi MMAs
// add to and the next drain of the same entry (by the same lane) folds in.
// So the pair accumulators together with the correction accumulators hold
// the sum as a float-float value with no low part in shared memory.  Entries
// a lane does not fold get a zero carry.
// Element offsets of the pair accumulators (pair_index(p, q) * 8 + (2 row +
// col) * 2 + re/im) split into a per-lane part and a part in b and j:
//   b >= a:  ku + 8 b + 2 j,  ku = 8 (a na - a (a - 1) / 2 - a) + 4 i + h
//   b <  a:  8 R_b + kl + 4 j,  kl = 8 a + 2 i + h,  R_b = b na - b (b - 1) / 2 - b
// PACK (at most 32 antennas, two channels per CTA): rows 64 c + 2 a + i and
// columns 64 c + 2 b + j hold channel c; only its diagonal block is
// drained, into the pair accumulators of channel c (c npairs Jones on).
template <bool PACK>
__device__ void tc_drain(const FusedArgs<float>& A, uint32_t tmem, float* sVf, bool carry, int nch) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int q = warp & 3, jw = warp >> 2;  // lane quarter, and the warp's index among its 3 warps
  const int r = 32 * q + lane, i = r & 1;
  const int c = PACK ? (r >> 6) : 0, a = PACK ? ((r >> 1) & 31) : (r >> 1);
  const int na = A.na;
  const bool row_ok = a < na && c < nch;
  if (PACK) sVf += size_t(c) * (na * (na + 1) / 2) * 8;
  const int dmax = (na - 1) / 2 + ((na % 2 == 0 && a < na / 2) ? 1 : 0);
  const int up_hi = row_ok ? min(a + dmax, na - 1) : -1;
  const int wrap_end = row_ok ? a + dmax - na : -1;
  const int ku0 = 8 * (a * na - (a * (a - 1)) / 2 - a) + 4 * i;
  const int kl0 = 8 * a + 2 * i;
  // 8 tasks (matrix h, column block blk of 16 antennas) per lane quarter
  // (PACK: 4, the blocks of the quarter's channel), dealt to its warps
  constexpr int kTasks = PACK ? 4 : 8;
#pragma unroll 1
  for (int task = jw; task < kTasks; task += 3) {
    const int h = PACK ? task >> 1 : task >> 2, blk = PACK ? task & 1 : task & 3;
    const int ku = ku0 + h, kl = kl0 + h;
    const float sgn = h ? -1.f : 1.f;
    const uint32_t lane_addr = tmem + (uint32_t(32 * q) << 16) + uint32_t(h * 128) + uint32_t(PACK ? 64 * c : 0);
    const int b_lo = 16 * blk;
    const bool need = (max(a, b_lo) <= min(up_hi, b_lo + 15)) || (wrap_end >= b_lo);
    if (!__any_sync(0xffffffffu, need)) continue;  // warp-uniform: the loads are collective
    float v[32], w[32];
    tc::tmem_ld32x2(lane_addr + 32 * blk, lane_addr + 256 + 32 * blk, v, w);
#pragma unroll
    for (int k = 0; k < 32; k += 2) {
      const float2 m = __fadd2_rn(make_float2(v[k], v[k + 1]), make_float2(w[k], w[k + 1]));  // main + correction
      v[k] = m.x;
      v[k + 1] = m.y;
      w[k] = w[k + 1] = 0.f;  // carries
    }
    if (need) {
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        const int b = b_lo + c;
        const float2 x = make_float2(v[2 * c], v[2 * c + 1]);
        float2 r = make_float2(0.f, 0.f);
        if (b >= a && b <= up_hi) {
          const int e = ku + 8 * b;
          r = fold_carry2(sVf + e, sVf + e + 2, x);
        } else if (b <= wrap_end) {
          const int e = 8 * (b * na - (b * (b - 1)) / 2 - b) + kl;
          r = fold_carry2(sVf + e, sVf + e + 4, make_float2(sgn * x.x, sgn * x.y));
          r = make_float2(sgn * r.x, sgn * r.y);
        }
        w[2 * c] = r.x;
        w[2 * c + 1] = r.y;
      }
    }
    if (carry) {
      uint32_t wb[32];
#pragma unroll
      for (int k = 0; k < 32; ++k) wb[k] = __float_as_uint(w[k]);
      tc::tmem_st32(lane_addr + 256 + 32 * blk, wb);
    }
  }
  if (carry) tc::tmem_wait_st();
}

// Source terms needed for a point source's J at (time t, channel ch).
__device__ __forceinline__ SrcInfo<float> point_source_info(const FusedArgs<float>& A, int t, int ch, int s,
                                                           float log2_ratio) {
  SrcInfo<float> si;
  si.l = __ldg(A.lm + 2 * s);
  si.m = __ldg(A.lm + 2 * s + 1);
  if (A.bsq0) {  // sqrt(B) = (nu/nu_ref)^(alpha/2) sqrt(B)(nu_ref)
    const float* b = A.bsq0 + kBsqVals * (size_t(s) * A.ntime + t);
    const float4 q = __ldg(reinterpret_cast<const float4*>(b));
    const float sp = exp2f(__ldg(b + 4) * log2_ratio);
    si.B.a = {sp * q.x, 0.f};
    si.B.b = {sp * q.z, sp * q.w};
    si.B.c = {sp * q.z, -sp * q.w};
    si.B.d = {sp * q.y, 0.f};
    return si;
  }
  const size_t st = size_t(s) * A.ltime + t;
  const float* S = A.stokes + 4 * st;
  const float power = mb_pow(__ldg(A.freq + ch) / __ldg(A.ref_freq + ch), __ldg(A.alpha + st));
  si.B = brightness_sqrt<float>(__ldg(S), __ldg(S + 1), __ldg(S + 2), __ldg(S + 3), power);
  return si;
}

// Source terms for the point-source chain at (time t, channel ch): those of
// point_source_info plus l / n and m / n from the sqrt(B) table.
__device__ __forceinline__ SrcInfo<float> point_source_chain_info(const FusedArgs<float>& A, int t, int ch, int s,
                                                                 float log2_ratio) {
  SrcInfo<float> si = point_source_info(A, t, ch, s, log2_ratio);
  if (A.bsq0) {
    const float2 q = __ldg(reinterpret_cast<const float2*>(A.bsq0 + kBsqVals * (size_t(s) * A.ntime + t) + 6));
    si.l_over_n = q.x;
    si.m_over_n = q.y;
  } else {
    const double l = si.l, m = si.m, n = sqrt(1.0 - l * l - m * m);
    si.l_over_n = float(l / n);
    si.m_over_n = float(m / n);
  }
  return si;
}

// Stokes parameters, power and sqrt(B) of point source s at (t, ch), FP32.
__device__ __forceinline__ SrcInfo<float> point_source_stokes(const FusedArgs<float>& A, int t, int ch, int s,
                                                             float log2_ratio) {
  SrcInfo<float> si = point_source_info(A, t, ch, s, log2_ratio);
  const size_t st = size_t(s) * A.ltime + t;
  const float* S = A.stokes + 4 * st;
  si.I = S[0]; si.Q = S[1]; si.U = S[2]; si.V = S[3];
  si.power = mb_pow(__ldg(A.freq + ch) / __ldg(A.ref_freq + ch), __ldg(A.alpha + st));
  return si;
}

// PACK (at most 32 antennas): a CTA takes the unit pair (t, 2k), (t, 2k + 1);
// operand rows 64 c + 2 a + i hold channel c (producer lane a, rep c), so one
// MMA sequence and one drain pass serve both channels.
template <int MODE, bool BATCHED, bool PACK>
__global__ void __launch_bounds__(kTcThreads) coh_tc_fwd_kernel(FusedArgs<float> A_in, SmemPlan S, TcPlan P) {
  constexpr int kRowBytes = TcGeom<MODE>::kRowBytes;
  constexpr int KAPPA = TcGeom<MODE>::kSlots;  // source slots per stage
  constexpr int NSRC = kTcProducerWarps;       // sources per stage
  using L = StageLayout<MODE, kRowBytes>;
  static_assert(L::kKT == 4 * KAPPA, "stage rows hold Re and Im of every slot");
  extern __shared__ __align__(16) unsigned char smem[];
  AntInfo<float>* sa = reinterpret_cast<AntInfo<float>*>(smem + S.off_ant);
  SrcInfo<float>* ss = reinterpret_cast<SrcInfo<float>*>(smem + S.off_src);
  Jones<float>* sV = reinterpret_cast<Jones<float>*>(smem + S.off_V);
  Jones<float>* sVlo = reinterpret_cast<Jones<float>*>(smem + P.off_vlo32);  // extended sources
  int* items = reinterpret_cast<int*>(smem + S.off_items);
  double* red = reinterpret_cast<double*>(smem + S.off_red);
  unsigned char* stage = smem + P.off_stage;
  Jones<float>* sJ = reinterpret_cast<Jones<float>*>(stage);  // extended sources, after the tensor-core phase
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + P.off_bar);
  uint64_t* full = bars;                    // [kTcStages], producers -> MMA
  uint64_t* empty = bars + kTcStages;       // [kTcStages], MMA commit -> producers
  uint64_t* accfull = bars + 2 * kTcStages;  // MMA commit -> drain
  uint64_t* accfree = accfull + 1;           // drain (all threads) -> MMA
  uint64_t* done = accfull + 2;              // last MMA commit
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  int* abort_flag = reinterpret_cast<int*>(tmem_slot + 1);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  FusedArgs<float> A = A_in;
  int cta = blockIdx.x;
  if constexpr (BATCHED) cta = cta_unit(A);
  constexpr int NCH = PACK ? 2 : 1;  // channels per CTA
  int t, ch, nch = 1;                // time, first channel, channels of this CTA
  if (PACK) {
    const int npc = (A.nchan + 1) / 2;
    t = cta / npc;
    ch = 2 * (cta - t * npc);
    nch = min(2, A.nchan - ch);
  } else {
    t = cta / A.nchan;
    ch = cta - t * A.nchan;
  }
  const int unit = t * A.nchan + ch;  // the first channel's unit; the second is unit + 1
  if (tid == 0) *abort_flag = A.err ? *reinterpret_cast<volatile int*>(A.err) : 0;
  __syncthreads();
  if (*abort_flag) {  // an earlier CTA timed out: do no work
    if (tid < nch) A.partial[unit + tid] = double(NAN);
    return;
  }
  __syncthreads();
  for (int c = 0; c < nch; ++c) load_antennas(A, t, ch + c, sa + c * A.na);
  for (int i = tid; i < NCH * S.npairs; i += blockDim.x) sV[i] = jzero<float>();
  // the stage buffers' unused slots are read by the MMAs as zeros
  for (int i = tid; i < int(kTcStages * 2 * L::kMatBytes / 16); i += blockDim.x)
    reinterpret_cast<uint4*>(stage)[i] = make_uint4(0u, 0u, 0u, 0u);
  if (tid == 0) {
    const int npt = (A.na + 1) / 2, nqt = (A.na + 3) / 4;
    int k = 0;
    for (int ip = 0; ip < npt; ++ip)
      for (int jq = (ip * 2) / 4; jq < nqt; ++jq) items[k++] = ip | (jq << 16);
    for (int i = 0; i < kTcStages; ++i) {
      tc::mbar_init(full + i, kTcProducers);
      tc::mbar_init(empty + i, 1);
    }
    tc::mbar_init(accfull, 1);
    tc::mbar_init(accfree, kTcThreads);
    tc::mbar_init(done, 1);
  }
  tc::fence_proxy_async_smem();
  if (warp == kTcProducerWarps) tc::tmem_alloc(tmem_slot, kTcCols);
  tc::fence_before_thread_sync();
  __syncthreads();
  tc::fence_after_thread_sync();
  const uint32_t tmem = *tmem_slot;

  float fc[NCH], log2_ratio[NCH];
  NuC nu[NCH];
  ChanPos<float> cp[NCH];
#pragma unroll
  for (int c = 0; c < NCH; ++c) {
    const int chc = min(ch + c, A.nchan - 1);
    fc[c] = A.freq[chc];
    nu[c] = make_nuc(double(fc[c]) / kLightSpeed);
    cp[c] = chan_pos<float>(fc[c], A.lfreq, A.ufreq, A.nud);
    log2_ratio[c] = log2f(fc[c] / A.ref_freq[chc]);
  }
  const int nstages = (A.npsrc + NSRC - 1) / NSRC;
  const int group = P.group;
  const uint32_t wlim = g_pipe_wait_limit;
  bool bad = false;

  if (warp < kTcProducerWarps) {
    // ---- producers -------------------------------------------------------
    // No barrier joins the warps inside the loop: every wait is a bounded
    // mbarrier wait, and each warp drains TMEM into pair accumulator entries
    // no other thread touches.  Warp w fills source slot w of every stage,
    // lane l antennas l and l + 32; rows are written starting from row
    // i0 = lane bit 2, so that 8 lanes of a store cover the 8 rows of a core
    // matrix.
    const int sl = warp;
    const int i0 = (lane >> 2) & 1;
    // A producer whose wait gave up (bad) skips all further waits and work;
    // the MMA warp's waits then give up too, and everyone reaches the end.
    for (int g = 0; g < nstages; ++g) {
      const int slot = g % kTcStages, use = g / kTcStages;
      const int s0 = g * NSRC, ns = min(NSRC, A.npsrc - s0);
      if (g + 1 < nstages && A.phi != nullptr) {  // the next stage's source terms into L1
        const int sn = s0 + NSRC + sl;
        if (sn < A.npsrc) {
          const double* pn = A.phi + (size_t(t) * A.nsrc + sn) * A.na_glob;
          if (lane < A.na) tc::prefetch_l1(pn + gant(A, lane));
          if (lane + 32 < A.na) tc::prefetch_l1(pn + gant(A, lane + 32));
          if (lane == 0) {
            tc::prefetch_l1(A.lm + 2 * sn);
            if (A.bsq0) tc::prefetch_l1(A.bsq0 + kBsqVals * (size_t(sn) * A.ntime + t));
          }
        }
      }
      if (!bad) bad = !tc::mbar_wait(empty + slot, (use & 1) ^ 1, wlim);
      if (!bad) {
        unsigned char* hi = stage + size_t(slot) * 2 * L::kMatBytes;
        unsigned char* lo = hi + L::kMatBytes;
        // the source's terms, the same for both antennas of the lane (PACK:
        // per channel)
        SrcInfo<float> src;
        if (!PACK && sl < ns) src = point_source_info(A, t, ch, s0 + sl, log2_ratio[0]);
#pragma unroll
        for (int rep = 0; rep < 2; ++rep) {
          const int c = PACK ? rep : 0;
          const int a = PACK ? lane : lane + 32 * rep;  // antenna
          const int ra = lane + 32 * rep;               // its rows 2 ra, 2 ra + 1
          Jones<float> J = jzero<float>();
          if (a < A.na && sl < ns && c < nch) {
            if (PACK) src = point_source_info(A, t, ch + c, s0 + sl, log2_ratio[c]);
            J = compute_jones(A, t, s0 + sl, a, src, sa[c * A.na + a], fc[c], nu[c], cp[c], ch + c);
          }
          // row 2a holds J00, J01; row 2a + 1 holds J10, J11
          const Cx<float> r0a = i0 ? J.c : J.a, r0b = i0 ? J.d : J.b;
          const Cx<float> r1a = i0 ? J.a : J.c, r1b = i0 ? J.b : J.d;
          L::put2(hi, lo, 2 * ra + i0, 2 * sl, r0a.r, r0b.r);
          L::put2(hi, lo, 2 * ra + i0, 2 * KAPPA + 2 * sl, r0a.i, r0b.i);
          L::put2(hi, lo, 2 * ra + 1 - i0, 2 * sl, r1a.r, r1b.r);
          L::put2(hi, lo, 2 * ra + 1 - i0, 2 * KAPPA + 2 * sl, r1a.i, r1b.i);
        }
        tc::fence_proxy_async_smem();
        tc::mbar_arrive(full + slot);
      }
      // A group is drained once the first stage of the next one is staged,
      // so the group's last MMAs run while the warps produce that stage.
      if ((g % group) == 0 && g > 0) {
        if (!bad) bad = !tc::mbar_wait(accfull, ((g / group) - 1) & 1, wlim);
        tc::fence_after_thread_sync();
        bad = __any_sync(0xffffffffu, bad);  // the drain's TMEM loads are warp-collective
        if (!bad) tc_drain<PACK>(A, tmem, reinterpret_cast<float*>(sV), true, nch);
        tc::fence_before_thread_sync();
        if (!bad) tc::mbar_arrive(accfree);
      }
    }
    if (nstages > 0) {  // the last group
      if (!bad) bad = !tc::mbar_wait(accfull, ((nstages - 1) / group) & 1, wlim);
      tc::fence_after_thread_sync();
      bad = __any_sync(0xffffffffu, bad);
      if (!bad) tc_drain<PACK>(A, tmem, reinterpret_cast<float*>(sV), false, nch);
      tc::fence_before_thread_sync();
      if (!bad) tc::mbar_arrive(accfree);
    }
  } else {
    // ---- MMA issue (lane 0); the whole warp drains with the producers ------
    const uint32_t idesc = L::instr(128, 128);
    const uint32_t idesc_neg = idesc | (1u << 13);  // negate A
    const int half = L::kKSteps / 2;
    bool issued = false;
    for (int g = 0; g < nstages; ++g) {
      const int slot = g % kTcStages, use = g / kTcStages;
      const bool first = (g % group) == 0, last = (g % group) == group - 1 || g == nstages - 1;
      if (first && g > 0) {  // the previous group, as the producers drain it
        if (!bad) bad = !tc::mbar_wait(accfull, ((g / group) - 1) & 1, wlim);
        tc::fence_after_thread_sync();
        bad = __any_sync(0xffffffffu, bad);
        if (!bad) tc_drain<PACK>(A, tmem, reinterpret_cast<float*>(sV), true, nch);
        tc::fence_before_thread_sync();
        if (!bad) tc::mbar_arrive(accfree);
      }
      if (lane == 0 && !bad) {
        if (first && g > 0) {
          bad = !tc::mbar_wait(accfree, ((g / group) - 1) & 1, wlim);
          tc::fence_after_thread_sync();
        }
        if (!bad) bad = !tc::mbar_wait(full + slot, use & 1, wlim);
        if (!bad) {
          tc::fence_after_thread_sync();
          const uint32_t hi = tc::smem_addr(stage + size_t(slot) * 2 * L::kMatBytes);
          const uint32_t lo = hi + L::kMatBytes;
          // the main accumulators restart with every group; the correction
          // accumulators only with the first stage (they carry the drains'
          // rounding errors from group to group)
          const uint32_t acc0 = (first ? 0u : 1u), cacc0 = (g == 0 ? 0u : 1u);
#pragma unroll
          for (int kk = 0; kk < L::kKSteps; ++kk) {
            const uint32_t o = kk * L::kKStepBytes;
            const uint64_t ah = L::desc(hi + o), al = L::desc(lo + o);
            const uint32_t acc = kk == 0 ? acc0 : 1u, cacc = kk == 0 ? cacc0 : 1u;
            L::mma(tmem, ah, ah, idesc, acc);
            L::mma(tmem + 256, ah, al, idesc, cacc);
            L::mma(tmem + 256, al, ah, idesc, 1u);
          }
#pragma unroll
          for (int kk = 0; kk < half; ++kk) {
            const uint32_t oi = (kk + half) * L::kKStepBytes, orr = kk * L::kKStepBytes;
            const uint64_t ih = L::desc(hi + oi), il = L::desc(lo + oi);
            const uint64_t rh = L::desc(hi + orr), rl = L::desc(lo + orr);
            const uint32_t acc = kk == 0 ? acc0 : 1u, cacc = kk == 0 ? cacc0 : 1u;
            // D_im += A_im A_re^T
            L::mma(tmem + 128, ih, rh, idesc, acc);
            L::mma(tmem + 384, ih, rl, idesc, cacc);
            L::mma(tmem + 384, il, rh, idesc, 1u);
            // D_im += (-A_re) A_im^T
            L::mma(tmem + 128, rh, ih, idesc_neg, 1u);
            L::mma(tmem + 384, rh, il, idesc_neg, 1u);
            L::mma(tmem + 384, rl, ih, idesc_neg, 1u);
          }
          issued = true;
          tc::mma_commit(empty + slot);
          if (last) tc::mma_commit(accfull);
        }
      }
    }
    bad = __any_sync(0xffffffffu, bad);
    if (nstages > 0) {  // the last group
      if (!bad) bad = !tc::mbar_wait(accfull, ((nstages - 1) / group) & 1, wlim);
      tc::fence_after_thread_sync();
      bad = __any_sync(0xffffffffu, bad);
      if (!bad) tc_drain<PACK>(A, tmem, reinterpret_cast<float*>(sV), false, nch);
      tc::fence_before_thread_sync();
      if (!bad) tc::mbar_arrive(accfree);
    }
    if (lane == 0 && issued) {  // all MMAs finished before TMEM is released
      tc::mma_commit(done);
      if (!tc::mbar_wait(done, 0)) bad = true;
    }
  }
  if (bad) *abort_flag = 1;
  tc::fence_before_thread_sync();
  __syncthreads();
  tc::fence_after_thread_sync();
  if (warp == kTcProducerWarps) tc::tmem_dealloc(tmem, kTcCols);
  const bool aborted = *abort_flag != 0;

  // ---- extended sources on the CUDA cores, then the epilogue, per channel --
  // they accumulate with FP32 low parts in the stage region
  for (int c = 0; c < nch; ++c) {
    Jones<float>* sVc = sV + c * S.npairs;
    const AntInfo<float>* sac = sa + c * A.na;
    {
      float* vlo = reinterpret_cast<float*>(sVlo);
      for (int i = tid; i < S.npairs * 8; i += blockDim.x) vlo[i] = 0.f;
    }
    __syncthreads();
    const float kg = A.gauss_scale * fc[c], ks = A.two_pi_over_c * fc[c];
    for (int s0 = A.npsrc; s0 < A.nsrc && A.tc_ext && !aborted;) {
      const int s1 = min(s0 + S.st, A.nsrc), ns = s1 - s0;
      load_sources(A, t, ch + c, s0, ns, ss);
      __syncthreads();
      produce_jones(A, S, t, ch + c, s0, ns, ss, sac, sJ, cp[c]);
      __syncthreads();
      consume_pairs<float, 2, 4, false>(A, S, ns, ss, sac, sJ, sVc, sVlo, items, true, kg, ks);
      __syncthreads();
      s0 = s1;
    }
    for (int i = tid; i < S.npairs; i += blockDim.x) sVc[i] = jadd(sVc[i], sVlo[i]);
    __syncthreads();
    epilogue<false>(A, t, ch + c, unit + c, sVc, sJ, red);
    __syncthreads();
    if (aborted && tid == 0) {
      A.partial[unit + c] = double(NAN);
      if (A.err) atomicExch(A.err, int(MB_ERR_TIMEOUT));
    }
  }
}

// ---------------------------------------------------------------------------
// Adjoint
// ---------------------------------------------------------------------------
// Y_ab: the Hermitian completion of the pair matrix X (see file header).
template <typename T>
__device__ __forceinline__ Jones<T> y_entry(const Jones<T>* sX, int a, int b, int na) {
  if (a < b) return sX[pair_index(a, b, na)];
  if (a > b) return jherm(sX[pair_index(b, a, na)]);
  Jones<T> x = sX[pair_index(a, a, na)];
  return jadd(x, jherm(x));
}

template <typename T>
__device__ __forceinline__ Jones<T> y_at(const Jones<T>* sY, int a, int b, int na) {
  if (AdjTile<T>::FULL_Y) return jload<T>(y_full(reinterpret_cast<const T*>(sY), a, b, na));
  return y_entry(sY, a, b, na);
}

// dJ_a (s) = sum_b Y_ab J_b (s) for the point sources of a tile, with the
// complete Y in shared memory.  Work item: 2 antennas x 4 sources x a
// quarter of the b sum; the 4 quarters sit in adjacent lanes and are
// combined with shuffles.
template <typename T>
__device__ void adj_consume_point_full(const FusedArgs<T>& A, const SmemPlan& S, int ns, const Jones<T>* sJ,
                                       const Jones<T>* sY, Jones<T>* sgJ) {
  constexpr int TA = 2, TS = 4, NB = 4;
  const int nat = S.nap / TA, nsg = (S.st + TS - 1) / TS;
  const int total = nat * nsg * NB;
  const int rounds = (total + blockDim.x - 1) / blockDim.x;
  for (int round = 0; round < rounds; ++round) {
    const int k = round * blockDim.x + threadIdx.x;
    const bool active = k < total;
    const int bq = k & 3, rest = k >> 2;
    const int at = rest % nat, sg = rest / nat;
    const int a0 = at * TA, sb = sg * TS;
    Jones<T> acc[TA][TS];
#pragma unroll
    for (int r = 0; r < TA; ++r)
#pragma unroll
      for (int c = 0; c < TS; ++c) acc[r][c] = jzero<T>();
    if (active) {
      for (int b = bq; b < A.na; b += NB) {
        Jones<T> Y[TA], J[TS];
#pragma unroll
        for (int r = 0; r < TA; ++r)
          Y[r] = (a0 + r < A.na) ? jload<T>(y_full(reinterpret_cast<const T*>(sY), a0 + r, b, A.na)) : jzero<T>();
#pragma unroll
        for (int c = 0; c < TS; ++c) {
          const int si = min(sb + c, ns - 1);
          J[c] = jload<T>(reinterpret_cast<const T*>(jtile(sJ, S, si, b)));
        }
#pragma unroll
        for (int r = 0; r < TA; ++r)
#pragma unroll
          for (int c = 0; c < TS; ++c) jmac(acc[r][c], Y[r], J[c]);
      }
    }
    // combine the 4 partial sums over b (all lanes take part)
#pragma unroll
    for (int r = 0; r < TA; ++r)
#pragma unroll
      for (int c = 0; c < TS; ++c) {
        T* v = reinterpret_cast<T*>(&acc[r][c]);
#pragma unroll
        for (int e = 0; e < 8; ++e) {
          v[e] += __shfl_xor_sync(0xffffffffu, v[e], 1);
          v[e] += __shfl_xor_sync(0xffffffffu, v[e], 2);
        }
      }
    if (active) {
      // lane bq writes outputs (r, c) with (r * TS + c) % NB == bq
#pragma unroll
      for (int r = 0; r < TA; ++r)
#pragma unroll
        for (int c = 0; c < TS; ++c)
          if (((r * TS + c) & (NB - 1)) == bq && sb + c < ns) *jtile(sgJ, S, sb + c, a0 + r) = acc[r][c];
    }
  }
}

// Beam value and its derivatives with respect to the l and m grid offsets.
template <typename T>
__device__ void beam_interp_d(const T* __restrict__ E_beam, const BeamGeom& G, const GridPos<T>& gl,
                              const GridPos<T>& gm, const ChanPos<T>& cp, Jones<T>& E, Jones<T>& dEl,
                              Jones<T>& dEm) {
  Jones<T> sum = jzero<T>(), dsl = jzero<T>(), dsm = jzero<T>();
  T amp[4] = {0, 0, 0, 0}, dal[4] = {0, 0, 0, 0}, dam[4] = {0, 0, 0, 0};
  const T ld = gl.d, md = gm.d, cd = cp.d;
#pragma unroll
  for (int corner = 0; corner < 8; ++corner) {
    const bool hl = corner & 1, hm = corner & 2, hc = corner & 4;
    const int il = hl ? gl.i1 : gl.i0, im = hm ? gm.i1 : gm.i0, ic = hc ? cp.c1 : cp.c0;
    const T fl = hl ? ld : T(1) - ld, fm = hm ? md : T(1) - md, fc = hc ? cd : T(1) - cd;
    const T w = fl * fm * fc, wl = (hl ? T(1) : T(-1)) * fm * fc, wm = fl * (hm ? T(1) : T(-1)) * fc;
    const T* p = E_beam + 8 * ((size_t(il) * G.mh + im) * G.nud + ic);
    Jones<T> e = jldg<T>(p);
    const Cx<T>* e4 = &e.a;
    Cx<T>* s4 = &sum.a; Cx<T>* l4 = &dsl.a; Cx<T>* m4 = &dsm.a;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      T ab = cabs_(e4[k]);
      s4[k] = s4[k] + e4[k] * w; amp[k] += w * ab;
      l4[k] = l4[k] + e4[k] * wl; dal[k] += wl * ab;
      m4[k] = m4[k] + e4[k] * wm; dam[k] += wm * ab;
    }
  }
  Cx<T>* E4 = &E.a; Cx<T>* dl4 = &dEl.a; Cx<T>* dm4 = &dEm.a;
  const Cx<T>* s4 = &sum.a; const Cx<T>* l4 = &dsl.a; const Cx<T>* m4 = &dsm.a;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    T inv = mb_rsqrt(s4[k].r * s4[k].r + s4[k].i * s4[k].i);
    if (isfinite(inv)) {
      E4[k] = s4[k] * (amp[k] * inv);
      T drl = cdot_re(s4[k], l4[k]) * inv, drm = cdot_re(s4[k], m4[k]) * inv;
      dl4[k] = (l4[k] * amp[k] + s4[k] * dal[k]) * inv - s4[k] * (amp[k] * drl * inv * inv);
      dm4[k] = (m4[k] * amp[k] + s4[k] * dam[k]) * inv - s4[k] * (amp[k] * drm * inv * inv);
    } else {
      E4[k] = s4[k] * amp[k];
      dl4[k] = l4[k] * amp[k] + s4[k] * dal[k];
      dm4[k] = m4[k] * amp[k] + s4[k] * dam[k];
    }
  }
}

// Same as beam_interp_d on the frequency-blended coefficient plane (see
// plane_cell): the bilinear values and their derivatives along the l and m
// grid axes, then the renormalisation and its derivatives.
template <typename T>
__device__ void beam_interp_plane_d(const T* __restrict__ plane, int mh, const GridPos<T>& gl, const GridPos<T>& gm,
                                    Jones<T>& E, Jones<T>& dEl, Jones<T>& dEm) {
  T v[kPlaneComp], vx[kPlaneComp], vy[kPlaneComp];
  plane_cell<T, true>(plane_cell_ptr(plane, mh, gl.i0, gm.i0), gl.d, gm.d, v, vx, vy);
  // E = s g with g = amp / |s|, and by the quotient rule
  //   dE/dx = g ds/dx + s inv (damp/dx - g inv Re(conj(s) ds/dx)),  inv = 1 / |s|;
  // a non-finite inv (s = 0) is replaced by 1, which gives the same value as
  // leaving out the normalisation (E = s amp, dE/dx = ds/dx amp + s damp/dx).
  Cx<T>* E4 = &E.a; Cx<T>* dl4 = &dEl.a; Cx<T>* dm4 = &dEm.a;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const Cx<T> s4{v[2 * k], v[2 * k + 1]}, l4{vx[2 * k], vx[2 * k + 1]}, m4{vy[2 * k], vy[2 * k + 1]};
    const T amp = v[8 + k], dal = vx[8 + k], dam = vy[8 + k];
    T inv = mb_rsqrt(s4.r * s4.r + s4.i * s4.i);
    inv = isfinite(inv) ? inv : T(1);
    const T g = amp * inv, gi = g * inv;
    const T hl = inv * (dal - gi * cdot_re(s4, l4));
    const T hm = inv * (dam - gi * cdot_re(s4, m4));
    if constexpr (sizeof(T) == 4) {  // (Re, Im) pairs by packed FP32x2 arithmetic
      const float2 s2 = make_float2(s4.r, s4.i), gg = make_float2(g, g);
      const float2 e = __fmul2_rn(s2, gg);
      const float2 dl = __ffma2_rn(s2, make_float2(hl, hl), __fmul2_rn(make_float2(l4.r, l4.i), gg));
      const float2 dm = __ffma2_rn(s2, make_float2(hm, hm), __fmul2_rn(make_float2(m4.r, m4.i), gg));
      E4[k] = {e.x, e.y};
      dl4[k] = {dl.x, dl.y};
      dm4[k] = {dm.x, dm.y};
    } else {
      E4[k] = s4 * g;
      dl4[k] = {l4.r * g + s4.r * hl, l4.i * g + s4.i * hl};
      dm4[k] = {m4.r * g + s4.r * hm, m4.i * g + s4.i * hm};
    }
  }
}

// Shape factor and its derivatives with respect to the 3 shape parameters.
template <typename T>
__device__ __forceinline__ T shape_and_grad(int type, T u, T v, T p0, T p1, T p2, T kg, T ks, T (&d)[3]) {
  if (type == SRC_GAUSS) {
    const T el = p0, em = p1, R = p2;
    T a1 = u * em - v * el;
    T u1 = a1 * kg * R, v1 = (u * el + v * em) * kg;
    T c = mb_exp(-(u1 * u1 + v1 * v1));
    d[0] = T(-2) * c * (u1 * (-v * kg * R) + v1 * (u * kg));
    d[1] = T(-2) * c * (u1 * (u * kg * R) + v1 * (v * kg));
    d[2] = T(-2) * c * (u1 * a1 * kg);
    return c;
  }
  const T e1 = p0, e2 = p1, R = p2;
  T den = T(1) - e1 * e1 - e2 * e2;
  T Sc = R / den;
  T a1 = u * (T(1) + e1) + v * e2, b1 = u * e2 + v * (T(1) - e1);
  T u1 = a1 * ks * Sc, v1 = b1 * ks * Sc;
  T dd = T(1) + u1 * u1 + v1 * v1;
  T c;
  if constexpr (sizeof(T) == 4) {
    const T r = mb_rsqrt(dd);
    c = r * r * r;
  } else {
    c = T(1) / (dd * mb_sqrt(dd));
  }
  T dS1 = Sc * T(2) * e1 / den, dS2 = Sc * T(2) * e2 / den;
  T du_e1 = ks * (u * Sc + a1 * dS1), dv_e1 = ks * (-v * Sc + b1 * dS1);
  T du_e2 = ks * (v * Sc + a1 * dS2), dv_e2 = ks * (u * Sc + b1 * dS2);
  T du_R = a1 * ks / den, dv_R = b1 * ks / den;
  T k3 = T(-3) * c / dd;
  d[0] = k3 * (u1 * du_e1 + v1 * dv_e1);
  d[1] = k3 * (u1 * du_e2 + v1 * dv_e2);
  d[2] = k3 * (u1 * du_R + v1 * dv_R);
  return c;
}

template <typename T, int RA, int RS>
__device__ void adj_consume_point(const FusedArgs<T>& A, const SmemPlan& S, int ns, const Jones<T>* sJ,
                                  const Jones<T>* sX, Jones<T>* sgJ) {
  const int nat = S.nap / RA, nsg = (ns + RS - 1) / RS;
  for (int k = threadIdx.x; k < nat * nsg; k += blockDim.x) {
    const int sg = k / nat, at = k - sg * nat;
    const int a0 = at * RA, sbase = sg * RS;
    Jones<T> acc[RA][RS];
#pragma unroll
    for (int r = 0; r < RA; ++r)
#pragma unroll
      for (int c = 0; c < RS; ++c) acc[r][c] = jzero<T>();
    for (int b = 0; b < A.na; ++b) {
      Jones<T> Y[RA], Jb[RS];
#pragma unroll
      for (int r = 0; r < RA; ++r) Y[r] = (a0 + r < A.na) ? y_entry(sX, a0 + r, b, A.na) : jzero<T>();
#pragma unroll
      for (int c = 0; c < RS; ++c) {
        int si = min(sbase + c, ns - 1);
        Jb[c] = jload<T>(reinterpret_cast<const T*>(jtile(sJ, S, si, b)));
      }
#pragma unroll
      for (int r = 0; r < RA; ++r)
#pragma unroll
        for (int c = 0; c < RS; ++c) jmac(acc[r][c], Y[r], Jb[c]);
    }
#pragma unroll
    for (int r = 0; r < RA; ++r)
#pragma unroll
      for (int c = 0; c < RS; ++c)
        if (sbase + c < ns) *jtile(sgJ, S, sbase + c, a0 + r) = acc[r][c];
  }
}

// Adds the NV values of every active lane to acc[key * kNAcc + first + j]
// (warp_keyed_add_stride with the per-source accumulator stride).
template <typename T, int NV>
__device__ __forceinline__ void warp_keyed_add(T* acc, int first, int key, T (&v)[NV]) {
  warp_keyed_add_stride<T, NV>(acc + first, kNAcc, key, v);
}

// Chain d chi^2 / dJ(s, a) through E and K: d chi^2 / d(l, m) of the item
// and gB = d chi^2 / d sqrt(B) (complex, per Jones entry).  Uses src.l, m,
// l_over_n, m_over_n and B.
template <typename T>
__device__ __forceinline__ void chain_core(const FusedArgs<T>& A, int t, int ch, int s, int a, const SrcInfo<T>& src,
                                           const AntInfo<T>& ai, const Jones<T>& gJ, T f, const NuC& nu,
                                           T dphase, const ChanPos<T>& cp, T& gl0, T& gm0, Jones<T>& gB) {
  const BeamGeom G{A.lw, A.mh, A.nud};
  Cx<T> K = phase_term(A, t, s, a, f, nu);
  T l, m;
  beam_lm<T>(src.l, src.m, ai.sin_pa, ai.cos_pa, ai.pe_l, ai.pe_m, ai.sc_l, ai.sc_m, l, m);
  GridPos<T> gl = grid_pos<T>(l, A.ll, A.ul, A.lscale, A.lw);
  GridPos<T> gm = grid_pos<T>(m, A.lmm, A.um, A.mscale, A.mh);
  Jones<T> E, dEl, dEm;
  if (A.plane)
    beam_interp_plane_d<T>(A.plane + size_t(ch) * A.lw * A.mh * kPlaneVals, A.mh, gl, gm, E, dEl, dEm);
  else
    beam_interp_d<T>(A.E_beam, G, gl, gm, cp, E, dEl, dEm);
  const Jones<T>& B = src.B;
  Jones<T> KB = {cmul(K, B.a), cmul(K, B.b), cmul(K, B.c), cmul(K, B.d)};
  // E
  Jones<T> gE = jmulh(gJ, KB);
  T g_ld = gl.inside ? jdot_re(gE, dEl) * A.lscale : T(0);
  T g_md = gm.inside ? jdot_re(gE, dEm) * A.mscale : T(0);
  gl0 = g_ld * ai.sc_l * ai.cos_pa + g_md * ai.sc_m * ai.sin_pa;
  gm0 = -g_ld * ai.sc_l * ai.sin_pa + g_md * ai.sc_m * ai.cos_pa;
  // K and sqrt(B)
  Jones<T> gKB = jhmul(E, gJ);
  Cx<T> gK = cmulc(gKB.a, B.a) + cmulc(gKB.b, B.b) + cmulc(gKB.c, B.c) + cmulc(gKB.d, B.d);
  T gphi = dphase * (gK.r * K.i - gK.i * K.r);
  gl0 += gphi * (ai.u - ai.w * src.l_over_n);
  gm0 += gphi * (ai.v - ai.w * src.m_over_n);
  Cx<T> Kc = conj(K);
  gB = {cmul(Kc, gKB.a), cmul(Kc, gKB.b), cmul(Kc, gKB.c), cmul(Kc, gKB.d)};
}

// d chi^2 / d(I, Q, U, V, alpha) of a source from gB = d chi^2 / d sqrt(B)
// at its (time, channel).  Linear in gB, so gB may be a sum over antennas.
// Uses src.B, I, Q, U, V and power.
template <typename T>
__device__ __forceinline__ void stokes_grads(const SrcInfo<T>& src, const Jones<T>& gB, T half_log_ratio,
                                             T (&g)[5]) {
  const T GB = jdot_re(gB, src.B);
  const T det0 = src.I * src.I - src.Q * src.Q - src.U * src.U - src.V * src.V;
  const T s0v = mb_sqrt(det0 > T(0) ? det0 : T(0));
  T gI = 0, gQ = 0, gU = 0, gVv = 0;
  if (s0v > T(0)) {
    T tt = mb_sqrt(T(2) * src.power * (src.I + s0v));
    T pt = src.power / tt;
    T tr1 = gB.a.r + gB.d.r;
    T q2 = GB / (T(2) * s0v * (src.I + s0v));
    gI = pt * (T(1) + src.I / s0v) * tr1 - GB / (T(2) * s0v);
    gQ = pt * ((gB.a.r - gB.d.r) - (src.Q / s0v) * tr1) + q2 * src.Q;
    gU = pt * ((gB.b.r + gB.c.r) - (src.U / s0v) * tr1) + q2 * src.U;
    gVv = pt * ((gB.b.i - gB.c.i) - (src.V / s0v) * tr1) + q2 * src.V;
  }
  g[0] = gI; g[1] = gQ; g[2] = gU; g[3] = gVv;
  g[4] = GB * half_log_ratio;
}

// Chain d chi^2 / dJ(s, a) through E, K and sqrt(B): the contributions to
// d chi^2 / d(l, m, I, Q, U, V, alpha) of source s.
template <typename T>
__device__ __forceinline__ void chain_item(const FusedArgs<T>& A, int t, int ch, int s, int a, const SrcInfo<T>& src,
                                           const AntInfo<T>& ai, const Jones<T>& gJ, T f, const NuC& nu, T dphase,
                                           T half_log_ratio, const ChanPos<T>& cp, T (&g)[7]) {
  Jones<T> gB;
  chain_core(A, t, ch, s, a, src, ai, gJ, f, nu, dphase, cp, g[0], g[1], gB);
  T gs[5];
  stokes_grads(src, gB, half_log_ratio, gs);
#pragma unroll
  for (int k = 0; k < 5; ++k) g[2 + k] = gs[k];
}

// Chain d chi^2 / dJ through E, K and sqrt(B) to the source parameters.
template <typename T>
__device__ void adj_chain(const FusedArgs<T>& A, const SmemPlan& S, int t, int ch, int s0, int ns,
                          const SrcInfo<T>* ss, const AntInfo<T>* sa, const Jones<T>* sgJ,
                          T* sacc, const ChanPos<T>& cp) {
  const T f = A.freq[ch];
  const NuC nu = make_nuc(double(f) / kLightSpeed);
  const T dphase = T(nu.dphase);  // |dK/dphi|
  const T half_log_ratio = T(0.5) * mb_log(f / A.ref_freq[ch]);
  const int n = ns * A.na;
  const int rounds = (n + blockDim.x - 1) / blockDim.x;
  for (int round = 0; round < rounds; ++round) {
    const int i = round * blockDim.x + threadIdx.x;
    const bool active = i < n;
    const int si = active ? i / A.na : 0, a = active ? i - si * A.na : 0;
    T g[7] = {T(0), T(0), T(0), T(0), T(0), T(0), T(0)};
    if (active)
      chain_item(A, t, ch, s0 + si, a, ss[si], sa[a], *jtile(sgJ, S, si, a), f, nu, dphase, half_log_ratio, cp, g);
    warp_keyed_add<T, 7>(sacc, 0, active ? si : -1, g);
  }
}

// Extended sources of a tile, consumed and chained in one pass: work item
// (source, antenna a), the lanes of a warp taking consecutive antennas,
// forms dJ_a(s) = sum_b shape_s(a, b) Y_ab J_b(s) with d chi^2 / d(shape
// parameters) from the pairs a < b, and chains dJ_a(s) through E, K and
// sqrt(B) to the source's l, m, I, Q, U, V, alpha at once (chain_item), so
// dJ never goes through shared memory.  All 10 per-source sums of an item
// are added with one keyed warp sum.
template <typename T>
__device__ void adj_ext_tile(const FusedArgs<T>& A, const SmemPlan& S, int t, int ch, int s0, int ns,
                             const SrcInfo<T>* ss, const AntInfo<T>* sa, const Jones<T>* sJ, const Jones<T>* sX,
                             T* sacc, T kg, T ks, const ChanPos<T>& cp) {
  const T f = A.freq[ch];
  const NuC nu = make_nuc(double(f) / kLightSpeed);
  const T dphase = T(nu.dphase);  // |dK/dphi|
  const T half_log_ratio = T(0.5) * mb_log(f / A.ref_freq[ch]);
  const int n = ns * A.na;
  const int rounds = (n + blockDim.x - 1) / blockDim.x;
  for (int round = 0; round < rounds; ++round) {
    const int k = round * blockDim.x + threadIdx.x;
    const bool active = k < n;
    const int si = active ? k / A.na : 0, a = active ? k - si * A.na : 0;
    T g[kNAcc];
#pragma unroll
    for (int e = 0; e < kNAcc; ++e) g[e] = T(0);
    if (active) {
      const SrcInfo<T>& src = ss[si];
      const Jones<T> Ja = *jtile(sJ, S, si, a);
      const T ua = sa[a].u, va = sa[a].v;
      Jones<T> acc = jzero<T>();
      for (int b = 0; b < A.na; ++b) {
        const Jones<T> P = jmul(y_at(sX, a, b, A.na), *jtile(sJ, S, si, b));
        T d[3];
        const T c = shape_and_grad<T>(src.type, sa[b].u - ua, sa[b].v - va, src.s0, src.s1, src.s2, kg, ks, d);
        jaxpy(acc, P, c);
        if (a < b) {
          const T gc = jdot_re(Ja, P);
          g[7] += gc * d[0]; g[8] += gc * d[1]; g[9] += gc * d[2];
        }
      }
      T gc7[7];
      chain_item(A, t, ch, s0 + si, a, src, sa[a], acc, f, nu, dphase, half_log_ratio, cp, gc7);
#pragma unroll
      for (int e = 0; e < 7; ++e) g[e] = gc7[e];
    }
    warp_keyed_add<T, kNAcc>(sacc, 0, active ? si : -1, g);
  }
}

template <typename T>
__device__ void adj_flush(const FusedArgs<T>& A, int t, int s0, int ns, T* sacc) {
  for (int i = threadIdx.x; i < ns * kNAcc; i += blockDim.x) {
    const int si = i / kNAcc, k = i - si * kNAcc, s = s0 + si;
    const double val = double(sacc[i]);
    sacc[i] = T(0);
    if (val == 0.0) continue;
    if (k < 2) atomicAdd(&A.acc_lm[2 * s + k], val);
    else if (k < 6) atomicAdd(&A.acc_stokes[(size_t(s) * A.ntime + t) * 4 + (k - 2)], val);
    else if (k == 6) atomicAdd(&A.acc_alpha[size_t(s) * A.ntime + t], val);
    else {
      int st = src_type(A, s);
      if (st == SRC_GAUSS) atomicAdd(&A.acc_gauss[(k - 7) * A.ngsrc + (s - A.npsrc)], val);
      else if (st == SRC_SERSIC) atomicAdd(&A.acc_sersic[(k - 7) * A.nssrc + (s - A.npsrc - A.ngsrc)], val);
    }
  }
}

template <typename T, int RA, int RS, bool BATCHED>
__global__ void __launch_bounds__(AdjTile<T>::THREADS) coh_adj_kernel(FusedArgs<T> A_in, SmemPlan S) {
  extern __shared__ __align__(16) unsigned char smem[];
  AntInfo<T>* sa = reinterpret_cast<AntInfo<T>*>(smem + S.off_ant);
  SrcInfo<T>* ss = reinterpret_cast<SrcInfo<T>*>(smem + S.off_src);
  Jones<T>* sJ = reinterpret_cast<Jones<T>*>(smem + S.off_J);
  Jones<T>* sgJ = reinterpret_cast<Jones<T>*>(smem + S.off_gJ);
  Jones<T>* sX = reinterpret_cast<Jones<T>*>(smem + S.off_V);
  T* sacc = reinterpret_cast<T*>(smem + S.off_acc);

  FusedArgs<T> A = A_in;
  int unit = blockIdx.x;
  if constexpr (BATCHED) unit = cta_unit(A);
  const int t = unit / A.nchan, ch = unit - t * A.nchan;
  load_antennas(A, t, ch, sa);
  const int nx = AdjTile<T>::FULL_Y ? A.na * y_row_vals<T>(A.na) : 8 * S.npairs;
  for (int i = threadIdx.x; i < nx; i += blockDim.x) reinterpret_cast<T*>(sX)[i] = T(0);
  for (int i = threadIdx.x; i < S.st * kNAcc; i += blockDim.x) sacc[i] = T(0);
  __syncthreads();
  for (int bl = threadIdx.x; bl < A.nbl; bl += blockDim.x) {
    size_t tbl = size_t(t) * A.lnbl + bl;
    int p, q;
    if (!local_baseline(A, A.ant1[tbl], A.ant2[tbl], p, q)) continue;
    Jones<T> g = jload<T>(A.gV + 8 * ((size_t(t) * A.nbl + bl) * A.nchan + ch));
    if (AdjTile<T>::FULL_Y) {
      // baseline (p, q): Y_pq += gV, Y_qp += gV^H (p == q: both terms)
      atomic_add_jones(reinterpret_cast<Jones<T>*>(y_full(reinterpret_cast<T*>(sX), p, q, A.na)), g);
      atomic_add_jones(reinterpret_cast<Jones<T>*>(y_full(reinterpret_cast<T*>(sX), q, p, A.na)), jherm(g));
    } else if (p <= q) {
      atomic_add_jones(&sX[pair_index(p, q, A.na)], g);
    } else {
      atomic_add_jones(&sX[pair_index(q, p, A.na)], jherm(g));
    }
  }
  __syncthreads();

  const T f = A.freq[ch];
  const ChanPos<T> cp = chan_pos<T>(f, A.lfreq, A.ufreq, A.nud);
  const T kg = A.gauss_scale * f, ks = A.two_pi_over_c * f;
  for (int s0 = A.sbeg; s0 < A.nsrc;) {
    int s1 = s0 < A.npsrc ? min(s0 + S.st, A.npsrc) : min(s0 + S.st, A.nsrc);
    int ns = s1 - s0;
    load_sources(A, t, ch, s0, ns, ss);
    __syncthreads();
    produce_jones(A, S, t, ch, s0, ns, ss, sa, sJ, cp);
    __syncthreads();
    if (s0 < A.npsrc) {
      if (AdjTile<T>::FULL_Y) adj_consume_point_full<T>(A, S, ns, sJ, sX, sgJ);
      else adj_consume_point<T, RA, RS>(A, S, ns, sJ, sX, sgJ);
      __syncthreads();
      adj_chain<T>(A, S, t, ch, s0, ns, ss, sa, sgJ, sacc, cp);
    } else {
      adj_ext_tile<T>(A, S, t, ch, s0, ns, ss, sa, sJ, sX, sacc, kg, ks, cp);
    }
    __syncthreads();
    adj_flush<T>(A, t, s0, ns, sacc);
    __syncthreads();
    s0 = s1;
  }
}

// ---------------------------------------------------------------------------
// Split-precision adjoint: dJ = Y J for point sources on the tensor cores
// ---------------------------------------------------------------------------
// Y (2na x 2na complex, rows (a, i), columns (b, j)) is the Hermitian matrix
// of d chi^2 / dV.  As a real operand (128 rows x 256 K, BF16 hi + lo), held
// in TMEM as the MMAs' A operand (columns 0-127 hi, 128-255 lo, two K values
// per column):
//   Yop[(a,i), (b,j)] = Re Y_ab[i][j],  Yop[(a,i), 128 + (b,j)] = -Im Y_ab[i][j].
// Per tile of kTaKappa sources the producers stage
//   Jop[(s,k), (b,j)] = Re J_sb[j][k],  Jop[(s,k), 128 + (b,j)] = Im J_sb[j][k]
// and one MMA warp forms, in TMEM,
//   D_re = Yop Jop^T                          = Re (Y J)
//   D_im = (-Yop_im) Jop_re^T + Yop_re Jop_im^T = Im (Y J)
// (the second with the instruction's negate-A bit), each operand as
// hi.hi + hi.lo + lo.hi.
//
// The 12 worker warps form three groups of four (one warp per TMEM lane
// quarter) that take every third tile.  Worker lane (a, i) = TMEM lane 2a + i handles
// the items (source 4i + u, antenna a), u = 0..3, of its group's tile: it
// computes E, dE/dl, dE/dm, K and J once, stages J for the MMA and parks
//   EK = E K,  DL = dE/dl K,  DM = dE/dm K
// in shared memory (6 float4 per item) until dJ arrives in TMEM.
// Then, with gJ = dJ and W = gJ sqrt(B),
//   d sqrt(B) = EK^H gJ,  d/dl_beam = Re tr(W^H DL),  d/dm_beam = Re tr(W^H DM),
//   d/dphi = 2 pi nu / c * Im tr(d sqrt(B)^H sqrt(B)).
// Lane 0 of the group's first and second warps issue the Re and Im MMA
// chains once the group has staged its tile (group barrier); while one group
// waits for its MMAs the others compute.  Y itself is formed at the start of
// the CTA from d chi^2 / dV (the forward's epilogue output) and stays in TMEM.
constexpr int kTaRowBytes = 512;      // 256 BF16 values of K per operand row
constexpr int kTaKappa = 8;           // sources per tile (16 operand rows)
constexpr int kTaGroups = 3;          // worker groups = stages = TMEM regions
constexpr int kTaGroupThreads = 128;  // 4 warps, one per TMEM lane quarter
constexpr int kTaWorkers = kTaGroups * kTaGroupThreads;
constexpr int kTaThreads = kTaWorkers;
constexpr int kTaItems = 4;           // items per worker lane and tile
// TMEM: the Y operand in columns 0-255, then per group the two dJ
// accumulation chains (2 x 32 columns) from kTaYCols + 64 * group.
constexpr uint32_t kTaYCols = 256;
constexpr uint32_t kTaGroupCols = 64;
constexpr uint32_t kTaCols = 512;
static_assert(kTaYCols + kTaGroups * kTaGroupCols <= kTaCols, "TMEM columns of Y and the worker groups");
constexpr int kTaPark = 6;            // float4 of parked state per item
// Per-source sums: d/dl, d/dm and the Hermitian part of gB = d chi^2 /
// d sqrt(B) that the Stokes and alpha gradients depend on (sqrt(B) is
// Hermitian with real diagonal): Re gB00, Re gB11, Re (gB01 + gB10),
// Im (gB01 - gB10).
constexpr int kTaAcc = 6;
static_assert(kTaAcc <= 8, "per-source sums fit the 8-value reduce-scatter");
// The J operand (16 hi rows, then 16 lo rows) with K-adjacent core matrices
// 144 bytes apart and 8-row groups 4672 bytes apart: a worker lane (a, i)
// stores 4 bytes at K = 2a of row 2 (4 i + u), so a warp's 32 stores fall on
// 32 distinct banks (dense 128 / 4096 put them on 4: an 8-way conflict).
constexpr int kTaLBO = 144, kTaSBO = 32 * kTaLBO + 64;
using TaGeom = StageGeometry<kTaRowBytes, kTaLBO, kTaSBO>;
using TaLayout = StageLayout<MB_MODE_SPLIT_BF16, kTaRowBytes, kTaLBO, kTaSBO>;
constexpr size_t kJopBytes = 4 * size_t(kTaSBO);  // hi + lo, 16 rows each
constexpr int kTaParkBytes = int(sizeof(float4)) * kTaGroups * kTaItems * kTaPark * 128;
// Bytes per row of Y (na Jones + 32) while it is formed in the park region.
constexpr int kTaYRowBytes = 64 * int(sizeof(Jones<float>)) + 32;
static_assert(64 * kTaYRowBytes <= kTaParkBytes, "Y of 64 antennas fits the park region");

// Sum of v[k] over the 16 lanes that share lane bit 0, by reduce-scatter
// over lane bits 4, 3, 2 and a plain sum over bit 1 (8 shuffles for 8
// values).  Afterwards both lanes whose bits 4..2 read k hold the sum of
// value k; *k is returned.
__device__ __forceinline__ float reduce_scatter8(const float (&w8)[8], int lane, int* k) {
  const bool b4 = lane & 16, b3 = lane & 8, b2 = lane & 4;
  float w4[4], w2[2];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const float r = __shfl_xor_sync(0xffffffffu, b4 ? w8[j] : w8[j + 4], 16);
    w4[j] = (b4 ? w8[j + 4] : w8[j]) + r;
  }
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    const float r = __shfl_xor_sync(0xffffffffu, b3 ? w4[j] : w4[j + 2], 8);
    w2[j] = (b3 ? w4[j + 2] : w4[j]) + r;
  }
  const float r = __shfl_xor_sync(0xffffffffu, b2 ? w2[0] : w2[1], 4);
  float x = (b2 ? w2[1] : w2[0]) + r;
  x += __shfl_xor_sync(0xffffffffu, x, 2);
  *k = (b4 ? 4 : 0) + (b3 ? 2 : 0) + (b2 ? 1 : 0);
  return x;
}

// Barrier over the 4 warps of worker group `grp` (ids 1, 2) that ORs a
// predicate across them.
__device__ __forceinline__ bool group_sync_or(int grp, bool x) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\t"
      "bar.red.or.pred q, %2, %3, p;\n\tselp.u32 %0, 1, 0, q;\n\t}"
      : "=r"(r)
      : "r"(uint32_t(x)), "r"(1 + grp), "n"(kTaGroupThreads)
      : "memory");
  return r != 0;
}

struct TaPlan {
  size_t off_park, off_stage, off_ant, off_acc, off_src, off_bar, total;
};

// Per-source terms of a tile shared by a worker group's items:
// sqrt(B) (Re B00, Re B11, Re B01, Im B01; B10 = conj B01) and l, m, l / n,
// m / n.  Eight lanes fill a tile's entries, a tile ahead.
struct TaSrc {
  float4 b, lm;
};

__device__ __forceinline__ void ta_fill_src(const FusedArgs<float>& A, int t, int ch, int s, float log2_ratio,
                                            TaSrc* dst) {
  const SrcInfo<float> si = point_source_chain_info(A, t, ch, s, log2_ratio);
  dst->b = make_float4(si.B.a.r, si.B.d.r, si.B.b.r, si.B.b.i);
  dst->lm = make_float4(si.l, si.m, si.l_over_n, si.m_over_n);
}

// The MMAs of one tile for one chain of dJ = Y J, from the Y operand in
// TMEM (ytm: column 0, lane 0) and the tile's J operand at jsm (shared-memory
// address of the hi part; the lo part follows, and J's lo rows sit where
// rows 16-31 of a 32-row operand would, so one N = 32 MMA forms
// Y_hi [J_hi; J_lo]^T).  Per K step (16 values: 8 TMEM columns of Y):
//   D[0:16] += Y_hi J_hi^T,  D[16:32] += Y_hi J_lo^T   (N = 32)
//   D[0:16] += Y_lo J_hi^T                             (N = 16)
// Chain Re (im = false) accumulates at d over all K steps; chain Im (im =
// true) at d as -Y_im Re J (negate-A bit) plus Y_re Im J.  dJ = D[0:16] +
// D[16:32].  The two chains go to different accumulators and are issued by
// different threads, in parallel.
__device__ __forceinline__ void ta_issue_chain(bool im, uint32_t d, uint32_t ytm, uint32_t jsm) {
  constexpr uint32_t id32 = TaLayout::instr(128, 32), id16 = TaLayout::instr(128, 16);
  const uint32_t neg = im ? (1u << 13) : 0u;  // negate A for -Y_im
  const uint32_t yh = ytm, yl = ytm + 128;
  const uint64_t jh = TaGeom::desc(jsm);
  constexpr uint64_t kStep = TaGeom::kKStepBytes >> 4;
  constexpr int half = TaGeom::kKSteps / 2;
#pragma unroll
  for (int kk = 0; kk < half; ++kk) {
    const uint64_t ore = kk * kStep, oim = (kk + half) * kStep;  // J descriptor steps
    const uint32_t cre = 8 * kk, cim = 8 * (kk + half);          // Y columns
    const uint32_t acc = kk == 0 ? 0u : 1u;
    // Re: Y_re Re J + (-Y_im) Im J;  Im: (-Y_im) Re J (negated: Y_im Re J) + Y_re Im J
    const uint32_t c1 = im ? cim : cre, c2 = im ? cre : cim;
    tc::mma_f16_ta(d, yh + c1, jh + ore, id32 | neg, acc);
    tc::mma_f16_ta(d, yl + c1, jh + ore, id16 | neg, 1u);
    tc::mma_f16_ta(d, yh + c2, jh + oim, id32, 1u);
    tc::mma_f16_ta(d, yl + c2, jh + oim, id16, 1u);
  }
}

// PACK (at most 32 antennas): a CTA takes the unit pair (t, 2k), (t, 2k + 1);
// TMEM lane 64 c + 2 a + i works on channel c, antenna a, and Y is the
// block-diagonal matrix of both channels over 64 virtual antennas 32 c + a,
// so one sequence of MMAs serves both channels.
template <bool BATCHED, bool PACK>
__global__ void __launch_bounds__(kTaThreads, 1) coh_tc_adj_kernel(FusedArgs<float> A_in, TaPlan P) {
  extern __shared__ __align__(16) unsigned char smem[];
  float4* park = reinterpret_cast<float4*>(smem + P.off_park);  // [group][item][kTaPark][128 lanes]
  unsigned char* stage = smem + P.off_stage;  // [kTaGroups][kJopBytes]
  AntInfo<float>* sa = reinterpret_cast<AntInfo<float>*>(smem + P.off_ant);
  float* sacc = reinterpret_cast<float*>(smem + P.off_acc);  // [kTaGroups][2][NCH][kTaKappa][kTaAcc]
  TaSrc* ssrc = reinterpret_cast<TaSrc*>(smem + P.off_src);   // [kTaGroups][2][NCH][kTaKappa]
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + P.off_bar);
  uint64_t* dfull = bars;               // [kTaGroups] MMA commit -> group (dJ in TMEM)
  uint64_t* done = dfull + kTaGroups;   // [kTaGroups] last MMAs of a group
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + kTaGroups);
  int* abort_flag = reinterpret_cast<int*>(tmem_slot + 1);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  FusedArgs<float> A = A_in;
  int cta = blockIdx.x;
  if constexpr (BATCHED) cta = cta_unit(A);
  constexpr int NCH = PACK ? 2 : 1;  // channels per CTA
  int t, ch, nch = 1;                // time, first channel, channels of this CTA
  if (PACK) {
    const int npc = (A.nchan + 1) / 2;
    t = cta / npc;
    ch = 2 * (cta - t * npc);
    nch = min(2, A.nchan - ch);
  } else {
    t = cta / A.nchan;
    ch = cta - t * A.nchan;
  }
  const int unit = t * A.nchan + ch;
  if (tid == 0) *abort_flag = A.err ? *reinterpret_cast<volatile int*>(A.err) : 0;
  __syncthreads();
  if (*abort_flag) return;
  __syncthreads();

  for (int c = 0; c < nch; ++c) load_antennas(A, t, ch + c, sa + c * A.na);
  for (int i = tid; i < kTaGroups * 2 * NCH * kTaKappa * kTaAcc; i += blockDim.x) sacc[i] = 0.f;
  if (tid == 0) {
    for (int g = 0; g < kTaGroups; ++g) {
      tc::mbar_init(dfull + g, 2);  // one commit per chain issuer
      tc::mbar_init(done + g, 2);
    }
  }
  tc::fence_proxy_async_smem();
  if (warp == 0) tc::tmem_alloc(tmem_slot, kTaCols);
  tc::fence_before_thread_sync();
  __syncthreads();
  tc::fence_after_thread_sync();
  const uint32_t tmem = *tmem_slot;
  // Y of this unit from d chi^2 / dV, formed in the park region (unused until
  // the tile sweep): baseline (p, q) adds gV to Y_pq and gV^H to Y_qp (both to
  // Y_pp for an autocorrelation; repeated pairs sum).  Rows of Y are padded
  // by 32 bytes, so the 16-byte loads of 4 rows x 2 Jones rows that a
  // quarter warp makes below meet distinct banks.  Then each TMEM lane r =
  // (a, i) takes its row of the BF16 hi + lo operand: word kp of the hi half
  // (columns 0-127) holds K = 2 kp, 2 kp + 1, i.e. Re Y_ab[i][0], Re Y_ab[i][1]
  // for b = kp < 64 and -Im of them for b = kp - 64; the lo half (columns
  // 128-255) likewise.  The three warps of a lane quarter share the row's 8
  // runs of 32 words.
  // PACK: virtual antennas 32 c + a, off-diagonal channel blocks zero.
  {
    unsigned char* ybase = reinterpret_cast<unsigned char*>(park);
    const int na = PACK ? 64 : A.na, yrow = kTaYRowBytes;
    for (int x = tid; x < na * yrow / 16; x += blockDim.x)
      reinterpret_cast<uint4*>(ybase)[x] = make_uint4(0u, 0u, 0u, 0u);
    __syncthreads();
    for (int x = tid; x < nch * A.nbl; x += blockDim.x) {
      const int c = PACK ? x / A.nbl : 0, bl = PACK ? x - c * A.nbl : x;
      const size_t tbl = size_t(t) * A.lnbl + bl;
      int p, q;
      if (!local_baseline(A, A.ant1[tbl], A.ant2[tbl], p, q)) continue;
      p += 32 * c;
      q += 32 * c;
      const Jones<float> g = jload<float>(A.gV + 8 * ((size_t(t) * A.nbl + bl) * A.nchan + ch + c));
      atomic_add_jones(reinterpret_cast<Jones<float>*>(ybase + size_t(p) * yrow) + q, g);
      atomic_add_jones(reinterpret_cast<Jones<float>*>(ybase + size_t(q) * yrow) + p, jherm(g));
    }
    __syncthreads();
    const int q = warp & 3, part = warp >> 2;
    const int r = 32 * q + lane, a = r >> 1, i = r & 1;
    const float* yr = reinterpret_cast<const float*>(ybase + size_t(a < na ? a : 0) * yrow) + 4 * i;
    for (int run = part; run < 8; run += kTaGroups) {
      const bool lo_half = run >= 4, im = (run & 3) >= 2;
      const int b0 = 32 * (run & 1);
      uint32_t w[32];
#pragma unroll
      for (int k = 0; k < 32; ++k) {
        const int b = b0 + k;
        float x0 = 0.f, x1 = 0.f;
        if (a < na && b < na) {
          const float4 y4 = *reinterpret_cast<const float4*>(yr + 8 * b);  // Y_ab[i][0], Y_ab[i][1]
          x0 = im ? -y4.y : y4.x;
          x1 = im ? -y4.w : y4.z;
        }
        __nv_bfloat16 h0, l0, h1, l1;
        tc::split_bf16(x0, h0, l0);
        tc::split_bf16(x1, h1, l1);
        w[k] = lo_half ? (uint32_t(__bfloat16_as_ushort(l0)) | (uint32_t(__bfloat16_as_ushort(l1)) << 16))
                       : (uint32_t(__bfloat16_as_ushort(h0)) | (uint32_t(__bfloat16_as_ushort(h1)) << 16));
      }
      tc::tmem_st32(tmem + (uint32_t(32 * q) << 16) + uint32_t(32 * run), w);
    }
    tc::tmem_wait_st();
  }
  tc::fence_before_thread_sync();
  __syncthreads();
  tc::fence_after_thread_sync();

  const int ntiles = (A.npsrc + kTaKappa - 1) / kTaKappa;
  const uint32_t wlim = g_pipe_wait_limit;
  // Units start their tile sweep at different tiles, so that the CTAs in
  // flight (neighbouring channels) do not update the same sources' FP64
  // accumulators at the same time.
  const int rot = int((unsigned(unit) * 2654435761u) % unsigned(max(ntiles, 1)));
  auto tile_of = [&](int g) { const int x = g + rot; return x >= ntiles ? x - ntiles : x; };

  {
    const int grp = warp >> 2, q = warp & 3;
    const bool issuer = q < 2 && lane == 0;  // warp q = 0 issues chain Re, q = 1 chain Im
    bool issued = false;
    // TMEM lane r = (va, i): virtual antenna va = antenna a (PACK: 32 c + a,
    // channel c, the same for the whole warp)
    const int r = 32 * q + lane, va = r >> 1, i = r & 1;
    const int c = PACK ? va >> 5 : 0, a = PACK ? va & 31 : va;
    const int chl = min(ch + c, A.nchan - 1);  // this lane's channel
    const bool ant_ok = a < A.na && c < nch;
    const AntInfo<float> ai = sa[c * A.na + (ant_ok ? a : 0)];
    const float f = A.freq[chl];
    const NuC nu = make_nuc(double(f) / kLightSpeed);
    const ChanPos<float> cp = chan_pos<float>(f, A.lfreq, A.ufreq, A.nud);
    const float dphase = float(nu.dphase);
    unsigned char* hi = stage + size_t(grp) * kJopBytes;
    unsigned char* lo = hi + kJopBytes / 2;
    const BeamGeom G{A.lw, A.mh, A.nud};
    const float* plane = A.plane ? A.plane + size_t(chl) * A.lw * A.mh * kPlaneVals : nullptr;
    const uint32_t tlane = tmem + (uint32_t(32 * q) << 16) + kTaYCols + uint32_t(kTaGroupCols * grp);
    float4* mypark = park + size_t(grp) * kTaItems * kTaPark * 128 + r;
    TaSrc* gsrc = ssrc + size_t(grp) * 2 * NCH * kTaKappa;  // this group's two tiles of source terms
    const int ct = tid - grp * kTaGroupThreads;              // thread index within the group
    // the source terms of a tile are filled by NCH * kTaKappa threads of the
    // group: thread ct takes source ct % kTaKappa at channel ct / kTaKappa
    const int fc_ = ct / kTaKappa, fs_ = ct - fc_ * kTaKappa;
    const int fch = min(ch + fc_, A.nchan - 1);
    const float flog2 = log2f(A.freq[fch] / A.ref_freq[fch]);
    const float fhalf_log = 0.5f * logf(A.freq[fch] / A.ref_freq[fch]);
    const bool filler = ct < NCH * kTaKappa && fc_ < nch;
    if (filler && grp < ntiles) {
      const int s = tile_of(grp) * kTaKappa + fs_;
      if (s < A.npsrc) ta_fill_src(A, t, fch, s, flog2, gsrc + ct);
    }
    bool bad = group_sync_or(grp, false);
    int k = 0;  // this group's tile count
    for (int g = grp; g < ntiles; g += kTaGroups, ++k) {
      const int s0 = tile_of(g) * kTaKappa, ns = min(kTaKappa, A.npsrc - s0);
      const TaSrc* tsrc = gsrc + ((k & 1) * NCH + c) * kTaKappa;  // this tile's source terms (lane's channel)
      if (filler && g + kTaGroups < ntiles) {  // the next tile's, before the staging barrier
        const int s = tile_of(g + kTaGroups) * kTaKappa + fs_;
        if (s < A.npsrc) ta_fill_src(A, t, fch, s, flog2, gsrc + ((k + 1) & 1) * NCH * kTaKappa + ct);
      }
      if (ant_ok && g + kTaGroups < ntiles && A.phi) {  // the items' path lengths, a tile ahead
        const int sn0 = tile_of(g + kTaGroups) * kTaKappa;
#pragma unroll
        for (int u = 0; u < kTaItems; ++u)
          if (sn0 + 4 * i + u < A.npsrc)
            tc::prefetch_l1(A.phi + (size_t(t) * A.nsrc + sn0 + 4 * i + u) * A.na_glob + gant(A, a));
      }
      if (ct < kTaKappa && g + 2 * kTaGroups < ntiles) {  // the source terms' table entries, two tiles ahead
        const int s = tile_of(g + 2 * kTaGroups) * kTaKappa + ct;
        if (s < A.npsrc) {
          if (A.bsq0) tc::prefetch_l1(A.bsq0 + kBsqVals * (size_t(s) * A.ntime + t));
          tc::prefetch_l1(A.lm + 2 * s);
        }
      }
      // ---- forward step: J of the items, staged for the MMA -------------
#pragma unroll
      for (int u = 0; u < kTaItems; ++u) {
        const int sl = 4 * i + u;
        Jones<float> J = jzero<float>();
        float st[3][8];  // EK, Pl, Pm
#pragma unroll
        for (int e = 0; e < 8; ++e) st[0][e] = st[1][e] = st[2][e] = 0.f;
        if (!bad && ant_ok && sl < ns) {
          const int sg = s0 + sl;
          const float4 tb = tsrc[sl].b, tlm = tsrc[sl].lm;
          const Cx<float> K = phase_term(A, t, sg, a, f, nu);
          float l, m;
          beam_lm<float>(tlm.x, tlm.y, ai.sin_pa, ai.cos_pa, ai.pe_l, ai.pe_m, ai.sc_l, ai.sc_m, l, m);
          const GridPos<float> gl = grid_pos<float>(l, A.ll, A.ul, A.lscale, A.lw);
          const GridPos<float> gm = grid_pos<float>(m, A.lmm, A.um, A.mscale, A.mh);
          Jones<float> E, dEl, dEm;
          if (plane) beam_interp_plane_d<float>(plane, A.mh, gl, gm, E, dEl, dEm);
          else beam_interp_d<float>(A.E_beam, G, gl, gm, cp, E, dEl, dEm);
          // J = (E K) sqrt(B); the beam derivatives are parked times K (zero
          // where the grid coordinate was clamped), sqrt(B) joins in the chain
          const Jones<float> EK = {cmul(E.a, K), cmul(E.b, K), cmul(E.c, K), cmul(E.d, K)};
          J = jmul_herm_real_diag(EK, tb.x, tb.y, Cx<float>{tb.z, tb.w});
          const Cx<float> Kl = gl.inside ? K : Cx<float>{0.f, 0.f}, Km = gm.inside ? K : Cx<float>{0.f, 0.f};
          const Jones<float> DL = {cmul(dEl.a, Kl), cmul(dEl.b, Kl), cmul(dEl.c, Kl), cmul(dEl.d, Kl)};
          const Jones<float> DM = {cmul(dEm.a, Km), cmul(dEm.b, Km), cmul(dEm.c, Km), cmul(dEm.d, Km)};
#pragma unroll
          for (int e = 0; e < 8; ++e) {
            st[0][e] = reinterpret_cast<const float*>(&EK)[e];
            st[1][e] = reinterpret_cast<const float*>(&DL)[e];
            st[2][e] = reinterpret_cast<const float*>(&DM)[e];
          }
        }
        // park the item's state in shared memory (lane-contiguous float4)
#pragma unroll
        for (int x = 0; x < 3; ++x) {
          mypark[(u * kTaPark + 2 * x) * 128] = make_float4(st[x][0], st[x][1], st[x][2], st[x][3]);
          mypark[(u * kTaPark + 2 * x + 1) * 128] = make_float4(st[x][4], st[x][5], st[x][6], st[x][7]);
        }
        // row (s, k): K = (va, 0), (va, 1) hold J[0][k], J[1][k]
        TaLayout::put2(hi, lo, 2 * sl, 2 * va, J.a.r, J.c.r);
        TaLayout::put2(hi, lo, 2 * sl, 128 + 2 * va, J.a.i, J.c.i);
        TaLayout::put2(hi, lo, 2 * sl + 1, 2 * va, J.b.r, J.d.r);
        TaLayout::put2(hi, lo, 2 * sl + 1, 128 + 2 * va, J.b.i, J.d.i);
      }
      tc::fence_proxy_async_smem();
      tc::fence_before_thread_sync();
      if (group_sync_or(grp, bad)) { bad = true; break; }
      if (issuer) {
        tc::fence_after_thread_sync();
        ta_issue_chain(q == 1, tmem + kTaYCols + uint32_t(kTaGroupCols * grp) + uint32_t(32 * q), tmem,
                       tc::smem_addr(hi));
        tc::mma_commit(dfull + grp);
        issued = true;
      }
      // ---- dJ of the tile: TMEM buffer grp ------------------------------
      if (!bad) bad = !tc::mbar_wait(dfull + grp, k & 1, wlim);
      tc::fence_after_thread_sync();
      float v[32];  // v[2s + kc] = Re dJ(s)[i][kc], v[16 + 2s + kc] = Im
      if (!__any_sync(0xffffffffu, bad)) {  // warp-collective loads, only of finished MMAs
        float re[32], im[32];
        tc::tmem_ld32(tlane, re);
        tc::tmem_ld32(tlane + 32, im);
#pragma unroll
        for (int e = 0; e < 16; ++e) {
          v[e] = re[e] + re[16 + e];
          v[16 + e] = im[e] + im[16 + e];
        }
      } else {
        bad = true;
#pragma unroll
        for (int e = 0; e < 32; ++e) v[e] = 0.f;
      }
      // own row i of dJ for sources 4i + u; the partner lane (a, 1 - i)
      // holds row 1 - i.  Give it row i of its sources 4(1 - i) + u.
      float recv[16];
#pragma unroll
      for (int u = 0; u < kTaItems; ++u)
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          const int own = 2 * u + e, oth = 8 + 2 * u + e;  // column of source u / 4 + u
          recv[4 * u + e] = __shfl_xor_sync(0xffffffffu, i ? v[own] : v[oth], 1);
          recv[4 * u + 2 + e] = __shfl_xor_sync(0xffffffffu, i ? v[16 + own] : v[16 + oth], 1);
        }
      // ---- chain step ------------------------------------------------------
      float* tacc = sacc + (size_t(grp) * 2 + (k & 1)) * NCH * kTaKappa * kTaAcc;  // this tile's sums
      float* acc = tacc + c * kTaKappa * kTaAcc;                                    // the lane's channel
#pragma unroll
      for (int u = 0; u < kTaItems; ++u) {
        const int sl = 4 * i + u;
        // own row: column 2 sl + kc of v, sl = 4i + u (constant indices, lane select)
        const int c0 = 2 * u, c1 = 8 + 2 * u;
        const Cx<float> o0{i ? v[c1] : v[c0], i ? v[16 + c1] : v[16 + c0]};
        const Cx<float> o1{i ? v[c1 + 1] : v[c0 + 1], i ? v[16 + c1 + 1] : v[16 + c0 + 1]};
        const Cx<float> p0{recv[4 * u], recv[4 * u + 2]}, p1{recv[4 * u + 1], recv[4 * u + 3]};
        Jones<float> gJ;
        gJ.a = i ? p0 : o0; gJ.b = i ? p1 : o1;
        gJ.c = i ? o0 : p0; gJ.d = i ? o1 : p1;
        float gsum[8];  // kTaAcc values, zero padded for the reduce-scatter
#pragma unroll
        for (int e = 0; e < 8; ++e) gsum[e] = 0.f;
        float sv[24];  // parked EK, DL, DM of the item
#pragma unroll
        for (int x = 0; x < kTaPark; ++x) {
          const float4 p4 = mypark[(u * kTaPark + x) * 128];
          sv[4 * x] = p4.x; sv[4 * x + 1] = p4.y; sv[4 * x + 2] = p4.z; sv[4 * x + 3] = p4.w;
        }
        if (!bad && ant_ok && sl < ns) {
          const float4 tb = tsrc[sl].b, tlm = tsrc[sl].lm;
          Jones<float> EK, DL, DM;
#pragma unroll
          for (int e = 0; e < 8; ++e) {
            reinterpret_cast<float*>(&EK)[e] = sv[e];
            reinterpret_cast<float*>(&DL)[e] = sv[8 + e];
            reinterpret_cast<float*>(&DM)[e] = sv[16 + e];
          }
          const Jones<float> gB = jhmul(EK, gJ);
          // Re tr(gJ^H dE K sqrt(B)) = Re tr((gJ sqrt(B))^H dE K), sqrt(B) Hermitian
          const Jones<float> W = jmul_herm_real_diag(gJ, tb.x, tb.y, Cx<float>{tb.z, tb.w});
          const float g_ld = A.lscale * jdot_re(W, DL), g_md = A.mscale * jdot_re(W, DM);
          // Im tr(gB^H B), B = [[a, b], [conj(b), d]] with a, d real
          const float imt = -gB.a.i * tb.x - gB.d.i * tb.y + (gB.b.r * tb.w - gB.b.i * tb.z) -
                            (gB.c.r * tb.w + gB.c.i * tb.z);
          const float gphi = dphase * imt;
          gsum[0] = g_ld * ai.sc_l * ai.cos_pa + g_md * ai.sc_m * ai.sin_pa +
                    gphi * (ai.u - ai.w * tlm.z);
          gsum[1] = -g_ld * ai.sc_l * ai.sin_pa + g_md * ai.sc_m * ai.cos_pa +
                    gphi * (ai.v - ai.w * tlm.w);
          gsum[2] = gB.a.r;
          gsum[3] = gB.d.r;
          gsum[4] = gB.b.r + gB.c.r;
          gsum[5] = gB.b.i - gB.c.i;
        }
        // sum over the warp's 16 antennas (lane bits 1-4)
        int e;
        const float x = reduce_scatter8(gsum, lane, &e);
        if (e < kTaAcc && !(lane & 2)) atomicAdd(acc + sl * kTaAcc + e, x);
      }
      if (group_sync_or(grp, bad)) { bad = true; break; }
      // flush the tile's per-source sums to the FP64 accumulators; the
      // other accumulator buffer takes the group's next tile
      if (filler) {  // thread ct: source fs_ at channel fch
        float* rr = tacc + ct * kTaAcc;
        if (fs_ < ns) {
          const int sg = s0 + fs_;
          if (rr[0] != 0.f) atomicAdd(&A.acc_lm[2 * sg], double(rr[0]));
          if (rr[1] != 0.f) atomicAdd(&A.acc_lm[2 * sg + 1], double(rr[1]));
          const SrcInfo<float> src = point_source_stokes(A, t, fch, sg, flog2);
          // a Hermitian gB with the summed parts (all the gradients read)
          const Jones<float> gB = {{rr[2], 0.f}, {0.5f * rr[4], 0.5f * rr[5]}, {0.5f * rr[4], -0.5f * rr[5]},
                                   {rr[3], 0.f}};
          float gs[5];
          stokes_grads(src, gB, fhalf_log, gs);
          double* st = &A.acc_stokes[(size_t(sg) * A.ntime + t) * 4];
#pragma unroll
          for (int e = 0; e < 4; ++e)
            if (gs[e] != 0.f) atomicAdd(st + e, double(gs[e]));
          if (gs[4] != 0.f) atomicAdd(&A.acc_alpha[size_t(sg) * A.ntime + t], double(gs[4]));
        }
#pragma unroll
        for (int e = 0; e < kTaAcc; ++e) rr[e] = 0.f;
      }
    }
    // every MMA of the group has completed before TMEM is released
    if (issued) {
      tc::mma_commit(done + grp);
      if (!tc::mbar_wait(done + grp, 0)) bad = true;
    }
    if (bad && lane == 0) *abort_flag = 1;
  }
  tc::fence_before_thread_sync();
  __syncthreads();
  tc::fence_after_thread_sync();
  if (warp == 0) tc::tmem_dealloc(tmem, kTaCols);
  if (*abort_flag && tid == 0 && A.err) atomicExch(A.err, int(MB_ERR_TIMEOUT));
}

// ---------------------------------------------------------------------------
// Small kernels: phase path lengths, gradient finalisation
// ---------------------------------------------------------------------------
// Frequency-blended beam plane per active channel as bilinear coefficients
// per (l, m) cell (see plane_cell), formed in FP64 from the cube.
template <typename T>
__global__ void beam_plane_kernel(FusedArgs<T> A, T* __restrict__ plane) {
  const size_t cells = size_t(A.lw) * A.mh;
  const size_t total = size_t(A.nchan) * cells;
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < total; i += size_t(gridDim.x) * blockDim.x) {
    const int ch = int(i / cells);
    const size_t cell = i - size_t(ch) * cells;
    const int il = int(cell / A.mh), im = int(cell % A.mh);
    const int il1 = min(il + 1, A.lw - 1), im1 = min(im + 1, A.mh - 1);
    const ChanPos<T> cp = chan_pos<T>(A.freq[ch], A.lfreq, A.ufreq, A.nud);
    const double w0 = 1.0 - double(cp.d), w1 = double(cp.d);
    double v[4][kPlaneComp];  // corners (il, im), (il1, im), (il, im1), (il1, im1)
    const int cl[4] = {il, il1, il, il1}, cm[4] = {im, im, im1, im1};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const size_t c = size_t(cl[k]) * A.mh + cm[k];
      const T* e0 = A.E_beam + 8 * (c * A.nud + cp.c0);
      const T* e1 = A.E_beam + 8 * (c * A.nud + cp.c1);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const double ar = e0[2 * q], ai = e0[2 * q + 1], br = e1[2 * q], bi = e1[2 * q + 1];
        v[k][2 * q] = w0 * ar + w1 * br;
        v[k][2 * q + 1] = w0 * ai + w1 * bi;
        v[k][8 + q] = w0 * sqrt(ar * ar + ai * ai) + w1 * sqrt(br * br + bi * bi);
      }
    }
    T* out = plane + kPlaneVals * i;
#pragma unroll
    for (int q = 0; q < kPlaneComp; ++q) {
      const double b = v[2][q] - v[0][q];
      out[q] = T(v[0][q]);
      out[kPlaneComp + q] = T(v[1][q] - v[0][q]);
      out[2 * kPlaneComp + q] = T(b);
      out[3 * kPlaneComp + q] = T(v[3][q] - v[1][q] - b);
    }
  }
}

// sqrt(B) at nu = nu_ref, and alpha / 2, per (source, time):
// sqrt(B)(nu) = (nu / nu_ref)^(alpha / 2) * sqrt(B)(nu_ref).  Layout
// [s][t][8] = ((I+Q+s0)/tau, (I-Q+s0)/tau, U/tau, V/tau, alpha/2, 0, 0, 0):
// 32-byte entries, so the first four values are one aligned 16-byte load.
template <typename T>
__global__ void bsqrt_ref_kernel(FusedArgs<T> A_in, T* __restrict__ tab) {
  FusedArgs<T> A = A_in;
  if (A.bsets) {  // batched: grid.y = set, the set's own table
    use_set(A, A.bsets[blockIdx.y]);
    tab = const_cast<T*>(A.bsq0);
  }
  const size_t total = size_t(A.nsrc) * A.ntime;
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < total; i += size_t(gridDim.x) * blockDim.x) {
    const int s = int(i / A.ntime), t = int(i % A.ntime);
    const size_t st = size_t(s) * A.ltime + t;
    const T* S = A.stokes + 4 * st;
    const Jones<T> B = brightness_sqrt<T>(S[0], S[1], S[2], S[3], T(1));
    T* o = tab + kBsqVals * i;
    o[0] = B.a.r; o[1] = B.d.r; o[2] = B.b.r; o[3] = B.b.i;
    o[4] = T(0.5) * A.alpha[st];
    // l / n, m / n with n = sqrt(1 - l^2 - m^2) (phase gradient), in FP64
    const double l = A.lm[2 * s], m = A.lm[2 * s + 1], n = sqrt(1.0 - l * l - m * m);
    o[5] = T(0);
    o[6] = T(l / n);
    o[7] = T(m / n);
  }
}

template <typename T>
__global__ void phi_kernel(FusedArgs<T> A_in, double* __restrict__ phi) {
  FusedArgs<T> A = A_in;
  if (A.bsets) {  // batched: grid.y = set, the set's own table
    use_set(A, A.bsets[blockIdx.y]);
    phi = const_cast<double*>(A.phi);
  }
  size_t total = size_t(A.ntime) * A.nsrc * A.na;
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < total; i += size_t(gridDim.x) * blockDim.x) {
    int a = int(i % A.na);
    int s = int((i / A.na) % A.nsrc);
    int t = int(i / (size_t(A.na) * A.nsrc));
    double l = A.lm[2 * s], m = A.lm[2 * s + 1];
    double n = sqrt(1.0 - l * l - m * m) - 1.0;
    const T* p = A.uvw + 3 * (size_t(t) * A.lna + a);
    const double v = l * double(p[0]) + m * double(p[1]) + n * double(p[2]);
    if constexpr (sizeof(T) == 4) reinterpret_cast<float2*>(phi)[i] = split_f64(v);  // see phase_term
    else phi[i] = v;
  }
}

template <typename T>
__global__ void finalize_grads_kernel(FusedArgs<T> A_in, double scale, T* __restrict__ g_lm, T* __restrict__ g_stokes,
                                      T* __restrict__ g_alpha, T* __restrict__ g_gauss, T* __restrict__ g_sersic,
                                      T* __restrict__ g_G) {
  FusedArgs<T> A = A_in;
  if (A.bsets) {  // batched: grid.y = set, the set's accumulators and outputs
    const BatchSet<T>& b = A.bsets[blockIdx.y];
    use_set(A, b);
    g_lm = b.g_lm; g_stokes = b.g_stokes; g_alpha = b.g_alpha;
    g_gauss = b.g_gauss; g_sersic = b.g_sersic; g_G = b.g_G;
  }
  const size_t n_lm = size_t(A.nsrc) * 2, n_st = size_t(A.nsrc) * A.ntime;
  const size_t n_g = size_t(3) * A.ngsrc, n_x = size_t(3) * A.nssrc;
  const size_t n_G = size_t(A.ntime) * A.na * A.nchan;
  const size_t total = n_lm + n_st + n_g + n_x + n_G;
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < total; i += size_t(gridDim.x) * blockDim.x) {
    size_t j = i;
    if (j < n_lm) { if (g_lm) g_lm[j] = T(A.acc_lm[j] * scale); continue; }
    j -= n_lm;
    if (j < n_st) {
      size_t s = j / A.ntime, t = j % A.ntime;
      size_t dst = s * A.ltime + t;
      if (g_stokes)
        for (int k = 0; k < 4; ++k) g_stokes[4 * dst + k] = T(A.acc_stokes[4 * j + k] * scale);
      if (g_alpha) g_alpha[dst] = T(A.acc_alpha[j] * scale);
      continue;
    }
    j -= n_st;
    if (j < n_g) { if (g_gauss) g_gauss[(j / A.ngsrc) * A.lgsrc + j % A.ngsrc] = T(A.acc_gauss[j] * scale); continue; }
    j -= n_g;
    if (j < n_x) { if (g_sersic) g_sersic[(j / A.nssrc) * A.lssrc + j % A.nssrc] = T(A.acc_sersic[j] * scale); continue; }
    j -= n_x;
    if (g_G) {
      size_t ch = j % A.nchan, a = (j / A.nchan) % A.na, t = j / (size_t(A.nchan) * A.na);
      const T* src = A.dG + 8 * j;
      T* dst = g_G + 8 * ((t * A.lna + a) * A.lchan + ch);
      for (int k = 0; k < 8; ++k) dst[k] = T(double(src[k]) * scale);
    }
  }
}

// chi^2 of every set of a batch: block b sums set b's unit partials in a
// fixed order (deterministic), X2[b] = scale * sum.
template <typename T>
__global__ void sum_partials_sets_kernel(const BatchSet<T>* __restrict__ sets, int units, double scale,
                                         double* __restrict__ X2) {
  __shared__ double red[32];
  const double* partial = sets[blockIdx.x].partial;
  double acc = 0.0;
  for (int i = threadIdx.x; i < units; i += blockDim.x) acc += partial[i];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    acc = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (threadIdx.x == 0) X2[blockIdx.x] = acc * scale;
  }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
// Antenna sub-arrays.  The fused kernels hold one (time, channel) unit's
// pair sums (or, in the adjoint, its matrix of d chi^2 / dV) for at most
// kSubMaxNa antennas: the tensor-core kernels' 128-row MMA tile and the
// CUDA-core kernels' shared memory.  A larger array is split into blocks of
// kSubBlock antennas and evaluated as one launch per pair of blocks I < J on
// the antennas of both; that launch owns the baselines between I and J, and
// those within I when J = I + 1 and within J for the last pair, so each
// baseline is summed, written and differentiated exactly once.  Per-antenna
// work is repeated in each launch that holds the antenna (nb - 1 times for
// nb blocks); chi^2 partials are kept per launch and dchi^2/dG is summed
// over them.
constexpr int kSubMaxNa = 64;
constexpr int kSubBlock = 32;

int sub_blocks(int na) { return (na + kSubBlock - 1) / kSubBlock; }
int sub_count(int na) {
  if (na <= kSubMaxNa) return 1;
  const int nb = sub_blocks(na);
  return nb * (nb - 1) / 2;
}

// Arguments of sub-array launch k (of sub_count(A.na)) over `units` units.
template <typename T>
FusedArgs<T> sub_args(const FusedArgs<T>& A, int k, int units) {
  if (A.na_glob <= kSubMaxNa) return A;
  const int na = A.na_glob, nb = sub_blocks(na);
  int I = 0, r = k;  // launch k is the k-th pair (I, J), I < J, in row-major order
  while (r >= nb - 1 - I) {
    r -= nb - 1 - I;
    ++I;
  }
  const int J = I + 1 + r;
  FusedArgs<T> S = A;
  S.sub_blk = kSubBlock;
  S.sub_i = I;
  S.sub_j = J;
  S.sub_off0 = I * kSubBlock;
  S.sub_off1 = J * kSubBlock;
  S.sub_n0 = std::min(kSubBlock, na - S.sub_off0);
  S.na = S.sub_n0 + std::min(kSubBlock, na - S.sub_off1);
  S.sub_diag = (J == I + 1 ? 1 : 0) | (I == nb - 2 && J == nb - 1 ? 2 : 0);
  if (A.partial) S.partial = A.partial + size_t(k) * units;
  return S;
}

struct WsLayout {
  size_t phi, plane, bsq0, partial, gV, dG, acc_lm, acc_stokes, acc_alpha, acc_gauss, acc_sersic, acc_end, err,
      vis_ext, total;
};

WsLayout ws_layout(mb_dtype dtype, mb_mode mode, const mb_dims* d, bool want_grad) {
  const size_t es = dtype == MB_FLOAT64 ? 8 : 4;
  const size_t nt = ext(d->ntime), na = ext(d->na), nbl = ext(d->nbl), nc = ext(d->nchan);
  const size_t ns = ext(d->nsrc), ng = ext(d->ngsrc), nx = ext(d->nssrc);
  WsLayout L;
  size_t o = 0;
  auto take = [&o](size_t bytes) { size_t r = o; o = align_up(o + bytes, 256); return r; };
  L.phi = take(nt * ns * na * 8);
  L.plane = take(nc * size_t(d->beam_lw.local_size) * d->beam_mh.local_size * kPlaneVals * es);
  L.bsq0 = take(dtype == MB_FLOAT32 ? ns * nt * kBsqVals * es : 0);
  L.partial = take(nt * nc * size_t(sub_count(int(na))) * 8);
  L.gV = take(want_grad ? nt * nbl * nc * 8 * es : 0);
  L.dG = take(want_grad ? nt * na * nc * 8 * es : 0);
  L.acc_lm = take(want_grad ? ns * 2 * 8 : 0);
  L.acc_stokes = take(want_grad ? ns * nt * 4 * 8 : 0);
  L.acc_alpha = take(want_grad ? ns * nt * 8 : 0);
  L.acc_gauss = take(want_grad ? 3 * ng * 8 : 0);
  L.acc_sersic = take(want_grad ? 3 * nx * 8 : 0);
  L.acc_end = o;
  L.err = take(sizeof(int));
  // split forms: the extended sources' visibility sums (local strides, as
  // the epilogue indexes visibilities)
  L.vis_ext = take(mode != MB_MODE_NATIVE && dtype == MB_FLOAT32 && (ng + nx) > 0
                       ? size_t(d->ntime.local_size) * d->nbl.local_size * d->nchan.local_size * 8 * es
                       : 0);
  L.total = o;
  return L;
}

template <typename T>
mb_status fill_args(FusedArgs<T>& A, const mb_dims* d, const mb_props* P, uint32_t options,
                    const mb_rime_inputs* in, void* model_vis, void* chi2, bool want_grad, void* ws,
                    const WsLayout& L) {
  A.ntime = ext(d->ntime); A.na = ext(d->na); A.nbl = ext(d->nbl); A.nchan = ext(d->nchan);
  A.nsrc = ext(d->nsrc); A.npsrc = ext(d->npsrc); A.ngsrc = ext(d->ngsrc); A.nssrc = ext(d->nssrc);
  A.ltime = d->ntime.local_size; A.lna = d->na.local_size; A.lnbl = d->nbl.local_size;
  A.lchan = d->nchan.local_size; A.lgsrc = d->ngsrc.local_size; A.lssrc = d->nssrc.local_size;
  A.lw = d->beam_lw.local_size; A.mh = d->beam_mh.local_size; A.nud = d->beam_nud.local_size;
  A.sbeg = 0;
  A.bsets = nullptr; A.bitems = nullptr;
  A.na_glob = A.na; A.sub_blk = 0; A.sub_i = A.sub_j = 0; A.sub_n0 = A.na;
  A.sub_off0 = A.sub_off1 = 0; A.sub_diag = 3;
  A.accumulate_in = d->nsrc.lower_extent > 0;
  A.partial_out = d->nsrc.upper_extent < d->nsrc.global_size;
  A.weights = options & MB_APPLY_WEIGHTS;
  A.residuals = options & MB_RESIDUALS;
  A.src_tile = 4 << ((options & MB_SOURCE_TILE_MASK) >> MB_SOURCE_TILE_SHIFT);  // 8, 16, 32
  if (!(options & MB_SOURCE_TILE_MASK)) A.src_tile = 0;
  A.want_grad = want_grad;
  A.ll = T(P->beam_ll); A.lmm = T(P->beam_lm); A.ul = T(P->beam_ul); A.um = T(P->beam_um);
  A.lfreq = T(P->beam_lfreq); A.ufreq = T(P->beam_ufreq);
  A.lscale = T(A.lw - 1) / (A.ul - A.ll);
  A.mscale = T(A.mh - 1) / (A.um - A.lmm);
  A.gauss_scale = T(P->gauss_scale); A.two_pi_over_c = T(P->two_pi_over_c);
  A.inv_sigma2 = 1.0 / P->sigma_sqrd;
  A.uvw = (const T*)in->uvw; A.freq = (const T*)in->frequency; A.ref_freq = (const T*)in->ref_frequency;
  A.pa = (const T*)in->parallactic_angles; A.pe = (const T*)in->point_errors; A.sc = (const T*)in->antenna_scaling;
  A.E_beam = (const T*)in->E_beam; A.G = (const T*)in->G_term; A.lm = (const T*)in->lm;
  A.stokes = (const T*)in->stokes; A.alpha = (const T*)in->alpha; A.gauss = (const T*)in->gauss_shape;
  A.sersic = (const T*)in->sersic_shape; A.weight = (const T*)in->weight_vector; A.obs = (const T*)in->observed_vis;
  A.ant1 = in->antenna1; A.ant2 = in->antenna2; A.flag = in->flag;
  A.model_vis = (T*)model_vis; A.chi2 = (T*)chi2;
  A.vis_in = (const T*)model_vis; A.tc_ext = true;
  A.err = nullptr;
  A.phi = nullptr; A.partial = nullptr; A.gV = nullptr; A.dG = nullptr;
  A.plane = nullptr; A.bsq0 = nullptr;
  A.acc_lm = A.acc_stokes = A.acc_alpha = A.acc_gauss = A.acc_sersic = nullptr;
  if (ws == nullptr) return MB_OK;
  char* w = static_cast<char*>(ws);
  A.phi = reinterpret_cast<const double*>(w + L.phi);
  A.plane = reinterpret_cast<const T*>(w + L.plane);
  A.bsq0 = sizeof(T) == 4 ? reinterpret_cast<const T*>(w + L.bsq0) : nullptr;
  A.partial = reinterpret_cast<double*>(w + L.partial);
  A.gV = want_grad ? reinterpret_cast<T*>(w + L.gV) : nullptr;
  A.dG = want_grad ? reinterpret_cast<T*>(w + L.dG) : nullptr;
  A.acc_lm = reinterpret_cast<double*>(w + L.acc_lm);
  A.acc_stokes = reinterpret_cast<double*>(w + L.acc_stokes);
  A.acc_alpha = reinterpret_cast<double*>(w + L.acc_alpha);
  A.acc_gauss = reinterpret_cast<double*>(w + L.acc_gauss);
  A.acc_sersic = reinterpret_cast<double*>(w + L.acc_sersic);
  A.err = reinterpret_cast<int*>(w + L.err);
  return MB_OK;
}

mb_status check_inputs(const mb_dims* d, const mb_props* P, uint32_t options, const mb_rime_inputs* in,
                       const void* model_vis) {
  MB_CHECK(check_dims(d, true));
  MB_REQUIRE(P, "props"); MB_REQUIRE(in, "inputs");
  MB_REQUIRE(in->uvw, "uvw"); MB_REQUIRE(in->antenna1, "antenna1"); MB_REQUIRE(in->antenna2, "antenna2");
  MB_REQUIRE(in->frequency, "frequency"); MB_REQUIRE(in->ref_frequency, "ref_frequency");
  MB_REQUIRE(in->parallactic_angles, "parallactic_angles"); MB_REQUIRE(in->point_errors, "point_errors");
  MB_REQUIRE(in->antenna_scaling, "antenna_scaling"); MB_REQUIRE(in->E_beam, "E_beam");
  MB_REQUIRE(in->lm, "lm"); MB_REQUIRE(in->stokes, "stokes"); MB_REQUIRE(in->alpha, "alpha");
  if (ext(d->ngsrc) > 0) MB_REQUIRE(in->gauss_shape, "gauss_shape");
  if (ext(d->nssrc) > 0) MB_REQUIRE(in->sersic_shape, "sersic_shape");
  const bool partial_out = d->nsrc.upper_extent < d->nsrc.global_size;
  if (partial_out || d->nsrc.lower_extent > 0) MB_REQUIRE(model_vis, "model_vis (source batches accumulate in it)");
  if (!partial_out) {
    MB_REQUIRE(in->G_term, "G_term"); MB_REQUIRE(in->flag, "flag"); MB_REQUIRE(in->observed_vis, "observed_vis");
    if (options & MB_APPLY_WEIGHTS) MB_REQUIRE(in->weight_vector, "weight_vector");
  }
  if (options & ~(MB_APPLY_WEIGHTS | MB_RESIDUALS | MB_SOURCE_TILE_MASK))
    return fail(MB_ERR_INVALID_ARG, "unknown option bits 0x%x", options);
  if (!(P->sigma_sqrd > 0.0) && !(options & MB_APPLY_WEIGHTS))
    return fail(MB_ERR_INVALID_ARG, "sigma_sqrd must be > 0 (got %g)", P->sigma_sqrd);
  if (ext(d->na) > 0xffff) return fail(MB_ERR_UNSUPPORTED, "na > 65535");
  MB_ALIGNED(in->E_beam, 16, "E_beam"); MB_ALIGNED(in->G_term, 16, "G_term");
  MB_ALIGNED(in->observed_vis, 16, "observed_vis"); MB_ALIGNED(model_vis, 16, "model_vis");
  MB_ALIGNED(in->flag, 4, "flag");
  return MB_OK;
}

// Per-call tables shared by the forward and the adjoint: the path lengths
// (formed in FP64; stored as FP32 pairs for the FP32 kernels), the
// frequency-blended beam plane, and (FP32) sqrt(B) at the reference
// frequency.
template <typename T>
mb_status launch_prep(const FusedArgs<T>& A, void* ws, const WsLayout& L, cudaStream_t stream) {
  char* w = static_cast<char*>(ws);
  auto blocks_for = [](size_t n) { return int(std::min<size_t>((n + 255) / 256, 1u << 20)); };
  size_t n = size_t(A.ntime) * A.nsrc * A.na;
  if (n > 0) {
    {
      KernelScope ks_("phi_kernel", stream);
      phi_kernel<T><<<blocks_for(n), 256, 0, stream>>>(A, reinterpret_cast<double*>(w + L.phi));
    }
    MB_CHECK(check_launch("phi_kernel"));
  }
  n = size_t(A.nchan) * A.lw * A.mh;
  if (n > 0) {
    {
      KernelScope ks_("beam_plane_kernel", stream);
      beam_plane_kernel<T><<<blocks_for(n), 256, 0, stream>>>(A, reinterpret_cast<T*>(w + L.plane));
    }
    MB_CHECK(check_launch("beam_plane_kernel"));
  }
  n = size_t(A.nsrc) * A.ntime;
  if (sizeof(T) == 4 && n > 0) {
    {
      KernelScope ks_("bsqrt_ref_kernel", stream);
      bsqrt_ref_kernel<T><<<blocks_for(n), 256, 0, stream>>>(A, reinterpret_cast<T*>(w + L.bsq0));
    }
    MB_CHECK(check_launch("bsqrt_ref_kernel"));
  }
  return MB_OK;
}

// Kernel launchers over `grid` CTAs: a single problem's (time, channel)
// units, or a batched launch's (set, unit) items (A.bitems).

// The tensor-core kernels pack two channels per CTA when the (sub-)array has
// at most 32 antennas (its 64 operand rows then fill the 128-row MMA tile).
bool tc_pack(int na) { return na <= 32; }
// CTAs of a tensor-core launch over ntime x nchan units.
int tc_ctas(int na, int ntime, int nchan) { return tc_pack(na) ? ntime * ((nchan + 1) / 2) : ntime * nchan; }

// Split-precision forward: point sources on the tensor cores, extended
// sources on the CUDA cores in the same CTA.
mb_status run_tc_fwd(const FusedArgs<float>& A, mb_mode mode, int grid, cudaStream_t stream) {
  if (A.na > 64)
    return fail(MB_ERR_UNSUPPORTED, "split-precision modes handle up to 64 antennas (got %d)", A.na);
  // The stage region holds the operand stages during the tensor-core phase,
  // then the extended sources' Jones tile and the FP32 low parts of the pair
  // accumulators.  All regions 128-byte aligned.  The extended sources take
  // 32-source tiles (fewer tile passes and barriers; 35.1 -> 24.6 ms on the
  // 100 x 27 x 64 mixed workload) unless the source-tile option asks
  // otherwise or the layout does not fit, then 16 or 8.
  const size_t row_bytes = mode == MB_MODE_SPLIT_TF32 ? TcGeom<MB_MODE_SPLIT_TF32>::kRowBytes
                                                      : TcGeom<MB_MODE_SPLIT_BF16>::kRowBytes;
  const size_t stage_bytes = size_t(kTcStages) * 2 * 128 * row_bytes;
  SmemPlan S;
  TcPlan P;
  for (int tile = A.src_tile ? A.src_tile : 32;; tile /= 2) {
    S = make_plan<float>(A.na, false, false, tile);
    // The tensor-core kernel runs with kTcThreads threads; its extended-source
    // phase uses the same pair-tile plan with that thread count.
    S.nthreads = kTcThreads;
    S.groups = S.nitems <= kTcThreads ? std::min(8, std::max(1, kTcThreads / S.nitems)) : 1;
    P.group = kTcGroup;
    const size_t jbytes = align_up(size_t(S.jrow) * S.st, 128);
    const size_t vbytes = sizeof(Jones<float>) * S.npairs;
    size_t o = 0;
    auto take = [&o](size_t b) { size_t r = o; o = align_up(o + b, 128); return r; };
    P.off_stage = take(std::max(stage_bytes, jbytes + vbytes));
    P.off_vlo32 = P.off_stage + jbytes;
    S.off_J = P.off_stage;
    S.off_Vlo = P.off_vlo32;
    const int nch = tc_pack(A.na) ? 2 : 1;
    S.off_ant = take(sizeof(AntInfo<float>) * A.na * nch);
    S.off_src = take(sizeof(SrcInfo<float>) * S.st);
    S.off_V = take(vbytes * nch);
    S.off_items = take(sizeof(int) * (S.nitems + 128));
    S.off_red = take(sizeof(double) * 32);
    P.off_bar = take((2 * kTcStages + 3) * sizeof(uint64_t) + 16);
    P.total = o;
    if (P.total <= kMaxDynamicSmem || tile <= 8) break;
  }
  if (P.total > kMaxDynamicSmem)
    return fail(MB_ERR_UNSUPPORTED, "split-precision kernel needs %zu bytes of shared memory for na=%d",
                P.total, A.na);
  if (grid == 0) return MB_OK;
  const bool b = A.bitems != nullptr, pk = tc_pack(A.na);
  auto kern = mode == MB_MODE_SPLIT_TF32
                  ? (b ? (pk ? coh_tc_fwd_kernel<MB_MODE_SPLIT_TF32, true, true>
                             : coh_tc_fwd_kernel<MB_MODE_SPLIT_TF32, true, false>)
                       : (pk ? coh_tc_fwd_kernel<MB_MODE_SPLIT_TF32, false, true>
                             : coh_tc_fwd_kernel<MB_MODE_SPLIT_TF32, false, false>))
                  : (b ? (pk ? coh_tc_fwd_kernel<MB_MODE_SPLIT_BF16, true, true>
                             : coh_tc_fwd_kernel<MB_MODE_SPLIT_BF16, true, false>)
                       : (pk ? coh_tc_fwd_kernel<MB_MODE_SPLIT_BF16, false, true>
                             : coh_tc_fwd_kernel<MB_MODE_SPLIT_BF16, false, false>));
  MB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(P.total)));
  { KernelScope ks_("coh_tc_fwd_kernel", stream); kern<<<grid, kTcThreads, P.total, stream>>>(A, S, P); }
  return check_launch("coh_tc_fwd_kernel");
}

// CUDA-core forward (FP64, plain FP32).
template <typename T>
mb_status run_fwd(const FusedArgs<T>& A, int grid, cudaStream_t stream) {
  constexpr int RP = FwdTile<T>::RP, RQ = FwdTile<T>::RQ;
  SmemPlan S = make_plan<T>(A.na, false, true, A.src_tile);
  if (S.total > kMaxDynamicSmem)
    return fail(MB_ERR_UNSUPPORTED, "fused forward needs %zu bytes of shared memory for na=%d (max 232448)",
                S.total, A.na);
  if (grid == 0) return MB_OK;
  auto kern = A.bitems ? coh_fwd_kernel<T, RP, RQ, true> : coh_fwd_kernel<T, RP, RQ, false>;
  MB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(S.total)));
  { KernelScope ks_("coh_fwd_kernel", stream); kern<<<grid, S.nthreads, S.total, stream>>>(A, S); }
  return check_launch("coh_fwd_kernel");
}

// Split-precision adjoint of the point sources: dJ = Y J on the tensor cores.
mb_status run_tc_adj(const FusedArgs<float>& A, int grid, cudaStream_t stream) {
  if (A.na > 64)
    return fail(MB_ERR_UNSUPPORTED, "split-precision modes handle up to 64 antennas (got %d)", A.na);
  if (grid == 0) return MB_OK;
  TaPlan P;
  size_t o = 0;
  auto take = [&o](size_t bytes) { size_t r = o; o = align_up(o + bytes, 128); return r; };
  P.off_park = take(kTaParkBytes);
  P.off_stage = take(size_t(kTaGroups) * kJopBytes);
  const int nch = tc_pack(A.na) ? 2 : 1;
  P.off_ant = take(sizeof(AntInfo<float>) * A.na * nch);
  P.off_acc = take(sizeof(float) * kTaGroups * 2 * nch * kTaKappa * kTaAcc);
  P.off_src = take(sizeof(TaSrc) * kTaGroups * 2 * nch * kTaKappa);
  P.off_bar = take(2 * kTaGroups * sizeof(uint64_t) + 16);
  P.total = o;
  const bool b = A.bitems != nullptr, pk = tc_pack(A.na);
  auto kern = b ? (pk ? coh_tc_adj_kernel<true, true> : coh_tc_adj_kernel<true, false>)
                : (pk ? coh_tc_adj_kernel<false, true> : coh_tc_adj_kernel<false, false>);
  MB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(P.total)));
  { KernelScope ks_("coh_tc_adj_kernel", stream); kern<<<grid, kTaThreads, P.total, stream>>>(A, P); }
  return check_launch("coh_tc_adj_kernel");
}

// CUDA-core adjoint: all sources from A.sbeg (FP64, plain FP32), or only the
// extended sources of a split-precision call (ext_only: no dchi^2/dJ tile,
// 32-source tiles by default).
template <typename T>
mb_status run_adj(const FusedArgs<T>& A, bool ext_only, int grid, cudaStream_t stream) {
  constexpr int RA = AdjTile<T>::RA, RS = AdjTile<T>::RS;
  SmemPlan S = ext_only ? make_plan<T>(A.na, true, true, A.src_tile ? A.src_tile : 32, false)
                        : make_plan<T>(A.na, true, true, A.src_tile);
  if (S.total > kMaxDynamicSmem)
    return fail(MB_ERR_UNSUPPORTED, "fused adjoint needs %zu bytes of shared memory for na=%d", S.total, A.na);
  if (grid == 0) return MB_OK;
  // Where the shared memory of two CTAs fits an SM, CTAs of half the threads
  // (the registers of one 512-thread CTA): two per SM, so that one computes
  // while the other waits at its tile barriers.
  if (sizeof(T) == 4 && 2 * S.total <= kMaxDynamicSmem) S.nthreads = AdjTile<T>::THREADS / 2;
  auto kern = A.bitems ? coh_adj_kernel<T, RA, RS, true> : coh_adj_kernel<T, RA, RS, false>;
  MB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(S.total)));
  { KernelScope ks_("coh_adj_kernel", stream); kern<<<grid, S.nthreads, S.total, stream>>>(A, S); }
  return check_launch("coh_adj_kernel");
}

template <typename T>
mb_status launch_forward(const FusedArgs<T>& A, mb_mode mode, double* X2, void* ws, const WsLayout& L,
                         cudaStream_t stream) {
  const int units = A.ntime * A.nchan;
  if (A.err) MB_CUDA(cudaMemsetAsync(A.err, 0, sizeof(int), stream));
  if (units == 0) {
    MB_CUDA(cudaMemsetAsync(X2, 0, sizeof(double), stream));
    return MB_OK;
  }
  MB_CHECK(launch_prep(A, ws, L, stream));
  const int nsub = sub_count(A.na);
  // sub-arrays add their dchi^2/dG terms into it
  if (nsub > 1 && A.want_grad && A.dG)
    MB_CUDA(cudaMemsetAsync(A.dG, 0, size_t(A.ntime) * A.na * A.nchan * 8 * sizeof(T), stream));
  // Split forms with extended sources: the CUDA-core forward sums the
  // extended sources first (onto the caller's partial sums, if any) into
  // the workspace's visibility region, and the tensor-core forward adds its
  // point sources to those and finishes (G, flags, chi^2).  The CUDA-core
  // kernel runs several CTAs per SM; inside the tensor-core CTA the same
  // sums ran at a fraction of its speed.
  const bool ext_first = mode != MB_MODE_NATIVE && A.nsrc > A.npsrc && L.vis_ext != L.total;
  T* vis_ext = reinterpret_cast<T*>(static_cast<char*>(ws) + L.vis_ext);
  for (int k = 0; k < nsub; ++k) {
    const FusedArgs<T> Ak = sub_args(A, k, units);
    bool done = false;
    if constexpr (sizeof(T) == 4) {
      if (mode != MB_MODE_NATIVE) {
        FusedArgs<T> At = Ak;
        if (ext_first) {
          FusedArgs<T> Ae = Ak;
          Ae.sbeg = Ak.npsrc;
          Ae.partial_out = true;
          Ae.model_vis = vis_ext;
          Ae.chi2 = nullptr;
          Ae.want_grad = false;
          MB_CHECK(run_fwd(Ae, units, stream));
          At.tc_ext = false;
          At.accumulate_in = true;
          At.vis_in = vis_ext;
        }
        MB_CHECK(run_tc_fwd(At, mode, tc_ctas(At.na, At.ntime, At.nchan), stream));
        done = true;
      }
    }
    if (!done) MB_CHECK(run_fwd(Ak, units, stream));
  }
  {
    KernelScope ks_("sum_partials_kernel", stream);
    sum_partials_kernel<<<1, 1024, 0, stream>>>(A.partial, units * nsub, A.weights ? 1.0 : A.inv_sigma2, X2);
  }
  return check_launch("sum_partials_kernel");
}

// Split-precision adjoint: point sources on the tensor cores, extended
// sources on the CUDA cores (same FP64 accumulators).
mb_status launch_tc_adjoint(const FusedArgs<float>& A, cudaStream_t stream) {
  const int units = A.ntime * A.nchan;
  // the error word is the forward's (cleared there): an adjoint after a
  // forward whose waits gave up does no work and keeps reporting it
  for (int k = 0, nsub = sub_count(A.na); k < nsub; ++k) {
    FusedArgs<float> Ak = sub_args(A, k, units);
    if (Ak.npsrc > 0) MB_CHECK(run_tc_adj(Ak, tc_ctas(Ak.na, Ak.ntime, Ak.nchan), stream));
    if (Ak.nsrc > Ak.npsrc) {
      Ak.sbeg = Ak.npsrc;
      MB_CHECK(run_adj(Ak, true, units, stream));
    }
  }
  return MB_OK;
}

template <typename T>
mb_status launch_adjoint(const FusedArgs<T>& A, mb_mode mode, double grad_scale, const mb_rime_grads* g,
                         void* ws, const WsLayout& L, cudaStream_t stream) {
  char* w = static_cast<char*>(ws);
  MB_CUDA(cudaMemsetAsync(w + L.acc_lm, 0, L.acc_end - L.acc_lm, stream));
  const int units = A.ntime * A.nchan;
  bool done_sources = false;
  if constexpr (sizeof(T) == 4) {
    if (mode != MB_MODE_NATIVE && units > 0 && A.nsrc > 0) {
      MB_CHECK(launch_tc_adjoint(A, stream));
      done_sources = true;
    }
  }
  if (units > 0 && A.nsrc > 0 && !done_sources)
    for (int k = 0, nsub = sub_count(A.na); k < nsub; ++k) MB_CHECK(run_adj(sub_args(A, k, units), false, units, stream));
  size_t total = size_t(A.nsrc) * 2 + size_t(A.nsrc) * A.ntime + 3 * size_t(A.ngsrc) + 3 * size_t(A.nssrc) +
                 size_t(A.ntime) * A.na * A.nchan;
  if (total > 0) {
    int blocks = int(std::min<size_t>((total + 255) / 256, 1u << 16));
    {
      KernelScope ks_("finalize_grads_kernel", stream);
      finalize_grads_kernel<T><<<blocks, 256, 0, stream>>>(A, grad_scale, (T*)g->lm, (T*)g->stokes, (T*)g->alpha,
                                                           (T*)g->gauss_shape, (T*)g->sersic_shape, (T*)g->G_term);
    }
    MB_CHECK(check_launch("finalize_grads_kernel"));
  }
  return MB_OK;
}

// ---------------------------------------------------------------------------
// Batched likelihood (mb_rime_batch)
// ---------------------------------------------------------------------------
// Workspace: the beam plane and error word shared by all sets, the device
// table of BatchSet entries, the (set, unit) item lists of the launches, all
// sets' FP64 gradient accumulators (one contiguous region, cleared by one
// memset), then per set its path-length table, sqrt(B) table (FP32), unit
// partials, d chi^2 / dV and d chi^2 / dG.
// kBatchExtFwd: the extended sources of split-form sets on the CUDA cores,
// into the set's vis_ext, before their tensor-core forward.
enum BatchKind { kBatchExtFwd, kBatchFwd, kBatchTcFwd, kBatchAdj, kBatchTcAdj, kBatchExtAdj };

struct BatchGroup {
  int kind, mode, tile;
  size_t first;  // first item of the group in the item list
  int count;     // items (CTAs)
};

struct SetOffsets {
  size_t phi, bsq0, partial, gV, dG, acc_lm, acc_stokes, acc_alpha, acc_gauss, acc_sersic, vis_ext;
};

struct BatchPlan {
  size_t plane = 0, err = 0, sets = 0, items = 0, acc_begin = 0, acc_end = 0, total = 0;
  size_t max_phi = 0, max_bsq = 0, max_grad = 0;  // largest per-set sizes of the set-grid kernels
  std::vector<SetOffsets> off;
  std::vector<int> order;  // sets by decreasing source count, so the longest CTAs start first
  std::vector<BatchGroup> groups;
  size_t nitems = 0;
};

int tile_of_options(uint32_t o) {
  return (o & MB_SOURCE_TILE_MASK) ? 4 << ((o & MB_SOURCE_TILE_MASK) >> MB_SOURCE_TILE_SHIFT) : 0;
}

mb_status batch_plan(mb_dtype dtype, const mb_dims* d, const mb_batch_set* sets, int nsets, BatchPlan& B) {
  if (dtype != MB_FLOAT32 && dtype != MB_FLOAT64) return fail(MB_ERR_UNSUPPORTED_DTYPE, "dtype %d", int(dtype));
  if (nsets < 0) return fail(MB_ERR_INVALID_ARG, "nsets < 0");
  if (nsets > 0) MB_REQUIRE(sets, "sets");
  if (nsets > 65535) return fail(MB_ERR_UNSUPPORTED, "at most 65535 sets per batch (got %d)", nsets);
  const size_t es = dtype == MB_FLOAT64 ? 8 : 4;
  const size_t nt = ext(d->ntime), na = ext(d->na), nbl = ext(d->nbl), nc = ext(d->nchan);
  const size_t units = nt * nc;
  const size_t tc_units = size_t(tc_ctas(int(na), int(nt), int(nc)));  // CTAs of a tensor-core launch per set
  for (int i = 0; i < nsets; ++i) {
    const mb_batch_set& s = sets[i];
    const uint64_t n = uint64_t(s.npsrc) + s.ngsrc + s.nssrc;
    if (n > 0x7fffffffu) return fail(MB_ERR_INVALID_ARG, "set %d: too many sources", i);
    if (s.mode != MB_MODE_NATIVE && s.mode != MB_MODE_SPLIT_TF32 && s.mode != MB_MODE_SPLIT_BF16)
      return fail(MB_ERR_INVALID_ARG, "set %d: mode %u", i, s.mode);
    if (s.mode != MB_MODE_NATIVE && dtype != MB_FLOAT32)
      return fail(MB_ERR_UNSUPPORTED, "set %d: split-precision modes take FLOAT32 data", i);
    if (na > size_t(kSubMaxNa))
      return fail(MB_ERR_UNSUPPORTED, "batched calls handle up to %d antennas (got %zu)", kSubMaxNa, na);
    if (s.options & ~MB_SOURCE_TILE_MASK)
      return fail(MB_ERR_INVALID_ARG, "set %d: options may only hold source-tile bits (0x%x)", i, s.options);
    if (s.reserved != 0) return fail(MB_ERR_INVALID_ARG, "set %d: reserved must be 0", i);
    if (n > 0) {
      MB_REQUIRE(s.lm, "set lm"); MB_REQUIRE(s.stokes, "set stokes"); MB_REQUIRE(s.alpha, "set alpha");
    }
    if (s.ngsrc > 0) MB_REQUIRE(s.gauss_shape, "set gauss_shape");
    if (s.nssrc > 0) MB_REQUIRE(s.sersic_shape, "set sersic_shape");
  }
  if (units * size_t(nsets) > size_t(0x7fffffff))
    return fail(MB_ERR_UNSUPPORTED, "a batch of %d sets x %zu units exceeds 2^31 CTAs", nsets, units);
  size_t o = 0;
  auto take = [&o](size_t bytes) { size_t r = o; o = align_up(o + bytes, 256); return r; };
  B.plane = take(nc * size_t(d->beam_lw.local_size) * d->beam_mh.local_size * kPlaneVals * es);
  B.err = take(sizeof(int));
  B.sets = take(size_t(nsets) * sizeof(BatchSet<float>));
  B.order.resize(nsets);
  for (int i = 0; i < nsets; ++i) B.order[i] = i;
  auto nsrc_of = [&](int i) { return uint64_t(sets[i].npsrc) + sets[i].ngsrc + sets[i].nssrc; };
  std::stable_sort(B.order.begin(), B.order.end(), [&](int a, int b) { return nsrc_of(a) > nsrc_of(b); });
  // launch groups: forward groups, then adjoint groups, each in first-seen order
  B.groups.clear();
  auto group_of = [&](int kind, int mode, int tile) -> BatchGroup& {
    for (auto& g : B.groups)
      if (g.kind == kind && g.mode == mode && g.tile == tile) return g;
    B.groups.push_back(BatchGroup{kind, mode, tile, 0, 0});
    return B.groups.back();
  };
  for (int pass = 0; pass < 3; ++pass) {
    for (int i : B.order) {
      const mb_batch_set& s = sets[i];
      const int tile = tile_of_options(s.options);
      const bool tc = s.mode != MB_MODE_NATIVE;
      if (pass == 0) {
        if (tc && s.ngsrc + s.nssrc > 0) group_of(kBatchExtFwd, 0, tile).count += int(units);
      } else if (pass == 1) {
        group_of(tc ? kBatchTcFwd : kBatchFwd, tc ? int(s.mode) : 0, tile).count += int(tc ? tc_units : units);
      } else {
        if (tc && s.npsrc > 0) group_of(kBatchTcAdj, 0, 0).count += int(tc_units);
        if (tc && s.ngsrc + s.nssrc > 0) group_of(kBatchExtAdj, 0, tile).count += int(units);
        if (!tc && nsrc_of(i) > 0) group_of(kBatchAdj, 0, tile).count += int(units);
      }
    }
  }
  B.nitems = 0;
  for (auto& g : B.groups) {
    g.first = B.nitems;
    B.nitems += size_t(g.count);
  }
  B.items = take(B.nitems * sizeof(int2));
  B.off.assign(nsets, SetOffsets{});
  B.acc_begin = o;
  for (int i = 0; i < nsets; ++i) {
    const size_t ns = nsrc_of(i);
    SetOffsets& so = B.off[i];
    so.acc_lm = take(ns * 2 * 8);
    so.acc_stokes = take(ns * nt * 4 * 8);
    so.acc_alpha = take(ns * nt * 8);
    so.acc_gauss = take(3 * size_t(sets[i].ngsrc) * 8);
    so.acc_sersic = take(3 * size_t(sets[i].nssrc) * 8);
  }
  B.acc_end = o;
  B.max_phi = B.max_bsq = B.max_grad = 0;
  for (int i = 0; i < nsets; ++i) {
    const size_t ns = nsrc_of(i);
    SetOffsets& so = B.off[i];
    so.phi = take(nt * ns * na * 8);
    so.bsq0 = take(dtype == MB_FLOAT32 ? ns * nt * kBsqVals * es : 0);
    so.partial = take(units * 8);
    so.gV = take(nt * nbl * nc * 8 * es);
    so.dG = take(nt * na * nc * 8 * es);
    const bool ext_first = sets[i].mode != MB_MODE_NATIVE && sets[i].ngsrc + sets[i].nssrc > 0;
    so.vis_ext = ext_first ? take(size_t(d->ntime.local_size) * d->nbl.local_size * d->nchan.local_size * 8 * es)
                           : 0;
    B.max_phi = std::max(B.max_phi, nt * ns * na);
    B.max_bsq = std::max(B.max_bsq, ns * nt);
    B.max_grad = std::max(B.max_grad, ns * 2 + ns * nt + 3 * size_t(sets[i].ngsrc) + 3 * size_t(sets[i].nssrc) +
                                          nt * na * nc);
  }
  B.total = o;
  return MB_OK;
}

// The observation's dims with the sources taken out (the sets bring theirs).
mb_dims batch_obs_dims(const mb_dims* d) {
  mb_dims o = *d;
  const mb_dim none = {0, 0, 0, 0};
  o.nsrc = o.npsrc = o.ngsrc = o.nssrc = none;
  return o;
}

template <typename T>
mb_status batch_prepare(const mb_dims* d, const mb_batch_set* sets, int nsets, void* ws, const BatchPlan& B,
                        cudaStream_t stream) {
  char* w = static_cast<char*>(ws);
  const int units = int(ext(d->ntime) * ext(d->nchan));
  const int tc_units = tc_ctas(int(ext(d->na)), int(ext(d->ntime)), int(ext(d->nchan)));
  std::vector<BatchSet<T>> bs(nsets);
  for (int i = 0; i < nsets; ++i) {
    const mb_batch_set& s = sets[i];
    const SetOffsets& so = B.off[i];
    BatchSet<T>& b = bs[i];
    b.lm = static_cast<const T*>(s.lm); b.stokes = static_cast<const T*>(s.stokes);
    b.alpha = static_cast<const T*>(s.alpha); b.gauss = static_cast<const T*>(s.gauss_shape);
    b.sersic = static_cast<const T*>(s.sersic_shape);
    b.phi = reinterpret_cast<const double*>(w + so.phi);
    b.bsq0 = sizeof(T) == 4 ? reinterpret_cast<const T*>(w + so.bsq0) : nullptr;
    b.partial = reinterpret_cast<double*>(w + so.partial);
    b.gV = reinterpret_cast<T*>(w + so.gV);
    b.dG = reinterpret_cast<T*>(w + so.dG);
    b.acc_lm = reinterpret_cast<double*>(w + so.acc_lm);
    b.acc_stokes = reinterpret_cast<double*>(w + so.acc_stokes);
    b.acc_alpha = reinterpret_cast<double*>(w + so.acc_alpha);
    b.acc_gauss = reinterpret_cast<double*>(w + so.acc_gauss);
    b.acc_sersic = reinterpret_cast<double*>(w + so.acc_sersic);
    b.g_lm = static_cast<T*>(s.grads.lm); b.g_stokes = static_cast<T*>(s.grads.stokes);
    b.g_alpha = static_cast<T*>(s.grads.alpha); b.g_gauss = static_cast<T*>(s.grads.gauss_shape);
    b.g_sersic = static_cast<T*>(s.grads.sersic_shape); b.g_G = static_cast<T*>(s.grads.G_term);
    const bool ext_first = s.mode != MB_MODE_NATIVE && s.ngsrc + s.nssrc > 0;
    b.vis_ext = ext_first ? reinterpret_cast<T*>(w + so.vis_ext) : nullptr;
    b.npsrc = int(s.npsrc); b.ngsrc = int(s.ngsrc); b.nssrc = int(s.nssrc); b.pad = 0;
  }
  std::vector<int2> items(B.nitems);
  for (const BatchGroup& g : B.groups) {
    size_t k = g.first;
    for (int i : B.order) {
      const mb_batch_set& s = sets[i];
      const bool tc = s.mode != MB_MODE_NATIVE;
      const int tile = tile_of_options(s.options);
      const uint64_t n = uint64_t(s.npsrc) + s.ngsrc + s.nssrc;
      bool in = false;
      switch (g.kind) {
        case kBatchExtFwd: in = tc && s.ngsrc + s.nssrc > 0 && g.tile == tile; break;
        case kBatchFwd: in = !tc && g.tile == tile; break;
        case kBatchTcFwd: in = tc && g.mode == int(s.mode) && g.tile == tile; break;
        case kBatchTcAdj: in = tc && s.npsrc > 0; break;
        case kBatchExtAdj: in = tc && s.ngsrc + s.nssrc > 0 && g.tile == tile; break;
        case kBatchAdj: in = !tc && n > 0 && g.tile == tile; break;
      }
      if (!in) continue;
      // the tensor-core kernels' CTAs may cover two channels each
      const int nu = (g.kind == kBatchTcFwd || g.kind == kBatchTcAdj) ? tc_units : units;
      for (int u = 0; u < nu; ++u) items[k++] = make_int2(i, u);
    }
    if (k != g.first + size_t(g.count)) return fail(MB_ERR_INVALID_ARG, "batch plan: item count mismatch");
  }
  if (nsets > 0)
    MB_CUDA(cudaMemcpyAsync(w + B.sets, bs.data(), sizeof(BatchSet<T>) * nsets, cudaMemcpyHostToDevice, stream));
  if (!items.empty())
    MB_CUDA(cudaMemcpyAsync(w + B.items, items.data(), sizeof(int2) * items.size(), cudaMemcpyHostToDevice, stream));
  MB_CUDA(cudaStreamSynchronize(stream));
  return MB_OK;
}

template <typename T>
mb_status batch_run(const mb_dims* d, const mb_props* P, uint32_t options, const mb_rime_inputs* in, int nsets,
                    double* X2, double grad_scale, void* ws, const BatchPlan& B, cudaStream_t stream) {
  char* w = static_cast<char*>(ws);
  const mb_dims od = batch_obs_dims(d);
  WsLayout unused{};
  FusedArgs<T> A;
  fill_args(A, &od, P, options, in, nullptr, nullptr, true, nullptr, unused);
  A.plane = reinterpret_cast<const T*>(w + B.plane);
  A.err = reinterpret_cast<int*>(w + B.err);
  A.bsets = reinterpret_cast<const BatchSet<T>*>(w + B.sets);
  const int2* items = reinterpret_cast<const int2*>(w + B.items);
  const int units = A.ntime * A.nchan;
  MB_CUDA(cudaMemsetAsync(A.err, 0, sizeof(int), stream));
  if (B.acc_end > B.acc_begin) MB_CUDA(cudaMemsetAsync(w + B.acc_begin, 0, B.acc_end - B.acc_begin, stream));
  if (nsets == 0) return MB_OK;
  auto blocks_for = [](size_t n) { return unsigned(std::max<size_t>(1, std::min<size_t>((n + 255) / 256, 4096))); };
  // shared beam plane, then the per-set tables (grid.y = set)
  size_t n = size_t(A.nchan) * A.lw * A.mh;
  if (n > 0) {
    { KernelScope ks_("beam_plane_kernel", stream);
      beam_plane_kernel<T><<<blocks_for(n), 256, 0, stream>>>(A, const_cast<T*>(A.plane)); }
    MB_CHECK(check_launch("beam_plane_kernel"));
  }
  if (B.max_phi > 0) {
    { KernelScope ks_("phi_kernel", stream);
      phi_kernel<T><<<dim3(blocks_for(B.max_phi), nsets), 256, 0, stream>>>(A, nullptr); }
    MB_CHECK(check_launch("phi_kernel"));
  }
  if (sizeof(T) == 4 && B.max_bsq > 0) {
    { KernelScope ks_("bsqrt_ref_kernel", stream);
      bsqrt_ref_kernel<T><<<dim3(blocks_for(B.max_bsq), nsets), 256, 0, stream>>>(A, nullptr); }
    MB_CHECK(check_launch("bsqrt_ref_kernel"));
  }
  // forward: one launch per (form, source tile) over all its sets' units;
  // first the split-form sets' extended sources on the CUDA cores, which the
  // tensor-core launch then adds its point sources to
  for (const BatchGroup& g : B.groups) {
    if (g.kind != kBatchExtFwd && g.kind != kBatchFwd && g.kind != kBatchTcFwd) continue;
    FusedArgs<T> Ag = A;
    Ag.src_tile = g.tile;
    Ag.bitems = items + g.first;
    if constexpr (sizeof(T) == 4) {
      if (g.kind == kBatchTcFwd) {
        Ag.tc_ext = false;
        Ag.accumulate_in = true;  // the set's vis_ext where it has one
        MB_CHECK(run_tc_fwd(Ag, mb_mode(g.mode), g.count, stream));
        continue;
      }
    }
    if (g.kind == kBatchExtFwd) {
      Ag.sbeg = -1;  // each set's extended sources
      Ag.partial_out = true;  // into the set's vis_ext
      Ag.chi2 = nullptr;
      Ag.want_grad = false;
      MB_CHECK(run_fwd(Ag, g.count, stream));
    } else if (g.kind == kBatchFwd) {
      MB_CHECK(run_fwd(Ag, g.count, stream));
    }
  }
  if (units > 0) {
    { KernelScope ks_("sum_partials_kernel", stream);
      sum_partials_sets_kernel<T><<<nsets, 256, 0, stream>>>(A.bsets, units, A.weights ? 1.0 : A.inv_sigma2, X2); }
    MB_CHECK(check_launch("sum_partials_sets_kernel"));
  } else {
    MB_CUDA(cudaMemsetAsync(X2, 0, sizeof(double) * nsets, stream));
  }
  // adjoint: point sources on the tensor cores, extended sources of those
  // sets, CUDA-core sets
  for (const BatchGroup& g : B.groups) {
    if (g.kind == kBatchExtFwd || g.kind == kBatchFwd || g.kind == kBatchTcFwd) continue;
    FusedArgs<T> Ag = A;
    Ag.src_tile = g.tile;
    Ag.bitems = items + g.first;
    if constexpr (sizeof(T) == 4) {
      if (g.kind == kBatchTcAdj) {
        MB_CHECK(run_tc_adj(Ag, g.count, stream));
        continue;
      }
    }
    if (g.kind == kBatchExtAdj) {
      Ag.sbeg = -1;  // each set's extended sources
      MB_CHECK(run_adj(Ag, true, g.count, stream));
    } else if (g.kind == kBatchAdj) {
      MB_CHECK(run_adj(Ag, false, g.count, stream));
    }
  }
  if (B.max_grad > 0) {
    { KernelScope ks_("finalize_grads_kernel", stream);
      finalize_grads_kernel<T><<<dim3(blocks_for(B.max_grad), nsets), 256, 0, stream>>>(
          A, grad_scale, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr); }
    MB_CHECK(check_launch("finalize_grads_kernel"));
  }
  return MB_OK;
}

}  // namespace

size_t fused_workspace_size(mb_dtype dtype, mb_mode mode, const mb_dims* d, bool want_grad) {
  return ws_layout(dtype, mode, d, want_grad).total;
}

// ---------------------------------------------------------------------------
// Allocation-free forward (mb_rime_forward_noalloc)
// ---------------------------------------------------------------------------
// Its only scratch, one FP64 chi^2 partial per (time, channel) unit, lives in
// this file-scope device array.  Every GPU that loads the library holds the
// array (1 MiB) until the process exits.  All calls share it: calls whose
// kernels overlap on the GPU (different streams, no ordering between them)
// race on it.  Every slot a call reads is written by the same call first, so
// nothing needs clearing between calls.
constexpr size_t kNoallocMaxUnits = 131072;
static __device__ __align__(256) double g_noalloc_partials[kNoallocMaxUnits];

constexpr int kMaxDevices = 256;
static std::mutex g_noalloc_mutex;
static double* g_noalloc_ptr[kMaxDevices] = {};

// Device address of g_noalloc_partials on the current device.  In host code
// the symbol names a host-side stand-in, so the address is looked up with
// cudaGetSymbolAddress (with the device current).  Outside stream capture it
// is looked up on every call (cheap, and still right after a
// cudaDeviceReset reloaded the module); during capture the address of the
// last uncaptured call on the device is used.
mb_status noalloc_scratch(double** out, cudaStream_t stream) {
  int dev = 0;
  MB_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(MB_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  MB_CUDA(cudaStreamIsCapturing(stream, &cap));
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (cap == cudaStreamCaptureStatusNone || g_noalloc_ptr[dev] == nullptr) {
    if (cap != cudaStreamCaptureStatusNone)
      return fail(MB_ERR_INVALID_ARG, "mb_rime_forward_noalloc: call it once on this device before stream capture");
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
    if (e != cudaSuccess)
      return fail(MB_ERR_CUDA, "cudaGetSymbolAddress(g_noalloc_partials): %s", cudaGetErrorString(e));
    g_noalloc_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_noalloc_ptr[dev];
  return MB_OK;
}

namespace {
template <typename T>
mb_status launch_forward_noalloc(FusedArgs<T> A, double* partials, double* X2, cudaStream_t stream) {
  A.phi = nullptr;  // path lengths formed in the kernel instead of a table
  A.partial = partials;
  A.want_grad = false;
  const int units = A.ntime * A.nchan;
  if (units == 0) {
    {
      KernelScope ks_("sum_partials_kernel", stream);
      sum_partials_kernel<<<1, 1024, 0, stream>>>(partials, 0, 1.0, X2);
    }
    return check_launch("sum_partials_kernel");
  }
  constexpr int RP = FwdTile<T>::RP, RQ = FwdTile<T>::RQ;
  SmemPlan S = make_plan<T>(A.na, false, true, A.src_tile);
  if (S.total > kMaxDynamicSmem)
    return fail(MB_ERR_UNSUPPORTED, "fused forward needs %zu bytes of shared memory for na=%d (max 232448)",
                S.total, A.na);
  auto kern = coh_fwd_kernel<T, RP, RQ, false>;
  MB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(S.total)));
  { KernelScope ks_("coh_fwd_kernel", stream); kern<<<units, S.nthreads, S.total, stream>>>(A, S); }
  MB_CHECK(check_launch("coh_fwd_kernel"));
  {
    KernelScope ks_("sum_partials_kernel", stream);
    sum_partials_kernel<<<1, 1024, 0, stream>>>(partials, units, A.weights ? 1.0 : A.inv_sigma2, X2);
  }
  return check_launch("sum_partials_kernel");
}
}  // namespace

}  // namespace mb

using namespace mb;

extern "C" {

size_t mb_rime_workspace_size(mb_dtype dtype, mb_mode mode, const mb_dims* dims, int want_grad) {
  if (check_dims(dims, true) != MB_OK) return 0;
  return fused_workspace_size(dtype, mode, dims, want_grad != 0);
}

mb_status mb_rime_forward(mb_dtype dtype, mb_mode mode, const mb_dims* dims, const mb_props* props,
                          uint32_t options, const mb_rime_inputs* in, void* model_vis, void* chi_sqrd_result,
                          double* X2, int want_grad, void* workspace, size_t workspace_bytes, void* stream) {
  MB_CHECK(check_inputs(dims, props, options, in, model_vis));
  MB_REQUIRE(X2, "X2");
  if (dtype != MB_FLOAT32 && dtype != MB_FLOAT64) return fail(MB_ERR_UNSUPPORTED_DTYPE, "dtype %d", int(dtype));
  if (mode != MB_MODE_NATIVE && mode != MB_MODE_SPLIT_TF32 && mode != MB_MODE_SPLIT_BF16)
    return fail(MB_ERR_INVALID_ARG, "mode %d", int(mode));
  if (mode != MB_MODE_NATIVE && dtype != MB_FLOAT32)
    return fail(MB_ERR_UNSUPPORTED, "split-precision modes take FLOAT32 data");
  const bool grad = want_grad != 0;
  if (grad && dims->nsrc.upper_extent < dims->nsrc.global_size)
    return fail(MB_ERR_INVALID_ARG, "gradients need the last source batch (upper_extent == global_size)");
  WsLayout L = ws_layout(dtype, mode, dims, grad);
  if (workspace == nullptr || workspace_bytes < L.total || (reinterpret_cast<uintptr_t>(workspace) & 255))
    return fail(MB_ERR_WORKSPACE, "workspace must be >= %zu bytes and 256-byte aligned (got %zu)", L.total,
                workspace_bytes);
  cudaStream_t s = as_stream(stream);
  if (dtype == MB_FLOAT32) {
    FusedArgs<float> A;
    fill_args(A, dims, props, options, in, model_vis, chi_sqrd_result, grad, workspace, L);
    return launch_forward(A, mode, X2, workspace, L, s);
  }
  FusedArgs<double> A;
  fill_args(A, dims, props, options, in, model_vis, chi_sqrd_result, grad, workspace, L);
  return launch_forward(A, mode, X2, workspace, L, s);
}

mb_status mb_rime_adjoint(mb_dtype dtype, mb_mode mode, const mb_dims* dims, const mb_props* props,
                          uint32_t options, const mb_rime_inputs* in, double grad_scale, const mb_rime_grads* grads,
                          void* workspace, size_t workspace_bytes, void* stream) {
  MB_CHECK(check_inputs(dims, props, options, in, nullptr));
  MB_REQUIRE(grads, "grads");
  if (dtype != MB_FLOAT32 && dtype != MB_FLOAT64) return fail(MB_ERR_UNSUPPORTED_DTYPE, "dtype %d", int(dtype));
  if (dims->nsrc.lower_extent > 0 || dims->nsrc.upper_extent < dims->nsrc.global_size)
    return fail(MB_ERR_INVALID_ARG, "the adjoint takes the whole source set in one call");
  WsLayout L = ws_layout(dtype, mode, dims, true);
  if (workspace == nullptr || workspace_bytes < L.total || (reinterpret_cast<uintptr_t>(workspace) & 255))
    return fail(MB_ERR_WORKSPACE, "workspace must be >= %zu bytes and 256-byte aligned (got %zu)", L.total,
                workspace_bytes);
  cudaStream_t s = as_stream(stream);
  if (dtype == MB_FLOAT32) {
    FusedArgs<float> A;
    fill_args(A, dims, props, options, in, nullptr, nullptr, true, workspace, L);
    return launch_adjoint(A, mode, grad_scale, grads, workspace, L, s);
  }
  FusedArgs<double> A;
  fill_args(A, dims, props, options, in, nullptr, nullptr, true, workspace, L);
  return launch_adjoint(A, mode, grad_scale, grads, workspace, L, s);
}

mb_status mb_rime_status(mb_dtype dtype, mb_mode mode, const mb_dims* dims, int want_grad, const void* workspace,
                         size_t workspace_bytes, void* stream) {
  MB_CHECK(check_dims(dims, true));
  if (dtype != MB_FLOAT32 && dtype != MB_FLOAT64) return fail(MB_ERR_UNSUPPORTED_DTYPE, "dtype %d", int(dtype));
  WsLayout L = ws_layout(dtype, mode, dims, want_grad != 0);
  if (workspace == nullptr || workspace_bytes < L.total || (reinterpret_cast<uintptr_t>(workspace) & 255))
    return fail(MB_ERR_WORKSPACE, "workspace must be >= %zu bytes and 256-byte aligned (got %zu)", L.total,
                workspace_bytes);
  cudaStream_t s = as_stream(stream);
  int word = 0;
  MB_CUDA(cudaMemcpyAsync(&word, static_cast<const char*>(workspace) + L.err, sizeof(int), cudaMemcpyDeviceToHost,
                          s));
  MB_CUDA(cudaStreamSynchronize(s));
  if (word == int(MB_ERR_TIMEOUT))
    return fail(MB_ERR_TIMEOUT,
                "a bounded wait of the tensor-core kernels gave up: chi^2, model visibilities and gradients of "
                "this call are invalid");
  if (word != 0) return fail(MB_ERR_CUDA, "unexpected device error word %d", word);
  return MB_OK;
}

mb_status mb_set_wait_limit(uint32_t polls) {
  MB_CUDA(cudaMemcpyToSymbol(g_pipe_wait_limit, &polls, sizeof(polls)));
  return MB_OK;
}

uint32_t mb_default_wait_limit(void) { return 1u << 20; }

}  // extern "C"

extern "C" {

size_t mb_rime_noalloc_max_units(void) { return kNoallocMaxUnits; }

mb_status mb_rime_forward_noalloc(mb_dtype dtype, const mb_dims* dims, const mb_props* props, uint32_t options,
                                  const mb_rime_inputs* in, void* model_vis, void* chi_sqrd_result, double* X2,
                                  void* stream) {
  MB_CHECK(check_inputs(dims, props, options, in, model_vis));
  MB_REQUIRE(X2, "X2");
  if (dtype != MB_FLOAT32 && dtype != MB_FLOAT64) return fail(MB_ERR_UNSUPPORTED_DTYPE, "dtype %d", int(dtype));
  const size_t units = size_t(ext(dims->ntime)) * ext(dims->nchan);
  if (units > kNoallocMaxUnits)
    return fail(MB_ERR_UNSUPPORTED,
                "mb_rime_forward_noalloc handles at most %zu (time, channel) units (got %zu = %u x %u); "
                "split the call over time or use mb_rime_forward with a workspace",
                kNoallocMaxUnits, units, ext(dims->ntime), ext(dims->nchan));
  cudaStream_t s = as_stream(stream);
  double* partials = nullptr;
  MB_CHECK(noalloc_scratch(&partials, s));
  WsLayout L = ws_layout(dtype, MB_MODE_NATIVE, dims, false);
  if (dtype == MB_FLOAT32) {
    FusedArgs<float> A;
    fill_args(A, dims, props, options, in, model_vis, chi_sqrd_result, false, nullptr, L);
    return launch_forward_noalloc(A, partials, X2, s);
  }
  FusedArgs<double> A;
  fill_args(A, dims, props, options, in, model_vis, chi_sqrd_result, false, nullptr, L);
  return launch_forward_noalloc(A, partials, X2, s);
}

}  // extern "C"

extern "C" {

size_t mb_rime_batch_workspace_size(mb_dtype dtype, const mb_dims* dims, const mb_batch_set* sets, int nsets) {
  if (check_dims(dims, true) != MB_OK) return 0;
  BatchPlan B;
  if (batch_plan(dtype, dims, sets, nsets, B) != MB_OK) return 0;
  return B.total;
}

mb_status mb_rime_batch_prepare(mb_dtype dtype, const mb_dims* dims, const mb_batch_set* sets, int nsets,
                                void* workspace, size_t workspace_bytes, void* stream) {
  MB_CHECK(check_dims(dims, true));
  BatchPlan B;
  MB_CHECK(batch_plan(dtype, dims, sets, nsets, B));
  if (workspace == nullptr || workspace_bytes < B.total || (reinterpret_cast<uintptr_t>(workspace) & 255))
    return fail(MB_ERR_WORKSPACE, "workspace must be >= %zu bytes and 256-byte aligned (got %zu)", B.total,
                workspace_bytes);
  cudaStream_t s = as_stream(stream);
  if (dtype == MB_FLOAT32) return batch_prepare<float>(dims, sets, nsets, workspace, B, s);
  return batch_prepare<double>(dims, sets, nsets, workspace, B, s);
}

mb_status mb_rime_batch(mb_dtype dtype, const mb_dims* dims, const mb_props* props, uint32_t options,
                        const mb_rime_inputs* shared, const mb_batch_set* sets, int nsets, double* X2,
                        double grad_scale, void* workspace, size_t workspace_bytes, void* stream) {
  MB_CHECK(check_dims(dims, true));
  MB_REQUIRE(props, "props"); MB_REQUIRE(shared, "shared inputs");
  // the observation's inputs, with a stand-in for the per-set source arrays
  mb_rime_inputs in = *shared;
  const mb_dims od = batch_obs_dims(dims);
  static const double dummy[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  in.lm = in.stokes = in.alpha = dummy;
  in.gauss_shape = in.sersic_shape = nullptr;
  if (options & MB_SOURCE_TILE_MASK)
    return fail(MB_ERR_INVALID_ARG, "source tiles are chosen per set (mb_batch_set.options)");
  MB_CHECK(check_inputs(&od, props, options, &in, nullptr));
  if (nsets > 0) MB_REQUIRE(X2, "X2");
  BatchPlan B;
  MB_CHECK(batch_plan(dtype, dims, sets, nsets, B));
  if (workspace == nullptr || workspace_bytes < B.total || (reinterpret_cast<uintptr_t>(workspace) & 255))
    return fail(MB_ERR_WORKSPACE, "workspace must be >= %zu bytes and 256-byte aligned (got %zu)", B.total,
                workspace_bytes);
  cudaStream_t s = as_stream(stream);
  if (dtype == MB_FLOAT32) return batch_run<float>(dims, props, options, shared, nsets, X2, grad_scale, workspace, B, s);
  return batch_run<double>(dims, props, options, shared, nsets, X2, grad_scale, workspace, B, s);
}

}  // extern "C"
