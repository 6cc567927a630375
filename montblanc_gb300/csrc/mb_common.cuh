// Device-side building blocks shared by the stage kernels and the fused
// kernels: complex / 2x2 Jones arithmetic and the per-(source, time,
// antenna, channel) terms of the RIME v4 measurement equation.
//
// Conventions (identical to the reference's v4 arrays,
// montblanc/impl/rime/v4/config.py:131-247): C order, complex values
// interleaved (re, im), 2x2 Jones matrices stored row-major as
// [00, 01, 10, 11] (XX, XY, YX, YY for visibilities).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/montblanc_gb300.h"

namespace mb {

constexpr double kLightSpeed = 299792458.0;  // montblanc/__init__.py:52-59
constexpr double kPi = 3.141592653589793238462643383279502884;

template <typename T> struct Vec2;
template <> struct Vec2<float> { using type = float2; };
template <> struct Vec2<double> { using type = double2; };

template <typename T>
struct Cx {
  T r, i;
};

template <typename T> __host__ __device__ __forceinline__ Cx<T> cx(T r, T i) { return Cx<T>{r, i}; }
template <typename T> __device__ __forceinline__ Cx<T> operator+(Cx<T> a, Cx<T> b) { return {a.r + b.r, a.i + b.i}; }
template <typename T> __device__ __forceinline__ Cx<T> operator-(Cx<T> a, Cx<T> b) { return {a.r - b.r, a.i - b.i}; }
template <typename T> __device__ __forceinline__ Cx<T> operator*(Cx<T> a, T s) { return {a.r * s, a.i * s}; }
template <typename T> __device__ __forceinline__ Cx<T> conj(Cx<T> a) { return {a.r, -a.i}; }
// a * b
template <typename T> __device__ __forceinline__ Cx<T> cmul(Cx<T> a, Cx<T> b) {
  return {a.r * b.r - a.i * b.i, a.r * b.i + a.i * b.r};
}
// a * conj(b)
template <typename T> __device__ __forceinline__ Cx<T> cmulc(Cx<T> a, Cx<T> b) {
  return {a.r * b.r + a.i * b.i, a.i * b.r - a.r * b.i};
}
// acc += a * b
template <typename T> __device__ __forceinline__ void cmac(Cx<T>& acc, Cx<T> a, Cx<T> b) {
  acc.r = fma(a.r, b.r, fma(-a.i, b.i, acc.r));
  acc.i = fma(a.r, b.i, fma(a.i, b.r, acc.i));
}
// acc += a * conj(b)
template <typename T> __device__ __forceinline__ void cmacc(Cx<T>& acc, Cx<T> a, Cx<T> b) {
  acc.r = fma(a.r, b.r, fma(a.i, b.i, acc.r));
  acc.i = fma(a.i, b.r, fma(-a.r, b.i, acc.i));
}
// Re(conj(a) * b)
template <typename T> __device__ __forceinline__ T cdot_re(Cx<T> a, Cx<T> b) { return a.r * b.r + a.i * b.i; }

// FP32: a complex value is an FP32x2 pair (re, im) for the packed FMAs of
// sm_100 and later (each lane rounded as fmaf).  An operand may be a
// broadcast scalar, the swapped pair or have one lane negated at no extra
// instruction, so a complex product or multiply-add is 2 instructions
// instead of 4.
__device__ __forceinline__ float2 as_f2(Cx<float> z) { return make_float2(z.r, z.i); }
__device__ __forceinline__ Cx<float> as_cx(float2 v) { return {v.x, v.y}; }
// (a.r b.r - a.i b.i, a.i b.r + a.r b.i)
template <> __device__ __forceinline__ Cx<float> cmul<float>(Cx<float> a, Cx<float> b) {
  const float2 p = __fmul2_rn(as_f2(a), make_float2(b.r, b.r));
  return as_cx(__ffma2_rn(make_float2(a.i, a.r), make_float2(-b.i, b.i), p));
}
// (a.r b.r + a.i b.i, a.i b.r - a.r b.i)
template <> __device__ __forceinline__ Cx<float> cmulc<float>(Cx<float> a, Cx<float> b) {
  const float2 p = __fmul2_rn(as_f2(a), make_float2(b.r, b.r));
  return as_cx(__ffma2_rn(make_float2(a.i, a.r), make_float2(b.i, -b.i), p));
}
template <> __device__ __forceinline__ void cmac<float>(Cx<float>& acc, Cx<float> a, Cx<float> b) {
  float2 p = __ffma2_rn(make_float2(a.i, a.r), make_float2(-b.i, b.i), as_f2(acc));
  acc = as_cx(__ffma2_rn(as_f2(a), make_float2(b.r, b.r), p));
}
template <> __device__ __forceinline__ void cmacc<float>(Cx<float>& acc, Cx<float> a, Cx<float> b) {
  float2 p = __ffma2_rn(make_float2(a.i, a.r), make_float2(b.i, -b.i), as_f2(acc));
  acc = as_cx(__ffma2_rn(as_f2(a), make_float2(b.r, b.r), p));
}

// 2x2 complex Jones matrix, row-major [00, 01, 10, 11].
template <typename T>
struct Jones {
  Cx<T> a, b, c, d;
};

template <typename T> __device__ __forceinline__ Jones<T> jzero() {
  Jones<T> z;
  z.a = z.b = z.c = z.d = Cx<T>{T(0), T(0)};
  return z;
}
template <typename T> __device__ __forceinline__ Jones<T> jadd(const Jones<T>& x, const Jones<T>& y) {
  return {x.a + y.a, x.b + y.b, x.c + y.c, x.d + y.d};
}
template <typename T> __device__ __forceinline__ Jones<T> jscale(const Jones<T>& x, T s) {
  return {x.a * s, x.b * s, x.c * s, x.d * s};
}
template <> __device__ __forceinline__ Jones<float> jscale<float>(const Jones<float>& x, float s) {
  const float2 ss = make_float2(s, s);
  return {as_cx(__fmul2_rn(as_f2(x.a), ss)), as_cx(__fmul2_rn(as_f2(x.b), ss)), as_cx(__fmul2_rn(as_f2(x.c), ss)),
          as_cx(__fmul2_rn(as_f2(x.d), ss))};
}
// acc += x s
template <typename T> __device__ __forceinline__ void jaxpy(Jones<T>& acc, const Jones<T>& x, T s) {
  acc = jadd(acc, jscale(x, s));
}
template <> __device__ __forceinline__ void jaxpy<float>(Jones<float>& acc, const Jones<float>& x, float s) {
  const float2 ss = make_float2(s, s);
  acc.a = as_cx(__ffma2_rn(as_f2(x.a), ss, as_f2(acc.a)));
  acc.b = as_cx(__ffma2_rn(as_f2(x.b), ss, as_f2(acc.b)));
  acc.c = as_cx(__ffma2_rn(as_f2(x.c), ss, as_f2(acc.c)));
  acc.d = as_cx(__ffma2_rn(as_f2(x.d), ss, as_f2(acc.d)));
}
// X * Y
template <typename T> __device__ __forceinline__ Jones<T> jmul(const Jones<T>& X, const Jones<T>& Y) {
  Jones<T> R;
  R.a = cmul(X.a, Y.a); cmac(R.a, X.b, Y.c);
  R.b = cmul(X.a, Y.b); cmac(R.b, X.b, Y.d);
  R.c = cmul(X.c, Y.a); cmac(R.c, X.d, Y.c);
  R.d = cmul(X.c, Y.b); cmac(R.d, X.d, Y.d);
  return R;
}
// X * Y^H
template <typename T> __device__ __forceinline__ Jones<T> jmulh(const Jones<T>& X, const Jones<T>& Y) {
  Jones<T> R;
  R.a = cmulc(X.a, Y.a); cmacc(R.a, X.b, Y.b);
  R.b = cmulc(X.a, Y.c); cmacc(R.b, X.b, Y.d);
  R.c = cmulc(X.c, Y.a); cmacc(R.c, X.d, Y.b);
  R.d = cmulc(X.c, Y.c); cmacc(R.d, X.d, Y.d);
  return R;
}
// X^H * Y
template <typename T> __device__ __forceinline__ Jones<T> jhmul(const Jones<T>& X, const Jones<T>& Y) {
  Jones<T> R;
  // (X^H)_{ij} = conj(X_{ji})
  R.a = cmul(conj(X.a), Y.a); cmac(R.a, conj(X.c), Y.c);
  R.b = cmul(conj(X.a), Y.b); cmac(R.b, conj(X.c), Y.d);
  R.c = cmul(conj(X.b), Y.a); cmac(R.c, conj(X.d), Y.c);
  R.d = cmul(conj(X.b), Y.b); cmac(R.d, conj(X.d), Y.d);
  return R;
}
// acc += X * Y^H
template <typename T> __device__ __forceinline__ void jmac_h(Jones<T>& acc, const Jones<T>& X, const Jones<T>& Y) {
  cmacc(acc.a, X.a, Y.a); cmacc(acc.a, X.b, Y.b);
  cmacc(acc.b, X.a, Y.c); cmacc(acc.b, X.b, Y.d);
  cmacc(acc.c, X.c, Y.a); cmacc(acc.c, X.d, Y.b);
  cmacc(acc.d, X.c, Y.c); cmacc(acc.d, X.d, Y.d);
}
// acc += X * Y
template <typename T> __device__ __forceinline__ void jmac(Jones<T>& acc, const Jones<T>& X, const Jones<T>& Y) {
  cmac(acc.a, X.a, Y.a); cmac(acc.a, X.b, Y.c);
  cmac(acc.b, X.a, Y.b); cmac(acc.b, X.b, Y.d);
  cmac(acc.c, X.c, Y.a); cmac(acc.c, X.d, Y.c);
  cmac(acc.d, X.c, Y.b); cmac(acc.d, X.d, Y.d);
}
// X^H
template <typename T> __device__ __forceinline__ Jones<T> jherm(const Jones<T>& X) {
  return {conj(X.a), conj(X.c), conj(X.b), conj(X.d)};
}
// Re <X, Y> = Re sum_ij conj(X_ij) Y_ij
template <typename T> __device__ __forceinline__ T jdot_re(const Jones<T>& X, const Jones<T>& Y) {
  return cdot_re(X.a, Y.a) + cdot_re(X.b, Y.b) + cdot_re(X.c, Y.c) + cdot_re(X.d, Y.d);
}
template <> __device__ __forceinline__ float jdot_re<float>(const Jones<float>& X, const Jones<float>& Y) {
  float2 p = __fmul2_rn(as_f2(X.a), as_f2(Y.a));
  p = __ffma2_rn(as_f2(X.b), as_f2(Y.b), p);
  p = __ffma2_rn(as_f2(X.c), as_f2(Y.c), p);
  p = __ffma2_rn(as_f2(X.d), as_f2(Y.d), p);
  return p.x + p.y;
}

// ---- loads / stores of interleaved complex Jones -------------------------
template <typename T> __device__ __forceinline__ Jones<T> jload(const T* p);
template <> __device__ __forceinline__ Jones<float> jload<float>(const float* p) {
  float4 u = *reinterpret_cast<const float4*>(p);
  float4 v = *reinterpret_cast<const float4*>(p + 4);
  return {{u.x, u.y}, {u.z, u.w}, {v.x, v.y}, {v.z, v.w}};
}
template <> __device__ __forceinline__ Jones<double> jload<double>(const double* p) {
  double2 u = *reinterpret_cast<const double2*>(p);
  double2 v = *reinterpret_cast<const double2*>(p + 2);
  double2 w = *reinterpret_cast<const double2*>(p + 4);
  double2 x = *reinterpret_cast<const double2*>(p + 6);
  return {{u.x, u.y}, {v.x, v.y}, {w.x, w.y}, {x.x, x.y}};
}
template <typename T> __device__ __forceinline__ Jones<T> jldg(const T* p);
template <> __device__ __forceinline__ Jones<float> jldg<float>(const float* p) {
  float4 u = __ldg(reinterpret_cast<const float4*>(p));
  float4 v = __ldg(reinterpret_cast<const float4*>(p + 4));
  return {{u.x, u.y}, {u.z, u.w}, {v.x, v.y}, {v.z, v.w}};
}
template <> __device__ __forceinline__ Jones<double> jldg<double>(const double* p) {
  double2 u = __ldg(reinterpret_cast<const double2*>(p));
  double2 v = __ldg(reinterpret_cast<const double2*>(p + 2));
  double2 w = __ldg(reinterpret_cast<const double2*>(p + 4));
  double2 x = __ldg(reinterpret_cast<const double2*>(p + 6));
  return {{u.x, u.y}, {v.x, v.y}, {w.x, w.y}, {x.x, x.y}};
}
template <typename T> __device__ __forceinline__ void jstore(T* p, const Jones<T>& J);
template <> __device__ __forceinline__ void jstore<float>(float* p, const Jones<float>& J) {
  *reinterpret_cast<float4*>(p) = make_float4(J.a.r, J.a.i, J.b.r, J.b.i);
  *reinterpret_cast<float4*>(p + 4) = make_float4(J.c.r, J.c.i, J.d.r, J.d.i);
}
template <> __device__ __forceinline__ void jstore<double>(double* p, const Jones<double>& J) {
  *reinterpret_cast<double2*>(p) = make_double2(J.a.r, J.a.i);
  *reinterpret_cast<double2*>(p + 2) = make_double2(J.b.r, J.b.i);
  *reinterpret_cast<double2*>(p + 4) = make_double2(J.c.r, J.c.i);
  *reinterpret_cast<double2*>(p + 6) = make_double2(J.d.r, J.d.i);
}

// ---- scalar helpers -------------------------------------------------------
__device__ __forceinline__ float mb_sqrt(float x) { return sqrtf(x); }
// 1 / sqrt(x): the hardware reciprocal square root in FP32 (a few ulp), the
// correctly rounded quotient in FP64.  +inf for x == 0 in both.
__device__ __forceinline__ float mb_rsqrt(float x) { return rsqrtf(x); }
__device__ __forceinline__ double mb_rsqrt(double x) { return 1.0 / sqrt(x); }
__device__ __forceinline__ double mb_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float mb_exp(float x) { return expf(x); }
__device__ __forceinline__ double mb_exp(double x) { return exp(x); }
__device__ __forceinline__ float mb_pow(float x, float y) { return powf(x, y); }
__device__ __forceinline__ double mb_pow(double x, double y) { return pow(x, y); }
__device__ __forceinline__ float mb_floor(float x) { return floorf(x); }
__device__ __forceinline__ double mb_floor(double x) { return floor(x); }
__device__ __forceinline__ float mb_log(float x) { return logf(x); }
__device__ __forceinline__ double mb_log(double x) { return log(x); }
template <typename T> __device__ __forceinline__ T mb_clamp(T x, T lo, T hi) { return x < lo ? lo : (x > hi ? hi : x); }
template <typename T> __device__ __forceinline__ T cabs_(Cx<T> z) { return mb_sqrt(z.r * z.r + z.i * z.i); }

// X B for a Hermitian B = [[a, b], [conj(b), d]] with real a, d (a
// brightness square root).
template <typename T>
__device__ __forceinline__ Jones<T> jmul_herm_real_diag(const Jones<T>& X, T a, T d, Cx<T> b) {
  const Cx<T> bc = conj(b);
  return {X.a * a + cmul(X.b, bc), cmul(X.a, b) + X.b * d, X.c * a + cmul(X.d, bc), cmul(X.c, b) + X.d * d};
}
// Row (x0, x1) of X times [[a, b], [conj b, d]] is (x0 a + x1 conj b, x0 b + x1 d).
template <>
__device__ __forceinline__ Jones<float> jmul_herm_real_diag<float>(const Jones<float>& X, float a, float d,
                                                                   Cx<float> b) {
  Jones<float> R;
  const Cx<float>* x = &X.a;
  Cx<float>* y = &R.a;
#pragma unroll
  for (int row = 0; row < 2; ++row) {
    const Cx<float> x0 = x[2 * row], x1 = x[2 * row + 1];
    float2 p = __fmul2_rn(as_f2(x0), make_float2(a, a));
    p = __ffma2_rn(as_f2(x1), make_float2(b.r, b.r), p);
    y[2 * row] = as_cx(__ffma2_rn(make_float2(x1.i, x1.r), make_float2(b.i, -b.i), p));
    float2 q = __fmul2_rn(as_f2(x1), make_float2(d, d));
    q = __ffma2_rn(as_f2(x0), make_float2(b.r, b.r), q);
    y[2 * row + 1] = as_cx(__ffma2_rn(make_float2(x0.i, x0.r), make_float2(-b.i, b.i), q));
  }
  return R;
}

// ---- brightness square root (a1) -----------------------------------------
// B = [[I+Q, U+iV], [U-iV, I-Q]] * (nu/nu_ref)^alpha,
// sqrt(B) = (B + s*1) / t with s = sqrt(det B), t = sqrt(tr B + 2 s); t := 1
// when s == t == 0.  CPUSolver.py:235-317, brightness.cuh:108-164.
// A determinant that rounds below zero is clamped to zero.
template <typename T>
__device__ __forceinline__ Jones<T> brightness_sqrt(T I, T Q, T U, T V, T power) {
  T b0 = (I + Q) * power, b3 = (I - Q) * power;
  T ur = U * power, vi = V * power;
  T trace = b0 + b3;
  T det = b0 * b3 - (ur * ur + vi * vi);
  det = det < T(0) ? T(0) : det;
  T s = mb_sqrt(det);
  T t = mb_sqrt(trace + T(2) * s);
  if (s == T(0) && t == T(0)) t = T(1);
  T rt = T(1) / t;
  Jones<T> R;
  R.a = {(b0 + s) * rt, T(0)};
  R.b = {ur * rt, vi * rt};
  R.c = {ur * rt, -vi * rt};
  R.d = {(b3 + s) * rt, T(0)};
  return R;
}

// ---- phase (a2) ----------------------------------------------------------
// K = exp(-2 pi i phi nu / c), phi = u l + v m + w (n - 1).  The phase
// argument is always formed in FP64 (CPUSolver.py:162-195); in the FP32
// forms its reduction to [-1/2, 1/2] cycles is exact on that FP64 value
// (fp64_frac_nearest) and only the reduced argument is rounded to FP32.
template <typename T> __device__ __forceinline__ Cx<T> phase_from_phi(double phi, double freq);
// FP64: exp(i * ((-2 pi phi) nu) / c), in the oracle's evaluation order.
template <> __device__ __forceinline__ Cx<double> phase_from_phi<double>(double phi, double freq) {
  double arg = ((-2.0 * kPi) * phi * freq) / kLightSpeed;
  double s, c;
  sincos(arg, &s, &c);
  return {c, s};
}
// FP32: cycles = phi nu / c in FP64 and its exact reduction, then an FP32
// sincospi of the reduced argument.
__device__ __forceinline__ float fp64_frac_nearest(double x);
template <> __device__ __forceinline__ Cx<float> phase_from_phi<float>(double phi, double freq) {
  const float frac = fp64_frac_nearest(phi * freq / kLightSpeed);
  float s, c;
  sincospif(-2.0f * frac, &s, &c);
  return {c, s};
}

// Same, with nu / c precomputed per channel (fused kernels).
template <typename T> __device__ __forceinline__ Cx<T> phase_from_cycles(double phi, double nu_over_c);
template <> __device__ __forceinline__ Cx<double> phase_from_cycles<double>(double phi, double nu_over_c) {
  double cycles = phi * nu_over_c;
  double frac = cycles - rint(cycles);
  double s, c;
  sincospi(-2.0 * frac, &s, &c);
  return {c, s};
}
// r = x - rint(x) for an FP64 x, rounded to FP32 (a tie may come out as
// +1/2 or -1/2; both give the same phase factor).  The reduction is exact:
// it keeps the bits of x's 53-bit significand below the binary point,
// working on the bit pattern with integer instructions, so the only FP64
// instruction of the phase is the product forming x.
__device__ __forceinline__ float fp64_frac_nearest(double x) {
  const long long bits = __double_as_longlong(x);
  const int ex = int((bits >> 52) & 0x7ff);
  if (ex == 0x7ff) return __int_as_float(0x7fc00000);  // NaN / inf input stays NaN
  const int f = 1075 - ex;               // fraction bits of the significand
  if (ex == 0 || f <= 0) return 0.f;     // zero or subnormal, or an integer
  if (f > 62) return float(x);           // |x| < 2^-9: nothing to reduce
  const long long m = (bits & 0xFFFFFFFFFFFFFLL) | (1LL << 52);
  long long fb = m & ((1LL << f) - 1);
  if (fb >= (1LL << (f - 1))) fb -= (1LL << f);
  if (bits < 0) fb = -fb;
  const int sh = f > 31 ? f - 31 : 0;     // keep 31 bits: |fb >> sh| <= 2^30
  const int r32 = int(fb >> sh);
  return float(r32) * __int_as_float((127 + sh - f) << 23);  // * 2^(sh - f), exact
}

template <> __device__ __forceinline__ Cx<float> phase_from_cycles<float>(double phi, double nu_over_c) {
  const float frac = fp64_frac_nearest(phi * nu_over_c);
  float s, c;
  sincospif(-2.0f * frac, &s, &c);
  return {c, s};
}

// An FP64 value as the FP32 pair (hi, lo) = (float(x), float(x - hi)):
// 48 significant bits in the 8 bytes of the double.
__device__ __forceinline__ float2 split_f64(double x) {
  const float h = float(x);
  return make_float2(h, float(x - double(h)));
}

// cycles = phi nu / c reduced to about [-1/2, 1/2], from the FP32 pairs
// (ph, pl) of phi and (nh, nl) of nu / c, on the FP32 pipe only.  With p the
// rounded product ph nh, e0 = ph nh - p is exact (one FMA), p - rint(p) is
// exact (Sterbenz), and the small terms e0 + ph nl + pl nh are added to it;
// the dropped pl nl and the pairs' own truncation leave an absolute error
// of about |cycles| 2^-47 before the final FP32 rounding (2^-25): 4e-10
// cycles at |cycles| = 5e4.  (The FP64 product and its exact reduction
// leave |cycles| 2^-53.)  p is formed by __fmul_rn so that it is not fused
// into the subtraction, which would count e0 twice.  The result lies within
// 3 |p| 2^-24 of [-1/2, 1/2] (the three small terms are each at most about
// |p| 2^-24; above 2^23 cycles p is an integer and they are all that is
// left); the sincospi that takes it reduces the rest exactly.
__device__ __forceinline__ float frac_cycles_df(float ph, float pl, float nh, float nl) {
  const float p = __fmul_rn(ph, nh);
  float e = fmaf(ph, nh, -p);
  e = fmaf(ph, nl, e);
  e = fmaf(pl, nh, e);
  return __fadd_rn(__fsub_rn(p, rintf(p)), e);
}

// K from the pairs of the path length (as split_f64 stores it) and of nu / c.
__device__ __forceinline__ Cx<float> phase_from_pair(float2 phi, float2 n) {
  float s, c;
  sincospif(-2.0f * frac_cycles_df(phi.x, phi.y, n.x, n.y), &s, &c);
  return {c, s};
}

// nu / c of one channel with what the per-item terms take from it formed
// once per channel (FP64 arithmetic costs 64 FP32 operations on GB300):
// its FP32 pair for phase_from_pair and 2 pi nu / c = |dK/dphi|.
struct NuC {
  double d;
  float2 p;
  double dphase;
};
__device__ __forceinline__ NuC make_nuc(double nu_over_c) {
  return {nu_over_c, split_f64(nu_over_c), 2.0 * kPi * nu_over_c};
}

// ---- beam cube (a3) ------------------------------------------------------
// Beam grid position along one axis: scale * (x - lower), clamped to
// [0, n-1], split into the lower grid index, the upper grid index and the
// offset.  CPUSolver.py:394-414 (the oracle form ((n-1)(x-lo))/(hi-lo) is
// used in FP64, the pre-scaled form in FP32).
template <typename T>
struct GridPos {
  int i0, i1;
  T d;
  bool inside;  // strictly inside (0, n-1): derivative w.r.t. x is non-zero
};

template <typename T>
__device__ __forceinline__ GridPos<T> grid_pos(T x, T lower, T upper, T scale, int n) {
  T v;
  if (sizeof(T) == 8) v = (T(n - 1) * (x - lower)) / (upper - lower);
  else v = scale * (x - lower);
  GridPos<T> g;
  g.inside = (v > T(0)) && (v < T(n - 1));
  v = mb_clamp(v, T(0), T(n - 1));
  T f0 = mb_floor(v);
  // The integer clamp keeps a NaN coordinate (invalid input) inside the cube.
  g.i0 = min(max(static_cast<int>(f0), 0), n - 1);
  g.i1 = min(g.i0 + 1, n - 1);
  g.d = v - f0;
  return g;
}

// Channel grid of the beam cube for one frequency.
template <typename T>
struct ChanPos {
  int c0, c1;
  T d;
};

template <typename T>
__device__ __forceinline__ ChanPos<T> chan_pos(T freq, T lfreq, T ufreq, int nud) {
  T v = (T(nud - 1) * (freq - lfreq)) / (ufreq - lfreq);
  v = mb_clamp(v, T(0), T(nud - 1));
  T f0 = mb_floor(v);
  ChanPos<T> c;
  c.c0 = min(max(static_cast<int>(f0), 0), nud - 1);
  c.c1 = min(c.c0 + 1, nud - 1);
  c.d = v - f0;
  return c;
}

struct BeamGeom {
  int lw, mh, nud;
};

// Weighted gather of the 4 correlations of one beam-cube corner.
template <typename T>
__device__ __forceinline__ void beam_corner(const T* __restrict__ E_beam, const BeamGeom& G,
                                            int il, int im, int ic, T w, Jones<T>& sum, T (&amp)[4]) {
  const T* p = E_beam + 8 * ((static_cast<size_t>(il) * G.mh + im) * G.nud + ic);
  Jones<T> e = jldg<T>(p);
  sum.a = sum.a + e.a * w; amp[0] += w * cabs_(e.a);
  sum.b = sum.b + e.b * w; amp[1] += w * cabs_(e.b);
  sum.c = sum.c + e.c * w; amp[2] += w * cabs_(e.c);
  sum.d = sum.d + e.d * w; amp[3] += w * cabs_(e.d);
}

template <typename T>
__device__ __forceinline__ Cx<T> renorm(Cx<T> z, T amp) {
  T norm = mb_rsqrt(z.r * z.r + z.i * z.i);
  if (!isfinite(norm)) norm = T(1);
  return z * (norm * amp);
}

// Trilinear, amplitude-renormalised beam value at grid positions gl, gm
// and channel position ch (CPUSolver.py:416-475, RimeEBeam.py:94-116,
// 287-339).  Corner order and weights follow the oracle.
template <typename T>
__device__ __forceinline__ Jones<T> beam_interp(const T* __restrict__ E_beam, const BeamGeom& G,
                                                const GridPos<T>& gl, const GridPos<T>& gm,
                                                const ChanPos<T>& ch) {
  Jones<T> sum = jzero<T>();
  T amp[4] = {T(0), T(0), T(0), T(0)};
  T ld = gl.d, md = gm.d, cd = ch.d;
  beam_corner(E_beam, G, gl.i0, gm.i0, ch.c0, (T(1) - ld) * (T(1) - md) * (T(1) - cd), sum, amp);
  beam_corner(E_beam, G, gl.i1, gm.i0, ch.c0, ld * (T(1) - md) * (T(1) - cd), sum, amp);
  beam_corner(E_beam, G, gl.i0, gm.i1, ch.c0, (T(1) - ld) * md * (T(1) - cd), sum, amp);
  beam_corner(E_beam, G, gl.i1, gm.i1, ch.c0, ld * md * (T(1) - cd), sum, amp);
  beam_corner(E_beam, G, gl.i0, gm.i0, ch.c1, (T(1) - ld) * (T(1) - md) * cd, sum, amp);
  beam_corner(E_beam, G, gl.i1, gm.i0, ch.c1, ld * (T(1) - md) * cd, sum, amp);
  beam_corner(E_beam, G, gl.i0, gm.i1, ch.c1, (T(1) - ld) * md * cd, sum, amp);
  beam_corner(E_beam, G, gl.i1, gm.i1, ch.c1, ld * md * cd, sum, amp);
  Jones<T> E;
  E.a = renorm(sum.a, amp[0]);
  E.b = renorm(sum.b, amp[1]);
  E.c = renorm(sum.c, amp[2]);
  E.d = renorm(sum.d, amp[3]);
  return E;
}

// The beam cube blended along frequency for one channel, stored per (l, m)
// grid cell as bilinear coefficients.  Per cell (i, j), the 12 values v
// (the 4 correlations of E, complex, and of |E|), each linearly
// interpolated between the two cube planes the channel falls between, give
//   f00 = v(i, j),  a = v(i1, j) - v(i, j),  b = v(i, j1) - v(i, j),
//   c = v(i1, j1) - v(i1, j) - b,   i1 = min(i + 1, lw - 1), j1 = min(j + 1, mh - 1),
// stored as [f00 | a | b | c] (12 values each, 48 per cell), so that the
// trilinear interpolation of the cube at (i + x, j + y, channel) is
//   v = f00 + x a + y (b + x c),  dv/dx = a + y c,  dv/dy = b + x c:
// the same weights as the 8-corner sum (the blend along frequency first),
// three FMAs per value, and one contiguous cell per lookup.
constexpr int kPlaneComp = 12;  // values per coefficient (E: 8, |E|: 4)
constexpr int kPlaneVals = 4 * kPlaneComp;

// The 12 bilinear values (and optionally their x and y derivatives) of the
// coefficient cell at p for offsets x, y.
template <typename T, bool DERIV>
__device__ __forceinline__ void plane_cell(const T* __restrict__ p, T x, T y, T (&v)[kPlaneComp],
                                           T (&dx)[kPlaneComp], T (&dy)[kPlaneComp]) {
  if constexpr (sizeof(T) == 4) {
    // two values per packed FP32x2 FMA (each lane rounded as fmaf)
    const float4* q = reinterpret_cast<const float4*>(p);
    const float2 xx = make_float2(x, x), yy = make_float2(y, y);
#pragma unroll
    for (int r = 0; r < 3; ++r) {  // float4 runs: E.a E.b | E.c E.d | |E|
      const float4 f4 = __ldg(q + r), a4 = __ldg(q + 3 + r), b4 = __ldg(q + 6 + r), c4 = __ldg(q + 9 + r);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const float2 f = h ? make_float2(f4.z, f4.w) : make_float2(f4.x, f4.y);
        const float2 a = h ? make_float2(a4.z, a4.w) : make_float2(a4.x, a4.y);
        const float2 b = h ? make_float2(b4.z, b4.w) : make_float2(b4.x, b4.y);
        const float2 c = h ? make_float2(c4.z, c4.w) : make_float2(c4.x, c4.y);
        const float2 fy = __ffma2_rn(xx, c, b);
        const float2 vv = __ffma2_rn(yy, fy, __ffma2_rn(xx, a, f));
        const int k = 4 * r + 2 * h;
        v[k] = vv.x;
        v[k + 1] = vv.y;
        if (DERIV) {
          const float2 d = __ffma2_rn(yy, c, a);
          dx[k] = d.x;
          dx[k + 1] = d.y;
          dy[k] = fy.x;
          dy[k + 1] = fy.y;
        }
      }
    }
  } else {
#pragma unroll
    for (int k = 0; k < kPlaneComp; ++k) {
      const T f = __ldg(p + k), a = __ldg(p + kPlaneComp + k), b = __ldg(p + 2 * kPlaneComp + k),
              c = __ldg(p + 3 * kPlaneComp + k);
      const T fy = b + x * c;
      v[k] = f + x * a + y * fy;
      if (DERIV) {
        dx[k] = a + y * c;
        dy[k] = fy;
      }
    }
  }
}

template <typename T>
__device__ __forceinline__ const T* plane_cell_ptr(const T* plane, int mh, int il, int im) {
  return plane + kPlaneVals * (size_t(il) * mh + im);
}

template <typename T>
__device__ __forceinline__ Jones<T> beam_interp_plane(const T* __restrict__ plane, int mh, const GridPos<T>& gl,
                                                      const GridPos<T>& gm) {
  T v[kPlaneComp], unused[kPlaneComp];
  plane_cell<T, false>(plane_cell_ptr(plane, mh, gl.i0, gm.i0), gl.d, gm.d, v, unused, unused);
  Jones<T> E;
  E.a = renorm(Cx<T>{v[0], v[1]}, v[8]);
  E.b = renorm(Cx<T>{v[2], v[3]}, v[9]);
  E.c = renorm(Cx<T>{v[4], v[5]}, v[10]);
  E.d = renorm(Cx<T>{v[6], v[7]}, v[11]);
  return E;
}

// Rotate (l, m) by the parallactic angle, add the pointing error and scale
// by the antenna scaling (CPUSolver.py:367-390).
template <typename T>
__device__ __forceinline__ void beam_lm(T l0, T m0, T sin_pa, T cos_pa, T pe_l, T pe_m, T sc_l, T sc_m,
                                        T& l, T& m) {
  l = (l0 * cos_pa - m0 * sin_pa + pe_l) * sc_l;
  m = (l0 * sin_pa + m0 * cos_pa + pe_m) * sc_m;
}

// ---- source shapes (a5) --------------------------------------------------
// Gaussian: exp(-((u1 k R)^2 + (v1 k)^2)), u1 = u em - v el, v1 = u el + v em,
// k = gauss_scale * nu (CPUSolver.py:59-103).
template <typename T>
__device__ __forceinline__ T gauss_shape(T u, T v, T el, T em, T R, T k) {
  T u1 = (u * em - v * el) * k * R;
  T v1 = (u * el + v * em) * k;
  return mb_exp(-(u1 * u1 + v1 * v1));
}
// Sersic: 1 / (d sqrt d), d = 1 + (u1 k S)^2 + (v1 k S)^2, u1 = u(1+e1) + v e2,
// v1 = u e2 + v(1-e1), S = R / (1 - e1^2 - e2^2), k = 2 pi nu / c
// (CPUSolver.py:105-160).
template <typename T>
__device__ __forceinline__ T sersic_shape(T u, T v, T e1, T e2, T R, T k) {
  T S = R / (T(1) - e1 * e1 - e2 * e2);
  T u1 = (u * (T(1) + e1) + v * e2) * k * S;
  T v1 = (u * e2 + v * (T(1) - e1)) * k * S;
  T d = T(1) + u1 * u1 + v1 * v1;
  if constexpr (sizeof(T) == 4) {
    const T r = mb_rsqrt(d);
    return r * r * r;
  }
  return T(1) / (d * mb_sqrt(d));
}

// Source type of global source index s (point, gaussian, sersic order,
// montblanc/src_types.py:40-44).
enum SrcType { SRC_POINT = 0, SRC_GAUSS = 1, SRC_SERSIC = 2 };

// Index of unordered antenna pair (p <= q) in the packed upper triangle.
__host__ __device__ __forceinline__ int pair_index(int p, int q, int na) {
  return p * na - (p * (p - 1)) / 2 + (q - p);
}

}  // namespace mb
