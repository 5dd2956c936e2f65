// ddf.cuh -- double-float ("float-float") arithmetic: a value is the unevaluated sum hi + lo of two
// FP32 numbers (|lo| <= ulp(hi)/2, ~48-bit significand).  GB300's FP64 pipe runs at 1/64 of its FP32
// rate, so FP64-grade arithmetic built from FP32 instructions (~15 per fused multiply-add) is several
// times faster for the FP64 step's matrix products (3.97x on chained 3x3 complex products, measured).
// Algorithms: Dekker's product (TwoProd, here exact by FMA) and Knuth's TwoSum, with a Fast2Sum
// renormalisation (Dekker, Numer. Math. 18 (1971) 224; Knuth, TAOCP vol. 2, 4.2.2).
// The operators below let the templated SU(3) arithmetic of su3.cuh run on ddf unchanged.
#pragma once

#include <cuda_runtime.h>

#include <type_traits>

#include "su3.cuh"

namespace glasma {

using ::fma;  // the native overloads stay visible beside fma(ddf, ddf, ddf) below

struct ddf {
  float hi, lo;
  ddf() = default;
  // from a double: hi its nearest float, lo the nearest float to the remainder (constants fold)
  // explicit: a double never becomes a ddf silently (glasma::fma(ddf, ddf, ddf) must not capture
  // the FP64 code's fma calls)
  __host__ __device__ __forceinline__ explicit ddf(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
  __host__ __device__ __forceinline__ ddf(float h, float l) : hi(h), lo(l) {}
};

// Bit-level conversions, so that moving FP64 fields in and out of double-float costs no FP64
// instruction but the one addition of a store (GB300's conversions between FP64 and FP32 run at the
// FP64 rate).
__host__ __device__ __forceinline__ unsigned long long ddf_bits64(double d) {
#ifdef __CUDA_ARCH__
  return (unsigned long long)__double_as_longlong(d);
#else
  unsigned long long b;
  __builtin_memcpy(&b, &d, 8);
  return b;
#endif
}
__host__ __device__ __forceinline__ double ddf_double_from_bits(unsigned long long b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double d;
  __builtin_memcpy(&d, &b, 8);
  return d;
#endif
}
__host__ __device__ __forceinline__ unsigned ddf_bits32(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  unsigned b;
  __builtin_memcpy(&b, &f, 4);
  return b;
#endif
}
__host__ __device__ __forceinline__ float ddf_float_from_bits(unsigned b) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(b);
#else
  float f;
  __builtin_memcpy(&f, &b, 4);
  return f;
#endif
}

// d = head + tail: head = the leading 24 bits of d's significand (exponent rebiased), tail = the
// remaining 29 bits as t 2^(e-1075), rounded to a float; then renormalised (Fast2Sum).  Outside
// 2^-74 <= |d| < 2^128 the FP64 conversion is used instead: zero stays zero, tiny values keep fewer
// bits, and |d| >= 2^128 (beyond FP32's exponent range, as in any double-float format) becomes
// +-inf.  Field values of the evolution are far inside the range.
__host__ __device__ __forceinline__ ddf ddf_from_double(double d) {
  const unsigned long long b = ddf_bits64(d);
  const unsigned hi32 = (unsigned)(b >> 32), lo32 = (unsigned)b;
  const int e = (int)((hi32 >> 20) & 0x7ffu);  // biased exponent
  if (e < 949 || e > 1150) return ddf(d);
  const unsigned sign = hi32 & 0x80000000u;
  const unsigned top23 = ((hi32 & 0xfffffu) << 3) | (lo32 >> 29);
  const float head = ddf_float_from_bits(sign | ((unsigned)(e - 896) << 23) | top23);
  const float scale = ddf_float_from_bits((unsigned)(e - 948) << 23);  // 2^(e - 1075)
  float tail = (float)(lo32 & 0x1fffffffu) * scale;
  tail = sign ? -tail : tail;
  const float h = head + tail;
  return ddf(h, tail - (h - head));
}
// exact float -> double by bits (normal floats; zero, subnormal, inf and nan by conversion)
__host__ __device__ __forceinline__ double ddf_widen(float x) {
  const unsigned u = ddf_bits32(x);
  const unsigned e = (u >> 23) & 0xffu;
  if (e == 0u || e == 255u) return (double)x;
  return ddf_double_from_bits(((unsigned long long)(u & 0x80000000u) << 32) |
                              ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)(u & 0x7fffffu) << 29));
}
__host__ __device__ __forceinline__ double to_double(ddf a) { return ddf_widen(a.hi) + ddf_widen(a.lo); }

// s = a + b exactly as s.hi + s.lo (TwoSum), then the low parts, then renormalised
__device__ __forceinline__ ddf operator+(ddf a, ddf b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  float e = (a.hi - (s - bb)) + (b.hi - bb);
  e += a.lo + b.lo;
  const float hi = s + e;
  return ddf(hi, e - (hi - s));
}
__device__ __forceinline__ ddf operator-(ddf a) { return ddf(-a.hi, -a.lo); }
__device__ __forceinline__ ddf operator-(ddf a, ddf b) { return a + (-b); }
// a b: the exact product of the high parts by FMA, plus the cross terms (lo*lo is below the precision)
__device__ __forceinline__ ddf operator*(ddf a, ddf b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  const float hi = p + e;
  return ddf(hi, e - (hi - p));
}
// c + a b with one renormalisation
__device__ __forceinline__ ddf fma(ddf a, ddf b, ddf c) {
  const float p = a.hi * b.hi;
  float pe = fmaf(a.hi, b.hi, -p);
  pe = fmaf(a.hi, b.lo, pe);
  pe = fmaf(a.lo, b.hi, pe);
  const float s = c.hi + p;
  const float bb = s - c.hi;
  float e = (c.hi - (s - bb)) + (p - bb);
  e += c.lo + pe;
  const float hi = s + e;
  return ddf(hi, e - (hi - s));
}
__device__ __forceinline__ ddf& operator+=(ddf& a, ddf b) { return a = a + b; }
__device__ __forceinline__ ddf& operator-=(ddf& a, ddf b) { return a = a - b; }
__device__ __forceinline__ ddf& operator*=(ddf& a, ddf b) { return a = a * b; }

// storage type <-> compute type
template <typename TC, typename T>
__device__ __forceinline__ TC to_compute(T x) {
  if constexpr (std::is_same<TC, ddf>::value && std::is_same<T, double>::value)
    return ddf_from_double(x);
  else
    return TC(x);
}
template <typename T>
__device__ __forceinline__ T from_compute(T x) {
  return x;
}
template <typename T>
__device__ __forceinline__ T from_compute(ddf x);
template <>
__device__ __forceinline__ double from_compute<double>(ddf x) {
  return to_double(x);
}

// The double-float 3x3 products run as out-of-line functions: fully unrolled and inlined at every use
// the force kernel's code overflowed the instruction cache (ncu: "no instruction" the dominant stall,
// 22 % issue); one copy of each product serves every call.
static __device__ __noinline__ void ddf_mul_nn(const Mat<ddf>& A, const Mat<ddf>& B, Mat<ddf>& C);
static __device__ __noinline__ void ddf_mul_dn(const Mat<ddf>& A, const Mat<ddf>& B, Mat<ddf>& C);
static __device__ __noinline__ void ddf_mul_nn_herm(const Mat<ddf>& A, const Mat<ddf>& B, Mat<ddf>& C);
static __device__ __noinline__ void ddf_mul_nd_traceless(const Mat<ddf>& A, const Mat<ddf>& B, Mat<ddf>& C);
template <>
__device__ __forceinline__ void mul_nn<ddf>(const Mat<ddf>& A, const Mat<ddf>& B, Mat<ddf>& C) {
  ddf_mul_nn(A, B, C);
}
template <>
__device__ __forceinline__ void mul_dn<ddf>(const Mat<ddf>& A, const Mat<ddf>& B, Mat<ddf>& C) {
  ddf_mul_dn(A, B, C);
}
template <>
__device__ __forceinline__ void mul_nn_herm<ddf>(const Mat<ddf>& A, const Mat<ddf>& B, Mat<ddf>& C) {
  ddf_mul_nn_herm(A, B, C);
}
template <>
__device__ __forceinline__ void mul_nd_traceless<ddf>(const Mat<ddf>& A, const Mat<ddf>& B, Mat<ddf>& C) {
  ddf_mul_nd_traceless(A, B, C);
}
// the bodies: the generic products' own arithmetic, on ddf
static __device__ __noinline__ void ddf_mul_nn(const Mat<ddf>& A, const Mat<ddf>& B, Mat<ddf>& C) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      cx<ddf> acc = mk<ddf>(ddf(0.0), ddf(0.0));
#pragma unroll
      for (int k = 0; k < 3; k++) cfma(acc, A.e[i + 3 * k], B.e[k + 3 * j]);
      C.e[i + 3 * j] = acc;
    }
}
static __device__ __noinline__ void ddf_mul_dn(const Mat<ddf>& A, const Mat<ddf>& B, Mat<ddf>& C) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      cx<ddf> acc = mk<ddf>(ddf(0.0), ddf(0.0));
#pragma unroll
      for (int k = 0; k < 3; k++) cfma_cn(acc, A.e[k + 3 * i], B.e[k + 3 * j]);
      C.e[i + 3 * j] = acc;
    }
}
static __device__ __noinline__ void ddf_mul_nn_herm(const Mat<ddf>& A, const Mat<ddf>& B, Mat<ddf>& C) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = i; j < 3; j++) {
      cx<ddf> acc = mk<ddf>(ddf(0.0), ddf(0.0));
      if (i == j) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
          acc.re = fma(A.e[i + 3 * k].re, B.e[k + 3 * j].re, acc.re);
          acc.re = fma(-A.e[i + 3 * k].im, B.e[k + 3 * j].im, acc.re);
        }
      } else {
#pragma unroll
        for (int k = 0; k < 3; k++) cfma(acc, A.e[i + 3 * k], B.e[k + 3 * j]);
      }
      C.e[i + 3 * j] = acc;
    }
}
static __device__ __noinline__ void ddf_mul_nd_traceless(const Mat<ddf>& A, const Mat<ddf>& B, Mat<ddf>& C) {
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      cx<ddf> acc = mk<ddf>(ddf(0.0), ddf(0.0));
      if (i == j) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
          acc.im = fma(-A.e[i + 3 * k].re, B.e[j + 3 * k].im, acc.im);
          acc.im = fma(A.e[i + 3 * k].im, B.e[j + 3 * k].re, acc.im);
        }
      } else {
#pragma unroll
        for (int k = 0; k < 3; k++) cfma_nc(acc, A.e[i + 3 * k], B.e[j + 3 * k]);
      }
      C.e[i + 3 * j] = acc;
    }
}

// links of FP64 fields loaded and split out of line: p points at element 0 of the link, the nine
// complex elements `stride` apart
static __device__ __noinline__ void ddf_load_link9(const cx<double>* __restrict__ p, long long stride, Mat<ddf>& m) {
#pragma unroll
  for (int k = 0; k < 9; k++) {
    const cx<double> v = p[(long long)k * stride];
    m.e[k] = mk<ddf>(ddf_from_double(v.re), ddf_from_double(v.im));
  }
}

template <>
struct Consts<ddf> {
  static __device__ __forceinline__ ddf inv_sqrt3() { return ddf(0.57735026918962576450914878050195745564760175127013); }
  static __device__ __forceinline__ ddf inv_sqrt2() { return ddf(0.70710678118654752440084436210484903928483593768847); }
};

// V^dagger (t.e) V in double-float, out of line (six per site in the force kernel)
template <typename T>
__device__ __forceinline__ void herm_from_alg(const Alg<T>& al, Mat<T>& M);
template <typename T>
__device__ __forceinline__ void alg_from_herm(const Mat<T>& W, Alg<T>& out);
static __device__ __noinline__ void ddf_inv_adj_mul(const Mat<ddf>& V, const Alg<ddf>& e, Alg<ddf>& out) {
  Mat<ddf> M, W, R;
  herm_from_alg(e, M);
  ddf_mul_dn(V, M, W);
  ddf_mul_nn_herm(W, V, R);
  alg_from_herm(R, out);
}
template <>
__device__ __forceinline__ void inv_adj_mul<ddf>(const Mat<ddf>& V, const Alg<ddf>& e, Alg<ddf>& out) {
  ddf_inv_adj_mul(V, e, out);
}

}  // namespace glasma
