// Float-float ("double-float") numbers: a value is hi + lo with |lo| <= ulp(hi)/2, both FP32.
//
// GB300 runs FP64 at about 1/56 of its FP32 rate, so the mixed-precision path keeps its state,
// stencils and refinement residuals in this representation (about 48 significant bits,
// FP32 exponent range) and does all of their arithmetic on the FP32 pipe.  The algorithms are
// the classical error-free transformations: Knuth's TwoSum, Dekker's Fast2Sum and the
// FMA-based exact product (as in Dekker 1971, Hida-Li-Bailey 2001).
#pragma once

#include <cuda_runtime.h>

namespace ib {

struct df64 {
  float hi, lo;

  df64() = default;
  __host__ __device__ constexpr df64(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ constexpr df64(float v) : hi(v), lo(0.0f) {}
  // nearest float-float of a double (two roundings); exact for doubles with <= 48 bits
  __host__ __device__ constexpr df64(double v)
      : hi(static_cast<float>(v)), lo(static_cast<float>(v - static_cast<double>(static_cast<float>(v)))) {}
  __host__ __device__ constexpr df64(int v) : df64(static_cast<double>(v)) {}

  __host__ __device__ explicit operator double() const { return static_cast<double>(hi) + static_cast<double>(lo); }
  __host__ __device__ explicit operator float() const { return hi + lo; }
};

// s + e = a + b exactly
__device__ __forceinline__ df64 two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  const float e = (a - (s - bb)) + (b - bb);
  return df64(s, e);
}
// s + e = a + b exactly, given |a| >= |b|
__device__ __forceinline__ df64 fast_two_sum(float a, float b) {
  const float s = a + b;
  return df64(s, b - (s - a));
}
// p + e = a * b exactly
__device__ __forceinline__ df64 two_prod(float a, float b) {
  const float p = a * b;
  return df64(p, fmaf(a, b, -p));
}

// accurate sum (error relative to the result, also under cancellation)
__device__ __forceinline__ df64 add_accurate(df64 a, df64 b) {
  df64 s = two_sum(a.hi, b.hi);
  const df64 t = two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = fast_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return fast_two_sum(s.hi, s.lo);
}
// Dekker's add: error below 2 ulp of max(|a|, |b|) in the float-float sense, i.e. about 2^-46
// relative to the larger operand (not to the sum); enough wherever the sum's absolute error
// is what matters, which is every use in this library (the arithmetic operators use it).
__device__ __forceinline__ df64 add_sloppy(df64 a, df64 b) {
  df64 s = two_sum(a.hi, b.hi);
  s.lo += a.lo + b.lo;
  return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df64 operator+(df64 a, df64 b) { return add_sloppy(a, b); }
__device__ __forceinline__ df64 operator-(df64 a) { return df64(-a.hi, -a.lo); }
__device__ __forceinline__ df64 operator-(df64 a, df64 b) { return add_sloppy(a, -b); }
__device__ __forceinline__ df64 operator*(df64 a, df64 b) {
  df64 p = two_prod(a.hi, b.hi);
  p.lo = fmaf(a.hi, b.lo, p.lo);
  p.lo = fmaf(a.lo, b.hi, p.lo);
  return fast_two_sum(p.hi, p.lo);
}
// 4 c - (w + e + s + n) of five floats, to float-float accuracy: the neighbour sum is formed
// with error-free sums (its three small parts add up in float with an error ~2^-48 of the
// sum), the difference with the exactly scaled centre with one more error-free sum.
__device__ __forceinline__ df64 lap5_exact(float c, float w, float e, float s, float n) {
  const df64 a = two_sum(w, e);
  const df64 b = two_sum(s, n);
  const df64 t = two_sum(a.hi, b.hi);
  const float small = (a.lo + b.lo) + t.lo;
  const df64 u = two_sum(4.0f * c, -t.hi);
  return fast_two_sum(u.hi, u.lo - small);
}

__device__ __forceinline__ df64& operator+=(df64& a, df64 b) { return a = a + b; }
__device__ __forceinline__ df64& operator-=(df64& a, df64 b) { return a = a - b; }
__device__ __forceinline__ df64& operator*=(df64& a, df64 b) { return a = a * b; }

template <typename T> struct is_df64 { static constexpr bool value = false; };
template <> struct is_df64<df64> { static constexpr bool value = true; };

// the exact-arithmetic partner of a storage type: FP64 path -> double, mixed path -> df64
template <typename T> struct acc_of { using type = double; };
template <> struct acc_of<df64> { using type = df64; };

}  // namespace ib
