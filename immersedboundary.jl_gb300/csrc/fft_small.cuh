// Small in-register forward DFTs (e^{-2 pi i / R}) and helpers shared by the sine-transform
// kernels (dst.cu: shared-memory Stockham passes; dstw.cuh: warp-per-line passes).
#pragma once

#include "ib_common.cuh"

namespace ib {

template <typename T, int R> struct Dft;

template <typename T> struct Dft<T, 2> {
  template <typename V> __device__ __forceinline__ static void run(V* v) {
    V a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  }
};

template <typename T> struct Dft<T, 4> {
  template <typename V> __device__ __forceinline__ static void run(V* v) {
    V t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
    V t2 = cadd(v[1], v[3]), t3 = cmul_mi(csub(v[1], v[3]));
    v[0] = cadd(t0, t2);
    v[2] = csub(t0, t2);
    v[1] = cadd(t1, t3);
    v[3] = csub(t1, t3);
  }
};

template <typename T> struct Dft<T, 8> {
  template <typename V> __device__ __forceinline__ static void run(V* v) {
    const T r2 = T(0.70710678118654752440);
    V e[4] = {v[0], v[2], v[4], v[6]};
    V o[4] = {v[1], v[3], v[5], v[7]};
    Dft<T, 4>::run(e);
    Dft<T, 4>::run(o);
    // o1 *= (1 - i)/sqrt2 ; o2 *= -i ; o3 *= (-1 - i)/sqrt2
    V o1 = mk<V>(r2 * (o[1].x + o[1].y), r2 * (o[1].y - o[1].x));
    V o2 = cmul_mi(o[2]);
    V o3 = mk<V>(r2 * (o[3].y - o[3].x), -r2 * (o[3].x + o[3].y));
    v[0] = cadd(e[0], o[0]);
    v[4] = csub(e[0], o[0]);
    v[1] = cadd(e[1], o1);
    v[5] = csub(e[1], o1);
    v[2] = cadd(e[2], o2);
    v[6] = csub(e[2], o2);
    v[3] = cadd(e[3], o3);
    v[7] = csub(e[3], o3);
  }
};

template <typename T> struct Dft<T, 3> {
  template <typename V> __device__ __forceinline__ static void run(V* v) {
    const T s = T(0.86602540378443864676);
    V t1 = cadd(v[1], v[2]);
    V d = csub(v[1], v[2]);
    V t2 = mk<V>(v[0].x - T(0.5) * t1.x, v[0].y - T(0.5) * t1.y);
    V t3 = mk<V>(s * d.y, -s * d.x);  // -i s (x1 - x2)
    v[0] = cadd(v[0], t1);
    v[1] = cadd(t2, t3);
    v[2] = csub(t2, t3);
  }
};

template <typename T> struct Dft<T, 5> {
  template <typename V> __device__ __forceinline__ static void run(V* v) {
    const T c1 = T(0.30901699437494742410), c2 = T(-0.80901699437494742410);
    const T s1 = T(0.95105651629515357212), s2 = T(0.58778525229247312917);
    V a1 = cadd(v[1], v[4]), b1 = csub(v[1], v[4]);
    V a2 = cadd(v[2], v[3]), b2 = csub(v[2], v[3]);
    V x0 = v[0];
    V r1 = mk<V>(x0.x + c1 * a1.x + c2 * a2.x, x0.y + c1 * a1.y + c2 * a2.y);
    V r2 = mk<V>(x0.x + c2 * a1.x + c1 * a2.x, x0.y + c2 * a1.y + c1 * a2.y);
    V i1 = mk<V>(s1 * b1.x + s2 * b2.x, s1 * b1.y + s2 * b2.y);
    V i2 = mk<V>(s2 * b1.x - s1 * b2.x, s2 * b1.y - s1 * b2.y);
    v[0] = mk<V>(x0.x + a1.x + a2.x, x0.y + a1.y + a2.y);
    // y = r -/+ i*ii :  -i*(a+ib) = (b, -a)
    v[1] = mk<V>(r1.x + i1.y, r1.y - i1.x);
    v[4] = mk<V>(r1.x - i1.y, r1.y + i1.x);
    v[2] = mk<V>(r2.x + i2.y, r2.y - i2.x);
    v[3] = mk<V>(r2.x - i2.y, r2.y + i2.x);
  }
};

template <typename T> __device__ __forceinline__ T fmaT(T a, T b, T c);
template <> __device__ __forceinline__ double fmaT(double a, double b, double c) { return fma(a, b, c); }
template <> __device__ __forceinline__ float fmaT(float a, float b, float c) { return fmaf(a, b, c); }


}  // namespace ib
