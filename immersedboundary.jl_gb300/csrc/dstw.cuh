// Warp-per-line sine transforms: the DST-I passes of the Poisson / Crank-Nicolson solves for
// axes of n = 64 P cells, P in {1, 2, 4, 8, 16, 32} or {3, 6, 12, 24} (the same transform as
// dst.cu, see there).
//
// One warp owns one line in shared memory and keeps it in registers between the exchanges, so
// the transform needs no block-wide barrier.  With M = n/2 = 32 P complex points, lane l holds
// z_m = u_{2m} + i u_{2m+1} for m = l + 32 r (r < P) and the length-M FFT is a four-step
// factorisation M = P x 32:
//   1. DFT_P over r in registers, twiddle e^{-2 pi i l a / M}
//   2. shared-memory transpose (row stride 32 + G, G = 32 / P, conflict-free both ways) so that
//      the G lanes of group a' hold the 32 values of sub-transform a', interleaved by lane
//   3. DFT_P in registers, twiddle e^{-2 pi i g c / 32}, then DFT_G across the group's lanes
//      (radix-2 decimation in frequency with shuffles; output index bit-reversed in the lane)
//   (P = 3 2^k does not divide 32: steps 2-3 become one 32-point transform across all lanes,
//   done with shuffles, and step 1's index a is the final one)
//   4. store in natural order, split the real transform into the even outputs and the
//      differences D_k, and form the odd outputs as the compensated prefix sum of D
// Tables come from global memory in lane order (coalesced, L1-resident).
#pragma once

#include "fft_small.cuh"
#include "ib_common.cuh"

#include <type_traits>

namespace ib {
namespace wdst {

constexpr unsigned kFull = 0xffffffffu;
#ifndef IB_WDST_LINES
#define IB_WDST_LINES 4
#endif
constexpr int kLines = IB_WDST_LINES;  // lines per block
// resident blocks per SM of the pass kernels: IB_WDST_XMINB / IB_WDST_YMINB (ib_common.cuh)

// (lanes per line, values per lane) pairs with compiled passes: one warp per line, or two
// (IBGB300_LINE_LANES=64, axes with M = 64 P, P = 2..16)
#define IB_WDST_COMBOS(X) \
  X(32, 1) X(32, 2) X(32, 3) X(32, 4) X(32, 6) X(32, 8) X(32, 12) X(32, 16) X(32, 24) X(32, 32) \
  X(64, 2) X(64, 4) X(64, 8) X(64, 16)
// loads in flight per lane in the line copies (ring-transfer kernels, FP64 lines, two-warp lines:
// more would spill)
constexpr int kLB = 8;
// FP32 one-warp lines of n = 64 P values: the whole line in one round trip per lane, 2 P loads
// (at most 32).  Measured on GB300 (device time per mixed step): 1.167-1.180 / 4.56-4.62 ms at
// 1024^2 x 4 / 2048^2 x 5 against 1.202 / 4.74 with 8 loads per round.
template <typename T, int P, int NL>
__host__ __device__ constexpr int line_lb() {
  return (sizeof(T) == 4 && NL == 32) ? (2 * P < 32 ? 2 * P : 32) : kLB;
}

// cos(2 pi t / 96) for t = 0..24 (a quarter period); the rest by symmetry.  96 = lcm of the
// in-lane transform sizes 2^k and 3 2^k (k <= 5).
__host__ __device__ constexpr double cos96_q(int t) {
  constexpr double c[25] = {
      1.00000000000000000000, 0.997858923238603506738, 0.991444861373810411145, 0.980785280403230449126,
      0.965925826289068286750, 0.946930129495105664256, 0.923879532511286756128, 0.896872741532688303894,
      0.866025403784438646764, 0.831469612302545237079, 0.793353340291235164580, 0.751839807478977396407,
      0.707106781186547524401, 0.659345815100068868425, 0.608761429008720639416, 0.555570233019602224743,
      0.500000000000000000000, 0.442288690219001281995, 0.382683432365089771728, 0.321439465303161580701,
      0.258819045102520762349, 0.195090322016128267848, 0.130526192220051591548, 0.0654031292301430668153,
      0.0};
  return c[t];
}
__host__ __device__ constexpr double cos96(int t) {
  return (t % 96) <= 24 ? cos96_q(t % 96)
       : (t % 96) <= 48 ? -cos96_q(48 - (t % 96))
       : (t % 96) <= 72 ? -cos96_q((t % 96) - 48)
       : cos96_q(96 - (t % 96));
}

// x * e^{-2 pi i e / P} with e, P known after unrolling (trivial factors without multiplies)
template <typename T, int P>
__device__ __forceinline__ c2_t<T> wmul(c2_t<T> x, int e) {
  using V = c2_t<T>;
  static_assert(96 % P == 0, "in-lane transform size must divide 96");
  const int t = ((e % P) * (96 / P)) % 96;
  if (t == 0) return x;
  if (t == 24) return cmul_mi(x);
  if (t == 48) return mk<V>(-x.x, -x.y);
  if (t == 72) return mk<V>(-x.y, x.x);
  const T c = T(cos96(t)), s = -T(cos96(t + 72));
  return mk<V>(x.x * c - x.y * s, x.x * s + x.y * c);
}

// In-register DFT of P points, natural order in and out.
template <typename T, int P> struct LaneDft;
template <typename T> struct LaneDft<T, 1> {
  __device__ __forceinline__ static void run(c2_t<T>*) {}
};
template <typename T> struct LaneDft<T, 2> {
  __device__ __forceinline__ static void run(c2_t<T>* v) { Dft<T, 2>::run(v); }
};
template <typename T> struct LaneDft<T, 4> {
  __device__ __forceinline__ static void run(c2_t<T>* v) { Dft<T, 4>::run(v); }
};
template <typename T> struct LaneDft<T, 8> {
  __device__ __forceinline__ static void run(c2_t<T>* v) { Dft<T, 8>::run(v); }
};
template <typename T> struct LaneDft<T, 3> {
  __device__ __forceinline__ static void run(c2_t<T>* v) { Dft<T, 3>::run(v); }
};
// P = A B: x[m1 + A m2] -> DFT_B over m2, twiddle W_P^{m1 k2}, DFT_A over m1 -> X[k2 + B k1]
template <typename T, int P, int A, int B>
__device__ __forceinline__ void four_step(c2_t<T>* v) {
  using V = c2_t<T>;
  V t[A * B];
#pragma unroll
  for (int m1 = 0; m1 < A; ++m1) {
    V s[B];
#pragma unroll
    for (int m2 = 0; m2 < B; ++m2) s[m2] = v[m1 + A * m2];
    Dft<T, B>::run(s);
#pragma unroll
    for (int k2 = 0; k2 < B; ++k2) t[m1 * B + k2] = wmul<T, P>(s[k2], m1 * k2);
  }
#pragma unroll
  for (int k2 = 0; k2 < B; ++k2) {
    V s[A];
#pragma unroll
    for (int m1 = 0; m1 < A; ++m1) s[m1] = t[m1 * B + k2];
    Dft<T, A>::run(s);
#pragma unroll
    for (int k1 = 0; k1 < A; ++k1) v[k2 + B * k1] = s[k1];
  }
}
template <typename T> struct LaneDft<T, 16> {
  __device__ __forceinline__ static void run(c2_t<T>* v) { four_step<T, 16, 4, 4>(v); }
};
template <typename T> struct LaneDft<T, 32> {
  __device__ __forceinline__ static void run(c2_t<T>* v) { four_step<T, 32, 4, 8>(v); }
};
template <typename T> struct LaneDft<T, 6> {
  __device__ __forceinline__ static void run(c2_t<T>* v) { four_step<T, 6, 2, 3>(v); }
};
template <typename T> struct LaneDft<T, 12> {
  __device__ __forceinline__ static void run(c2_t<T>* v) { four_step<T, 12, 4, 3>(v); }
};
template <typename T> struct LaneDft<T, 24> {
  __device__ __forceinline__ static void run(c2_t<T>* v) { four_step<T, 24, 8, 3>(v); }
};

constexpr int ilog2(int x) { return x <= 1 ? 0 : 1 + ilog2(x / 2); }

// Synchronisation of the NL threads of one line: the warp itself, or (two warps) a named
// barrier of the line (ids 1.. kLines; 0 is __syncthreads).
template <int NL>
__device__ __forceinline__ void line_sync(int bar) {
  if constexpr (NL == 32) {
    __syncwarp();
  } else {
    asm volatile("bar.sync %0, %1;" ::"r"(bar), "n"(NL) : "memory");
  }
}

// Shared-memory shape of one line of NL lanes (NL = 32: one warp, 64: two warps), in elements.
template <typename T, int P, int NL>
struct Shape {
  // P dividing NL: transpose + G = NL / P lanes per sub-transform (G <= 32, inside a warp).
  // P = 3 2^k (NL = 32 only): no transpose, the second factor is a 32-point transform across
  // all lanes (shuffles only).
  static constexpr bool kShuffle = (NL % P) != 0;
  static_assert(!kShuffle || NL == 32, "3 2^k lines use one warp");
  static constexpr int M = NL * P, N = 2 * M, G = kShuffle ? 32 : NL / P, S = NL + G, LG = ilog2(G);
  static_assert(G <= 32, "cross-lane stage must stay inside a warp");
  // line / transpose / natural-order spectrum share one buffer: max(n + 1, 2 P S) = n + 2 NL
  static constexpr int kU = N + 2 * NL;
  // prefix-sum workspace, chunk of P padded by one (index k + k / P), plus the warp-total slot
  static constexpr int kD = M + NL + 4;
  // per-line stride: 16-byte aligned and 32 / kLines (mod 32) words apart, so that the lines
  // of a block sit in different banks for the column-wise (transposing) copies
  static constexpr int words = (int)(sizeof(T) / 4);
  static constexpr int stride_from(int s) {
    return ((s * words) % 32 == 32 / kLines && (s * (int)sizeof(T)) % 16 == 0) ? s : stride_from(s + 1);
  }
  static constexpr int kStride = stride_from(kU + kD);
};

// In-place DST-I (F convention) of U[1..n-1] by the NL threads of a line (lane = 0..NL-1, bar
// = the line's barrier id); U[0] and U[n] are read as zero.  U: Shape::kU elements, D:
// Shape::kD, both private to the line.
template <typename T, int P, int NL>
__device__ __forceinline__ void line_dst(T* U, T* D, const DstAxis<T>& ax, int lane, int bar) {
  using V = c2_t<T>;
  using Sh = Shape<T, P, NL>;
  constexpr int M = Sh::M, N = Sh::N, G = Sh::G, S = Sh::S;
  const int wl = lane & 31;  // lane within its warp
  V z[P];
  // 1. u_j = sin(pi j/n)(y_j + y_{n-j}) + (y_j - y_{n-j})/2, paired into complex points
#pragma unroll
  for (int r = 0; r < P; ++r) {
    const int m = lane + NL * r;
    const int j0 = 2 * m, j1 = j0 + 1;
    const T a0 = j0 ? U[j0] : T(0);
    const T b0 = j0 ? U[N - j0] : T(0);
    const T a1 = U[j1], b1 = U[N - j1];
    const V sn = __ldg(&ax.wsn[r * NL + lane]);
    z[r] = mk<V>(fmaT(sn.x, a0 + b0, T(0.5) * (a0 - b0)), fmaT(sn.y, a1 + b1, T(0.5) * (a1 - b1)));
  }
  line_sync<NL>(bar);
  // 2. DFT_P over r, twiddle, transpose
  LaneDft<T, P>::run(z);
#pragma unroll
  for (int a = 1; a < P; ++a) z[a] = cmul(z[a], __ldg(&ax.wtw1[a * NL + lane]));
  V* X = reinterpret_cast<V*>(U);
  // P = 3 2^k: the sub-transform index stays a = c, one group of 32 lanes
  const int ap = Sh::kShuffle ? 0 : lane / G, g = Sh::kShuffle ? lane : lane % G;
  if constexpr (!Sh::kShuffle) {
#pragma unroll
    for (int a = 0; a < P; ++a) X[a * S + lane] = z[a];
    line_sync<NL>(bar);
#pragma unroll
    for (int i = 0; i < P; ++i) z[i] = X[ap * S + g + G * i];
    // 3. DFT_P over i, twiddle
    LaneDft<T, P>::run(z);
#pragma unroll
    for (int c = 1; c < P; ++c)
      if (G > 1) z[c] = cmul(z[c], __ldg(&ax.wtw2[c * NL + lane]));
  }
  // DFT_G across the group (its G lanes are consecutive inside one warp)
  if (G > 1) {
#pragma unroll
    for (int s = 0; s < Sh::LG; ++s) {
      const int h = G >> (s + 1);
      const bool upper = (lane & h) != 0;
      const V w = __ldg(&ax.wtw3[s * NL + lane]);
#pragma unroll
      for (int c = 0; c < P; ++c) {
        V p;
        p.x = __shfl_xor_sync(kFull, z[c].x, h);
        p.y = __shfl_xor_sync(kFull, z[c].y, h);
        z[c] = upper ? cmul(csub(p, z[c]), w) : cadd(z[c], p);
      }
    }
  }
  const int d = (G > 1) ? (int)(__brev((unsigned)g) >> (32 - Sh::LG)) : 0;
  line_sync<NL>(bar);
  // 4. natural order, real split (pairs k, M-k), prefix sum
  if constexpr (Sh::kShuffle) {
#pragma unroll
    for (int c = 0; c < P; ++c) X[c + P * d] = z[c];
  } else {
#pragma unroll
    for (int c = 0; c < P; ++c) X[ap + P * c + P * P * d] = z[c];
  }
  line_sync<NL>(bar);
  T* L = U;
#pragma unroll
  for (int t = 0; t < (P + 1) / 2; ++t) {
    const int k = lane + NL * t;
    if (2 * k >= M) break;  // P == 1: lanes NL/2.. have no pair
    const V zk = X[k];
    if (k == 0) {
      D[0] = T(0.5) * (zk.x + zk.y);  // D_0 / 2
    } else {
      const V zm = X[M - k];
      const T er = T(0.5) * (zk.x + zm.x), ei = T(0.5) * (zk.y - zm.y);
      const T orr = T(0.5) * (zk.y + zm.y), oi = T(0.5) * (zm.x - zk.x);
      const V w = __ldg(&ax.post[k]);
      const T tr = w.x * orr - w.y * oi, ti = w.x * oi + w.y * orr;
      L[2 * k] = -(ei + ti);
      D[k + k / P] = er + tr;
      L[2 * (M - k)] = ei - ti;
      D[(M - k) + (M - k) / P] = er - tr;
    }
  }
  if (lane == 0) {
    const V zh = X[M / 2];
    L[M] = zh.y;                      // F_M
    D[M / 2 + (M / 2) / P] = zh.x;
  }
  line_sync<NL>(bar);
  // F_{2k+1} = D_0/2 + D_1 + ... + D_k: compensated chunk sums (chunk = P values per lane),
  // scan of the chunk totals across the warp (and across the pair of warps)
  T cs[P];
  T acc = T(0), comp = T(0);
#pragma unroll
  for (int i = 0; i < P; ++i) {
    const T y = D[lane * (P + 1) + i] - comp;
    const T tmp = acc + y;
    comp = (tmp - acc) - y;
    acc = tmp;
    cs[i] = acc;
  }
  T incl = acc;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T v = __shfl_up_sync(kFull, incl, o);
    if (wl >= o) incl += v;
  }
  T excl = __shfl_up_sync(kFull, incl, 1);
  if (wl == 0) excl = T(0);
  if constexpr (NL == 64) {
    T* wtot = D + Sh::kD - 2;
    if (lane == 31) wtot[0] = incl;
    line_sync<NL>(bar);
    if (lane >= 32) excl += wtot[0];
  }
#pragma unroll
  for (int i = 0; i < P; ++i) D[lane * (P + 1) + i] = cs[i] + excl;
  line_sync<NL>(bar);
#pragma unroll
  for (int t = 0; t < P; ++t) {
    const int k = lane + NL * t;
    L[2 * k + 1] = D[k + k / P];
  }
  line_sync<NL>(bar);
}

// lanes per line for an axis with warp-per-line tables (the tables are built for this width)
template <typename T> __host__ __device__ inline int line_lanes(const DstAxis<T>& ax) { return ax.wNL; }

}  // namespace wdst
}  // namespace ib
