// Sine transforms as BF16x3 split-precision GEMMs on the 5th-generation tensor cores (tcgen05),
// the dense form of the DST-I passes of the Poisson / Crank-Nicolson solves
// (reference: the FFTW RODFT00 plan of src/streamfcn/fluid-ops.jl:24-25, executed at :49, :51).
//
// A line transform F_k = sum_{j=1}^{n-1} u_j sin(pi j k / n), k = 1..n-1 (the half-scaled
// convention of the other passes), is one row of the product U S with the n x n sine matrix
// S[j][k] = sin(pi j k / n): index 0 of both factors is a zero row / column, so the product is an
// exact n x n x n GEMM per block of lines.  Both factors are split into BF16 parts, u = u_hi +
// u_lo, S = S_hi + S_lo, and the three products u_hi S_hi + u_hi S_lo + u_lo S_hi accumulate in
// FP32 in tensor memory (the dropped u_lo S_lo and the split remainders are ~2^-17 of the terms).
// The refinement sweeps of the mixed-precision solve take the result from there to float-float
// accuracy, as they do for the FP32 FFT passes.
//
// Kernel (one CTA = 128 lines x BN outputs, K = n in chunks of 64, two smem stages):
//   * all 8 warps load the chunk's line values (FP32, any row stride; one chunk ahead, so the
//     loads are in flight while the previous chunk's MMAs run), split them into BF16 hi / lo
//     and store them in the 128-byte-swizzled K-major layout the MMA reads (8-row x 128-byte
//     atoms, 16-byte units XOR-ed with the row in the atom);
//   * the sine operand is stored in global memory already in that tile image, per
//     (N tile, K chunk, part), and one thread brings each 32 KB part in with one bulk copy
//     (cp.async.bulk, completion counted on an mbarrier);
//   * one thread issues 4 K-steps x 3 products of tcgen05.mma (M 128, N BN, K 16, BF16 in, FP32
//     accumulate in TMEM) and commits them to the stage's mbarrier, which frees the stage;
//   * epilogue: the 8 warps read the accumulator with tcgen05.ld (warp w: TMEM lanes 32 (w mod
//     4).., column half w / 4) and store the tile row-major (optionally times a spectral
//     multiplier, or summed into a float-float iterate) or transposed.
// Every mbarrier wait is bounded (about one second of SM clock): on expiry the CTA records
// status[3], waits (bounded) for its own bulk copies and MMAs in flight, frees its tensor memory
// and returns.
#include "ib_common.cuh"
#include "tcgen05.cuh"

#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <vector>

namespace ib {
namespace {
using namespace tc;

constexpr int BM = 128;                 // lines per CTA (MMA M)
constexpr int BK = 64;                  // K per chunk: one 128-byte swizzle row of BF16
constexpr int kThreads = 256;
constexpr int kStages = 2;

template <int BN> struct Tile {
  static constexpr int kA = BM * BK * 2;       // bytes of one BF16 part of the line tile
  static constexpr int kB = BN * BK * 2;       // bytes of one BF16 part of the sine tile
  static constexpr int kStage = 2 * kA + 2 * kB;
  static constexpr int kSmem = kStages * kStage + 1024;  // + alignment slack
};

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major, M x N.
template <int BN>
__host__ __device__ constexpr uint32_t idesc_bf16() {
  return idesc_bf16_mn<BM, BN>();
}

template <int BN, int MODE>
__global__ void __launch_bounds__(kThreads, 1)
k_sgemm(SgIn in, SgOut o, const uint16_t* __restrict__ img, int n, int* __restrict__ status) {
  using TL = Tile<BN>;
  extern __shared__ unsigned char smem_raw[];
  __shared__ uint64_t full[kStages], empty[kStages];
  __shared__ uint32_t tmem_slot;
  unsigned char* sm = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023)) & 1023);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nt = blockIdx.x, m0 = blockIdx.y * BM;
  const int nkc = n / BK;
  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    fence_mbar_init();
    fence_async_smem();
  }
  if (warp == 0) tmem_alloc(&tmem_slot, BN);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  constexpr uint32_t kIdesc = idesc_bf16<BN>();
  // thread 0's record of asynchronous work in flight, for a bounded drain after a timeout
  int issued_b[kStages] = {0, 0}, waited_b[kStages] = {0, 0}, committed[kStages] = {0, 0}, drained[kStages] = {0, 0};
  bool bad = false;
  // line values of one K chunk: warp w owns rows 16 w .. 16 w + 15, lane l the K pair (2l, 2l+1)
  float va[16], vb[16];
  auto load_chunk = [&](int cc) {
    const int j0 = cc * BK + 2 * lane;  // K index of the pair's first element (input j0 - 1)
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const int r = m0 + warp * 16 + i;
      const float* row = in.a + (int64_t)r * in.lda;
      const bool ok = r < in.rows;
      va[i] = (ok && j0 >= 1 && j0 <= in.klen) ? row[j0 - 1] : 0.0f;
      vb[i] = (ok && j0 + 1 <= in.klen) ? row[j0] : 0.0f;
    }
  };
  load_chunk(0);
  int c = 0;
  for (; c < nkc; ++c) {
    const int s = c & 1;
    const uint32_t u = (uint32_t)(c >> 1);
    unsigned char* A_hi = sm + s * TL::kStage;
    unsigned char* A_lo = A_hi + TL::kA;
    unsigned char* B_hi = A_lo + TL::kA;
    unsigned char* B_lo = B_hi + TL::kB;
    // stage s was last read by the MMAs of chunk c - 2
    if (c >= 2) {
      if (!mbar_wait(&empty[s], (u - 1) & 1)) bad = true;
      else if (tid == 0) drained[s] = committed[s];
    }
    if (__syncthreads_or(bad)) break;
    if (tid == 0) {
      const uint16_t* src = img + ((int64_t)nt * nkc + c) * 2 * (BN * BK);
      mbar_expect_tx(&full[s], 2 * TL::kB);
      bulk_g2s(B_hi, src, TL::kB, &full[s]);
      bulk_g2s(B_lo, src + BN * BK, TL::kB, &full[s]);
      issued_b[s]++;
    }
    // the chunk's line values (loaded during the previous chunk) into the swizzled tiles, then
    // the next chunk's values into registers, in flight while this chunk's MMAs run
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const int rr = warp * 16 + i;
      uint32_t lo;
      const uint32_t hi = split_pair(va[i], vb[i], lo);
      const uint32_t off = sw128_off(rr, lane);
      *reinterpret_cast<uint32_t*>(A_hi + off) = hi;
      *reinterpret_cast<uint32_t*>(A_lo + off) = lo;
    }
    fence_async_smem();
    __syncthreads();
    if (c + 1 < nkc) load_chunk(c + 1);
    if (tid == 0) {
      if (!mbar_wait(&full[s], u & 1)) {
        bad = true;
      } else {
        waited_b[s]++;
        tc_fence_after();
        const uint32_t ah = smem_u32(A_hi), al = smem_u32(A_lo), bh = smem_u32(B_hi), bl = smem_u32(B_lo);
#pragma unroll
        for (int ks = 0; ks < BK / 16; ++ks) {
          const uint32_t o32 = ks * 32;  // 16 BF16 = 32 bytes along K inside the swizzle row
          const uint32_t acc0 = (c > 0 || ks > 0) ? 1u : 0u;
          umma_bf16(tmem, sw128_desc(ah + o32), sw128_desc(bl + o32), kIdesc, acc0);
          umma_bf16(tmem, sw128_desc(al + o32), sw128_desc(bh + o32), kIdesc, 1u);
          umma_bf16(tmem, sw128_desc(ah + o32), sw128_desc(bh + o32), kIdesc, 1u);
        }
        umma_commit(&empty[s]);
        committed[s]++;
      }
    }
  }
  // all MMAs done (the last commit covers every earlier one), or drain after a timeout
  bool ok = !bad;
  if (ok) {
    const int cl = nkc - 1;
    if (!mbar_wait(&empty[cl & 1], (uint32_t)(cl >> 1) & 1)) ok = false;
  }
  if (__syncthreads_or(!ok)) {
    if (tid == 0) {
      atomicExch(status + 3, 1);
      for (int s = 0; s < kStages; ++s) {
        // bulk copies issued and never waited for, MMAs committed and never waited for
        for (int k = waited_b[s]; k < issued_b[s]; ++k) mbar_wait(&full[s], (uint32_t)k & 1);
        for (int k = drained[s]; k < committed[s]; ++k) mbar_wait(&empty[s], (uint32_t)k & 1);
      }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, BN);
    return;
  }
  tc_fence_after();
  // epilogue: warp w reads TMEM lanes 32 (w & 3) .. + 31 (tile rows), columns of half w >> 2
  if (MODE == 1) {
    // transposed store: the 32 lanes (consecutive rows) write consecutive addresses
    const int q = warp & 3, half = warp >> 2;
    const int r = m0 + 32 * q + lane;
    const bool rok = r < in.rows;
    const uint32_t tb = tmem + ((uint32_t)(32 * q) << 16);
    const int slot = rok ? r / o.rpb : 0, rr = rok ? r - slot * o.rpb : 0;
#pragma unroll 1
    for (int cc = 0; cc < BN / 2; cc += 16) {
      const int col0 = half * (BN / 2) + cc;
      float v[16];
      tmem_ld16(tb + (uint32_t)col0, v);
      if (!rok) continue;
      const int cbase = nt * BN + col0;  // output index c of v[0]; stored at c - 1
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const int cidx = cbase + i;
        if (cidx >= 1 && cidx <= o.ncols)
          static_cast<float*>(o.out)[slot * o.bstride + (int64_t)(cidx - 1) * o.ld + rr] = v[i];
      }
    }
  } else {
    // row-major results: the tile goes through shared memory (the operand stages are free now;
    // row stride BN + 1 words, so a warp's 32 rows fall in 32 banks), then every warp stores
    // whole rows, 32 consecutive columns per instruction
    float* tile = reinterpret_cast<float*>(sm);
    constexpr int TS = BN + 1;
    {
      const int q = warp & 3, half = warp >> 2;
      const uint32_t tb = tmem + ((uint32_t)(32 * q) << 16);
      float* trow = tile + (32 * q + lane) * TS;
#pragma unroll 1
      for (int cc = 0; cc < BN / 2; cc += 16) {
        const int col0 = half * (BN / 2) + cc;
        float v[16];
        tmem_ld16(tb + (uint32_t)col0, v);
#pragma unroll
        for (int i = 0; i < 16; ++i) trow[col0 + i] = v[i];
      }
    }
    __syncthreads();
    const int c_lo = max(1, nt * BN), c_hi = min(o.ncols, nt * BN + BN - 1);  // output indices c
#pragma unroll 1
    for (int rr0 = warp; rr0 < BM; rr0 += kThreads / 32) {
      const int r = m0 + rr0;
      if (r >= in.rows) break;
      const float* trow = tile + rr0 * TS - nt * BN;  // indexed by c
      const int slot = r / o.rpb, rr = r - slot * o.rpb;
      for (int cidx = c_lo + lane; cidx <= c_hi; cidx += 32) {
        const float x = trow[cidx];
        const int64_t e = (int64_t)r * o.ld + (cidx - 1);
        if (MODE == 0) {
          const float m = o.mult ? __ldg(&o.mult[slot * o.mstride + (int64_t)rr * o.ld + (cidx - 1)]) : 1.0f;
          static_cast<float*>(o.out)[e] = o.mult ? x * m : x;
        } else {
          df64 xv = o.base ? two_sum(o.base[e], o.base2 ? o.base2[e] : 0.0f) : df64(0.0f);
          xv = two_sum(xv.hi, xv.lo + x);
          df64* dst = static_cast<df64*>(o.out);
          if (o.epi == kEpiSubAddBase) dst[e] = add_sloppy(o.sub_from[e], -xv);
          else if (o.epi == kEpiAddTo) dst[e] = add_sloppy(o.sub_from[e], xv);
          else dst[e] = xv;
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, BN);
}

// --------------------------------------------------------------------------------------------
// prologue of the forward x pass (the values a row is transformed from), written as FP32 rows:
// the same arithmetic as the warp-per-line x pass (dstw_x.cuh) with the float-float input
// --------------------------------------------------------------------------------------------
template <int PRO, bool kBC>
__global__ void k_gpro(Geometry g, XArgs a, float* __restrict__ u) {
  const int ncol = g.nx - 1, nrow = g.ny - 1;
  const int64_t nG = g.nG, tot = (int64_t)a.batch * nG;
  const df64* in = static_cast<const df64*>(a.in);
  df64* rout = static_cast<df64*>(a.resid_out);
  const df64 fac = df64(a.bcfac);
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(e / nG);
    const int64_t rem = e - (int64_t)b * nG;
    const int J = (int)(rem / ncol), I = (int)(rem - (int64_t)J * ncol);
    const int64_t off = (int64_t)b * a.stride + rem;
    df64 vv = in[off];
    if (kBC) {
      const df64* bc = static_cast<const df64*>(a.bc) + (int64_t)b * g.nbc;
      auto addbc = [&](df64 q) { vv = add_sloppy(vv, a.bcfac == 1.0 ? q : fac * q); };
      if (J == 0) addbc(bc[g.B + 1 + I]);
      if (J == nrow - 1) addbc(bc[g.T + 1 + I]);
      if (I == 0) addbc(bc[g.L + 1 + J]);
      if (I == ncol - 1) addbc(bc[g.R + 1 + J]);
    }
    if (PRO == kProLoad) {
      u[e] = (float)vv;
      continue;
    }
    // refinement residual r = b [+ bc] - M x, M x = mc x + ma (4 x - neighbours)
    df64 lap, xv;
    if (PRO == kProResidD) {
      const df64* xd = a.based + (int64_t)b * a.stride;
      const df64 z(0.0f);
      const int64_t k = rem;
      const df64 c = xd[k], w = I > 0 ? xd[k - 1] : z, ee = I < ncol - 1 ? xd[k + 1] : z;
      const df64 s = J > 0 ? xd[k - ncol] : z, nn = J < nrow - 1 ? xd[k + ncol] : z;
      lap = add_sloppy(lap5_exact(c.hi, w.hi, ee.hi, s.hi, nn.hi), lap5_exact(c.lo, w.lo, ee.lo, s.lo, nn.lo));
      xv = two_sum(c.hi, c.lo);
    } else {
      auto lapf = [&](const float* x) {
        const int64_t k = rem;
        return lap5_exact(x[k], I > 0 ? x[k - 1] : 0.0f, I < ncol - 1 ? x[k + 1] : 0.0f, J > 0 ? x[k - ncol] : 0.0f,
                          J < nrow - 1 ? x[k + ncol] : 0.0f);
      };
      const float* x0 = a.base + (int64_t)b * a.stride;
      lap = lapf(x0);
      xv = df64(x0[rem]);
      if (a.base2) {
        const float* x1 = a.base2 + (int64_t)b * a.stride;
        lap = add_sloppy(lap, lapf(x1));
        xv = two_sum(xv.hi, x1[rem]);
      }
    }
    const double mcd = a.mc[b * a.mstep];
    const df64 mc = df64(mcd), ma = df64(a.ma[b * a.mstep]);
    df64 mx = ma * lap;
    if (mcd == 1.0) mx = add_sloppy(mx, xv);
    else if (mcd != 0.0) mx = add_sloppy(mx, mc * xv);
    u[e] = (vv.hi - mx.hi) + (vv.lo - mx.lo);
    if (rout) rout[off] = add_sloppy(vv, -mx);
  }
}

#define CE_RET(x)                \
  do {                           \
    cudaError_t e_ = (x);        \
    if (e_ != cudaSuccess) return e_; \
  } while (0)

int elem_blocks(int64_t n) {
  const int64_t b = (n + 255) / 256;
  return (int)(b > 8192 ? 8192 : (b < 1 ? 1 : b));
}

uint16_t f32_to_bf16(float f) {
  uint32_t x;
  std::memcpy(&x, &f, 4);
  if ((x & 0x7f800000u) == 0x7f800000u) return (uint16_t)(x >> 16);
  x += 0x7fffu + ((x >> 16) & 1u);
  return (uint16_t)(x >> 16);
}
float bf16_to_f32(uint16_t b) {
  const uint32_t x = (uint32_t)b << 16;
  float f;
  std::memcpy(&f, &x, 4);
  return f;
}

template <int BN, int MODE>
cudaError_t launch_bn(const SineGemm& ax, const SgIn& in, const SgOut& o, int* status, cudaStream_t s) {
  auto k = k_sgemm<BN, MODE>;
  cudaError_t e = set_smem_limit((const void*)k, Tile<BN>::kSmem);
  if (e != cudaSuccess) return e;
  dim3 grid(ax.n / BN, (in.rows + BM - 1) / BM);
  k<<<grid, kThreads, Tile<BN>::kSmem, s>>>(in, o, ax.img, ax.n, status);
  return cudaGetLastError();
}

}  // namespace

bool sgemm_axis_supported(int n) { return n >= 128 && n <= 4096 && n % 128 == 0; }

cudaError_t SineGemm::build(int n_) {
  release();
  if (!sgemm_axis_supported(n_)) return cudaErrorInvalidValue;
  n = n_;
  bn = (n % 256 == 0) ? 256 : 128;
  const int nkc = n / BK, nnt = n / bn;
  const size_t tile = (size_t)bn * BK;
  std::vector<uint16_t> h((size_t)nnt * nkc * 2 * tile);
  for (int t = 0; t < nnt; ++t)
    for (int c = 0; c < nkc; ++c) {
      uint16_t* hi = h.data() + ((size_t)t * nkc + c) * 2 * tile;
      uint16_t* lo = hi + tile;
      for (int r = 0; r < bn; ++r)
        for (int kk = 0; kk < BK; ++kk) {
          const int64_t nn = (int64_t)t * bn + r, jj = (int64_t)c * BK + kk;
          const int64_t m = (nn * jj) % (2 * (int64_t)n);
          const double sv = std::sin(M_PI * (double)m / (double)n);
          const uint16_t bh = f32_to_bf16((float)sv);
          const uint16_t bl = f32_to_bf16((float)(sv - (double)bf16_to_f32(bh)));
          const uint32_t off = sw128_off(r, kk >> 1) / 2 + (kk & 1);  // in BF16 elements
          hi[off] = bh;
          lo[off] = bl;
        }
    }
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, h.size() * sizeof(uint16_t));
  if (e != cudaSuccess) return e;
  img = static_cast<uint16_t*>(p);
  return cudaMemcpy(img, h.data(), h.size() * sizeof(uint16_t), cudaMemcpyHostToDevice);
}

void SineGemm::release() {
  if (img) cudaFree(img);
  img = nullptr;
  n = bn = 0;
}

cudaError_t sgemm_pass(const SineGemm& ax, const SgIn& in, const SgOut& o, int* status, cudaStream_t s) {
  if (!ax.img || in.rows <= 0) return in.rows < 0 ? cudaErrorInvalidValue : cudaSuccess;
  if (in.klen > ax.n - 1 || o.ncols > ax.n - 1) return cudaErrorInvalidValue;
  switch (o.mode * 1000 + ax.bn) {
    case 256: return launch_bn<256, 0>(ax, in, o, status, s);
    case 128: return launch_bn<128, 0>(ax, in, o, status, s);
    case 1256: return launch_bn<256, 1>(ax, in, o, status, s);
    case 1128: return launch_bn<128, 1>(ax, in, o, status, s);
    case 2256: return launch_bn<256, 2>(ax, in, o, status, s);
    case 2128: return launch_bn<128, 2>(ax, in, o, status, s);
    default: return cudaErrorInvalidValue;
  }
}

// ---- the three passes of a solve in GEMM form ----------------------------------------------
// x forward: prologue rows u[b][J][I] (FP32, into `rows`) -> S_x -> transposed out[b][I][J]
cudaError_t gx_fwd(const Geometry& g, const SineGemm& ax, const XArgs& a, float* rows, int* status, cudaStream_t s) {
  if (a.batch <= 0) return cudaSuccess;
  if (a.stride != g.nG || ax.n != g.nx) return cudaErrorInvalidValue;
  ProfScope prof(kClassXPass, s);
  const int64_t tot = (int64_t)a.batch * g.nG;
  const bool bc = a.bc != nullptr;
  const int nb = elem_blocks(tot);
  switch (a.pro) {
    case kProLoad:
      if (bc) k_gpro<kProLoad, true><<<nb, 256, 0, s>>>(g, a, rows);
      else k_gpro<kProLoad, false><<<nb, 256, 0, s>>>(g, a, rows);
      break;
    case kProResid:
      if (!a.base || !a.mc || !a.ma) return cudaErrorInvalidValue;
      if (bc) k_gpro<kProResid, true><<<nb, 256, 0, s>>>(g, a, rows);
      else k_gpro<kProResid, false><<<nb, 256, 0, s>>>(g, a, rows);
      break;
    case kProResidD:
      if (!a.based || !a.mc || !a.ma) return cudaErrorInvalidValue;
      if (bc) k_gpro<kProResidD, true><<<nb, 256, 0, s>>>(g, a, rows);
      else k_gpro<kProResidD, false><<<nb, 256, 0, s>>>(g, a, rows);
      break;
    default: return cudaErrorInvalidValue;
  }
  CE_RET(cudaGetLastError());
  const int ncol = g.nx - 1, nrow = g.ny - 1;
  SgIn in{rows, ncol, a.batch * nrow, ncol};
  SgOut o{};
  o.mode = 1; o.out = a.out; o.ld = nrow; o.rpb = nrow; o.bstride = g.nG; o.ncols = ncol;
  return sgemm_pass(ax, in, o, status, s);
}

// y: transposed rows in[b][I][J] -> S_y, times m -> work -> S_y -> out[b][J][I] (row-major)
cudaError_t gy_pass(const Geometry& g, const SineGemm& ay, const YPassArgs<float>& a, float* work, int* status,
                    cudaStream_t s) {
  if (a.batch <= 0) return cudaSuccess;
  // a.out may be a.in1: the first product has read all of it before the second one writes
  if (a.stride != g.nG || ay.n != g.ny || a.op != SpecOp::kScale || a.out == work) return cudaErrorInvalidValue;
  ProfScope prof(kClassYPass, s);
  const int ncol = g.nx - 1, nrow = g.ny - 1;
  SgIn in{a.in1, nrow, a.batch * ncol, nrow};
  SgOut o{};
  o.mode = 0; o.out = work; o.ld = nrow; o.rpb = ncol; o.mult = a.m1; o.mstride = a.mstride; o.ncols = nrow;
  CE_RET(sgemm_pass(ay, in, o, status, s));
  SgIn in2{work, nrow, a.batch * ncol, nrow};
  SgOut o2{};
  o2.mode = 1; o2.out = a.out; o2.ld = ncol; o2.rpb = ncol; o2.bstride = g.nG; o2.ncols = nrow;
  return sgemm_pass(ay, in2, o2, status, s);
}

// x inverse: row-major in[b][J][I] -> S_x -> epilogue (FP32 store, or a float-float sum)
template <typename Tout>
cudaError_t gx_inv(const Geometry& g, const SineGemm& ax, const XArgs& a, int* status, cudaStream_t s) {
  if (a.batch <= 0) return cudaSuccess;
  if (a.stride != g.nG || ax.n != g.nx || a.bc) return cudaErrorInvalidValue;
  ProfScope prof(kClassXPass, s);
  const int ncol = g.nx - 1, nrow = g.ny - 1;
  SgIn in{static_cast<const float*>(a.in), ncol, a.batch * nrow, ncol};
  SgOut o{};
  o.out = a.out; o.ld = ncol; o.rpb = nrow; o.ncols = ncol;
  if constexpr (std::is_same<Tout, float>::value) {
    if (a.epi != kEpiStore) return cudaErrorInvalidValue;
    o.mode = 0;
  } else {
    if (a.epi != kEpiAddBase && a.epi != kEpiSubAddBase && a.epi != kEpiAddTo) return cudaErrorInvalidValue;
    if ((a.epi != kEpiAddBase) && !a.sub_from) return cudaErrorInvalidValue;
    o.mode = 2;
    o.base = a.base; o.base2 = a.base2; o.sub_from = static_cast<const df64*>(a.sub_from); o.epi = a.epi;
  }
  return sgemm_pass(ax, in, o, status, s);
}

template cudaError_t gx_inv<float>(const Geometry&, const SineGemm&, const XArgs&, int*, cudaStream_t);
template cudaError_t gx_inv<df64>(const Geometry&, const SineGemm&, const XArgs&, int*, cudaStream_t);

}  // namespace ib
