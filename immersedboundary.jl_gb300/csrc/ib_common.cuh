// Internal declarations shared by the translation units of libibgb300.
//
// Layout conventions (identical to the reference's column-major Julia arrays):
//   circulation / streamfunction level: (nx-1)*(ny-1), index i + (nx-1)*j, i fastest
//   flux level: [qx (nx+1)*ny ; qy nx*(ny+1)], each i fastest
//   boundary ring: 2(nx+1)+2(ny+1) values with offsets L=0, R=ny+1, B=2(ny+1), T=B+nx+1
//   body forces: [fx_1..fx_nb, fy_1..fy_nb]
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <cstdint>

#include "df64.cuh"
#include <string>
#include <vector>

// Resident blocks per SM the x / y pass kernels are compiled for, which caps their registers
// (x: 128 per thread, y: 85).  By measurement on GB300 (mixed step, device time): 1.355 ms per
// 1024^2 x 4 step and 0.541 ms per 512^2 x 4 step with (4, 6), against 1.405 / 0.587 uncapped
// (the residual x pass then used 168 registers, 3 blocks per SM) and 1.477 / 0.565 with x at 5.
// The FP32 inverse x pass alone at 6 or 8 blocks (80 / 64 registers, no or 4-8 byte spills):
// 1.201 / 1.205 ms per 1024^2 x 4 step and 4.72 / 4.86 ms per 2048^2 x 5 step, against 1.197 /
// 4.70 at 4: the passes are bound by instruction issue, not by resident warps.
#ifndef IB_WDST_XMINB
#define IB_WDST_XMINB 4
#endif
#ifndef IB_WDST_YMINB
#define IB_WDST_YMINB 6
#endif
// (the y pass is also compiled for 8 blocks per SM; the autotuner may choose it per grid)

namespace ib {

// ----------------------------------------------------------------------------------------------
// complex helpers (forward transforms use e^{-2 pi i / N})
// ----------------------------------------------------------------------------------------------
template <typename T> struct C2;
template <> struct C2<double> { using type = double2; };
template <> struct C2<float> { using type = float2; };
template <typename T> using c2_t = typename C2<T>::type;

template <typename V> __host__ __device__ __forceinline__ V mk(decltype(V::x) a, decltype(V::x) b) {
  V v; v.x = a; v.y = b; return v;
}
template <typename V> __device__ __forceinline__ V cadd(V a, V b) { return mk<V>(a.x + b.x, a.y + b.y); }
template <typename V> __device__ __forceinline__ V csub(V a, V b) { return mk<V>(a.x - b.x, a.y - b.y); }
template <typename V> __device__ __forceinline__ V cmul(V a, V b) {
  return mk<V>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// multiply by -i
template <typename V> __device__ __forceinline__ V cmul_mi(V a) { return mk<V>(a.y, -a.x); }

// ----------------------------------------------------------------------------------------------
// Transform tables for one axis: DST-I of the n-1 interior values of an n-cell axis,
// computed as a half-length (M = n/2) complex FFT (Stockham, mixed radix 8/4/2/3/5).
// ----------------------------------------------------------------------------------------------
constexpr int kMaxStages = 10;

template <typename T> struct DstAxis {
  int n;                    // cells along the axis (array length n-1)
  int M;                    // n/2, complex FFT length
  int nstages;
  int radix[kMaxStages];
  const c2_t<T>* tw;        // [M]      e^{-2 pi i p / M}
  const T* sintab;          // [n/2+1]  sin(pi j / n)
  const c2_t<T>* post;      // [M/2+1]  e^{-2 pi i k / n}
  // line-parallel transforms (dstw.cuh): M = wNL wP, wNL = 32 (one warp per line) or 64 (two);
  // wP = 0 for axes without them.  Tables in lane order (entry [s][lane] at s*wNL + lane),
  // G = wNL / wP (or 32 when wP does not divide wNL):
  int wP, wNL;
  int wMinB;                // y pass: resident blocks per SM of the compiled variant to use
  const c2_t<T>* wtw1;      // [wP][wNL]     e^{-2 pi i lane a / M}
  const c2_t<T>* wtw2;      // [wP][wNL]     e^{-2 pi i (lane mod G) c / wNL}
  const c2_t<T>* wtw3;      // [log2 G][wNL] radix-2 twiddles of the cross-lane stages
  const c2_t<T>* wsn;       // [wP][wNL]     (sin(pi 2m/n), sin(pi (2m+1)/n)), m = lane + wNL r
};

struct Geometry {
  int nx, ny, nlev;
  int nG, nq, nu, nbc;
  int L, R, B, T;           // ring offsets
  double h, x0, y0;
};

inline Geometry make_geometry(int nx, int ny, int nlev, double h, double x0, double y0) {
  Geometry g;
  g.nx = nx; g.ny = ny; g.nlev = nlev;
  g.nG = (nx - 1) * (ny - 1);
  g.nu = (nx + 1) * ny;
  g.nq = g.nu + nx * (ny + 1);
  g.nbc = 2 * (nx + 1) + 2 * (ny + 1);
  g.L = 0; g.R = ny + 1; g.B = 2 * (ny + 1); g.T = 2 * (ny + 1) + nx + 1;
  g.h = h; g.x0 = x0; g.y0 = y0;
  return g;
}

// Host-side owner of the device tables of one axis.
template <typename T> struct AxisTables {
  DstAxis<T> d{};
  void* mem = nullptr;
  cudaError_t build(int n);
  void release();
};

bool dst_axis_supported(int n);
// both axes have warp-per-line tables: the solves use the dstw passes (transposed intermediate)
bool wdst_axis_supported(int n);

// Raise a kernel's dynamic shared-memory limit (once per device; never inside stream capture).
cudaError_t set_smem_limit(const void* fn, size_t bytes);

// ----------------------------------------------------------------------------------------------
// DST passes (dst.cu)
// ----------------------------------------------------------------------------------------------
// Every pass takes arrays of (nx-1)*(ny-1) values; `batch` arrays live at stride nG.
// Spectral multipliers are stored per array slot with stride `mstride` (0 = shared).
enum class SpecOp : int {
  kScale = 0,      // out = S_y(m1 * S_y(in1))
  kFwd = 2,        // out = scal * S_y(in1)   (one transform only)
};

// x pass: a 1-D sine transform along x of every row of `batch` arrays (compute type T).
// prologue (how a row is formed before the transform):
//   kProLoad   row = in                                  (in: Tin)
//   kProResid  row = in - M x0, M x = mc*x + ma*rot(curl(x)), formed in FP64
//              (x0 = base, or base + base2 when base2 is given: an exact FP32 pair)
//   kProResidD the same with a float-float x0 (based; warp passes, float-float input)
// either optionally plus fac * apply_bc(bc) on the edges (bc != nullptr)
// epilogue (what is stored):
//   kEpiStore       out = row                              (out: Tout)
//   kEpiSub         out = sub_from - row
//   kEpiAddBase     out = base [+ base2] + row             (FP64 sum)
//   kEpiSubAddBase  out = sub_from - (base [+ base2] + row)
//   kEpiAddTo       out = sub_from + (base [+ base2] + row)  (float-float output; out may be sub_from)
enum XPro : int { kProLoad = 0, kProResid = 1, kProResidD = 2 };
enum XEpi : int { kEpiStore = 0, kEpiSub = 1, kEpiAddBase = 2, kEpiSubAddBase = 3, kEpiAddTo = 4 };

struct XArgs {
  const void* in;           // Tin
  void* out;                // Tout
  int batch;
  int64_t stride;           // elements between batch slots (in, out, base, sub_from)
  const void* bc;           // apply_bc ring per slot (stride nbc) or nullptr; element type is the
  double bcfac;             //   pass's exact type (double, or df64 in the mixed path)
  const void* sub_from;     // kEpiSub / kEpiSubAddBase (same element type as bc)
  const float* base;        // x0 of the refinement (kProResid, kEpiAddBase)
  const float* base2;       // optional second FP32 part of x0 (second refinement sweep)
  const df64* based;        // float-float x0 (kProResidD)
  const double* mc;         // residual operator per slot (stride mstep)
  const double* ma;
  int mstep;
  int pro, epi;
  void* resid_out;          // optional (warp passes, float-float input): the residual itself, float-float
  void* sub2;               // optional with kEpiAddTo (warp passes): sub2 -= out as well, float-float
};

template <typename T, typename Tin, typename Tout>
cudaError_t xpass(const Geometry& g, const DstAxis<T>& ax, const XArgs& a, cudaStream_t s);

template <typename T>
struct YPassArgs {
  const T* in1; T* out; int batch; int64_t stride;
  const T* m1; int64_t mstride;                // multipliers (per slot stride)
  SpecOp op;
  T scal;                                      // kFwd scale
};

template <typename T>
cudaError_t ypass(const Geometry& g, const DstAxis<T>& ax, const YPassArgs<T>& a, cudaStream_t s);

// Warp-per-line passes (dstw_*.cu), for axes with wdst_axis_supported.  The intermediate of a
// solve is stored transposed, column by column: element (I, J) of slot b at b*stride + I*(ny-1) + J.
//   wx_fwd: prologue (XArgs.pro, bc) -> x transform -> transposed store into a.out (type T)
//   wypass: per column of the transposed array: S_y, multiply (or scale), S_y (kScale only)
//   wx_inv: transposed load of a.in (type T) -> x transform -> epilogue (XArgs.epi) into a.out
template <typename T, typename Tin>
cudaError_t wx_fwd(const Geometry& g, const DstAxis<T>& ax, const XArgs& a, cudaStream_t s);
template <typename T>
cudaError_t wypass(const Geometry& g, const DstAxis<T>& ax, const YPassArgs<T>& a, cudaStream_t s);
template <typename T, typename Tout>
cudaError_t wx_inv(const Geometry& g, const DstAxis<T>& ax, const XArgs& a, cudaStream_t s);


// ----------------------------------------------------------------------------------------------
// Sine transforms as BF16x3 tensor-core GEMMs (sgemm.cu), for axes of n = 128 k cells
// ----------------------------------------------------------------------------------------------
// Operand rows: row r (r < rows) at a + r*lda holds the klen inputs u_1..u_klen of one line.
struct SgIn {
  const float* a;
  int64_t lda;
  int rows;
  int klen;
};
// Result of row r, output index c = 1..ncols (stored at c - 1):
//   mode 0: out[r*ld + c-1] (FP32), times mult[(r/rpb)*mstride + (r mod rpb)*ld + c-1] if given
//   mode 1: out[(r/rpb)*bstride + (c-1)*ld + r mod rpb] (FP32, transposed within each slot)
//   mode 2: out[r*ld + c-1] float-float = base [+ base2] + value (epi kEpiAddBase), or
//           sub_from -/+ that (kEpiSubAddBase / kEpiAddTo)
struct SgOut {
  int mode;
  void* out;
  int64_t ld;
  int rpb;
  int64_t bstride;
  const float* mult;
  int64_t mstride;
  int ncols;
  const float* base;
  const float* base2;
  const df64* sub_from;
  int epi;
};
// Device image of one axis' sine matrix S[k][j] = sin(pi j k / n), split into BF16 hi / lo parts,
// laid out as the tensor-core tiles of the transform (bn outputs x 64 inputs per tile).
struct SineGemm {
  int n = 0, bn = 0;
  uint16_t* img = nullptr;
  cudaError_t build(int n);
  void release();
};
bool sgemm_axis_supported(int n);
// one batched line transform (status[3] is set if a pipeline wait of the kernel ran out)
cudaError_t sgemm_pass(const SineGemm& ax, const SgIn& in, const SgOut& o, int* status, cudaStream_t s);
// The passes of a solve in GEMM form (stride == nG):
//   gx_fwd:  prologue (XArgs.pro, bc) into FP32 rows `rows` -> S_x -> a.out transposed [b][I][J]
//   gy_pass: a.in1 [b][I][J] -> S_y, times m1 -> work -> S_y -> a.out row-major [b][J][I]
//   gx_inv:  a.in row-major FP32 -> S_x -> FP32 store (kEpiStore) or float-float epilogue
cudaError_t gx_fwd(const Geometry& g, const SineGemm& ax, const XArgs& a, float* rows, int* status, cudaStream_t s);
cudaError_t gy_pass(const Geometry& g, const SineGemm& ay, const YPassArgs<float>& a, float* work, int* status,
                    cudaStream_t s);
template <typename Tout>
cudaError_t gx_inv(const Geometry& g, const SineGemm& ax, const XArgs& a, int* status, cudaStream_t s);

// ----------------------------------------------------------------------------------------------
// stencils (stencil.cu)
// ----------------------------------------------------------------------------------------------
template <typename T>
cudaError_t get_bc(const Geometry& g, const T* r, T* bc, int batch, T extra_scale, cudaStream_t s);
template <typename T>
cudaError_t apply_bc(const Geometry& g, T* r, const T* bc, T fac, int batch, cudaStream_t s);
template <typename T>
cudaError_t coarsify(const Geometry& g, T* gc, const T* gf, int batch, int64_t stride, cudaStream_t s);
template <typename T>
cudaError_t curl(const Geometry& g, const T* psi, const T* bc, T* q, int batch, cudaStream_t s);
template <typename T>
cudaError_t rot(const Geometry& g, const T* q, T* gam, int batch, cudaStream_t s);

// Trial-state explicit part for all levels at once.  For each level (0-based l):
//   nl_new[l] = rot(direct_product(avg_flux(q[l] + q0[l]), gamma[l], bcn[l])) / hc_l^2
//   rhs[l]    = A_l gamma[l] + dt*beta0*nl_new[l] + dt*beta1*nl_old[l] + rhsbc edges of level l
// where A_l = I - alpha_l * rot(curl(.)) (the 5-point Laplacian with zero boundary values,
// alpha_l = dt / (2 Re hc_l^2)) is the explicit Crank-Nicolson operator that the reference
// applies through its sine transform (its eigenvalues are 1 - alpha_l * lap_eigs).
// bcn[l] is the nonlinear boundary ring (zero for the coarsest level); rhsbc edges are
// given as 4 edge vectors per level (bottom/top: nx-1, left/right: ny-1).
template <typename T>
struct NonlinArgs {
  const T* q; const T* gamma; const T* bcn; const T* nl_old; const T* edges;
  T* nl_new; T* rhs;
  const double* q0;        // [nlev][2] (u hc, v hc)
  const double* inv_hc2;   // [nlev]
  const double* alpha;     // [nlev] dt/(2 Re hc^2); nullptr: rhs without the A_l gamma term
  double dtb0, dtb1;
};
template <typename T>
cudaError_t nonlin_rhs(const Geometry& g, const NonlinArgs<T>& a, cudaStream_t s);
// one stage of the Runge-Kutta-Chebyshev scheme (stencil.cu: k_rkc_stage)
cudaError_t rkc_stage(int64_t n, double* Y, const double* Y0, const double* Ym1, const double* Ym2, const double* G,
                      double* F0, double a0, double a1, double a2, double c1, double c0, bool store_f0, cudaStream_t s);

// Trial-step boundary rings: bcn[l] (nonlinear ring, already x0.25x0.25) for l < nlev-1 and
// the accumulated rhsbc edge vectors of every level (reference quirk: never reset).
template <typename T>
cudaError_t trial_rings(const Geometry& g, const T* gamma, T* bcn, T* edges, const double* fac,
                        cudaStream_t s, bool accumulate = true);

// ----------------------------------------------------------------------------------------------
// bodies (body.cu)
// ----------------------------------------------------------------------------------------------
constexpr int kSupp = 6;
constexpr int kWin = 2 * kSupp + 1;   // 13
constexpr int kWin2 = kWin * kWin;    // 169

// weights [nb][2][13][13] (component, y offset b, x offset a); body_idx [nb][2]
cudaError_t reg_update(const Geometry& g, const double* xb, int nb, int* body_idx, double* weight,
                       int* status, cudaStream_t s);
// E: fb[k + c*nb] = sum_w weight * q_c(window), with q = q1 + q0; q0 is a device pointer to the
// uniform level-1 base flux (q0x, q0y) or nullptr
template <typename T>
cudaError_t reg_gather(const Geometry& g, const T* q, const double* q0, const int* body_idx,
                       const double* weight, int nb, double* fb, int ncols, int64_t qstride,
                       int64_t fstride, cudaStream_t s);
// E^T followed by rot: gamma_out = rot(E^T f) (whole array written).  With box (4 ints of
// device memory) the scatter and the rot's reads cover only the face box of the points'
// windows, and qtmp is left unwritten outside it; the box is found on the device first unless
// box_ready (it already holds body_box of the current points).
template <typename T>
cudaError_t reg_scatter_rot(const Geometry& g, const double* f, const int* body_idx,
                            const double* weight, int nb, T* qtmp, T* gam, int ncols,
                            int64_t fstride, int* status, int* box, bool box_ready, cudaStream_t s);
// box = {i_lo, i_hi, j_lo, j_hi}: the flux faces every point's 13x13 window covers
cudaError_t body_box(const Geometry& g, const int* body_idx, int nb, int* box, cudaStream_t s);
// E^T alone (operator test entry point)
template <typename T>
cudaError_t reg_scatter(const Geometry& g, const double* f, const int* body_idx, const double* weight,
                        int nb, T* q, int* status, cudaStream_t s);
// unit-vector columns: f[c][r] = (r == col0 + c)
cudaError_t unit_columns(double* f, int nf, int col0, int ncols, cudaStream_t s);

// unit-force columns for the Schur assembly: gam[c] = rot(E^T e_{col0+c}), c < ncols
template <typename T>
cudaError_t unit_scatter_rot(const Geometry& g, const int* body_idx, const double* weight, int nb, int col0,
                             int ncols, T* gam, cudaStream_t s);

// forces -> coefficients (update_stress!): out[2b] = C_D, out[2b+1] = C_L of body b;
// stress (optional) = per-body column-major (n x 2) surface stress blocks
cudaError_t update_stress_hd(const double* fb, int nb, int nbodies, const int* body_start, const double* ds,
                             double h, double dt, double* cd_cl_out, double* stress_out, cudaStream_t s);

// ----------------------------------------------------------------------------------------------
// moving bodies and the Schur CG (cg.cu)
// ----------------------------------------------------------------------------------------------
// points of rigidly moving bodies: kin[6b..6b+5] = r0x, r0y, v0x, v0y, theta, omega; xb_body in
// the body frame; xb / vb stacked [x..., y...]
cudaError_t body_points(const double* xb_body, const double* kin, const int* body_of, int nb, double* xb,
                        double* vb, cudaStream_t s);
cudaError_t vec_axpy(double* y, const double* v, double a, int n, cudaStream_t s);
cudaError_t vec_dot(const double* a, const double* b, int n, double* out, cudaStream_t s);
// CG scalars in device memory sc[0] = r.r, sc[1] = p.Ap, sc[2] = r.r after the update
cudaError_t cg_update_xr(double* x, double* r, const double* p, const double* Ap, const double* sc, int n,
                         cudaStream_t s);
cudaError_t cg_update_p(double* p, const double* r, double* sc, int n, cudaStream_t s);
// device-side loop control of a captured CG (see cg.cu)
cudaError_t cg_start(double* sc, double* ctl, double tol, int* status, double* out, cudaGraphConditionalHandle cond,
                     cudaStream_t s);
cudaError_t cg_check(const double* sc, double* ctl, int maxiter, int* status, cudaGraphConditionalHandle cond,
                     cudaStream_t s);
cudaError_t cg_finish(const double* sc, const double* ctl, double* out, cudaStream_t s);

// ----------------------------------------------------------------------------------------------
// dense linear algebra (linalg.cu)
// ----------------------------------------------------------------------------------------------
// y = A x for row-major A (n x n), one warp per row, fixed reduction order
cudaError_t gemv_rowmajor(const double* A, const double* x, double* y, int n, cudaStream_t s);
// in-place inverse of a column-major n x n matrix (blocked Gauss-Jordan); status!=0 on a
// zero/non-finite pivot
cudaError_t invert_inplace(double* A, int n, double* work, int* status, cudaStream_t s);
size_t invert_workspace_bytes(int n);
cudaError_t transpose(const double* in, double* out, int rows, int cols, cudaStream_t s);

// ----------------------------------------------------------------------------------------------
// launch profiling: when a Prof is installed for the calling thread, launches of the selected
// kernel class are bracketed by CUDA events on their stream (used by ib_profile_steps)
// ----------------------------------------------------------------------------------------------
// Multilevel Vort2Flux with the levels solved together (v2f.cu; mixed precision, one-warp line
// passes on both axes).  Tables of the ring transfer and the work of the ring chain.
struct RingPlan {
  int Kx = 0, Ky = 0, nK = 0, nchunk = 0;  // sine modes kept per bottom/top (left/right) side
  int64_t qls = 0;                          // quarter-line values per level: 2 rows, 2 columns
  double* St = nullptr;                     // [Kx][nx-1] 2 sin(pi (k+1)(I+1)/nx), [Ky][ny-1] (y)
  double* Aring = nullptr;                  // [nK][nbc] ring entry per harmonic coefficient
  int4* pts = nullptr;                      // [nbc] {x0 index, quarter-line index} x (1 or 2)
  float *vrow = nullptr, *ucolp = nullptr, *ucol = nullptr, *qline = nullptr, *sidex = nullptr, *sidey = nullptr;
  double *ringd = nullptr, *coef = nullptr;  // change of each level's ring (FP64), its coefficients
  double* dring = nullptr;                   // the change as float-float (df64 pairs)
  cudaError_t build(const Geometry& g);
  void release();
};
cudaError_t v2f_yspec(const Geometry& g, const DstAxis<float>& ax, float* w, const float* m, int batch, float* vrow,
                      cudaStream_t s);
cudaError_t v2f_yring(const Geometry& g, const DstAxis<float>& axy, const DstAxis<float>& axx, float* w,
                      const float* m, int batch, const float* sidex, const float* sidey, cudaStream_t s);
cudaError_t v2f_colsum(const Geometry& g, const RingPlan& rp, const float* w, int batch, cudaStream_t s);
cudaError_t v2f_lines(const DstAxis<float>& ax, const float* in, int64_t in_b, int64_t in_s, float* out,
                      int64_t out_b, int64_t out_s, int nlines, cudaStream_t s);
cudaError_t v2f_ring_eval(const Geometry& g, const RingPlan& rp, int l, const df64* xp_up, const float* x0_up,
                          df64* ring_l, cudaStream_t s);
cudaError_t v2f_ring_coef(const Geometry& g, const RingPlan& rp, int l, cudaStream_t s);

// ----------------------------------------------------------------------------------------------
// Programmatic dependent launch: while g_pdl is set (the capture of a static step's graph), the
// step kernels are launched so that each one may be scheduled while its predecessor in the
// stream drains; every such kernel begins with pdl_begin(), which waits for the predecessor to
// complete and its writes to be visible before anything else, and lets the next kernel launch.
// Launched the ordinary way (g_pdl clear) pdl_begin() has nothing to wait for.
// ----------------------------------------------------------------------------------------------
extern thread_local bool g_pdl;

__device__ __forceinline__ void pdl_begin() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <typename... KArgs, typename... Args>
inline cudaError_t launch_k(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args... args) {
  if (!g_pdl) {
    k<<<grid, block, smem, s>>>(args...);
    return cudaGetLastError();
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k, args...);
}

enum KClass : int { kClassXPass = 0, kClassYPass = 1, kClassNonlin = 2, kClassCount = 3 };
struct Prof {
  int cls = -1;
  std::vector<cudaEvent_t> ev;
  size_t used = 0;
};
extern thread_local Prof* g_prof;
struct ProfScope {
  cudaEvent_t end = nullptr;
  cudaStream_t s;
  ProfScope(int cls, cudaStream_t st) : s(st) {
    Prof* p = g_prof;
    if (!p || p->cls != cls) return;
    if (p->used + 2 > p->ev.size()) {
      for (int i = 0; i < 64; ++i) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        p->ev.push_back(e);
      }
    }
    cudaEventRecord(p->ev[p->used], s);
    end = p->ev[p->used + 1];
    p->used += 2;
  }
  ~ProfScope() {
    if (end) cudaEventRecord(end, s);
  }
};

// ----------------------------------------------------------------------------------------------
// read-only view of a handle's Laplacian-inverse operator (geometry, FP64 tables, multipliers,
// stream) for entry points implemented outside solver.cu
// ----------------------------------------------------------------------------------------------
struct LapView {
  Geometry g;
  DstAxis<double> ax, ay;
  const double* mlap;
  cudaStream_t stream;
  int device;
  bool wdst;  // both axes use the warp-per-line passes (wx_fwd / wypass / wx_inv)
};

// Makes `dev` the current device for the lifetime of the guard and restores the caller's
// current device afterwards, so that entry points called from a foreign host (Julia, a
// Python program with its own device choice) leave that host's device selection unchanged.
struct DeviceGuard {
  int prev = -1;
  cudaError_t err = cudaSuccess;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != dev) err = cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
  DeviceGuard(const DeviceGuard&) = delete;
  DeviceGuard& operator=(const DeviceGuard&) = delete;
};

// An NVTX range over a host scope, so that setup, eager steps and their phases (trial state,
// forcing, projection, CG) show by name on a profiler's timeline.  Inside stream capture a
// range marks when the phase was captured, not its replays.  Without a profiler attached a
// range costs a test of a null function pointer.
struct Range {
  explicit Range(const char* name) { nvtxRangePushA(name); }
  ~Range() { nvtxRangePop(); }
  Range(const Range&) = delete;
  Range& operator=(const Range&) = delete;
};

// ----------------------------------------------------------------------------------------------
// misc
// ----------------------------------------------------------------------------------------------
template <typename T>
cudaError_t fill(T* p, T v, int64_t n, cudaStream_t s);
template <typename T>
cudaError_t axpby(T* y, const T* x, T a, T b, int64_t n, cudaStream_t s);  // y = a x + b y

}  // namespace ib

struct ib_handle;
// fills `v` from the handle; returns false for a null handle
bool ib_handle_lap_view(const ib_handle* h, ib::LapView* v);
// records `msg` as the handle's last error and returns `code`
int ib_handle_fail(ib_handle* h, int code, const char* msg);
