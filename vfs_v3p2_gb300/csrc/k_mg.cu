// Hot-path stencil kernels: the FP64 outer operator apply / residual and the
// multigrid preconditioner (y-line smoother, residual + restriction,
// prolongation + correction, coarsest-level dense solve), templated on the
// working precision (float for the mixed solver, double for the plain FP64
// solver).
//
// All stencil kernels walk the interior with a (32 x 8) thread tile in (i, j)
// and march a chunk of k planes per block: a warp reads 32 consecutive i of
// every coefficient row (coalesced), the x neighbours of the 19-point stencil
// come back through L1/L2.  Slots that are zero on the whole level (mask bit
// clear) are skipped with a warp-uniform branch, so a grid whose metric has
// no i-j or j-k cross terms streams 11 coefficient arrays instead of 19.
#include <type_traits>

#include "mg_tiles.cuh"
#include "mg_stage.h"
#include "vfs_common.cuh"
#include "vfs_kernels.h"
#include "vfs_proj.h"

namespace vfs {

// ---------------------------------------------------------------------------
// FP64 outer operator: y = A x, or y = b - A x.
// ---------------------------------------------------------------------------
template <unsigned MASK, typename TXin>
__global__ void __launch_bounds__(TX* TY, VFS_STENCIL_MINB) k_apply64(OpView<double> A, const TXin* __restrict__ x, const double* __restrict__ b,
                                                    double* __restrict__ y) {
  if (skipped(A.skip)) return;
  TILE_LOOP(A.d) {
    const double s = stencil_clamped<MASK, double>(A.d, A.coef, x, i, j, k);
    if (!_in) continue;
    const size_t c = cidx(A.d, i, j, k);
    y[c] = b ? b[c] - s : s;
  }
}

int launch_apply64(const OpView<double>& A, const double* x, const double* b, double* y, cudaStream_t s) {
  if (fits_ch(A.mask)) k_apply64<MASK_CH, double><<<tile_grid(A.d), dim3(TX, TY), 0, s>>>(A, x, b, y);
  else k_apply64<MASK_ALL, double><<<tile_grid(A.d), dim3(TX, TY), 0, s>>>(A, x, b, y);
  ++g_launches;
  return (int)cudaGetLastError();
}
int launch_apply64_xf(const OpView<double>& A, const float* x, const double* b, double* y, cudaStream_t s) {
  if (fits_ch(A.mask)) k_apply64<MASK_CH, float><<<tile_grid(A.d), dim3(TX, TY), 0, s>>>(A, x, b, y);
  else k_apply64<MASK_ALL, float><<<tile_grid(A.d), dim3(TX, TY), 0, s>>>(A, x, b, y);
  ++g_launches;
  return (int)cudaGetLastError();
}

// Outer operator inside the Krylov iteration: z (multigrid precision) is the
// V-cycle applied to the stored column V_j, so the flexible direction of the
// basis vector vs_j V_j is vs_j z; w = vs_j (A z) in FP64, and z is copied to
// its Krylov slot Z[st->j] (the solution update applies vs_j again); z[c] is
// loaded for the stencil's centre anyway.
template <unsigned MASK, typename T>
__global__ void __launch_bounds__(TX* TY, VFS_STENCIL_MINB) k_apply64_krylov(OpView<double> A, const T* __restrict__ z, T* __restrict__ Z,
                                                           const KrylovState* st, double* __restrict__ w) {
  if (skipped(A.skip)) return;
  T* zj = Z + (size_t)st->j * ncell(A.d);
  const double vs = st->vs[st->j];
  TILE_LOOP(A.d) {
    const double s = stencil_clamped<MASK, double>(A.d, A.coef, z, i, j, k);
    if (!_in) continue;
    const size_t c = cidx(A.d, i, j, k);
    w[c] = vs * s;
    zj[c] = z[c];
  }
}
template <typename T>
int launch_apply64_krylov(const OpView<double>& A, const T* z, T* Z, const KrylovState* st, double* w, cudaStream_t s) {
  if (fits_ch(A.mask)) k_apply64_krylov<MASK_CH, T><<<tile_grid(A.d), dim3(TX, TY), 0, s>>>(A, z, Z, st, w);
  else k_apply64_krylov<MASK_ALL, T><<<tile_grid(A.d), dim3(TX, TY), 0, s>>>(A, z, Z, st, w);
  ++g_launches;
  return (int)cudaGetLastError();
}
template int launch_apply64_krylov<float>(const OpView<double>&, const float*, float*, const KrylovState*, double*, cudaStream_t);
template int launch_apply64_krylov<double>(const OpView<double>&, const double*, double*, const KrylovState*, double*, cudaStream_t);

template <unsigned MASK, typename T>
__global__ void __launch_bounds__(TX* TY, VFS_STENCIL_MINB) k_apply_mg(OpView<T> A, const T* __restrict__ x, const T* __restrict__ b,
                                                     T* __restrict__ y) {
  if (skipped(A.skip)) return;
  TILE_LOOP(A.d) {
    const T s = stencil_clamped<MASK, T>(A.d, A.coef, x, i, j, k);
    if (!_in) continue;
    const size_t c = cidx(A.d, i, j, k);
    y[c] = b ? b[c] - s : s;
  }
}
template <typename T>
int launch_apply_mg(const OpView<T>& A, const T* x, const T* b, T* y, cudaStream_t s) {
  if (fits_ch(A.mask)) k_apply_mg<MASK_CH, T><<<tile_grid(A.d), dim3(TX, TY), 0, s>>>(A, x, b, y);
  else k_apply_mg<MASK_ALL, T><<<tile_grid(A.d), dim3(TX, TY), 0, s>>>(A, x, b, y);
  ++g_launches;
  return (int)cudaGetLastError();
}

// y = A x with the FP32 face form (11-slot levels; testing hook).
__global__ void __launch_bounds__(TX* TY) k_apply_face(OpView<float> A, const float* __restrict__ x,
                                                       float* __restrict__ y) {
  const bool all = A.ffc != nullptr;  // the general face form (set on levels with i-j or j-k cross terms)
  TILE_LOOP(A.d) {
    if (!_in) continue;
    FaceData f;
    float xv[19];
    if (all) {
      FaceX e;
      face_gather_all(A, x, i, j, k, f, e, xv);
      y[cidx(A.d, i, j, k)] = face_row_all(f, e, xv);
    } else {
      face_gather(A, x, i, j, k, f, xv);
      y[cidx(A.d, i, j, k)] = face_row(f, xv);
    }
  }
}
int launch_apply_face(const OpView<float>& A, const float* x, float* y, cudaStream_t s) {
  k_apply_face<<<tile_grid(A.d), dim3(TX, TY), 0, s>>>(A, x, y);
  ++g_launches;
  return (int)cudaGetLastError();
}


template <unsigned MASK, typename T, typename TC, bool PAIR, int UU, bool ZG>
__global__ void __launch_bounds__(VFS_SMOOTH_NT, PAIR ? VFS_SMOOTH_MINB_HALF : (UU > 1 ? 2 : VFS_SMOOTH_MINB))
    k_smooth(OpView<T> A, const T* __restrict__ lf, const T* __restrict__ xi, const T* __restrict__ b,
             T* __restrict__ xo, T omega, int TW) {
  if (skipped(A.skip)) return;
  extern __shared__ unsigned char smraw[];
  smooth_tile<MASK, T, TC, PAIR, UU, ZG>(A, lf, xi, b, xo, omega, TW, blockIdx.x, blockIdx.y, smraw);
}

// The face-form sweep with warp-row neighbours (smooth_tile_w): 30-column tiles.
template <int U>
__global__ void __launch_bounds__(VFS_SMOOTH_NT, VFS_SMOOTH_W_MINB)
    k_smooth_w(OpView<float> A, const float* __restrict__ lf, const float* __restrict__ xi,
               const float* __restrict__ b, float* __restrict__ xo, float omega) {
  if (skipped(A.skip)) return;
  extern __shared__ unsigned char smraw[];
  smooth_tile_w<U>(A, lf, xi, b, xo, omega, blockIdx.x, blockIdx.y, smraw);
}
template <unsigned MASK, typename T, typename TC, bool PAIR, int UU, bool ZG>
static void smooth_attrs1() {
  cudaFuncSetAttribute(k_smooth<MASK, T, TC, PAIR, UU, ZG>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  if (VFS_SMOOTH_CARVE >= 0)
    cudaFuncSetAttribute(k_smooth<MASK, T, TC, PAIR, UU, ZG>, cudaFuncAttributePreferredSharedMemoryCarveout,
                         VFS_SMOOTH_CARVE);
}
template <unsigned MASK, typename T, typename TC, bool PAIR>
static void smooth_attrs() {
  smooth_attrs1<MASK, T, TC, PAIR, VFS_SMOOTH_U, false>();
  smooth_attrs1<MASK, T, TC, PAIR, VFS_SMOOTH_U_SMALL, false>();
  smooth_attrs1<MASK, T, TC, PAIR, VFS_SMOOTH_U, true>();
}

// One launch of the sweep kernel with the per-level choices: U cells per
// thread batch (small levels) and the instantiation.
template <unsigned MASK, typename T, typename TC, bool PAIR>
static void smooth_launch(bool small, dim3 g, size_t sm, cudaStream_t s, const OpView<T>& A, const T* lf, const T* xi,
                          const T* b, T* xo, T omega, int tw) {
  if (!xi)
    k_smooth<MASK, T, TC, PAIR, VFS_SMOOTH_U, true><<<g, VFS_SMOOTH_NT, sm, s>>>(A, lf, xi, b, xo, omega, tw);
  else if (small && !PAIR)
    k_smooth<MASK, T, TC, PAIR, VFS_SMOOTH_U_SMALL, false><<<g, VFS_SMOOTH_NT, sm, s>>>(A, lf, xi, b, xo, omega, tw);
  else k_smooth<MASK, T, TC, PAIR, VFS_SMOOTH_U, false><<<g, VFS_SMOOTH_NT, sm, s>>>(A, lf, xi, b, xo, omega, tw);
}

template <typename T>
int launch_smooth(const OpView<T>& A, const T* lf, const T* xi, const T* b, T* xo, T omega, cudaStream_t s, int cols,
                  bool solo, int stage) {
  if constexpr (sizeof(T) == 4) {
    // the tensor-copy sweep; a configuration it cannot take (its launch
    // refused before running) falls back to the register-staged one
    if (stage == STAGE_TMA && A.ffi && xi && fits_ch(A.mask) &&
        (size_t)(A.d.mx - 2) * (A.d.my - 2) * (A.d.mz - 2) >= (size_t)VFS_STAGE_MINCELLS &&
        smooth_tma_stages(A.d) > 0 && smooth_tma_err() &&
        launch_smooth_tma(A, lf, xi, b, xo, omega, smooth_tma_err(), s) == (int)cudaSuccess)
      return (int)cudaSuccess;
  }
  static bool attr = false;
  if (!attr) {
    smooth_attrs<MASK_CH, T, T, false>();
    smooth_attrs<MASK_ALL, T, T, false>();
    if constexpr (sizeof(T) == 4) {
      smooth_attrs<MASK_CH, T, __half, false>();
      smooth_attrs<MASK_CH, T, __half, true>();
      smooth_attrs<MASK_ALL, T, __half, true>();
      smooth_attrs<MASK_CH, T, FaceOp, false>();
      smooth_attrs<MASK_ALL, T, FaceOp, false>();
    }
    attr = true;
  }
  const int nj = A.d.my - 2, ni = A.d.mx - 2, nk = A.d.mz - 2;
  const int tw = smooth_tw<T>(ni, nj, nk, cols, solo || VFS_SMOOTH_NARROW_SHARED);
  const size_t sm = smooth_smem<T>(tw, nj);
  dim3 g((ni + tw - 1) / tw, nk);
  const bool ch = fits_ch(A.mask);
  // two-cell batches only when the sweep has the GPU to itself (one grid
  // solving) and fewer than two blocks per SM: with other grids' kernels
  // beside it (batch, serving) the looser register budget costs concurrency
  const bool small = sizeof(T) == 4 && solo && (size_t)g.x * g.y < 2 * 152;  // (FP64: spills at two cells)
  bool done = false;
  if constexpr (sizeof(T) == 4) {
    if (A.ffi && ch && xi && cols == 0 && tw == 32 && !small && VFS_SMOOTH_W_U > 0) {
      // automatic full-width tiles on the face form: the warp-row sweep
      static bool wattr = false;
      if (!wattr) {
        cudaFuncSetAttribute(k_smooth_w<VFS_SMOOTH_W_U>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        wattr = true;
      }
      const dim3 gw((ni + SMOOTH_W_TW - 1) / SMOOTH_W_TW, nk);
      k_smooth_w<VFS_SMOOTH_W_U><<<gw, VFS_SMOOTH_NT, smooth_smem<float>(32, nj), s>>>(A, lf, xi, b, xo, omega);
      done = true;
    } else if (A.ffi && ch) {
      smooth_launch<MASK_CH, T, FaceOp, false>(small, g, sm, s, A, lf, xi, b, xo, omega, tw);
      done = true;
    } else if (A.ffi && A.ffc) {  // the general face form (one cell per batch: two would spill)
      smooth_launch<MASK_ALL, T, FaceOp, false>(false, g, sm, s, A, lf, xi, b, xo, omega, tw);
      done = true;
    } else if (A.hcoef) {
      if (!ch) smooth_launch<MASK_ALL, T, __half, true>(small, g, sm, s, A, lf, xi, b, xo, omega, tw);
      else if (ncell(A.d) <= (size_t)VFS_SMOOTH_PAIR_MAXN)
        smooth_launch<MASK_CH, T, __half, true>(small, g, sm, s, A, lf, xi, b, xo, omega, tw);
      else smooth_launch<MASK_CH, T, __half, false>(small, g, sm, s, A, lf, xi, b, xo, omega, tw);
      done = true;
    }
  }
  if (!done) {
    if (ch) smooth_launch<MASK_CH, T, T, false>(small, g, sm, s, A, lf, xi, b, xo, omega, tw);
    else smooth_launch<MASK_ALL, T, T, false>(small, g, sm, s, A, lf, xi, b, xo, omega, tw);
  }
  ++g_launches;
  return (int)cudaGetLastError();
}

// Thomas pivots of the y-line tridiagonal (a_j = SP, b_j = CP, c_j = NP) of
// every column, in FP64 from the aj-scaled FP64 operator, stored as T:
// lf[c] = 1/m_j with m_j = b_j - a_j c'_{j-1}, c'_j = c_j / m_j.  The sweep
// forms a_j/m_j and c'_j = c_j/m_j from its own coefficients, so that the
// forward substitution is y_j = r_j/m_j - (a_j/m_j) y_{j-1} and the backward
// one delta_j = y_j - c'_j delta_{j+1}.  Non-fluid cells are identity rows;
// j-periodic seam couplings stay off the line.
template <typename T>
__global__ void k_line_factors(Dims d, const double* __restrict__ mcoef, T* __restrict__ lf) {
  const size_t N = ncell(d);
  const int ni = d.mx - 2, nk = d.mz - 2;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ni * nk; t += gridDim.x * blockDim.x) {
    const int i = 1 + t % ni, k = 1 + t / ni;
    double cprev = 0.;
    for (int j = 1; j < d.my - 1; j++) {
      const size_t c = cidx(d, i, j, k);
      double a = (j > 1) ? mcoef[(size_t)SP * N + c] : 0.;
      double bb = mcoef[c];
      double cc = (j < d.my - 2) ? mcoef[(size_t)NP * N + c] : 0.;
      if (bb == 0.) { a = 0.; bb = 1.; cc = 0.; }
      const double m = bb - a * cprev;
      const double inv = 1. / m;
      cprev = cc * inv;
      lf[c] = (T)inv;
    }
  }
}
template <typename T>
int launch_line_factors(const Dims& d, const double* mcoef, T* lf, cudaStream_t s) {
  const int n = (d.mx - 2) * (d.mz - 2);
  k_line_factors<T><<<(n + 127) / 128, 128, 0, s>>>(d, mcoef, lf); ++g_launches;
  return (int)cudaGetLastError();
}

// ---------------------------------------------------------------------------
// FP16 diagonal-normalised multigrid operator (FP32 multigrid only).  Per
// fluid row c with diagonal D = mcoef[CP][c] of the aj-scaled FP64 operator:
// h_m = fp16(mcoef[m][c] / D) for every off-diagonal slot (round to nearest
// even), and h_CP = fp16(delta) with delta = sum_m (mcoef[m][c] / D - h_m)
// in FP64, slot order, so that 1 + delta + sum_m h_m equals the row sum of
// the normalised row up to one FP16 rounding of delta.  Keeping the row sums
// keeps the near-null space (smooth modes) of the level operator, which is
// what the coarse-grid correction relies on.  Non-fluid rows are all zero.
// Optional outputs: dinv = fp32(1 / D) and dval = fp32(D), 0 on non-fluid
// rows (the finest level's input scaling, the coarsest level's dense solve).
// A ratio or correction beyond 6e4 (near the FP16 maximum, 65504) sets
// *range: the solver then keeps the FP32 operator for the grid.
// ---------------------------------------------------------------------------
__global__ void k_half_operator(Dims d, const double* __restrict__ mcoef, __half* __restrict__ h,
                                float* __restrict__ dinv, float* __restrict__ dval, unsigned* range) {
  const size_t n = ncell(d), hs = hslot(d);
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(c % d.mx), j = (int)((c / d.mx) % d.my), k = (int)(c / ((size_t)d.mx * d.my));
    const size_t hc = hidx(d, i, j, k);
    const double D = mcoef[c];
    double delta = 0.;
    for (int m = 1; m < 19; m++) {
      const double a = D != 0. ? mcoef[(size_t)m * n + c] / D : 0.;
      if (!(fabs(a) <= 6.e4)) atomicOr(range, 1u);
      const __half hm = __double2half(a);
      delta = delta + (a - (double)__half2float(hm));
      h[(size_t)m * hs + hc] = hm;
    }
    if (!(fabs(delta) <= 6.e4)) atomicOr(range, 1u);
    h[hc] = __double2half(delta);
    if (dinv) dinv[c] = D != 0. ? (float)(1. / D) : 0.f;
    if (dval) dval[c] = (float)D;
  }
}
int launch_half_operator(const Dims& d, const double* mcoef, __half* h, float* dinv, float* dval, unsigned* range,
                         cudaStream_t s) {
  const size_t nb = (ncell(d) + 255) / 256;
  k_half_operator<<<(unsigned)(nb < 4096 ? nb : 4096), 256, 0, s>>>(d, mcoef, h, dinv, dval, range); ++g_launches;
  return (int)cudaGetLastError();
}

// Thomas pivots 1/m_j of the normalised y-line tridiagonal (a_j = h_SP,
// b_j = 1 + h_CP, c_j = h_NP), in FP64 from the stored FP16 values, as FP32;
// 1/m = 0 on non-fluid rows (the sweep's delta there is then 0), which act
// as identity rows of the recurrence.
__global__ void k_line_factors_half(Dims d, const __half* __restrict__ h, const double* __restrict__ mcoef,
                                    float* __restrict__ lf) {
  const size_t hs = hslot(d);
  const int ni = d.mx - 2, nk = d.mz - 2;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ni * nk; t += gridDim.x * blockDim.x) {
    const int i = 1 + t % ni, k = 1 + t / ni;
    double cprev = 0.;
    for (int j = 1; j < d.my - 1; j++) {
      const size_t c = cidx(d, i, j, k), hc = hidx(d, i, j, k);
      if (mcoef[c] == 0.) {
        lf[c] = 0.f;
        cprev = 0.;
        continue;
      }
      const double a = (j > 1) ? (double)__half2float(h[(size_t)SP * hs + hc]) : 0.;
      const double bb = 1. + (double)__half2float(h[hc]);
      const double cc = (j < d.my - 2) ? (double)__half2float(h[(size_t)NP * hs + hc]) : 0.;
      const double inv = 1. / (bb - a * cprev);
      cprev = cc * inv;
      lf[c] = (float)inv;
    }
  }
}
int launch_line_factors_half(const Dims& d, const __half* h, const double* mcoef, float* lf, cudaStream_t s) {
  const int n = (d.mx - 2) * (d.mz - 2);
  k_line_factors_half<<<(n + 127) / 128, 128, 0, s>>>(d, h, mcoef, lf); ++g_launches;
  return (int)cudaGetLastError();
}

// Restriction weights of the normalised operator: the fine residual is
// D_f r_n and the coarse right-hand side is divided by D_c, so the weight
// max(0, 1 - nvert_f) becomes fp32(max(0, 1 - nvert_f) D_f / D_c) with c the
// coarse cell the fine cell restricts into (0 when either row is non-fluid).
__global__ void k_restrict_weights_half(Dims f, Dims c, int si, int sj, int sk, const double* __restrict__ nvf,
                                        const double* __restrict__ mcf, const double* __restrict__ mcc,
                                        float* __restrict__ w) {
  const size_t n = ncell(f);
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % f.mx), j = (int)((t / f.mx) % f.my), k = (int)(t / ((size_t)f.mx * f.my));
    float v = 0.f;
    if (i >= 1 && i <= f.mx - 2 && j >= 1 && j <= f.my - 2 && k >= 1 && k <= f.mz - 2) {
      const int ic = si ? i : (i + 1) / 2, jc = sj ? j : (j + 1) / 2, kc = sk ? k : (k + 1) / 2;
      const double Df = mcf[t], Dc = mcc[cidx(c, ic, jc, kc)];
      if (Df != 0. && Dc != 0.) v = (float)(fmax(0., 1. - nvf[t]) * Df / Dc);
    }
    w[t] = v;
  }
}
int launch_restrict_weights_half(const Dims& f, const Dims& c, int si, int sj, int sk, const double* nvf,
                                 const double* mcf, const double* mcc, float* w, cudaStream_t s) {
  const size_t nb = (ncell(f) + 255) / 256;
  k_restrict_weights_half<<<(unsigned)(nb < 4096 ? nb : 4096), 256, 0, s>>>(f, c, si, sj, sk, nvf, mcf, mcc, w);
  ++g_launches;
  return (int)cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Residual + restriction (MyRestriction, poisson.c:364-471), one thread per
// coarse interior cell: bc = 0.125 * sum over the 8 children of
// (b - A x) * max(0, 1 - nvert_f), 0 on solid coarse cells; xc = 0.
// ---------------------------------------------------------------------------
template <unsigned MASK, typename T, typename TC>
__global__ void __launch_bounds__(TX* TY, VFS_STENCIL_MINB) k_resrestrict(OpView<T> A, const T* __restrict__ x, const T* __restrict__ b,
                                                        const T* __restrict__ rw, Dims c, const double* __restrict__ nvc,
                                                        int si, int sj, int sk, T* __restrict__ bc, T* __restrict__ xc) {
  if (skipped(A.skip)) return;
  const TC* __restrict__ coef = coef_ptr<TC>(A);
  const int ia = si ? 0 : 1, ja = sj ? 0 : 1, ka = sk ? 0 : 1;
  TILE_LOOP(c) {
    if (!_in) continue;
    const size_t q = cidx(c, i, j, k);
    T acc = T(0);
    if (!(nvc[q] > 0.1)) {
      const int ih = si ? i : 2 * i, jh = sj ? j : 2 * j, kh = sk ? k : 2 * k;
      const int oi[8] = {0, ia, 0, 0, ia, 0, ia, ia}, oj[8] = {0, 0, ja, 0, ja, ja, 0, ja},
                ok[8] = {0, 0, 0, ka, 0, ka, ka, ka};
#pragma unroll
      for (int t = 0; t < 8; t++) {
        const int fi = ih - oi[t], fj = jh - oj[t], fk = kh - ok[t];
        const size_t fc = cidx(A.d, fi, fj, fk);
        const T w = rw[fc];
        T ax = T(0);
        if (x) {
          TC cv[19];
          T xv[19];
          gather<MASK>(A.d, coef, x, fi, fj, fk, cv, xv);
          ax = row_dot<MASK, T>(cv, xv);
        }
        const T rr = (b[fc] - ax) * w;
        acc += (w != T(0)) ? rr : T(0);
      }
      acc *= T(0.125);
    }
    bc[q] = acc;
    xc[q] = T(0);
  }
}

// Full-coarsening fast path: a block owns a coarse tile of 32 x 4 x 1 cells,
// i.e. the fine tile 64 x 8 x 2.  Its 256 threads compute the 1024 fine
// residuals (four each, coalesced over fine i), weight them by
// max(0, 1 - nvert_f) into shared memory, and 128 threads sum the 2 x 2 x 2
// children of each coarse cell in the reference's order.
template <unsigned MASK, typename T, typename TC>
__global__ void __launch_bounds__(256, VFS_STENCIL_MINB) k_resrestrict_tiled(OpView<T> A, const T* __restrict__ x, const T* __restrict__ b,
                                                           const T* __restrict__ rw, Dims c,
                                                           const double* __restrict__ nvc, T* __restrict__ bc,
                                                           T* __restrict__ xc) {
  if (skipped(A.skip)) return;
  __shared__ T sr[2][8][64];
  resrestrict_tile<MASK, T, TC>(A, x, b, rw, c, nvc, bc, xc, blockIdx.x, blockIdx.y, blockIdx.z, sr);
}

template <typename T, typename TC>
static void launch_resrestrict_tc(const OpView<T>& A, const T* x, const T* b, const T* rw, const Dims& c,
                                  const double* nvc, int si, int sj, int sk, T* bc, T* xc, cudaStream_t s) {
  const bool ch = fits_ch(A.mask);
  if (!si && !sj && !sk) {
    dim3 g((c.mx - 2 + 31) / 32, (c.my - 2 + 3) / 4, c.mz - 2);
    if (ch) k_resrestrict_tiled<MASK_CH, T, TC><<<g, 256, 0, s>>>(A, x, b, rw, c, nvc, bc, xc);
    else k_resrestrict_tiled<MASK_ALL, T, TC><<<g, 256, 0, s>>>(A, x, b, rw, c, nvc, bc, xc);
  } else {
    if (ch) k_resrestrict<MASK_CH, T, TC><<<tile_grid(c), dim3(TX, TY), 0, s>>>(A, x, b, rw, c, nvc, si, sj, sk, bc, xc);
    else k_resrestrict<MASK_ALL, T, TC><<<tile_grid(c), dim3(TX, TY), 0, s>>>(A, x, b, rw, c, nvc, si, sj, sk, bc, xc);
  }
}

template <typename T>
int launch_residual_restrict(const OpView<T>& A, const T* x, const T* b, const T* rw, const Dims& c,
                             const double* nvc, int si, int sj, int sk, T* bc, T* xc, cudaStream_t s) {
  bool done = false;
  if constexpr (sizeof(T) == 4) {
    if (A.ffi && (fits_ch(A.mask) || A.ffc) && !si && !sj && !sk) {
      dim3 g((c.mx - 2 + 31) / 32, (c.my - 2 + 3) / 4, c.mz - 2);
      if (fits_ch(A.mask)) k_resrestrict_tiled<MASK_CH, T, FaceOp><<<g, 256, 0, s>>>(A, x, b, rw, c, nvc, bc, xc);
      else k_resrestrict_tiled<MASK_ALL, T, FaceOp><<<g, 256, 0, s>>>(A, x, b, rw, c, nvc, bc, xc);
      done = true;
    } else if (A.hcoef) {
      launch_resrestrict_tc<T, __half>(A, x, b, rw, c, nvc, si, sj, sk, bc, xc, s);
      done = true;
    }
  }
  if (!done) launch_resrestrict_tc<T, T>(A, x, b, rw, c, nvc, si, sj, sk, bc, xc, s);
  ++g_launches;
  return (int)cudaGetLastError();
}

// Restriction weights of a level, max(0, 1 - nvert) (MyRestriction), in both
// multigrid precisions; formed once per grid.
__global__ void k_restrict_weights(size_t n, const double* __restrict__ nv, float* __restrict__ w32,
                                   double* __restrict__ w64) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const double w = fmax(0., 1. - nv[t]);
    w32[t] = (float)w;
    w64[t] = w;
  }
}
int launch_restrict_weights(size_t n, const double* nv, float* w32, double* w64, cudaStream_t s) {
  k_restrict_weights<<<(unsigned)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096), 256, 0, s>>>(n, nv, w32, w64);
  ++g_launches;
  return (int)cudaGetLastError();
}

template <typename T>
__global__ void k_restrict_plain(Dims f, const T* __restrict__ x, const double* __restrict__ nvf, Dims c,
                                 const double* __restrict__ nvc, int si, int sj, int sk, T* __restrict__ out) {
  const int ia = si ? 0 : 1, ja = sj ? 0 : 1, ka = sk ? 0 : 1;
  TILE_LOOP(c) {
    if (!_in) continue;
    const size_t q = cidx(c, i, j, k);
    const int ih = si ? i : 2 * i, jh = sj ? j : 2 * j, kh = sk ? k : 2 * k;
    const int oi[8] = {0, ia, 0, 0, ia, 0, ia, ia}, oj[8] = {0, 0, ja, 0, ja, ja, 0, ja}, ok[8] = {0, 0, 0, ka, 0, ka, ka, ka};
    T acc = T(0);
#pragma unroll
    for (int t = 0; t < 8; t++) {
      const size_t fc = cidx(f, ih - oi[t], jh - oj[t], kh - ok[t]);
      acc += x[fc] * (T)fmax(0., 1. - nvf[fc]);
    }
    acc *= T(0.125);
    out[q] = (nvc[q] > 0.1) ? T(0) : acc;
  }
}
template <typename T>
int launch_restrict(const Dims& f, const T* x, const double* nvf, const Dims& c, const double* nvc, int si, int sj, int sk,
                    T* out, cudaStream_t s) {
  k_restrict_plain<T><<<tile_grid(c), dim3(TX, TY), 0, s>>>(f, x, nvf, c, nvc, si, sj, sk, out); ++g_launches;
  return (int)cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Prolongation + correction (MyInterpolation, poisson.c:526-669), one thread
// per fine interior cell, offsets from the precomputed code.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(TX* TY, VFS_STENCIL_MINB) k_prolong(Dims f, const uint8_t* __restrict__ code, Dims c,
                                                                      const T* __restrict__ xc, T* __restrict__ xf,
                                                                      int add, int si, int sj, int sk, const int* skip) {
  if (skipped(skip)) return;
  prolong_tile<T>(f, code, c, xc, xf, add, si, sj, sk, blockIdx.x, blockIdx.y, blockIdx.z, threadIdx.x, threadIdx.y);
}

template <typename T>
int launch_prolong(const Dims& f, const uint8_t* code, const Dims& c, const T* xc, T* xf, int add, const int* skip,
                   cudaStream_t s) {
  // semi-coarsening flags are implied by equal extents
  const int si = (c.mx == f.mx), sj = (c.my == f.my), sk = (c.mz == f.mz);
  k_prolong<T><<<tile_grid(f), dim3(TX, TY), 0, s>>>(f, code, c, xc, xf, add, si, sj, sk, skip); ++g_launches;
  return (int)cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Coarsest level: x = Binv b over the packed interior (dense, one warp per row).
// ---------------------------------------------------------------------------
// dsc (nullable): the level's diagonal, for a right-hand side of the
// normalised operator (Binv inverts the unnormalised one: x = Binv (D b)).
template <typename T>
__global__ void __launch_bounds__(256) k_coarse_gemv(Dims d, const T* __restrict__ Binv, int n, const T* __restrict__ b,
                                                     T* __restrict__ x, const T* __restrict__ dsc, const int* skip) {
  if (skipped(skip)) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  gemv_tile<T>(d, Binv, n, b, x, dsc, blockIdx.x, (T*)smraw);
}
template <typename T>
int launch_coarse_gemv(const Dims& d, const T* Binv, int n, const T* b, T* x, const T* dsc, const int* skip,
                       cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_coarse_gemv<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    attr = true;
  }
  k_coarse_gemv<T><<<(n + 7) / 8, 256, (size_t)n * sizeof(T), s>>>(d, Binv, n, b, x, dsc, skip); ++g_launches;
  return (int)cudaGetLastError();
}

// dinv (nullable): 1 / D of the FP16 normalised operator, applied after the
// rounding to T.
template <typename T>
__global__ void __launch_bounds__(TX* TY) k_scale_in(Dims d, const double* __restrict__ aj, const double* __restrict__ v,
                                                     T* __restrict__ out, const float* __restrict__ dinv,
                                                     const int* skip) {
  if (skipped(skip)) return;
  TILE_LOOP(d) {
    if (!_in) continue;
    const size_t c = cidx(d, i, j, k);
    const T t = (T)(aj ? aj[c] * v[c] : v[c]);
    out[c] = dinv ? t * (T)dinv[c] : t;
  }
}
template <typename T>
int launch_scale_in(const Dims& d, const double* aj, const double* v, T* out, const int* skip, cudaStream_t s,
                    const float* dinv) {
  k_scale_in<T><<<tile_grid(d), dim3(TX, TY), 0, s>>>(d, aj, v, out, dinv, skip); ++g_launches;
  return (int)cudaGetLastError();
}

#define INST(T)                                                                                                        \
  template int launch_apply_mg<T>(const OpView<T>&, const T*, const T*, T*, cudaStream_t);                            \
  template int launch_smooth<T>(const OpView<T>&, const T*, const T*, const T*, T*, T, cudaStream_t, int, bool, int);      \
  template int launch_line_factors<T>(const Dims&, const double*, T*, cudaStream_t);                                  \
  template int launch_residual_restrict<T>(const OpView<T>&, const T*, const T*, const T*, const Dims&,           \
                                           const double*, int, int, int, T*, T*, cudaStream_t);                       \
  template int launch_restrict<T>(const Dims&, const T*, const double*, const Dims&, const double*, int, int, int, T*, \
                                  cudaStream_t);                                                                      \
  template int launch_prolong<T>(const Dims&, const uint8_t*, const Dims&, const T*, T*, int, const int*, cudaStream_t); \
  template int launch_coarse_gemv<T>(const Dims&, const T*, int, const T*, T*, const T*, const int*, cudaStream_t);  \
  template int launch_scale_in<T>(const Dims&, const double*, const double*, T*, const int*, cudaStream_t,             \
                                  const float*);
INST(float)
INST(double)

}  // namespace vfs
