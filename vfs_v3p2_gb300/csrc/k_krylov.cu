// Flexible GMRES(m) in FP64 with all scalars on the device.
//
// The Krylov basis V (m+1 vectors) is FP64; the preconditioned directions Z
// are in the multigrid precision T.  Basis vector q is vs[q] * V_q: with one
// classical Gram-Schmidt pass (the default) the update sweep stores the
// orthogonalised column unnormalised, together with the multigrid input of
// the next iteration and its norm partials, and the scale 1 / ||.|| follows
// from the reduction; the matrix-vector product and the solution update
// apply vs.  With CGS2 (classical with one re-orthogonalisation pass) the
// columns are stored normalised (vs = 1).  Every pass is a deterministic
// multi-dot or norm (fixed block partials summed in index order by one
// block) or one fused update sweep.  The Hessenberg column, Givens rotations and the
// residual estimate live in a KrylovState in device memory and are updated
// by a single-block kernel, so the host enqueues iterations without reading
// anything back; every kernel returns immediately once st->done is set.
#include "vfs_common.cuh"
#include "vfs_proj.h"

namespace vfs {

constexpr int KB = 256;
constexpr int MAXCOL = 64;  // largest restart length

int krylov_nblocks(size_t n) {
  size_t b = (n + KB * 4 - 1) / (KB * 4);
  if (b > 152 * 4) b = 152 * 4;
  return (int)(b ? b : 1);
}

__device__ __forceinline__ bool is_done(const KrylovState* st) { return *(volatile const int*)&st->done; }
__device__ __forceinline__ bool met(const KrylovState* st, double r) {
  return r <= st->rtol * st->bnorm && (st->atol <= 0. || r <= st->atol);
}

// ||v||^2 partials; then finish: is_b ? bnorm : beta (+ g[0], done check).
__global__ void __launch_bounds__(KB) k_sq_partials(const KrylovState* st, const double* __restrict__ v, size_t n,
                                                     double* parts, int check_done) {
  if (check_done && is_done(st)) return;
  __shared__ double sh[32];
  double s = 0.;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    double a = v[t];
    s = fma(a, a, s);
  }
  s = block_sum(s, sh);
  if (threadIdx.x == 0) parts[blockIdx.x] = s;
}

__global__ void k_norm_finish(KrylovState* st, const double* __restrict__ parts, int nparts, int is_b) {
  if (!is_b && is_done(st)) return;
  __shared__ double sh[32];
  double s = 0.;
  for (int p = threadIdx.x; p < nparts; p += blockDim.x) s += parts[p];
  s = block_sum(s, sh);
  if (!is_b) {  // clear the Hessenberg matrix and g with the whole block
    const int m = st->m;
    for (int q = threadIdx.x; q <= m; q += blockDim.x) st->g[q] = 0.;
    for (int q = threadIdx.x; q < (m + 1) * m; q += blockDim.x) st->H[q] = 0.;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double nrm = sqrt(s);
    if (is_b) {
      st->bnorm = nrm;
      st->done = (nrm == 0.) ? 1 : 0;
      st->it = 0;
      st->j = 0;
    } else {
      st->beta = nrm;
      st->resid = nrm;
      st->g[0] = nrm;
      st->j = 0;
      st->inv_hn = nrm > 0. ? 1. / nrm : 0.;
      st->vs[0] = 1.;  // V_0 is stored normalised
      if (met(st, nrm)) st->done = 1;
    }
  }
}

int launch_norm_init(KrylovState* st, const double* r, size_t n, double* parts, int is_b, cudaStream_t s) {
  const int nb = krylov_nblocks(n);
  k_sq_partials<<<nb, KB, 0, s>>>(st, r, n, parts, !is_b); ++g_launches;
  k_norm_finish<<<1, KB, 0, s>>>(st, parts, nb, is_b); ++g_launches;
  return (int)cudaGetLastError();
}

// v0 = r * (1 / beta)
__global__ void k_scale_vec(const KrylovState* st, const double* __restrict__ r, double* __restrict__ v, size_t n) {
  if (is_done(st)) return;
  const double f = st->inv_hn;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) v[t] = r[t] * f;
}
int launch_vec_scale_first(KrylovState* st, const double* r, double* v0, size_t n, cudaStream_t s) {
  k_scale_vec<<<krylov_nblocks(n) * 4, KB, 0, s>>>(st, r, v0, n); ++g_launches;
  return (int)cudaGetLastError();
}
int launch_vnext(KrylovState* st, const double* w, double* vn, size_t n, cudaStream_t s) {
  k_scale_vec<<<krylov_nblocks(n) * 4, KB, 0, s>>>(st, w, vn, n); ++g_launches;
  return (int)cudaGetLastError();
}

// Multi-dot partials: parts[b * ld + q] = sum over the block's cells of V_q . w
// for q < nv, chunks of 4 columns per sweep (w is re-read from L2).
// nv < 0: use the device's current column count st->j + 1 (graph-replayable).
__device__ __forceinline__ int nv_of(const KrylovState* st, int nv) { return nv < 0 ? st->j + 1 : nv; }

// NQ consecutive basis columns V0 .. V0 + (NQ-1) n against w: two cells per
// turn (their loads in flight together), each thread's cells accumulated in
// increasing order.
template <int NQ>
__device__ __forceinline__ void dot_chunk(const double* __restrict__ V0, const double* __restrict__ w, size_t n,
                                          double* a) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  for (; t + stride < n; t += 2 * stride) {
    const size_t u = t + stride;
    const double wv = w[t], wu = w[u];
    double v[NQ], x[NQ];
#pragma unroll
    for (int q = 0; q < NQ; q++) {
      v[q] = V0[(size_t)q * n + t];
      x[q] = V0[(size_t)q * n + u];
    }
#pragma unroll
    for (int q = 0; q < NQ; q++) a[q] = fma(x[q], wu, fma(v[q], wv, a[q]));
  }
  if (t < n) {
    const double wv = w[t];
#pragma unroll
    for (int q = 0; q < NQ; q++) a[q] = fma(V0[(size_t)q * n + t], wv, a[q]);
  }
}

__global__ void __launch_bounds__(KB) k_multidot(const KrylovState* st, const double* __restrict__ V, int nv,
                                                 const double* __restrict__ w, size_t n, double* parts, int ld) {
  if (is_done(st)) return;
  nv = nv_of(st, nv);
  __shared__ double sh[32];
  for (int q0 = 0; q0 < nv; q0 += 4) {
    double a[4] = {0., 0., 0., 0.};
    const int nq = min(4, nv - q0);
    const double* V0 = V + (size_t)q0 * n;
    switch (nq) {
      case 4: dot_chunk<4>(V0, w, n, a); break;
      case 3: dot_chunk<3>(V0, w, n, a); break;
      case 2: dot_chunk<2>(V0, w, n, a); break;
      default: dot_chunk<1>(V0, w, n, a); break;
    }
    for (int q = 0; q < nq; q++) {
      const double r = block_sum(a[q], sh);
      if (threadIdx.x == 0) parts[(size_t)blockIdx.x * ld + q0 + q] = r;
    }
  }
}

// Sum the multi-dot partials into st->h (and accumulate the column in hacc).
// One warp per dot (q = warp, warp + 8, ...): each lane sums a fixed stride
// of the block partials, then the warp tree; no block barriers, and the
// order is fixed, so the result is deterministic.
__global__ void k_multidot_finish(KrylovState* st, const double* __restrict__ parts, int nparts, int nv, int ld, int pass) {
  if (is_done(st)) return;
  nv = nv_of(st, nv);
  const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int q = threadIdx.x >> 5; q < nv; q += nw) {
    double s = 0.;
    for (int p = lane; p < nparts; p += 32) s += parts[(size_t)p * ld + q];
    s = warp_sum(s) * st->vs[q];
    if (lane == 0) {
      st->h[q] = s;
      st->hacc[q] = (pass == 1) ? s : st->hacc[q] + s;
    }
  }
}

int launch_multidot(KrylovState* st, const double* V, int nv, const double* w, size_t n, double* parts, int pass,
                    cudaStream_t s) {
  const int nb = krylov_nblocks(n);
  const int ld = 72;
  k_multidot<<<nb, KB, 0, s>>>(st, V, nv, w, n, parts, ld); ++g_launches;
  k_multidot_finish<<<1, KB, 0, s>>>(st, parts, nb, nv, ld, pass); ++g_launches;
  return (int)cudaGetLastError();
}

// w -= sum_q h[q] V_q, with the partials of ||w||^2 after the update.
__global__ void __launch_bounds__(KB) k_gs_update(const KrylovState* st, const double* __restrict__ V, int nv,
                                                  double* __restrict__ w, size_t n, double* parts) {
  if (is_done(st)) return;
  nv = nv_of(st, nv);
  __shared__ double sh[32];
  __shared__ double hs[72];
  for (int q = threadIdx.x; q < nv; q += blockDim.x) hs[q] = st->h[q] * st->vs[q];
  __syncthreads();
  double s = 0.;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    double a = w[t];
    for (int q = 0; q < nv; q++) a = fma(-hs[q], V[(size_t)q * n + t], a);
    w[t] = a;
    s = fma(a, a, s);
  }
  s = block_sum(s, sh);
  if (threadIdx.x == 0) parts[blockIdx.x] = s;
}
int launch_gs_update(KrylovState* st, const double* V, int nv, double* w, size_t n, double* parts, int pass,
                     cudaStream_t s) {
  (void)pass;
  k_gs_update<<<krylov_nblocks(n), KB, 0, s>>>(st, V, nv, w, n, parts); ++g_launches;
  return (int)cudaGetLastError();
}

// One-pass classical Gram-Schmidt update of column j = st->j: the
// orthogonalised vector u = w - sum_q h_q vs_q V_q is stored unnormalised as
// V_{j+1}, its multigrid-precision copy as the next preconditioner input, and
// the partials of ||u||^2 go to parts (k_arnoldi_finish sets vs_{j+1}).
// dinv (nullable): 1 / D of the FP16 normalised multigrid operator, applied
// to the multigrid copy after its rounding to T.
template <typename T>
__global__ void __launch_bounds__(KB) k_cgs_update(const KrylovState* st, double* V, const double* __restrict__ w,
                                                   T* __restrict__ out, size_t n, double* parts,
                                                   const float* __restrict__ dinv) {
  if (is_done(st)) return;
  const int nv = st->j + 1;
  __shared__ double sh[32];
  __shared__ double hs[72];
  for (int q = threadIdx.x; q < nv; q += blockDim.x) hs[q] = st->h[q] * st->vs[q];
  __syncthreads();
  double* vn = V + (size_t)nv * n;
  double s = 0.;
  // two cells per turn (their basis loads in flight together), in cell order
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  for (; t + stride < n; t += 2 * stride) {
    double a0 = w[t], a1 = w[t + stride];
#pragma unroll 4
    for (int q = 0; q < nv; q++) {
      const double h = hs[q];
      const double v0 = V[(size_t)q * n + t], v1 = V[(size_t)q * n + t + stride];
      a0 = fma(-h, v0, a0);
      a1 = fma(-h, v1, a1);
    }
    vn[t] = a0;
    vn[t + stride] = a1;
    out[t] = dinv ? (T)a0 * (T)dinv[t] : (T)a0;
    out[t + stride] = dinv ? (T)a1 * (T)dinv[t + stride] : (T)a1;
    s = fma(a0, a0, s);
    s = fma(a1, a1, s);
  }
  if (t < n) {
    double a = w[t];
#pragma unroll 4
    for (int q = 0; q < nv; q++) a = fma(-hs[q], V[(size_t)q * n + t], a);
    vn[t] = a;
    out[t] = dinv ? (T)a * (T)dinv[t] : (T)a;
    s = fma(a, a, s);
  }
  s = block_sum(s, sh);
  if (threadIdx.x == 0) parts[blockIdx.x] = s;
}
template <typename T>
int launch_cgs_update(KrylovState* st, double* V, const double* w, T* out, size_t n, double* parts, cudaStream_t s,
                      const float* dinv) {
  k_cgs_update<T><<<krylov_nblocks(n), KB, 0, s>>>(st, V, w, out, n, parts, dinv); ++g_launches;
  return (int)cudaGetLastError();
}
template int launch_cgs_update<float>(KrylovState*, double*, const double*, float*, size_t, double*, cudaStream_t,
                                      const float*);
template int launch_cgs_update<double>(KrylovState*, double*, const double*, double*, size_t, double*, cudaStream_t,
                                       const float*);

// Fused CGS2 middle pass: w <- w - V h (h from the first pass), and the
// second pass's dots V_q . w computed on the updated element while the basis
// values are still in registers.  NV = compile-time capacity; the kernel does
// its work only when NV0 < nv <= NV, so a fixed sequence of launches with
// increasing capacities serves every column count (graph-replayable) while
// the FP64 FMAs issued stay within 4 of 2 nv per element.
template <int NV0, int NV>
__global__ void __launch_bounds__(KB) k_gs_update_dots(const KrylovState* st, const double* __restrict__ V, int nv,
                                                       double* __restrict__ w, size_t n, double* parts, int ld) {
  if (is_done(st)) return;
  nv = nv_of(st, nv);
  if (nv <= NV0 || nv > NV) return;
  __shared__ double hs[NV];
  __shared__ double red[KB / 32][NV];
  for (int q = threadIdx.x; q < NV; q += blockDim.x) hs[q] = q < nv ? st->h[q] * st->vs[q] : 0.;
  __syncthreads();
  double acc[NV];
#pragma unroll
  for (int q = 0; q < NV; q++) acc[q] = 0.;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    double v[NV];
    double a = w[t];
#pragma unroll
    for (int q = 0; q < NV; q++) {
      v[q] = q < nv ? V[(size_t)q * n + t] : 0.;
      a = fma(-hs[q], v[q], a);
    }
    w[t] = a;
#pragma unroll
    for (int q = 0; q < NV; q++) acc[q] = fma(v[q], a, acc[q]);
  }
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NV; q++) {
    double x = warp_sum(acc[q]);
    if (lane == 0) red[wp][q] = x;
  }
  __syncthreads();
  for (int q = threadIdx.x; q < nv; q += blockDim.x) {
    double x = 0.;
    for (int u = 0; u < KB / 32; u++) x += red[u][q];
    parts[(size_t)blockIdx.x * ld + q] = x;
  }
}

// nv < 0: device column count, capacity chosen from cap (>= the largest nv).
int launch_gs_update_dots(KrylovState* st, const double* V, int nv, double* w, size_t n, double* parts, cudaStream_t s,
                          int cap) {
  const int nb = krylov_nblocks(n);
  const int ld = 72;
  if (nv > 32 || (nv < 0 && cap > 32)) return -1;
  // nv >= 0: the one bucket holding nv; nv < 0: every bucket up to cap
  const int lo = nv < 0 ? 0 : nv, hi = nv < 0 ? cap : nv;
  if (lo <= 4) { k_gs_update_dots<0, 4><<<nb, KB, 0, s>>>(st, V, nv, w, n, parts, ld); ++g_launches; }
  if (lo <= 8 && hi > 4) { k_gs_update_dots<4, 8><<<nb, KB, 0, s>>>(st, V, nv, w, n, parts, ld); ++g_launches; }
  if (lo <= 16 && hi > 8) { k_gs_update_dots<8, 16><<<nb, KB, 0, s>>>(st, V, nv, w, n, parts, ld); ++g_launches; }
  if (lo <= 24 && hi > 16) { k_gs_update_dots<16, 24><<<nb, KB, 0, s>>>(st, V, nv, w, n, parts, ld); ++g_launches; }
  if (hi > 24) { k_gs_update_dots<24, 32><<<nb, KB, 0, s>>>(st, V, nv, w, n, parts, ld); ++g_launches; }
  k_multidot_finish<<<1, KB, 0, s>>>(st, parts, nb, nv, ld, 2); ++g_launches;
  return (int)cudaGetLastError();
}

// Close Arnoldi column j: ||w||, Hessenberg column, Givens rotation, residual
// estimate |g[j+1]|, convergence test, 1 / h[j+1][j] for the next basis vector.
// The column, the previous rotations and g[j] are staged in shared memory by
// the whole block first, so that the serial rotation loop of thread 0 reads
// no global memory.
__global__ void k_arnoldi_finish(KrylovState* st, const double* __restrict__ parts, int nparts) {
  if (is_done(st)) return;
  __shared__ double sh[32];
  __shared__ double hc[MAXCOL + 2], cq[MAXCOL + 1], sq[MAXCOL + 1];
  double s = 0.;
  for (int p = threadIdx.x; p < nparts; p += blockDim.x) s += parts[p];
  const int m = st->m, j = st->j;
  for (int q = threadIdx.x; q <= j; q += blockDim.x) hc[q] = st->hacc[q];
  for (int q = threadIdx.x; q < j; q += blockDim.x) {
    cq[q] = st->cs[q];
    sq[q] = st->sn[q];
  }
  s = block_sum(s, sh);  // (its barriers also order the staging)
  if (threadIdx.x != 0) return;
  const double hn = sqrt(s);
  double* Hc = st->H + (size_t)j * (m + 1);
  hc[j + 1] = hn;
  for (int q = 0; q < j; q++) {
    const double a = hc[q], b = hc[q + 1];
    hc[q] = cq[q] * a + sq[q] * b;
    hc[q + 1] = -sq[q] * a + cq[q] * b;
  }
  for (int q = 0; q < j; q++) Hc[q] = hc[q];
  const double a = hc[j], b = hc[j + 1];
  const double den = sqrt(a * a + b * b);
  const double c = den > 0. ? a / den : 1., sn = den > 0. ? b / den : 0.;
  st->cs[j] = c;
  st->sn[j] = sn;
  Hc[j] = den;
  Hc[j + 1] = 0.;
  st->g[j + 1] = -sn * st->g[j];
  st->g[j] = c * st->g[j];
  st->resid = fabs(st->g[j + 1]);
  st->hn = hn;
  st->inv_hn = hn > 0. ? 1. / hn : 0.;
  st->vs[j + 1] = st->orth2 ? 1. : st->inv_hn;  // CGS2 normalises the column in k_vnext_in
  st->j = j + 1;
  st->it += 1;
  if (met(st, st->resid) || hn == 0. || !(st->resid == st->resid)) st->done = 1;
}
int launch_arnoldi_finish(KrylovState* st, int nparts, const double* parts, cudaStream_t s) {
  k_arnoldi_finish<<<1, KB, 0, s>>>(st, parts, nparts); ++g_launches;
  return (int)cudaGetLastError();
}

// y = R^{-1} g over the st->j closed columns (runs whether or not done).
__global__ void k_lsq(KrylovState* st) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int m = st->m, J = st->j;
  for (int q = J - 1; q >= 0; q--) {
    double s = st->g[q];
    for (int p = q + 1; p < J; p++) s -= st->H[(size_t)p * (m + 1) + q] * st->y[p];
    st->y[q] = s / st->H[(size_t)q * (m + 1) + q];
  }
}
int launch_lsq_update(KrylovState* st, cudaStream_t s) {
  k_lsq<<<1, 32, 0, s>>>(st); ++g_launches;
  return (int)cudaGetLastError();
}

// x += sum_q y_q Z_q over the closed columns.
template <typename T>
__global__ void __launch_bounds__(KB) k_x_update(const KrylovState* st, const T* __restrict__ Z, size_t n, double* x) {
  __shared__ double ys[72];
  const int J = st->j;
  for (int q = threadIdx.x; q < J; q += blockDim.x) ys[q] = st->y[q] * st->vs[q];
  __syncthreads();
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    double a = x[t];
    for (int q = 0; q < J; q++) a = fma(ys[q], to_acc<double>(Z[(size_t)q * n + t]), a);
    x[t] = a;
  }
}
template <typename T>
int launch_x_update(KrylovState* st, const T* Z, size_t n, double* x, cudaStream_t s) {
  k_x_update<T><<<krylov_nblocks(n) * 4, KB, 0, s>>>(st, Z, n, x); ++g_launches;
  return (int)cudaGetLastError();
}
template int launch_x_update<float>(KrylovState*, const float*, size_t, double*, cudaStream_t);
template int launch_x_update<double>(KrylovState*, const double*, size_t, double*, cudaStream_t);

// Mark the closed columns as applied (a later x update adds nothing).
__global__ void k_restart_reset(KrylovState* st) {
  if (threadIdx.x == 0 && blockIdx.x == 0) st->j = 0;
}
int launch_restart_reset(KrylovState* st, cudaStream_t s) {
  k_restart_reset<<<1, 32, 0, s>>>(st); ++g_launches;
  return (int)cudaGetLastError();
}

// out = ||v||_2 (no Krylov state involved).
__global__ void k_sqrt_sum(const double* __restrict__ parts, int nparts, double* out) {
  __shared__ double sh[32];
  double s = 0.;
  for (int p = threadIdx.x; p < nparts; p += blockDim.x) s += parts[p];
  s = block_sum(s, sh);
  if (threadIdx.x == 0) *out = sqrt(s);
}
int launch_norm2(const double* v, size_t n, double* parts, double* out, cudaStream_t s) {
  const int nb = krylov_nblocks(n);
  k_sq_partials<<<nb, KB, 0, s>>>(nullptr, v, n, parts, 0); ++g_launches;
  k_sqrt_sum<<<1, KB, 0, s>>>(parts, nb, out); ++g_launches;
  return (int)cudaGetLastError();
}

// Next basis vector and multigrid input in one sweep: V_{j+1} = w / h_{j+1,j}
// and out = T(V_{j+1}) over the interior; ghost entries of w are zero.
// vn == nullptr: the target is V + st->j * n (the column just opened).
template <typename T>
__global__ void __launch_bounds__(KB) k_vnext_in(const KrylovState* st, const double* __restrict__ w, double* vn,
                                                  T* __restrict__ out, size_t n, double* V,
                                                  const float* __restrict__ dinv) {
  if (is_done(st)) return;
  const double f = st->inv_hn;
  if (!vn) vn = V + (size_t)st->j * n;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const double v = w[t] * f;
    vn[t] = v;
    out[t] = dinv ? (T)v * (T)dinv[t] : (T)v;
  }
}
template <typename T>
int launch_vnext_in(KrylovState* st, const double* w, double* vn, T* out, size_t n, cudaStream_t s, double* V,
                    const float* dinv) {
  k_vnext_in<T><<<krylov_nblocks(n) * 4, KB, 0, s>>>(st, w, vn, out, n, V, dinv); ++g_launches;
  return (int)cudaGetLastError();
}
template int launch_vnext_in<float>(KrylovState*, const double*, double*, float*, size_t, cudaStream_t, double*,
                                    const float*);
template int launch_vnext_in<double>(KrylovState*, const double*, double*, double*, size_t, cudaStream_t, double*,
                                     const float*);

// done and epoch (adjacent) to pinned host memory
int launch_status_copy(const KrylovState* st, int* hst, cudaStream_t s) {
  return (int)cudaMemcpyAsync(hst, &st->done, 2 * sizeof(int), cudaMemcpyDeviceToHost, s);
}

}  // namespace vfs
