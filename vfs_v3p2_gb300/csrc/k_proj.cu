// Per-step FP64 kernels around the solve: the divergence right-hand side and
// its compatibility fix, the immersed-boundary flux balance, null-space
// removal, the phi / pressure ghost fills, the contravariant velocity
// correction (Projection), Contra2Cart and the divergence check.
//
// Compiled with --fmad=false like k_setup.cu: each kernel performs the
// reference's multiplies and adds in the reference's order, so for equal
// inputs the outputs are bit-identical (reductions excepted, which sum in a
// fixed tree order instead of the reference's loop order).
#include <mutex>

#include "vfs_common.cuh"
#include "vfs_kernels.h"
#include "vfs_proj.h"

namespace vfs {

constexpr int RB = 256;  // reduction block size

#define GRID_LOOP(d)                                                                          \
  for (size_t _t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; _t < ncell(d);              \
       _t += (size_t)gridDim.x * blockDim.x)
// cells [c0, c1) of the grid, grid-stride
#define RANGE_LOOP(c0, c1)                                                                     \
  for (size_t _t = (c0) + blockIdx.x * (size_t)blockDim.x + threadIdx.x; _t < (c1);           \
       _t += (size_t)gridDim.x * blockDim.x)
// 32-bit index split (grids stay below 2^31 cells)
#define DECOMP(d, i, j, k)                          \
  const unsigned _u = (unsigned)_t;                 \
  const unsigned _q = _u / (unsigned)(d).mx;        \
  int i = (int)(_u - _q * (unsigned)(d).mx);        \
  int k = (int)(_q / (unsigned)(d).my);             \
  int j = (int)(_q - (unsigned)k * (unsigned)(d).my)

static inline int nblk(size_t n, int bs = 256) {
  size_t b = (n + bs - 1) / bs;
  if (b > 152 * 16) b = 152 * 16;
  return (int)(b ? b : 1);
}

// Sum per-block partials [nparts][q] in index order (one block).
__global__ void k_finish_sums(const double* __restrict__ parts, int nparts, int nq, double* out) {
  __shared__ double sh[32];
  for (int q = 0; q < nq; q++) {
    double s = 0.;
    for (int p = threadIdx.x; p < nparts; p += blockDim.x) s += parts[(size_t)p * nq + q];
    s = block_sum(s, sh);
    if (threadIdx.x == 0) out[q] = s;
    __syncthreads();
  }
}
__global__ void k_finish_max(const double* __restrict__ parts, int nparts, double* out) {
  __shared__ double sh[32];
  double s = 0.;
  for (int p = threadIdx.x; p < nparts; p += blockDim.x) s = fmax(s, parts[p]);
  s = block_max(s, sh);
  if (threadIdx.x == 0) *out = s;
}

// ---- AoS (reference Cmpnts) <-> SoA device layout ----
__global__ void k_aos2soa(size_t n, const double* __restrict__ a, double* x, double* y, double* z) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    x[t] = a[3 * t];
    y[t] = a[3 * t + 1];
    z[t] = a[3 * t + 2];
  }
}
__global__ void k_soa2aos(size_t n, const double* __restrict__ x, const double* __restrict__ y, const double* __restrict__ z,
                          double* a) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    a[3 * t] = x[t];
    a[3 * t + 1] = y[t];
    a[3 * t + 2] = z[t];
  }
}
int launch_aos2soa(size_t n, const double* aos, double* x, double* y, double* z, cudaStream_t s) {
  k_aos2soa<<<nblk(n), 256, 0, s>>>(n, aos, x, y, z); ++g_launches;
  return (int)cudaGetLastError();
}
int launch_soa2aos(size_t n, const double* x, const double* y, const double* z, double* aos, cudaStream_t s) {
  k_soa2aos<<<nblk(n), 256, 0, s>>>(n, x, y, z, aos); ++g_launches;
  return (int)cudaGetLastError();
}

// ---------------------------------------------------------------------------
// PoissonRHS2_hypre (poisson_hypre.c:342-429): b = div(U*) * st * coeff / dt
// on fluid cells, periodic wrap of the minus faces; partial sums of b and of
// the fluid count for the compatibility fix of PoissonRHS2 (poisson.c:1879-1903).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(RB) k_rhs(Dims d, Ucont u, const double* __restrict__ nvert, double dt, double st,
                                            double coeff, double* b, double* parts) {
  __shared__ double sh[32];
  __shared__ unsigned shc[32];
  double lsum = 0.;
  unsigned lcnt = 0;  // fluid cells, counted on the integer pipe (exact)
  GRID_LOOP(d) {
    DECOMP(d, i, j, k);
    double val = 0.;
    if (interior(d, i, j, k) && !(nvert[_t] >= 0.1)) {
      val -= u.x[_t];
      if (i == 1 && d.ip) val += u.x[cidx(d, d.mx - 2, j, k)];
      else val += u.x[cidx(d, i - 1, j, k)];
      val -= u.y[_t];
      if (j == 1 && d.jp) val += u.y[cidx(d, i, d.my - 2, k)];
      else val += u.y[cidx(d, i, j - 1, k)];
      val -= u.z[_t];
      if (k == 1 && d.kp) val += u.z[cidx(d, i, j, d.mz - 2)];
      else val += u.z[cidx(d, i, j, k - 1)];
      val *= -1.0 / dt * st * coeff;
      lsum += val;
      lcnt += 1;
    }
    b[_t] = val;
  }
  lsum = block_sum(lsum, sh);
  lcnt = block_sum(lcnt, shc);
  if (threadIdx.x == 0) {
    parts[2 * blockIdx.x] = lsum;
    parts[2 * blockIdx.x + 1] = (double)lcnt;
  }
}
// b += -sum / count on fluid interior cells (sc = {sum, count}).
__global__ void k_meanfix(Dims d, const double* __restrict__ nvert, const double* __restrict__ sc, double* b) {
  const double v = (sc[1] > 0.) ? -sc[0] / sc[1] : 0.;
  GRID_LOOP(d) {
    DECOMP(d, i, j, k);
    if (interior(d, i, j, k) && nvert[_t] < 0.1) b[_t] += v;
  }
}
int launch_rhs(const Dims& d, const Ucont& u, const double* nvert, double dt, double st, double coeff, int meanfix,
               double* b, double* parts, double* sc, cudaStream_t s, const int* comp, int ncomp) {
  const int nb = nblk(ncell(d), RB);
  k_rhs<<<nb, RB, 0, s>>>(d, u, nvert, dt, st, coeff, b, parts); ++g_launches;
  k_finish_sums<<<1, 256, 0, s>>>(parts, nb, 2, sc); ++g_launches;
  if (meanfix && comp && ncomp > 1) {
    // one compatibility fix per connected fluid region (sums in sc[2..3])
    return launch_remove_mean(d, nvert, b, parts, sc + 2, s, comp, ncomp);
  }
  if (meanfix) {
    k_meanfix<<<nblk(ncell(d)), 256, 0, s>>>(d, nvert, sc, b);
    ++g_launches;
  }
  return (int)cudaGetLastError();
}

// ---------------------------------------------------------------------------
// IB flux balance.  mode 1: VolumeFlux(flg = 0), poisson.c:2898-3240
// (immersed == 1).  mode 0: VolumeFlux(lUcor), poisson.c:2634-2828 with
// immersed == 0, which zeroes every fluid / non-fluid face.
// phase 0: (mode 1) zero faces with |U| <= 1e-10 and sum flux, area;
// phase 1: apply the correction flux / area and sum the corrected faces again
// (the reference's second measuring pass, fused: same values, same order).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double nrm3(const double* v, size_t c) {
  return sqrt(v[3 * c] * v[3 * c] + v[3 * c + 1] * v[3 * c + 1] + v[3 * c + 2] * v[3 * c + 2]);
}

// nb8 (nvert as bytes, every value an integer in [0, 127]) turns the FP64
// interface tests into exact integer ones: nv < 0.1 <=> 0, nv > 0.1 <=> >= 1,
// 0.1 < nv < 1.1 <=> 1.
__global__ void __launch_bounds__(RB) k_vflux(Dims d, int mode, int phase, Ucont u, const double* __restrict__ nv,
                                              const double* __restrict__ csi, const double* __restrict__ eta,
                                              const double* __restrict__ zet, const double* __restrict__ fa, double* parts,
                                              const uint8_t* __restrict__ nb8) {
  __shared__ double sh[32];
  const double eps = 1.e-10, ibmval = 1.1;
  double flux = 0., area = 0.;
  double corr = 0.;
  if (phase == 1) corr = (fa[1] > 1.e-15) ? fa[0] / fa[1] : 0.;
  GRID_LOOP(d) {
    DECOMP(d, i, j, k);
    if (!interior(d, i, j, k)) continue;
    const size_t c = _t;
    const size_t ce = cidx(d, i + 1, j, k), cn = cidx(d, i, j + 1, k), ct = cidx(d, i, j, k + 1);
    double* uf[3] = {u.x, u.y, u.z};
    const double* mt[3] = {csi, eta, zet};
    const size_t nb[3] = {ce, cn, ct};
    const bool lim1[3] = {i < d.mx - 2, j < d.my - 2, k < d.mz - 2};
    const bool lim0[3] = {i <= d.mx - 2, j <= d.my - 2, k <= d.mz - 2};
    for (int f = 0; f < 3; f++) {
      double* uu = uf[f];
      if (mode == 1) {
        bool plus, minus;
        if (nb8) {
          const int a = nb8[c], b = nb8[nb[f]];
          plus = a == 0 && b == 1 && lim1[f];
          minus = a == 1 && b == 0 && lim1[f];
        } else {
          plus = nv[c] < 0.1 && nv[nb[f]] > 0.1 && nv[nb[f]] < ibmval && lim1[f];
          minus = nv[c] > 0.1 && nv[c] < ibmval && nv[nb[f]] < 0.1 && lim1[f];
        }
        if (!(plus || minus)) continue;
        if (phase == 0) {
          if (fabs(uu[c]) > eps) {
            flux += plus ? uu[c] : -uu[c];
            area += nrm3(mt[f], c);
          } else uu[c] = 0.;
        } else {
          // phase 1: correct, and measure the corrected face at once (the
          // same values and order as a separate measuring pass)
          const double nr = nrm3(mt[f], c);
          if (fabs(uu[c]) > eps) {
            if (plus) uu[c] -= nr * corr;
            else uu[c] += nr * corr;
          }
          flux += plus ? uu[c] : -uu[c];
          area += nr;
        }
      } else {
        bool plus, minus;
        if (nb8) {
          const int a = nb8[c], b = nb8[nb[f]];
          plus = a == 0 && b != 0 && lim0[f];
          minus = a != 0 && b == 0 && lim0[f];
        } else {
          plus = nv[c] < VFS_THR && nv[nb[f]] > VFS_THR && lim0[f];
          minus = nv[c] > VFS_THR && nv[nb[f]] < VFS_THR && lim0[f];
        }
        if (!(plus || minus)) continue;
        if (phase == 1) uu[c] = 0.;  // and measured as such
        flux += plus ? uu[c] : -uu[c];
        area += nrm3(mt[f], c);
      }
    }
  }
  flux = block_sum(flux, sh);
  area = block_sum(area, sh);
  if (threadIdx.x == 0) {
    parts[2 * blockIdx.x] = flux;
    parts[2 * blockIdx.x + 1] = area;
  }
}
int launch_volume_flux(const Dims& d, int mode, const Ucont& u, const double* nvert, const double* M, double* parts,
                       double* fa4, cudaStream_t s, const uint8_t* nb8) {
  const size_t N = ncell(d);
  const int nb = nblk(N, RB);
  const double *csi = M + N * MP_CSI, *eta = M + N * MP_ETA, *zet = M + N * MP_ZET;
  k_vflux<<<nb, RB, 0, s>>>(d, mode, 0, u, nvert, csi, eta, zet, fa4, parts, nb8); ++g_launches;
  k_finish_sums<<<1, 256, 0, s>>>(parts, nb, 2, fa4); ++g_launches;
  k_vflux<<<nb, RB, 0, s>>>(d, mode, 1, u, nvert, csi, eta, zet, fa4, parts, nb8); ++g_launches;
  k_finish_sums<<<1, 256, 0, s>>>(parts, nb, 2, fa4 + 2); ++g_launches;
  return (int)cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Remove_Nullspace (poisson_hypre.c:207-270): subtract the fluid mean of phi.
// With comp (labels of the connected fluid regions), only region q: a grid
// cut apart by bodies has one constant null vector per region, as in the
// reference's two-region split of PoissonNullSpaceFunction
// (poisson.c:819-873, regions from FullyBlocked, poisson.c:1918-1998).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(RB) k_fluid_sum(Dims d, const double* __restrict__ nvert, const double* __restrict__ x,
                                                  double* parts, const int* __restrict__ comp, int q) {
  __shared__ double sh[32];
  __shared__ unsigned shc[32];
  double s = 0.;
  unsigned n = 0;  // counted on the integer pipe (exact)
  GRID_LOOP(d) {
    DECOMP(d, i, j, k);
    if (interior(d, i, j, k) && nvert[_t] < 0.1 && (!comp || comp[_t] == q)) {
      s += x[_t];
      n += 1;
    }
  }
  s = block_sum(s, sh);
  n = block_sum(n, shc);
  if (threadIdx.x == 0) {
    parts[2 * blockIdx.x] = s;
    parts[2 * blockIdx.x + 1] = (double)n;
  }
}
__global__ void k_sub_mean(Dims d, const double* __restrict__ nvert, const double* __restrict__ sc, double* x,
                           const int* __restrict__ comp, int q) {
  const double v = (sc[1] > 0.) ? -sc[0] / sc[1] : 0.;
  GRID_LOOP(d) {
    DECOMP(d, i, j, k);
    if (interior(d, i, j, k) && nvert[_t] < 0.1 && (!comp || comp[_t] == q)) x[_t] += v;
  }
}
int launch_remove_mean(const Dims& d, const double* nvert, double* x, double* parts, double* sc, cudaStream_t s,
                       const int* comp, int ncomp) {
  const int nb = nblk(ncell(d), RB);
  const int nq = (comp && ncomp > 1) ? ncomp : 1;
  const int* cm = nq > 1 ? comp : nullptr;
  for (int q = 0; q < nq; q++) {
    k_fluid_sum<<<nb, RB, 0, s>>>(d, nvert, x, parts, cm, q); ++g_launches;
    k_finish_sums<<<1, 256, 0, s>>>(parts, nb, 2, sc); ++g_launches;
    k_sub_mean<<<nblk(ncell(d)), 256, 0, s>>>(d, nvert, sc, x, cm, q); ++g_launches;
  }
  return (int)cudaGetLastError();
}

// Convert_Phi2_Phi (poisson.c:97-185): zero on boundary and non-fluid cells.
__global__ void k_phi_zero(Dims d, const double* __restrict__ nvert, double* phi) {
  GRID_LOOP(d) {
    DECOMP(d, i, j, k);
    if (!interior(d, i, j, k) || (int)nvert[_t] > VFS_THR) phi[_t] = 0.;
  }
}
// Periodic ghost fill of a scalar (poisson.c:146-181, 2580-2616).
__global__ void k_scalar_ghosts(Dims d, double* a) {
  GRID_LOOP(d) {
    DECOMP(d, i, j, k);
    int ai = wrapi(i, d.mx, d.ip), bj = wrapi(j, d.my, d.jp), ck = wrapi(k, d.mz, d.kp);
    if (ai != i || bj != j || ck != k) a[_t] = a[cidx(d, ai, bj, ck)];
  }
}
int launch_phi_finish(const Dims& d, const double* nvert, double* phi, cudaStream_t s) {
  k_phi_zero<<<nblk(ncell(d)), 256, 0, s>>>(d, nvert, phi); ++g_launches;
  k_scalar_ghosts<<<nblk(ncell(d)), 256, 0, s>>>(d, phi); ++g_launches;
  return (int)cudaGetLastError();
}

// UpdatePressure (poisson.c:2522-2548, non-PRIMITIVE branch, + ghost fill).
__global__ void k_update_p(Dims d, const double* __restrict__ nvert, const double* __restrict__ phi, double* p) {
  GRID_LOOP(d) {
    DECOMP(d, i, j, k);
    if (interior(d, i, j, k) && nvert[_t] < 0.1) p[_t] += phi[_t];
  }
}
int launch_update_pressure(const Dims& d, const double* nvert, const double* phi, double* p, cudaStream_t s) {
  k_update_p<<<nblk(ncell(d)), 256, 0, s>>>(d, nvert, phi, p); ++g_launches;
  k_scalar_ghosts<<<nblk(ncell(d)), 256, 0, s>>>(d, p); ++g_launches;
  return (int)cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Projection (poisson.c:2202-2397): U^xi -= (dpdc g11 + dpde g12 + dpdz g13)
// dt st / coeff at i faces (likewise j, k), with the LHS's one-sided /
// centred / zero regimes for the cross derivatives; faces touching nvert are
// left alone.  pd holds the nine metric dot products of each face family
// (icsi.icsi, ieta.icsi, izet.icsi, jcsi.jeta, jeta.jeta, jzet.jeta,
// kcsi.kzet, keta.kzet, kzet.kzet) and M the face Jacobians iaj, jaj, kaj,
// multiplied in the reference's order: (dpdc * dot) * iaj.
// ---------------------------------------------------------------------------
// x / coeff is skipped when coeff == 1 (x / 1.0 == x exactly), and x * st
// when st == 1 (x * 1.0 == x exactly); r1 = r2 = r3 = 1 (no level set), so
// their divisions are always exact and omitted.
__device__ __forceinline__ double div_c(double x, double coeff) { return coeff == 1.0 ? x : x / coeff; }
__device__ __forceinline__ double mul_st(double x, double st) { return st == 1.0 ? x : x * st; }

template <bool NVI>
__global__ void __launch_bounds__(128) k_projection(Dims d, size_t c0, size_t c1, const double* __restrict__ pd,
                             const double* __restrict__ iaj,
                             const double* __restrict__ jaj, const double* __restrict__ kaj, const double* __restrict__ nvert,
                             const uint8_t* __restrict__ nb8, const double* __restrict__ phi, double dt, double st,
                             double coeff, Ucont u) {
  const size_t N = ncell(d);
  const int mx = d.mx, my = d.my, mz = d.mz, ip = d.ip, jp = d.jp, kp = d.kp;
  const double THR = VFS_THR;
  auto gt2 = [&](size_t a, size_t b) -> bool {
    if (NVI) return (nb8[a] | nb8[b]) != 0;
    return nvert[a] + nvert[b] > THR;
  };
  auto lt2 = [&](size_t a, size_t b) -> bool {
    if (NVI) return (nb8[a] | nb8[b]) == 0;
    return nvert[a] + nvert[b] < THR;
  };
  RANGE_LOOP(c0, c1) {
    DECOMP(d, i, j, k);
    const size_t c = _t;
// nvert pair tests: with NVI every nvert is an integer in [0, 127] and nb8
// holds it as a byte, so a + b > 0.1 <=> (a | b) != 0 and a + b < 0.1 <=>
// (a | b) == 0 exactly (no FP64 add and compare)
#define NVX(ii, jj, kk) cidx(d, ii, jj, kk)
#define GT2(A, B) gt2(NVX A, NVX B)
#define LT2(A, B) lt2(NVX A, NVX B)
#define PH(ii, jj, kk) phi[cidx(d, ii, jj, kk)]
    double dpdc, dpde, dpdz;
    if (j > 0 && j < my - 1 && k > 0 && k < mz - 1)
      if ((i > 0 && i < mx - 2) || (ip && i == mx - 2)) {
        dpdc = PH(i + 1, j, k) - PH(i, j, k);
        if (i == mx - 2 && ip) dpdc = PH(1, j, k) - PH(i, j, k);
        dpde = 0.;
        dpdz = 0.;
        if ((j == my - 2 && !jp) || GT2((i, j + 1, k), (i + 1, j + 1, k))) {
          if (LT2((i, j - 1, k), (i + 1, j - 1, k)) && (j != 1))
            dpde = (PH(i, j, k) + PH(i + 1, j, k) - PH(i, j - 1, k) - PH(i + 1, j - 1, k)) * 0.5;
        } else if ((j == 1 && !jp) || GT2((i, j - 1, k), (i + 1, j - 1, k))) {
          if (LT2((i, j + 1, k), (i + 1, j + 1, k)))
            dpde = (PH(i, j + 1, k) + PH(i + 1, j + 1, k) - PH(i, j, k) - PH(i + 1, j, k)) * 0.5;
        } else {
          dpde = (PH(i, j + 1, k) + PH(i + 1, j + 1, k) - PH(i, j - 1, k) - PH(i + 1, j - 1, k)) * 0.25;
        }
        if ((k == mz - 2 && !kp) || GT2((i, j, k + 1), (i + 1, j, k + 1))) {
          if (LT2((i, j, k - 1), (i + 1, j, k - 1)) && (k != 1))
            dpdz = (PH(i, j, k) + PH(i + 1, j, k) - PH(i, j, k - 1) - PH(i + 1, j, k - 1)) * 0.5;
        } else if ((k == 1 && !kp) || GT2((i, j, k - 1), (i + 1, j, k - 1))) {
          if (LT2((i, j, k + 1), (i + 1, j, k + 1)))
            dpdz = (PH(i, j, k + 1) + PH(i + 1, j, k + 1) - PH(i, j, k) - PH(i + 1, j, k)) * 0.5;
        } else {
          dpdz = (PH(i, j, k + 1) + PH(i + 1, j, k + 1) - PH(i, j, k - 1) - PH(i + 1, j, k - 1)) * 0.25;
        }
        if (LT2((i, j, k), (i + 1, j, k))) {
          const double a = iaj[c];
          u.x[c] -= div_c(mul_st((dpdc * pd[0 * N + c] * a + dpde * pd[1 * N + c] * a + dpdz * pd[2 * N + c] * a) * dt, st), coeff);
        }
      }
    if (i > 0 && i < mx - 1 && k > 0 && k < mz - 1)
      if ((j > 0 && j < my - 2) || (jp && j == my - 2)) {
        dpdc = 0.;
        dpdz = 0.;
        if ((i == mx - 2 && !ip) || GT2((i + 1, j, k), (i + 1, j + 1, k))) {
          if (LT2((i - 1, j, k), (i - 1, j + 1, k)) && (i != 1))
            dpdc = (PH(i, j, k) + PH(i, j + 1, k) - PH(i - 1, j, k) - PH(i - 1, j + 1, k)) * 0.5;
        } else if ((i == 1 && !ip) || GT2((i - 1, j, k), (i - 1, j + 1, k))) {
          if (LT2((i + 1, j, k), (i + 1, j + 1, k)))
            dpdc = (PH(i + 1, j, k) + PH(i + 1, j + 1, k) - PH(i, j, k) - PH(i, j + 1, k)) * 0.5;
        } else {
          dpdc = (PH(i + 1, j, k) + PH(i + 1, j + 1, k) - PH(i - 1, j, k) - PH(i - 1, j + 1, k)) * 0.25;
        }
        if (j == my - 2 && jp) dpde = PH(i, 1, k) - PH(i, j, k);
        else dpde = PH(i, j + 1, k) - PH(i, j, k);
        if ((k == mz - 2 && !kp) || GT2((i, j, k + 1), (i, j + 1, k + 1))) {
          if (LT2((i, j, k - 1), (i, j + 1, k - 1)) && (k != 1))
            dpdz = (PH(i, j, k) + PH(i, j + 1, k) - PH(i, j, k - 1) - PH(i, j + 1, k - 1)) * 0.5;
        } else if ((k == 1 && !kp) || GT2((i, j, k - 1), (i, j + 1, k - 1))) {
          if (LT2((i, j, k + 1), (i, j + 1, k + 1)))
            dpdz = (PH(i, j, k + 1) + PH(i, j + 1, k + 1) - PH(i, j, k) - PH(i, j + 1, k)) * 0.5;
        } else {
          dpdz = (PH(i, j, k + 1) + PH(i, j + 1, k + 1) - PH(i, j, k - 1) - PH(i, j + 1, k - 1)) * 0.25;
        }
        if (LT2((i, j, k), (i, j + 1, k))) {
          const double a = jaj[c];
          u.y[c] -= div_c(mul_st((dpdc * pd[3 * N + c] * a + dpde * pd[4 * N + c] * a + dpdz * pd[5 * N + c] * a) * dt, st), coeff);
        }
      }
    if (i > 0 && i < mx - 1 && j > 0 && j < my - 1)
      if ((k > 0 && k < mz - 2) || (kp && k == mz - 2)) {
        dpdc = 0.;
        dpde = 0.;
        if ((i == mx - 2 && !ip) || GT2((i + 1, j, k), (i + 1, j, k + 1))) {
          if (LT2((i - 1, j, k), (i - 1, j, k + 1)) && (i != 1))
            dpdc = (PH(i, j, k) + PH(i, j, k + 1) - PH(i - 1, j, k) - PH(i - 1, j, k + 1)) * 0.5;
        } else if ((i == 1 && !ip) || GT2((i - 1, j, k), (i - 1, j, k + 1))) {
          if (LT2((i + 1, j, k), (i + 1, j, k + 1)))
            dpdc = (PH(i + 1, j, k) + PH(i + 1, j, k + 1) - PH(i, j, k) - PH(i, j, k + 1)) * 0.5;
        } else {
          dpdc = (PH(i + 1, j, k) + PH(i + 1, j, k + 1) - PH(i - 1, j, k) - PH(i - 1, j, k + 1)) * 0.25;
        }
        if ((j == my - 2 && !jp) || GT2((i, j + 1, k), (i, j + 1, k + 1))) {
          if (LT2((i, j - 1, k), (i, j - 1, k + 1)) && (j != 1))
            dpde = (PH(i, j, k) + PH(i, j, k + 1) - PH(i, j - 1, k) - PH(i, j - 1, k + 1)) * 0.5;
        } else if ((j == 1 && !jp) || GT2((i, j - 1, k), (i, j - 1, k + 1))) {
          if (LT2((i, j + 1, k), (i, j + 1, k + 1)))
            dpde = (PH(i, j + 1, k) + PH(i, j + 1, k + 1) - PH(i, j, k) - PH(i, j, k + 1)) * 0.5;
        } else {
          dpde = (PH(i, j + 1, k) + PH(i, j + 1, k + 1) - PH(i, j - 1, k) - PH(i, j - 1, k + 1)) * 0.25;
        }
        if (k == mz - 2 && kp) dpdz = PH(i, j, 1) - PH(i, j, k);
        else dpdz = PH(i, j, k + 1) - PH(i, j, k);
        if (LT2((i, j, k), (i, j, k + 1))) {
          const double a = kaj[c];
          u.z[c] -= div_c(mul_st((dpdc * pd[6 * N + c] * a + dpde * pd[7 * N + c] * a + dpdz * pd[8 * N + c] * a) * dt, st), coeff);
        }
      }
#undef PH
#undef NVX
#undef GT2
#undef LT2
  }
}

// ---------------------------------------------------------------------------
// Projection on precomputed face weights.  Every choice the reference's
// Projection makes per face (poisson.c:2221-2363: the face is skipped where
// nvert touches it, each cross derivative is centred, one-sided or zero by
// the nvert and wall tests) depends on the grid only, so it is made once
// (k_proj_weights, at the operator set-up): per face a normal weight
// dot * aj_face and two cross weights s * dot * aj_face (s = 0.25 centred,
// 0.5 one-sided, 0 none; all three 0 where the face is not projected), and
// per cross term two code bits choosing its upper and lower pair (the pair
// beside the face, or the face's own pair for a one-sided difference).  The
// step then applies, per face, U -= (wN dn + wA (Up_A - Lo_A) + wB (Up_B -
// Lo_B)) dt st / coeff with FMAs: at most 33 FP64 operations per cell
// instead of about 60, and no nvert loads.  The same
// products in a different order: the result differs from the reference's
// operation order by rounding (<= 1e-14 relative).
// pw: [9][N] (i face: normal, j cross, k cross | j face: normal, i cross,
// k cross | k face: normal, i cross, j cross); pc: two bits per cross term
// in that order (bit 0: the upper pair is the face's own, bit 1: the lower),
// then bits 12, 13, 14: the i, j, k face is projected (a face that is not
// keeps its flux bit for bit).
// ---------------------------------------------------------------------------
__global__ void k_proj_weights(Dims d, const double* __restrict__ pd, const double* __restrict__ iaj,
                               const double* __restrict__ jaj, const double* __restrict__ kaj,
                               const double* __restrict__ nvert, double* __restrict__ pw, uint16_t* __restrict__ pc) {
  const size_t N = ncell(d);
  const int mx = d.mx, my = d.my, mz = d.mz, ip = d.ip, jp = d.jp, kp = d.kp;
  const double THR = VFS_THR;
  GRID_LOOP(d) {
    DECOMP(d, i, j, k);
    const size_t c = _t;
#define NVX(ii, jj, kk) nvert[cidx(d, ii, jj, kk)]
#define GT2(a, b, cc, e, f, g_) (NVX(a, b, cc) + NVX(e, f, g_) > THR)
#define LT2(a, b, cc, e, f, g_) (NVX(a, b, cc) + NVX(e, f, g_) < THR)
    double w[9] = {0., 0., 0., 0., 0., 0., 0., 0., 0.};
    unsigned code = 0;
    // one cross term: up/low pairs (the face's own one where one-sided) and the scale
    auto cross = [&](bool top_blocked, bool low_ok, bool bot_blocked, bool up_ok, double& sc, unsigned& bits) {
      sc = 0.;
      bits = 0;
      if (top_blocked) {
        if (low_ok) sc = 0.5, bits = 1u;  // (own pair) - (lower pair)
      } else if (bot_blocked) {
        if (up_ok) sc = 0.5, bits = 2u;   // (upper pair) - (own pair)
      } else {
        sc = 0.25;                         // (upper pair) - (lower pair)
      }
    };
    if (j > 0 && j < my - 1 && k > 0 && k < mz - 1 && ((i > 0 && i < mx - 2) || (ip && i == mx - 2)) &&
        LT2(i, j, k, i + 1, j, k)) {  // i face, poisson.c:2221-2265
      double se, sz;
      unsigned be, bz;
      cross((j == my - 2 && !jp) || GT2(i, j + 1, k, i + 1, j + 1, k), LT2(i, j - 1, k, i + 1, j - 1, k) && j != 1,
            (j == 1 && !jp) || GT2(i, j - 1, k, i + 1, j - 1, k), LT2(i, j + 1, k, i + 1, j + 1, k), se, be);
      cross((k == mz - 2 && !kp) || GT2(i, j, k + 1, i + 1, j, k + 1), LT2(i, j, k - 1, i + 1, j, k - 1) && k != 1,
            (k == 1 && !kp) || GT2(i, j, k - 1, i + 1, j, k - 1), LT2(i, j, k + 1, i + 1, j, k + 1), sz, bz);
      const double a = iaj[c];
      w[0] = pd[0 * N + c] * a;
      w[1] = se * (pd[1 * N + c] * a);
      w[2] = sz * (pd[2 * N + c] * a);
      code |= be | (bz << 2) | (1u << 12);
    }
    if (i > 0 && i < mx - 1 && k > 0 && k < mz - 1 && ((j > 0 && j < my - 2) || (jp && j == my - 2)) &&
        LT2(i, j, k, i, j + 1, k)) {  // j face, poisson.c:2267-2314
      double sc, sz;
      unsigned bc, bz;
      cross((i == mx - 2 && !ip) || GT2(i + 1, j, k, i + 1, j + 1, k), LT2(i - 1, j, k, i - 1, j + 1, k) && i != 1,
            (i == 1 && !ip) || GT2(i - 1, j, k, i - 1, j + 1, k), LT2(i + 1, j, k, i + 1, j + 1, k), sc, bc);
      cross((k == mz - 2 && !kp) || GT2(i, j, k + 1, i, j + 1, k + 1), LT2(i, j, k - 1, i, j + 1, k - 1) && k != 1,
            (k == 1 && !kp) || GT2(i, j, k - 1, i, j + 1, k - 1), LT2(i, j, k + 1, i, j + 1, k + 1), sz, bz);
      const double a = jaj[c];
      w[3] = pd[4 * N + c] * a;
      w[4] = sc * (pd[3 * N + c] * a);
      w[5] = sz * (pd[5 * N + c] * a);
      code |= (bc << 4) | (bz << 6) | (1u << 13);
    }
    if (i > 0 && i < mx - 1 && j > 0 && j < my - 1 && ((k > 0 && k < mz - 2) || (kp && k == mz - 2)) &&
        LT2(i, j, k, i, j, k + 1)) {  // k face, poisson.c:2316-2363
      double sc, se;
      unsigned bc, be;
      cross((i == mx - 2 && !ip) || GT2(i + 1, j, k, i + 1, j, k + 1), LT2(i - 1, j, k, i - 1, j, k + 1) && i != 1,
            (i == 1 && !ip) || GT2(i - 1, j, k, i - 1, j, k + 1), LT2(i + 1, j, k, i + 1, j, k + 1), sc, bc);
      cross((j == my - 2 && !jp) || GT2(i, j + 1, k, i, j + 1, k + 1), LT2(i, j - 1, k, i, j - 1, k + 1) && j != 1,
            (j == 1 && !jp) || GT2(i, j - 1, k, i, j - 1, k + 1), LT2(i, j + 1, k, i, j + 1, k + 1), se, be);
      const double a = kaj[c];
      w[6] = pd[8 * N + c] * a;
      w[7] = sc * (pd[6 * N + c] * a);
      w[8] = se * (pd[7 * N + c] * a);
      code |= (bc << 8) | (be << 10) | (1u << 14);
    }
#undef NVX
#undef GT2
#undef LT2
#pragma unroll
    for (int q = 0; q < 9; q++) pw[(size_t)q * N + c] = w[q];
    pc[c] = (uint16_t)code;
  }
}

int launch_proj_weights(const Dims& d, const double* pd, const double* M, const double* nvert, double* pw, uint16_t* pc,
                        cudaStream_t s) {
  const size_t N = ncell(d);
  k_proj_weights<<<nblk(N), 256, 0, s>>>(d, pd, M + N * MP_IAJ, M + N * MP_JAJ, M + N * MP_KAJ, nvert, pw, pc);
  ++g_launches;
  return (int)cudaGetLastError();
}

// U -= sc (wN dn + wA (Up_A - Lo_A) + wB (Up_B - Lo_B)) on the projected
// faces of the cells [c0, c1) (interior planes; the face bits are set on
// interior cells only, and the normal difference wraps only on a periodic
// seam, where alone the last face is projected); a cross term of weight 0
// loads nothing; every phi read lies in the array (ghost layers included).
__global__ void __launch_bounds__(128) k_projection_fast(Dims d, size_t c0, size_t c1, const double* __restrict__ pw,
                                                         const uint16_t* __restrict__ pc,
                                                         const double* __restrict__ phi, double sc, Ucont u) {
  const size_t N = ncell(d);
  const int mx = d.mx, my = d.my, mz = d.mz;
  const int sy = mx, sz = mx * my;
  RANGE_LOOP(c0, c1) {
    DECOMP(d, i, j, k);
    const int c = (int)_t;
    const unsigned code = pc[c];
    // pair difference: (upper or own pair) - (lower or own pair), pairs along offset o from cells a, b
    auto pair = [&](int a, int b, int o, unsigned bits) -> double {
      const double own = phi[a] + phi[b];
      const double up = (bits & 1u) ? own : phi[a + o] + phi[b + o];
      const double lo = (bits & 2u) ? own : phi[a - o] + phi[b - o];
      return up - lo;
    };
    if (code & (1u << 12)) {
      const double wn = pw[c], wa = pw[N + c], wb = pw[2 * N + c];
      const int e = (i == mx - 2) ? c + 3 - mx : c + 1;
      double t = wn * (phi[e] - phi[c]);
      if (wa != 0.) t = fma(wa, pair(c, c + 1, sy, code & 3u), t);
      if (wb != 0.) t = fma(wb, pair(c, c + 1, sz, (code >> 2) & 3u), t);
      u.x[c] = fma(-t, sc, u.x[c]);
    }
    if (code & (1u << 13)) {
      const double wn = pw[3 * N + c], wa = pw[4 * N + c], wb = pw[5 * N + c];
      const int e = (j == my - 2) ? c + (3 - my) * sy : c + sy;
      double t = wn * (phi[e] - phi[c]);
      if (wa != 0.) t = fma(wa, pair(c, c + sy, 1, (code >> 4) & 3u), t);
      if (wb != 0.) t = fma(wb, pair(c, c + sy, sz, (code >> 6) & 3u), t);
      u.y[c] = fma(-t, sc, u.y[c]);
    }
    if (code & (1u << 14)) {
      const double wn = pw[6 * N + c], wa = pw[7 * N + c], wb = pw[8 * N + c];
      const int e = (k == mz - 2) ? c + (3 - mz) * sz : c + sz;
      double t = wn * (phi[e] - phi[c]);
      if (wa != 0.) t = fma(wa, pair(c, c + sz, 1, (code >> 8) & 3u), t);
      if (wb != 0.) t = fma(wb, pair(c, c + sz, sy, (code >> 10) & 3u), t);
      u.z[c] = fma(-t, sc, u.z[c]);
    }
  }
}

int launch_projection_fast(const Dims& d, const double* pw, const uint16_t* pc, const double* phi, double dt, double st,
                           double coeff, const Ucont& u, cudaStream_t s, int k0, int k1) {
  const size_t P = (size_t)d.mx * d.my;
  if (k1 < 0) k1 = d.mz;
  if (k0 < 0 || k0 >= k1 || k1 > d.mz) return (int)cudaErrorInvalidValue;
  const int p0 = k0 > 1 ? k0 : 1, p1 = k1 < d.mz - 1 ? k1 : d.mz - 1;
  if (p0 < p1) {
    const size_t c0 = p0 * P, c1 = p1 * P;
    const double sc = dt * st / coeff;
    k_projection_fast<<<nblk(c1 - c0, 128), 128, 0, s>>>(d, c0, c1, pw, pc, phi, sc, u);
    ++g_launches;
  }
  return launch_ucont_ghosts(d, u, k0, k1, s);
}

// periodic ghost sync of the flagged component (poisson.c:2398-2437) on
// cells [c0, c1).  Every source is interior in all periodic directions, so
// the sync never reads a cell it writes; the source of a cell on an interior
// plane k lies on plane k.
__global__ void k_ucont_ghosts(Dims d, size_t c0, size_t c1, Ucont u) {
  RANGE_LOOP(c0, c1) {
    DECOMP(d, i, j, k);
    int a = wrapi(i, d.mx, d.ip), b = wrapi(j, d.my, d.jp), cc = wrapi(k, d.mz, d.kp);
    if (a == i && b == j && cc == k) continue;
    size_t s = cidx(d, a, b, cc);
    if (a != i) u.x[_t] = u.x[s];
    if (b != j) u.y[_t] = u.y[s];
    if (cc != k) u.z[_t] = u.z[s];
  }
}

// The nine metric dot products of the projection (same expressions as the
// reference's Projection, poisson.c:2262-2360, without the Jacobian).
__global__ void k_proj_dots(Dims d, const double* __restrict__ M, double* pd) {
  const size_t N = ncell(d);
  GRID_LOOP(d) {
    const size_t c = _t;
    const double* A = M + N * MP_ICSI + 3 * c;
    const double* B = M + N * MP_IETA + 3 * c;
    const double* E = M + N * MP_IZET + 3 * c;
    pd[0 * N + c] = A[0] * A[0] + A[1] * A[1] + A[2] * A[2];
    pd[1 * N + c] = B[0] * A[0] + B[1] * A[1] + B[2] * A[2];
    pd[2 * N + c] = E[0] * A[0] + E[1] * A[1] + E[2] * A[2];
    A = M + N * MP_JCSI + 3 * c;
    B = M + N * MP_JETA + 3 * c;
    E = M + N * MP_JZET + 3 * c;
    pd[3 * N + c] = A[0] * B[0] + A[1] * B[1] + A[2] * B[2];
    pd[4 * N + c] = B[0] * B[0] + B[1] * B[1] + B[2] * B[2];
    pd[5 * N + c] = E[0] * B[0] + E[1] * B[1] + E[2] * B[2];
    A = M + N * MP_KCSI + 3 * c;
    B = M + N * MP_KETA + 3 * c;
    E = M + N * MP_KZET + 3 * c;
    pd[6 * N + c] = A[0] * E[0] + A[1] * E[1] + A[2] * E[2];
    pd[7 * N + c] = B[0] * E[0] + B[1] * E[1] + B[2] * E[2];
    pd[8 * N + c] = E[0] * E[0] + E[1] * E[1] + E[2] * E[2];
  }
}
int launch_proj_dots(const Dims& d, const double* M, double* pd, cudaStream_t s) {
  k_proj_dots<<<nblk(ncell(d)), 256, 0, s>>>(d, M, pd); ++g_launches;
  return (int)cudaGetLastError();
}

int launch_projection(const Dims& d, const double* pd, const double* M, const double* nvert, const uint8_t* nb8,
                      const double* phi, double dt, double st, double coeff, const Ucont& u, cudaStream_t s, int k0,
                      int k1) {
  const size_t N = ncell(d);
  const size_t P = (size_t)d.mx * d.my;
  if (k1 < 0) k1 = d.mz;
  if (k0 < 0 || k0 >= k1 || k1 > d.mz) return (int)cudaErrorInvalidValue;
  // planes 0 and mz-1 hold no projected face (every branch needs 0 < k < mz-1)
  const int p0 = k0 > 1 ? k0 : 1, p1 = k1 < d.mz - 1 ? k1 : d.mz - 1;
  if (p0 < p1) {
    const size_t c0 = p0 * P, c1 = p1 * P;
    if (nb8)
      k_projection<true><<<nblk(c1 - c0, 128), 128, 0, s>>>(d, c0, c1, pd, M + N * MP_IAJ, M + N * MP_JAJ,
                                                            M + N * MP_KAJ, nvert, nb8, phi, dt, st, coeff, u);
    else
      k_projection<false><<<nblk(c1 - c0, 128), 128, 0, s>>>(d, c0, c1, pd, M + N * MP_IAJ, M + N * MP_JAJ,
                                                             M + N * MP_KAJ, nvert, nb8, phi, dt, st, coeff, u);
    ++g_launches;
  }
  return launch_ucont_ghosts(d, u, k0, k1, s);
}

int launch_ucont_ghosts(const Dims& d, const Ucont& u, int k0, int k1, cudaStream_t s) {
  const size_t P = (size_t)d.mx * d.my;
  if (k0 < 0 || k0 >= k1 || k1 > d.mz) return (int)cudaErrorInvalidValue;
  k_ucont_ghosts<<<nblk((k1 - k0) * P), 256, 0, s>>>(d, k0 * P, k1 * P, u); ++g_launches;
  return (int)cudaGetLastError();
}

// Contra2Cart (rhs.c:144-183): Cartesian velocity at fluid cells, the
// solution of [csi; eta; zet] ucat = q for the cell-centred contravariant
// fluxes q.  The reference solves each cell's 3 x 3 system by Cramer's rule
// (three FP64 divisions); the metric is static, so its inverse (adjugate /
// determinant, same cofactors) is formed once per grid, with the 1/2 of the
// face average q = (U_f- + U_f+) / 2 folded in (an exact power-of-two
// scale), and the step applies it with three multiplies and six FMAs (this
// unit is built without automatic contraction; the FMAs are explicit).
// Agrees with Cramer's rule to rounding.
__global__ void k_inverse_metric(Dims d, const double* __restrict__ M, const double* __restrict__ nvert, double* minv) {
  const size_t N = ncell(d);
  GRID_LOOP(d) {
    DECOMP(d, i, j, k);
    double* o = minv + 9 * _t;
    if (!interior(d, i, j, k) || !(nvert[_t] < 0.1)) {
      for (int q = 0; q < 9; q++) o[q] = 0.;
      continue;
    }
    const size_t c = _t;
    const double* A = M + N * MP_CSI + 3 * c;
    const double* B = M + N * MP_ETA + 3 * c;
    const double* E = M + N * MP_ZET + 3 * c;
    const double det = A[0] * (B[1] * E[2] - B[2] * E[1]) - A[1] * (B[0] * E[2] - B[2] * E[0]) + A[2] * (B[0] * E[1] - B[1] * E[0]);
    const double r = 0.5 / det;
    o[0] = (B[1] * E[2] - B[2] * E[1]) * r;
    o[1] = -(A[1] * E[2] - A[2] * E[1]) * r;
    o[2] = (A[1] * B[2] - A[2] * B[1]) * r;
    o[3] = -(B[0] * E[2] - B[2] * E[0]) * r;
    o[4] = (A[0] * E[2] - A[2] * E[0]) * r;
    o[5] = -(A[0] * B[2] - A[2] * B[0]) * r;
    o[6] = (B[0] * E[1] - B[1] * E[0]) * r;
    o[7] = -(A[0] * E[1] - A[1] * E[0]) * r;
    o[8] = (A[0] * B[1] - A[1] * B[0]) * r;
  }
}
int launch_inverse_metric(const Dims& d, const double* M, const double* nvert, double* minv, cudaStream_t s) {
  k_inverse_metric<<<nblk(ncell(d)), 256, 0, s>>>(d, M, nvert, minv); ++g_launches;
  return (int)cudaGetLastError();
}

__global__ void k_contra2cart(Dims d, const double* __restrict__ minv, const double* __restrict__ nvert, Ucont u,
                              double* ucat) {
  GRID_LOOP(d) {
    DECOMP(d, i, j, k);
    if (!interior(d, i, j, k) || !(nvert[_t] < 0.1)) continue;
    const size_t c = _t;
    const double* m = minv + 9 * c;
    const double q0 = u.x[cidx(d, i - 1, j, k)] + u.x[c];  // twice the face averages
    const double q1 = u.y[cidx(d, i, j - 1, k)] + u.y[c];
    const double q2 = u.z[cidx(d, i, j, k - 1)] + u.z[c];
    ucat[3 * c] = fma(m[2], q2, fma(m[1], q1, m[0] * q0));
    ucat[3 * c + 1] = fma(m[5], q2, fma(m[4], q1, m[3] * q0));
    ucat[3 * c + 2] = fma(m[8], q2, fma(m[7], q1, m[6] * q0));
  }
}
int launch_contra2cart(const Dims& d, const double* minv, const double* nvert, const Ucont& u, double* ucat, cudaStream_t s) {
  k_contra2cart<<<nblk(ncell(d)), 256, 0, s>>>(d, minv, nvert, u, ucat); ++g_launches;
  return (int)cudaGetLastError();
}

// Divergence (main.c:1279-1349): max over cells of |div U| * aj, 0 where the
// cell or a face neighbour carries nvert.
// Cell c or one of its six face neighbours carries nvert (the reference's
// sum > 0.1 test).  With nb8 (every nvert an integer in [0, 127]) the sum of
// non-negative integers exceeds 0.1 exactly when one of them is nonzero, an
// integer or of the bytes.
__device__ __forceinline__ bool near_body(const Dims& d, const double* __restrict__ nvert,
                                          const uint8_t* __restrict__ nb8, size_t c, int i, int j, int k) {
  if (nb8)
    return (nb8[c] | nb8[cidx(d, i, j, k + 1)] | nb8[cidx(d, i, j, k - 1)] | nb8[cidx(d, i, j + 1, k)] |
            nb8[cidx(d, i, j - 1, k)] | nb8[cidx(d, i + 1, j, k)] | nb8[cidx(d, i - 1, j, k)]) != 0;
  return nvert[c] + nvert[cidx(d, i, j, k + 1)] + nvert[cidx(d, i, j, k - 1)] + nvert[cidx(d, i, j + 1, k)] +
             nvert[cidx(d, i, j - 1, k)] + nvert[cidx(d, i + 1, j, k)] + nvert[cidx(d, i - 1, j, k)] >
         0.1;
}

__global__ void __launch_bounds__(RB) k_divergence(Dims d, Ucont u, const double* __restrict__ aj,
                                                   const double* __restrict__ nvert, double* parts,
                                                   const uint8_t* __restrict__ nb8 = nullptr) {
  __shared__ double sh[32];
  double mxv = 0.;
  GRID_LOOP(d) {
    DECOMP(d, i, j, k);
    if (!interior(d, i, j, k)) continue;
    const size_t c = _t;
    if (near_body(d, nvert, nb8, c, i, j, k)) continue;
    const double v = fabs((u.x[c] - u.x[cidx(d, i - 1, j, k)] + u.y[c] - u.y[cidx(d, i, j - 1, k)] + u.z[c] -
                           u.z[cidx(d, i, j, k - 1)]) * aj[c]);
    mxv = fmax(mxv, v);
  }
  mxv = block_max(mxv, sh);
  if (threadIdx.x == 0) parts[blockIdx.x] = mxv;
}
int launch_divergence(const Dims& d, const Ucont& u, const double* aj, const double* nvert, double* parts, double* out,
                      cudaStream_t s, const uint8_t* nb8) {
  const int nb = nblk(ncell(d), RB);
  k_divergence<<<nb, RB, 0, s>>>(d, u, aj, nvert, parts, nb8); ++g_launches;
  k_finish_max<<<1, 256, 0, s>>>(parts, nb, out); ++g_launches;
  return (int)cudaGetLastError();
}

// max |r| over the cells the Divergence check keeps (main.c:1279-1349: the
// cell and its six face neighbours free of nvert): with st = 1 the projection
// leaves div u = dt / coeff * r there for the aj-scaled residual r.
__global__ void __launch_bounds__(RB) k_masked_absmax(Dims d, const double* __restrict__ r, const double* __restrict__ nvert,
                                                      double* parts, const uint8_t* __restrict__ nb8) {
  __shared__ double sh[32];
  double mxv = 0.;
  GRID_LOOP(d) {
    DECOMP(d, i, j, k);
    if (!interior(d, i, j, k)) continue;
    const size_t c = _t;
    if (near_body(d, nvert, nb8, c, i, j, k)) continue;
    mxv = fmax(mxv, fabs(r[c]));
  }
  mxv = block_max(mxv, sh);
  if (threadIdx.x == 0) parts[blockIdx.x] = mxv;
}
int launch_masked_absmax(const Dims& d, const double* r, const double* nvert, double* parts, double* out, cudaStream_t s,
                         const uint8_t* nb8) {
  const int nb = nblk(ncell(d), RB);
  k_masked_absmax<<<nb, RB, 0, s>>>(d, r, nvert, parts, nb8); ++g_launches;
  k_finish_max<<<1, 256, 0, s>>>(parts, nb, out); ++g_launches;
  return (int)cudaGetLastError();
}

int launch_finish_sums(const double* parts, int nparts, int nq, double* out, cudaStream_t s) {
  k_finish_sums<<<1, 256, 0, s>>>(parts, nparts, nq, out); ++g_launches;
  return (int)cudaGetLastError();
}

int partial_blocks(const Dims& d) { return nblk(ncell(d), RB); }

// ---- allocation-free divergence check (static device scratch) ----
// The block maxima of k_divergence live in this file-scope array instead of
// a grid's partials buffer.  nblk() caps a launch at 152 * 16 blocks, so the
// array always holds one partial per block; every block writes its partial
// before k_finish_max reads it, so nothing in it has to start at zero.
constexpr int STATIC_PARTS = 152 * 16;
static __device__ __align__(256) double g_static_parts[STATIC_PARTS];

int divergence_max_static(int device, const Dims& d, const Ucont& u, const double* aj, const double* nvert, double* out,
                          cudaStream_t s, const char** why) {
  constexpr int MAXDEV = 64;
  static std::mutex mu;
  static double* addr[MAXDEV] = {};
  if (device < 0 || device >= MAXDEV) {
    *why = "device index out of range";
    return 1;
  }
  int cur = -1;
  cudaError_t e = cudaGetDevice(&cur);
  if (e != cudaSuccess) {
    *why = cudaGetErrorString(e);
    return 2;
  }
  if (cur != device) {
    *why = "the device argument must be the calling thread's current device";
    return 1;
  }
  double* parts = nullptr;
  {
    std::lock_guard<std::mutex> lk(mu);
    if (!addr[device]) {
      // once per device, with that device current
      e = cudaGetSymbolAddress((void**)&addr[device], g_static_parts);
      if (e != cudaSuccess) {
        addr[device] = nullptr;
        *why = cudaGetErrorString(e);
        return 2;
      }
    }
    parts = addr[device];
  }
  const int nb = nblk(ncell(d), RB);
  if (nb > STATIC_PARTS) {  // unreachable while nblk caps the grid; kept as the stated limit
    *why = "more block partials than the static scratch holds";
    return 1;
  }
  k_divergence<<<nb, RB, 0, s>>>(d, u, aj, nvert, parts); ++g_launches;
  k_finish_max<<<1, 256, 0, s>>>(parts, nb, out); ++g_launches;
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    *why = cudaGetErrorString(e);
    return 2;
  }
  return 0;
}

}  // namespace vfs
