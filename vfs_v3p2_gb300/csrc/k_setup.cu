// Setup kernels: FormMetrics, the g tensor and PoissonLHSNew's 19-point
// assembly, plus the multigrid hierarchy (coarse nodes, nvert coarsening,
// prolongation codes, dense coarsest-level inverse).
//
// This translation unit is compiled with --fmad=false: every multiply and add
// rounds separately, in the reference's order, so the metrics, g tensor and
// operator coefficients are bit-identical to the reference's double
// arithmetic (a*b+c is never contracted to an FMA, as with the gcc build the
// reference uses on x86-64).
#include "vfs_common.cuh"
#include "vfs_kernels.h"

namespace vfs {

struct V3 {
  double x, y, z;
};
__device__ __forceinline__ V3 ld3(const double* a, size_t c) { return V3{a[3 * c], a[3 * c + 1], a[3 * c + 2]}; }
__device__ __forceinline__ void st3(double* a, size_t c, V3 v) {
  a[3 * c] = v.x;
  a[3 * c + 1] = v.y;
  a[3 * c + 2] = v.z;
}

#define GRID_LOOP(d)                                                                          \
  for (size_t _t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; _t < ncell(d);              \
       _t += (size_t)gridDim.x * blockDim.x)

#define DECOMP(d, i, j, k)               \
  int i = (int)(_t % (d).mx);            \
  int j = (int)((_t / (d).mx) % (d).my); \
  int k = (int)(_t / ((size_t)(d).mx * (d).my))

// ---------------------------------------------------------------------------
// FormMetrics, NEWMETRIC branch (metrics.c:4-1004).  Output pack m (43 x N
// doubles): csi eta zet (AoS) aj | icsi ieta izet iaj | jcsi jeta jzet jaj |
// kcsi keta kzet kaj | cent.
// ---------------------------------------------------------------------------
__global__ void k_metrics_cells(Dims d, const double* __restrict__ coor, double* M, double* tmp) {
  const size_t N = ncell(d);
  double* cent = M + N * MP_CENT;
  double *csit = tmp, *etat = tmp + 3 * N, *zett = tmp + 6 * N;
  GRID_LOOP(d) {
    DECOMP(d, i, j, k);
#define C(ii, jj, kk) ld3(coor, cidx(d, ii, jj, kk))
    if (interior(d, i, j, k)) {  // metrics.c:80-103
      V3 a = C(i, j, k), b = C(i, j - 1, k), c = C(i, j, k - 1), e = C(i, j - 1, k - 1);
      V3 f = C(i - 1, j, k), g = C(i - 1, j - 1, k), h = C(i - 1, j, k - 1), q = C(i - 1, j - 1, k - 1);
      V3 r;
      r.x = 0.125 * (a.x + b.x + c.x + e.x + f.x + g.x + h.x + q.x);
      r.y = 0.125 * (a.y + b.y + c.y + e.y + f.y + g.y + h.y + q.y);
      r.z = 0.125 * (a.z + b.z + c.z + e.z + f.z + g.z + h.z + q.z);
      st3(cent, _t, r);
    }
    if (k >= 1 && k < d.mz - 1 && j >= 1 && j < d.my - 1 && i < d.mx - 1) {  // metrics.c:190-214
      V3 p00 = C(i, j, k), p10 = C(i, j - 1, k), p01 = C(i, j, k - 1), p11 = C(i, j - 1, k - 1);
      double dxde = 0.5 * (p00.x + p01.x - p10.x - p11.x);
      double dyde = 0.5 * (p00.y + p01.y - p10.y - p11.y);
      double dzde = 0.5 * (p00.z + p01.z - p10.z - p11.z);
      double dxdz = 0.5 * (p10.x + p00.x - p11.x - p01.x);
      double dydz = 0.5 * (p10.y + p00.y - p11.y - p01.y);
      double dzdz = 0.5 * (p10.z + p00.z - p11.z - p01.z);
      st3(csit, _t, V3{dyde * dzdz - dzde * dydz, -dxde * dzdz + dzde * dxdz, dxde * dydz - dyde * dxdz});
    }
    if (k >= 1 && k < d.mz - 1 && j < d.my - 1 && i >= 1 && i < d.mx - 1) {  // metrics.c:218-245
      V3 a = C(i, j, k), b = C(i, j, k - 1), c = C(i - 1, j, k), e = C(i - 1, j, k - 1);
      double dxdc = 0.5 * (a.x + b.x - c.x - e.x);
      double dydc = 0.5 * (a.y + b.y - c.y - e.y);
      double dzdc = 0.5 * (a.z + b.z - c.z - e.z);
      double dxdz = 0.5 * (a.x + c.x - b.x - e.x);
      double dydz = 0.5 * (a.y + c.y - b.y - e.y);
      double dzdz = 0.5 * (a.z + c.z - b.z - e.z);
      st3(etat, _t, V3{dydz * dzdc - dzdz * dydc, -dxdz * dzdc + dzdz * dxdc, dxdz * dydc - dydz * dxdc});
    }
    if (k < d.mz - 1 && j >= 1 && j < d.my - 1 && i >= 1 && i < d.mx - 1) {  // metrics.c:248-269
      V3 a = C(i, j, k), b = C(i, j - 1, k), c = C(i - 1, j, k), e = C(i - 1, j - 1, k);
      double dxdc = 0.5 * (a.x + b.x - c.x - e.x);
      double dydc = 0.5 * (a.y + b.y - c.y - e.y);
      double dzdc = 0.5 * (a.z + b.z - c.z - e.z);
      double dxde = 0.5 * (a.x + c.x - b.x - e.x);
      double dyde = 0.5 * (a.y + c.y - b.y - e.y);
      double dzde = 0.5 * (a.z + c.z - b.z - e.z);
      st3(zett, _t, V3{dydc * dzde - dzdc * dyde, -dxdc * dzde + dzdc * dxde, dxdc * dyde - dydc * dxde});
    }
#undef C
  }
}

__global__ void k_metrics_centred(Dims d, const double* __restrict__ coor, double* M, const double* tmp) {
  const size_t N = ncell(d);
  double *csi = M + N * MP_CSI, *eta = M + N * MP_ETA, *zet = M + N * MP_ZET, *aj = M + N * MP_AJ;
  const double *csit = tmp, *etat = tmp + 3 * N, *zett = tmp + 6 * N;
  GRID_LOOP(d) {
    DECOMP(d, i, j, k);
    if (!interior(d, i, j, k)) continue;
    // metrics.c:291-297 (AxByC: 0.5*a + 0.5*b)
    V3 a = ld3(csit, _t), b = ld3(csit, cidx(d, i - 1, j, k));
    st3(csi, _t, V3{0.5 * a.x + 0.5 * b.x, 0.5 * a.y + 0.5 * b.y, 0.5 * a.z + 0.5 * b.z});
    a = ld3(etat, _t);
    b = ld3(etat, cidx(d, i, j - 1, k));
    st3(eta, _t, V3{0.5 * a.x + 0.5 * b.x, 0.5 * a.y + 0.5 * b.y, 0.5 * a.z + 0.5 * b.z});
    a = ld3(zett, _t);
    b = ld3(zett, cidx(d, i, j, k - 1));
    st3(zet, _t, V3{0.5 * a.x + 0.5 * b.x, 0.5 * a.y + 0.5 * b.y, 0.5 * a.z + 0.5 * b.z});
    // cell Jacobian, metrics.c:304-340
#define C(ii, jj, kk) ld3(coor, cidx(d, ii, jj, kk))
    V3 c000 = C(i, j, k), c010 = C(i, j - 1, k), c001 = C(i, j, k - 1), c011 = C(i, j - 1, k - 1);
    V3 c100 = C(i - 1, j, k), c110 = C(i - 1, j - 1, k), c101 = C(i - 1, j, k - 1), c111 = C(i - 1, j - 1, k - 1);
#undef C
    double dxdc = 0.25 * (c000.x + c010.x + c001.x + c011.x - c100.x - c110.x - c101.x - c111.x);
    double dydc = 0.25 * (c000.y + c010.y + c001.y + c011.y - c100.y - c110.y - c101.y - c111.y);
    double dzdc = 0.25 * (c000.z + c010.z + c001.z + c011.z - c100.z - c110.z - c101.z - c111.z);
    double dxde = 0.25 * (c000.x + c100.x + c001.x + c101.x - c010.x - c110.x - c011.x - c111.x);
    double dyde = 0.25 * (c000.y + c100.y + c001.y + c101.y - c010.y - c110.y - c011.y - c111.y);
    double dzde = 0.25 * (c000.z + c100.z + c001.z + c101.z - c010.z - c110.z - c011.z - c111.z);
    double dxdz = 0.25 * (c000.x + c010.x + c100.x + c110.x - c001.x - c011.x - c101.x - c111.x);
    double dydz = 0.25 * (c000.y + c010.y + c100.y + c110.y - c001.y - c011.y - c101.y - c111.y);
    double dzdz = 0.25 * (c000.z + c010.z + c100.z + c110.z - c001.z - c011.z - c101.z - c111.z);
    double det = dxdc * (dyde * dzdz - dzde * dydz) - dydc * (dxde * dzdz - dzde * dxdz) + dzdc * (dxde * dydz - dyde * dxdz);
    aj[_t] = 1. / det;
  }
}

// Mirror copies of csi/eta/zet/aj onto the boundary planes, metrics.c:373-453.
// axis 0, 1, 2 are launched in that order, as the reference loops them.
__global__ void k_metrics_mirror(Dims d, double* M, int axis) {
  const size_t N = ncell(d);
  double *csi = M + N * MP_CSI, *eta = M + N * MP_ETA, *zet = M + N * MP_ZET, *aj = M + N * MP_AJ;
  GRID_LOOP(d) {
    DECOMP(d, i, j, k);
    size_t s;
    if (axis == 0) {
      if (i == 0) s = cidx(d, 1, j, k);
      else if (i == d.mx - 1) s = cidx(d, d.mx - 2, j, k);
      else continue;
    } else if (axis == 1) {
      if (j == 0) s = cidx(d, i, 1, k);
      else if (j == d.my - 1) s = cidx(d, i, d.my - 2, k);
      else continue;
    } else {
      if (k == 0) s = cidx(d, i, j, 1);
      else if (k == d.mz - 1) s = cidx(d, i, j, d.mz - 2);
      else continue;
    }
    st3(csi, _t, ld3(csi, s));
    st3(eta, _t, ld3(eta, s));
    st3(zet, _t, ld3(zet, s));
    aj[_t] = aj[s];
  }
}

// The mirror copies are the final ghost values of the cell-centred metrics:
// the reference's periodic copies (metrics.c:470-510) go to its local vectors
// only, nothing reads them there (the face-metric fallbacks that would are
// commented out), and its closing scatter of the global vectors
// (metrics.c:1212-1244) restores the mirror values on every boundary plane.

__device__ __forceinline__ void face_metric(double dxdc, double dydc, double dzdc, double dxde, double dyde, double dzde,
                                            double dxdz, double dydz, double dzdz, double* M, size_t N, size_t t,
                                            int ocsi, int oeta, int ozet, int oaj) {
  st3(M + N * ocsi, t, V3{dyde * dzdz - dzde * dydz, -dxde * dzdz + dzde * dxdz, dxde * dydz - dyde * dxdz});
  st3(M + N * oeta, t, V3{dydz * dzdc - dzdz * dydc, -dxdz * dzdc + dzdz * dxdc, dxdz * dydc - dydz * dxdc});
  st3(M + N * ozet, t, V3{dydc * dzde - dzdc * dyde, -dxdc * dzde + dzdc * dxde, dxdc * dyde - dydc * dxde});
  double a = dxdc * (dyde * dzdz - dzde * dydz) - dydc * (dxde * dzdz - dzde * dxdz) + dzdc * (dxde * dydz - dyde * dxdz);
  M[N * oaj + t] = 1. / a;
}

// Face centres of the three face families (metrics.c:592-606, 735-748, 846-858).
__device__ __forceinline__ V3 fcent(const Dims& d, const double* coor, int fam, int i, int j, int k) {
#define C(ii, jj, kk) ld3(coor, cidx(d, ii, jj, kk))
  V3 a, b, c, e;
  if (fam == 0) {
    a = C(i, j, k); b = C(i, j, k - 1); c = C(i, j - 1, k); e = C(i, j - 1, k - 1);
  } else if (fam == 1) {
    a = C(i, j, k); b = C(i, j, k - 1); c = C(i - 1, j, k); e = C(i - 1, j, k - 1);
  } else {
    a = C(i, j, k); b = C(i, j - 1, k); c = C(i - 1, j, k); e = C(i - 1, j - 1, k);
  }
#undef C
  return V3{(a.x + b.x + c.x + e.x) * 0.25, (a.y + b.y + c.y + e.y) * 0.25, (a.z + b.z + c.z + e.z) * 0.25};
}
__device__ __forceinline__ V3 vsub(V3 p, V3 m) { return V3{p.x - m.x, p.y - m.y, p.z - m.z}; }
__device__ __forceinline__ V3 vhalf(V3 p, V3 m) { return V3{(p.x - m.x) * 0.5, (p.y - m.y) * 0.5, (p.z - m.z) * 0.5}; }
__device__ __forceinline__ V3 vseam(V3 a, V3 b, V3 c, V3 e) {
  return V3{(a.x - b.x + c.x - e.x) * 0.5, (a.y - b.y + c.y - e.y) * 0.5, (a.z - b.z + c.z - e.z) * 0.5};
}

// Face-centred metric sets I*, J*, K* (metrics.c:608-960).
__global__ void k_metrics_faces(Dims d, const double* __restrict__ coor, double* M) {
  const size_t N = ncell(d);
  GRID_LOOP(d) {
    DECOMP(d, i, j, k);
    const int mx = d.mx, my = d.my, mz = d.mz;
    // i faces: k, j in [1, m-2], i in [0, mx-2]
    if (k >= 1 && k < mz - 1 && j >= 1 && j < my - 1 && i < mx - 1) {
      V3 dc, de, dz;
      if (i == 0) dc = vsub(fcent(d, coor, 0, i + 1, j, k), fcent(d, coor, 0, i, j, k));
      else if (i == mx - 2) {
        if (d.ip) dc = vseam(fcent(d, coor, 0, 1, j, k), fcent(d, coor, 0, 0, j, k), fcent(d, coor, 0, i, j, k), fcent(d, coor, 0, i - 1, j, k));
        else dc = vsub(fcent(d, coor, 0, i, j, k), fcent(d, coor, 0, i - 1, j, k));
      } else dc = vhalf(fcent(d, coor, 0, i + 1, j, k), fcent(d, coor, 0, i - 1, j, k));
      if (j == 1) de = vsub(fcent(d, coor, 0, i, j + 1, k), fcent(d, coor, 0, i, j, k));
      else if (j == my - 2) de = vsub(fcent(d, coor, 0, i, j, k), fcent(d, coor, 0, i, j - 1, k));
      else de = vhalf(fcent(d, coor, 0, i, j + 1, k), fcent(d, coor, 0, i, j - 1, k));
      if (k == 1) dz = vsub(fcent(d, coor, 0, i, j, k + 1), fcent(d, coor, 0, i, j, k));
      else if (k == mz - 2) dz = vsub(fcent(d, coor, 0, i, j, k), fcent(d, coor, 0, i, j, k - 1));
      else dz = vhalf(fcent(d, coor, 0, i, j, k + 1), fcent(d, coor, 0, i, j, k - 1));
      face_metric(dc.x, dc.y, dc.z, de.x, de.y, de.z, dz.x, dz.y, dz.z, M, N, _t, MP_ICSI, MP_IETA, MP_IZET, MP_IAJ);
    }
    // j faces: k in [1, mz-2], j in [0, my-2], i in [1, mx-2]
    if (k >= 1 && k < mz - 1 && j < my - 1 && i >= 1 && i < mx - 1) {
      V3 dc, de, dz;
      if (i == 1) dc = vsub(fcent(d, coor, 1, i + 1, j, k), fcent(d, coor, 1, i, j, k));
      else if (i == mx - 2) dc = vsub(fcent(d, coor, 1, i, j, k), fcent(d, coor, 1, i - 1, j, k));
      else dc = vhalf(fcent(d, coor, 1, i + 1, j, k), fcent(d, coor, 1, i - 1, j, k));
      if (j == 0) de = vsub(fcent(d, coor, 1, i, j + 1, k), fcent(d, coor, 1, i, j, k));
      else if (j == my - 2) {
        if (d.jp) de = vseam(fcent(d, coor, 1, i, 1, k), fcent(d, coor, 1, i, 0, k), fcent(d, coor, 1, i, j, k), fcent(d, coor, 1, i, j - 1, k));
        else de = vsub(fcent(d, coor, 1, i, j, k), fcent(d, coor, 1, i, j - 1, k));
      } else de = vhalf(fcent(d, coor, 1, i, j + 1, k), fcent(d, coor, 1, i, j - 1, k));
      if (k == 1) dz = vsub(fcent(d, coor, 1, i, j, k + 1), fcent(d, coor, 1, i, j, k));
      else if (k == mz - 2) dz = vsub(fcent(d, coor, 1, i, j, k), fcent(d, coor, 1, i, j, k - 1));
      else dz = vhalf(fcent(d, coor, 1, i, j, k + 1), fcent(d, coor, 1, i, j, k - 1));
      face_metric(dc.x, dc.y, dc.z, de.x, de.y, de.z, dz.x, dz.y, dz.z, M, N, _t, MP_JCSI, MP_JETA, MP_JZET, MP_JAJ);
    }
    // k faces: k in [0, mz-2], j, i in [1, m-2]
    if (k < mz - 1 && j >= 1 && j < my - 1 && i >= 1 && i < mx - 1) {
      V3 dc, de, dz;
      if (i == 1) dc = vsub(fcent(d, coor, 2, i + 1, j, k), fcent(d, coor, 2, i, j, k));
      else if (i == mx - 2) dc = vsub(fcent(d, coor, 2, i, j, k), fcent(d, coor, 2, i - 1, j, k));
      else dc = vhalf(fcent(d, coor, 2, i + 1, j, k), fcent(d, coor, 2, i - 1, j, k));
      if (j == 1) de = vsub(fcent(d, coor, 2, i, j + 1, k), fcent(d, coor, 2, i, j, k));
      else if (j == my - 2) de = vsub(fcent(d, coor, 2, i, j, k), fcent(d, coor, 2, i, j - 1, k));
      else de = vhalf(fcent(d, coor, 2, i, j + 1, k), fcent(d, coor, 2, i, j - 1, k));
      if (k == 0) dz = vsub(fcent(d, coor, 2, i, j, k + 1), fcent(d, coor, 2, i, j, k));
      else if (k == mz - 2) {
        if (d.kp) dz = vseam(fcent(d, coor, 2, i, j, 1), fcent(d, coor, 2, i, j, 0), fcent(d, coor, 2, i, j, k), fcent(d, coor, 2, i, j, k - 1));
        else dz = vsub(fcent(d, coor, 2, i, j, k), fcent(d, coor, 2, i, j, k - 1));
      } else dz = vhalf(fcent(d, coor, 2, i, j, k + 1), fcent(d, coor, 2, i, j, k - 1));
      face_metric(dc.x, dc.y, dc.z, de.x, de.y, de.z, dz.x, dz.y, dz.z, M, N, _t, MP_KCSI, MP_KETA, MP_KZET, MP_KAJ);
    }
  }
}

// ---------------------------------------------------------------------------
// g tensor, poisson.c:1105-1141.  g[0..8][N] = g11 g12 g13 g21 g22 g23 g31 g32 g33.
// ---------------------------------------------------------------------------
__global__ void k_gtensor(Dims d, const double* __restrict__ M, double* g) {
  const size_t N = ncell(d);
  GRID_LOOP(d) {
    DECOMP(d, i, j, k);
    size_t s = cidx(d, wrapi(i, d.mx, d.ip), wrapi(j, d.my, d.jp), wrapi(k, d.mz, d.kp));
    V3 ic = ld3(M + N * MP_ICSI, s), ie = ld3(M + N * MP_IETA, s), iz = ld3(M + N * MP_IZET, s);
    V3 jc = ld3(M + N * MP_JCSI, s), je = ld3(M + N * MP_JETA, s), jz = ld3(M + N * MP_JZET, s);
    V3 kc = ld3(M + N * MP_KCSI, s), ke = ld3(M + N * MP_KETA, s), kz = ld3(M + N * MP_KZET, s);
    double iaj = M[N * MP_IAJ + s], jaj = M[N * MP_JAJ + s], kaj = M[N * MP_KAJ + s];
    g[0 * N + _t] = (ic.x * ic.x + ic.y * ic.y + ic.z * ic.z) * iaj;
    g[1 * N + _t] = (ie.x * ic.x + ie.y * ic.y + ie.z * ic.z) * iaj;
    g[2 * N + _t] = (iz.x * ic.x + iz.y * ic.y + iz.z * ic.z) * iaj;
    g[3 * N + _t] = (jc.x * je.x + jc.y * je.y + jc.z * je.z) * jaj;
    g[4 * N + _t] = (je.x * je.x + je.y * je.y + je.z * je.z) * jaj;
    g[5 * N + _t] = (jz.x * je.x + jz.y * je.y + jz.z * je.z) * jaj;
    g[6 * N + _t] = (kc.x * kz.x + kc.y * kz.y + kc.z * kz.z) * kaj;
    g[7 * N + _t] = (ke.x * kz.x + ke.y * kz.y + ke.z * kz.z) * kaj;
    g[8 * N + _t] = (kz.x * kz.x + kz.y * kz.y + kz.z * kz.z) * kaj;
  }
}

// Does stencil neighbour (i,j,k) carry a fluid id (setup_lidx2, poisson.c:237-300)?
// Periodic ghosts take their partner's id; walls and (int)nvert > 0.1 have none.
__device__ __forceinline__ bool has_id(const Dims& d, const double* nvert, int i, int j, int k) {
  int a = wrapi(i, d.mx, d.ip), b = wrapi(j, d.my, d.jp), c = wrapi(k, d.mz, d.kp);
  if (!interior(d, a, b, c)) return false;
  return !((int)nvert[cidx(d, a, b, c)] > VFS_THR);
}

// ---------------------------------------------------------------------------
// PoissonLHSNew (poisson.c:976-1630), built HYPRE body, matrix-free: the 19
// row entries of every fluid interior cell in the reference's summation
// order, after the drop rule of poisson.c:1607-1616.  Also writes the
// aj-scaled copies used by the multigrid levels (poisson.c:1560, the
// poisson == -1 branch the reference's PCMG path runs with) in FP64 and FP32,
// and ORs the nonzero slots of the level into *mask.
// ---------------------------------------------------------------------------
__global__ void k_assemble(Dims d, const double* __restrict__ g, const double* __restrict__ nvert,
                           const double* __restrict__ aj, double* coef, double* mcoef, float* mcoef32, unsigned* mask) {
  const size_t N = ncell(d);
  const int mx = d.mx, my = d.my, mz = d.mz, ip = d.ip, jp = d.jp, kp = d.kp;
  const double *g11 = g, *g12 = g + N, *g13 = g + 2 * N, *g21 = g + 3 * N, *g22 = g + 4 * N, *g23 = g + 5 * N;
  const double *g31 = g + 6 * N, *g32 = g + 7 * N, *g33 = g + 8 * N;
  const double THR = VFS_THR;
  unsigned mymask = 0;
  GRID_LOOP(d) {
    DECOMP(d, i, j, k);
    double vol[19];
#pragma unroll
    for (int m = 0; m < 19; m++) vol[m] = 0.;
    const bool row = interior(d, i, j, k) && !(nvert[_t] > THR);
    if (row) {
#define NV(ii, jj, kk) nvert[cidx(d, ii, jj, kk)]
      const double r = 1.0;
      const size_t c = _t;
      if (NV(i + 1, j, k) < THR && (i != mx - 2 || ip)) {
        vol[CP] -= g11[c] / r;
        vol[EP] += g11[c] / r;
        if ((j == my - 2 && !jp) || NV(i, j + 1, k) + NV(i + 1, j + 1, k) > THR) {
          if (NV(i, j - 1, k) + NV(i + 1, j - 1, k) < THR && j != 1) {
            vol[CP] += g12[c] * 0.5 / r; vol[EP] += g12[c] * 0.5 / r;
            vol[SP] -= g12[c] * 0.5 / r; vol[SE] -= g12[c] * 0.5 / r;
          }
        } else if ((j == 1 && !jp) || NV(i, j - 1, k) + NV(i + 1, j - 1, k) > THR) {
          if (NV(i, j + 1, k) + NV(i + 1, j + 1, k) < THR) {
            vol[NP] += g12[c] * 0.5 / r; vol[NE] += g12[c] * 0.5 / r;
            vol[CP] -= g12[c] * 0.5 / r; vol[EP] -= g12[c] * 0.5 / r;
          }
        } else {
          vol[NP] += g12[c] * 0.25 / r; vol[NE] += g12[c] * 0.25 / r;
          vol[SP] -= g12[c] * 0.25 / r; vol[SE] -= g12[c] * 0.25 / r;
        }
        if ((k == mz - 2 && !kp) || NV(i, j, k + 1) + NV(i + 1, j, k + 1) > THR) {
          if (NV(i, j, k - 1) + NV(i + 1, j, k - 1) < THR && k != 1) {
            vol[CP] += g13[c] * 0.5 / r; vol[EP] += g13[c] * 0.5 / r;
            vol[BP] -= g13[c] * 0.5 / r; vol[BE] -= g13[c] * 0.5 / r;
          }
        } else if ((k == 1 && !kp) || NV(i, j, k - 1) + NV(i + 1, j, k - 1) > THR) {
          if (NV(i, j, k + 1) + NV(i + 1, j, k + 1) < THR) {
            vol[TP] += g13[c] * 0.5 / r; vol[TE] += g13[c] * 0.5 / r;
            vol[CP] -= g13[c] * 0.5 / r; vol[EP] -= g13[c] * 0.5 / r;
          }
        } else {
          vol[TP] += g13[c] * 0.25 / r; vol[TE] += g13[c] * 0.25 / r;
          vol[BP] -= g13[c] * 0.25 / r; vol[BE] -= g13[c] * 0.25 / r;
        }
      }
      if (NV(i - 1, j, k) < THR && (i != 1 || ip)) {
        const size_t w = cidx(d, i - 1, j, k);
        vol[CP] -= g11[w] / r;
        vol[WP] += g11[w] / r;
        if ((j == my - 2 && !jp) || NV(i, j + 1, k) + NV(i - 1, j + 1, k) > THR) {
          if (NV(i, j - 1, k) + NV(i - 1, j - 1, k) < THR && j != 1) {
            vol[CP] -= g12[w] * 0.5 / r; vol[WP] -= g12[w] * 0.5 / r;
            vol[SP] += g12[w] * 0.5 / r; vol[SW] += g12[w] * 0.5 / r;
          }
        } else if ((j == 1 && !jp) || NV(i, j - 1, k) + NV(i - 1, j - 1, k) > THR) {
          if (NV(i, j + 1, k) + NV(i - 1, j + 1, k) < THR) {
            vol[NP] -= g12[w] * 0.5 / r; vol[NW] -= g12[w] * 0.5 / r;
            vol[CP] += g12[w] * 0.5 / r; vol[WP] += g12[w] * 0.5 / r;
          }
        } else {
          vol[NP] -= g12[w] * 0.25 / r; vol[NW] -= g12[w] * 0.25 / r;
          vol[SP] += g12[w] * 0.25 / r; vol[SW] += g12[w] * 0.25 / r;
        }
        if ((k == mz - 2 && !kp) || NV(i, j, k + 1) + NV(i - 1, j, k + 1) > THR) {
          if (NV(i, j, k - 1) + NV(i - 1, j, k - 1) < THR && k != 1) {
            vol[CP] -= g13[w] * 0.5 / r; vol[WP] -= g13[w] * 0.5 / r;
            vol[BP] += g13[w] * 0.5 / r; vol[BW] += g13[w] * 0.5 / r;
          }
        } else if ((k == 1 && !kp) || NV(i, j, k - 1) + NV(i - 1, j, k - 1) > THR) {
          if (NV(i, j, k + 1) + NV(i - 1, j, k + 1) < THR) {
            vol[TP] -= g13[w] * 0.5 / r; vol[TW] -= g13[w] * 0.5 / r;
            vol[CP] += g13[w] * 0.5 / r; vol[WP] += g13[w] * 0.5 / r;
          }
        } else {
          vol[TP] -= g13[w] * 0.25 / r; vol[TW] -= g13[w] * 0.25 / r;
          vol[BP] += g13[w] * 0.25 / r; vol[BW] += g13[w] * 0.25 / r;
        }
      }
      if (NV(i, j + 1, k) < THR && (j != my - 2 || jp)) {
        if ((i == mx - 2 && !ip) || NV(i + 1, j, k) + NV(i + 1, j + 1, k) > THR) {
          if (NV(i - 1, j, k) + NV(i - 1, j + 1, k) < THR && i != 1) {
            vol[CP] += g21[c] * 0.5 / r; vol[NP] += g21[c] * 0.5 / r;
            vol[WP] -= g21[c] * 0.5 / r; vol[NW] -= g21[c] * 0.5 / r;
          }
        } else if ((i == 1 && !ip) || NV(i - 1, j, k) + NV(i - 1, j + 1, k) > THR) {
          if (NV(i + 1, j, k) + NV(i + 1, j + 1, k) < THR) {
            vol[EP] += g21[c] * 0.5 / r; vol[NE] += g21[c] * 0.5 / r;
            vol[CP] -= g21[c] * 0.5 / r; vol[NP] -= g21[c] * 0.5 / r;
          }
        } else {
          vol[EP] += g21[c] * 0.25 / r; vol[NE] += g21[c] * 0.25 / r;
          vol[WP] -= g21[c] * 0.25 / r; vol[NW] -= g21[c] * 0.25 / r;
        }
        vol[CP] -= g22[c] / r;
        vol[NP] += g22[c] / r;
        if ((k == mz - 2 && !kp) || NV(i, j, k + 1) + NV(i, j + 1, k + 1) > THR) {
          if (NV(i, j, k - 1) + NV(i, j + 1, k - 1) < THR && k != 1) {
            vol[CP] += g23[c] * 0.5 / r; vol[NP] += g23[c] * 0.5 / r;
            vol[BP] -= g23[c] * 0.5 / r; vol[BN] -= g23[c] * 0.5 / r;
          }
        } else if ((k == 1 && !kp) || NV(i, j, k - 1) + NV(i, j + 1, k - 1) > THR) {
          if (NV(i, j, k + 1) + NV(i, j + 1, k + 1) < THR) {
            vol[TP] += g23[c] * 0.5 / r; vol[TN] += g23[c] * 0.5 / r;
            vol[CP] -= g23[c] * 0.5 / r; vol[NP] -= g23[c] * 0.5 / r;
          }
        } else {
          vol[TP] += g23[c] * 0.25 / r; vol[TN] += g23[c] * 0.25 / r;
          vol[BP] -= g23[c] * 0.25 / r; vol[BN] -= g23[c] * 0.25 / r;
        }
      }
      if (NV(i, j - 1, k) < THR && (j != 1 || jp)) {
        const size_t s = cidx(d, i, j - 1, k);
        if ((i == mx - 2 && !ip) || NV(i + 1, j, k) + NV(i + 1, j - 1, k) > THR) {
          if (NV(i - 1, j, k) + NV(i - 1, j - 1, k) < THR && i != 1) {
            vol[CP] -= g21[s] * 0.5 / r; vol[SP] -= g21[s] * 0.5 / r;
            vol[WP] += g21[s] * 0.5 / r; vol[SW] += g21[s] * 0.5 / r;
          }
        } else if ((i == 1 && !ip) || NV(i - 1, j, k) + NV(i - 1, j - 1, k) > THR) {
          if (NV(i + 1, j, k) + NV(i + 1, j - 1, k) < THR) {
            vol[EP] -= g21[s] * 0.5 / r; vol[SE] -= g21[s] * 0.5 / r;
            vol[CP] += g21[s] * 0.5 / r; vol[SP] += g21[s] * 0.5 / r;
          }
        } else {
          vol[EP] -= g21[s] * 0.25 / r; vol[SE] -= g21[s] * 0.25 / r;
          vol[WP] += g21[s] * 0.25 / r; vol[SW] += g21[s] * 0.25 / r;
        }
        vol[CP] -= g22[s] / r;
        vol[SP] += g22[s] / r;
        if ((k == mz - 2 && !kp) || NV(i, j, k + 1) + NV(i, j - 1, k + 1) > THR) {
          if (NV(i, j, k - 1) + NV(i, j - 1, k - 1) < THR && k != 1) {
            vol[CP] -= g23[s] * 0.5 / r; vol[SP] -= g23[s] * 0.5 / r;
            vol[BP] += g23[s] * 0.5 / r; vol[BS] += g23[s] * 0.5 / r;
          }
        } else if ((k == 1 && !kp) || NV(i, j, k - 1) + NV(i, j - 1, k - 1) > THR) {
          if (NV(i, j, k + 1) + NV(i, j - 1, k + 1) < THR) {
            vol[TP] -= g23[s] * 0.5 / r; vol[TS] -= g23[s] * 0.5 / r;
            vol[CP] += g23[s] * 0.5 / r; vol[SP] += g23[s] * 0.5 / r;
          }
        } else {
          vol[TP] -= g23[s] * 0.25 / r; vol[TS] -= g23[s] * 0.25 / r;
          vol[BP] += g23[s] * 0.25 / r; vol[BS] += g23[s] * 0.25 / r;
        }
      }
      if (NV(i, j, k + 1) < THR && (k != mz - 2 || kp)) {
        if ((i == mx - 2 && !ip) || NV(i + 1, j, k) + NV(i + 1, j, k + 1) > THR) {
          if (NV(i - 1, j, k) + NV(i - 1, j, k + 1) < THR && i != 1) {
            vol[CP] += g31[c] * 0.5 / r; vol[TP] += g31[c] * 0.5 / r;
            vol[WP] -= g31[c] * 0.5 / r; vol[TW] -= g31[c] * 0.5 / r;
          }
        } else if ((i == 1 && !ip) || NV(i - 1, j, k) + NV(i - 1, j, k + 1) > THR) {
          if (NV(i + 1, j, k) + NV(i + 1, j, k + 1) < THR) {
            vol[EP] += g31[c] * 0.5 / r; vol[TE] += g31[c] * 0.5 / r;
            vol[CP] -= g31[c] * 0.5 / r; vol[TP] -= g31[c] * 0.5 / r;
          }
        } else {
          vol[EP] += g31[c] * 0.25 / r; vol[TE] += g31[c] * 0.25 / r;
          vol[WP] -= g31[c] * 0.25 / r; vol[TW] -= g31[c] * 0.25 / r;
        }
        if ((j == my - 2 && !jp) || NV(i, j + 1, k) + NV(i, j + 1, k + 1) > THR) {
          if (NV(i, j - 1, k) + NV(i, j - 1, k + 1) < THR && j != 1) {
            vol[CP] += g32[c] * 0.5 / r; vol[TP] += g32[c] * 0.5 / r;
            vol[SP] -= g32[c] * 0.5 / r; vol[TS] -= g32[c] * 0.5 / r;
          }
        } else if ((j == 1 && !jp) || NV(i, j - 1, k) + NV(i, j - 1, k + 1) > THR) {
          if (NV(i, j + 1, k) + NV(i, j + 1, k + 1) < THR) {
            vol[NP] += g32[c] * 0.5 / r; vol[TN] += g32[c] * 0.5 / r;
            vol[CP] -= g32[c] * 0.5 / r; vol[TP] -= g32[c] * 0.5 / r;
          }
        } else {
          vol[NP] += g32[c] * 0.25 / r; vol[TN] += g32[c] * 0.25 / r;
          vol[SP] -= g32[c] * 0.25 / r; vol[TS] -= g32[c] * 0.25 / r;
        }
        vol[CP] -= g33[c] / r;
        vol[TP] += g33[c] / r;
      }
      if (NV(i, j, k - 1) < THR && (k != 1 || kp)) {
        const size_t b = cidx(d, i, j, k - 1);
        if ((i == mx - 2 && !ip) || NV(i + 1, j, k) + NV(i + 1, j, k - 1) > THR) {
          if (NV(i - 1, j, k) + NV(i - 1, j, k - 1) < THR && i != 1) {
            vol[CP] -= g31[b] * 0.5 / r; vol[BP] -= g31[b] * 0.5 / r;
            vol[WP] += g31[b] * 0.5 / r; vol[BW] += g31[b] * 0.5 / r;
          }
        } else if ((i == 1 && !ip) || NV(i - 1, j, k) + NV(i - 1, j, k - 1) > THR) {
          if (NV(i + 1, j, k) + NV(i + 1, j, k - 1) < THR) {
            vol[EP] -= g31[b] * 0.5 / r; vol[BE] -= g31[b] * 0.5 / r;
            vol[CP] += g31[b] * 0.5 / r; vol[BP] += g31[b] * 0.5 / r;
          }
        } else {
          vol[EP] -= g31[b] * 0.25 / r; vol[BE] -= g31[b] * 0.25 / r;
          vol[WP] += g31[b] * 0.25 / r; vol[BW] += g31[b] * 0.25 / r;
        }
        if ((j == my - 2 && !jp) || NV(i, j + 1, k) + NV(i, j + 1, k - 1) > THR) {
          if (NV(i, j - 1, k) + NV(i, j - 1, k - 1) < THR && j != 1) {
            vol[CP] -= g32[b] * 0.5 / r; vol[BP] -= g32[b] * 0.5 / r;
            vol[SP] += g32[b] * 0.5 / r; vol[BS] += g32[b] * 0.5 / r;
          }
        } else if ((j == 1 && !jp) || NV(i, j - 1, k) + NV(i, j - 1, k - 1) > THR) {
          if (NV(i, j + 1, k) + NV(i, j + 1, k - 1) < THR) {
            vol[NP] -= g32[b] * 0.5 / r; vol[BN] -= g32[b] * 0.5 / r;
            vol[CP] += g32[b] * 0.5 / r; vol[BP] += g32[b] * 0.5 / r;
          }
        } else {
          vol[NP] -= g32[b] * 0.25 / r; vol[BN] -= g32[b] * 0.25 / r;
          vol[SP] += g32[b] * 0.25 / r; vol[BS] += g32[b] * 0.25 / r;
        }
        vol[CP] -= g33[b] / r;
        vol[BP] += g33[b] / r;
      }
#undef NV
      // drop rule, poisson.c:1607-1616: the unscaled row (the built HYPRE
      // path) drops |v| <= 1e-10; the aj-scaled row (the multigrid path,
      // poisson == -1) is scaled first (poisson.c:1560) and the same rule
      // applies to the scaled values
      const double a = aj[_t];
#pragma unroll
      for (int m = 0; m < 19; m++) {
        const bool col = (m == CP) || has_id(d, nvert, i + slot_di(m), j + slot_dj(m), k + slot_dk(m));
        const double s = vol[m] * a;
        const bool keep_u = (m == CP) || (fabs(vol[m]) > 1.e-10 && col);
        const bool keep_s = (m == CP) || (fabs(s) > 1.e-10 && col);
        coef[(size_t)m * N + _t] = keep_u ? vol[m] : 0.;
        mcoef[(size_t)m * N + _t] = keep_s ? s : 0.;
        mcoef32[(size_t)m * N + _t] = keep_s ? (float)s : 0.f;
        if ((keep_u && vol[m] != 0.) || (keep_s && s != 0.)) mymask |= 1u << m;
      }
      continue;
    }
#pragma unroll
    for (int m = 0; m < 19; m++) {
      coef[(size_t)m * N + _t] = 0.;
      mcoef[(size_t)m * N + _t] = 0.;
      mcoef32[(size_t)m * N + _t] = 0.f;
    }
  }
  atomicOr(mask, mymask);
}

// ---------------------------------------------------------------------------
// Face form of a level's aj-scaled operator for the FP32 multigrid.  The
// assembly above builds every row from six face fluxes, each computed
// identically by the two cells that share the face (poisson.c:1173-1558: the
// i+1 branch of cell c and the i-1 branch of cell c+1 test the same cells and
// walls), so on a level whose i-j and j-k cross terms vanish (the 11-slot
// operator)
//   (A x)_c = F_i(c) - F_i(c-i) + F_j(c) - F_j(c-j) + F_k(c) - F_k(c-k),
//   F_i(c) = gi (x_E - x_C) + gik (U - L)      (the k cross term of g13)
//   F_j(c) = gj (x_N - x_C)
//   F_k(c) = gk (x_T - x_C) + gki (R - Lf)     (the i cross term of g31)
// with gi = g11, gj = g22, gk = g33 where the face exists (both cells fluid,
// not a non-periodic wall) and 0 elsewhere, and the cross term's regime
// folded into its weight (0.25 centred, 0.5 one-sided, 0 none) and two code
// bits: U is the pair at k+1 (x_T + x_TE) or, one-sided, the centre pair
// (x_C + x_E); L the pair at k-1 or the centre pair; likewise R / Lf for the
// pairs at i+1 / i-1 of the k face.  A cell owns its +i, +j, +k faces; the
// row is scaled by aj.  The four code bits ride in the low mantissa bits of
// the FP32 aj (a relative change of at most 2^-19 of aj; the bits are
// cleared before aj is used), so a row streams 5 FP32 face weights and aj
// (24 bytes) instead of 11 FP32 coefficients (44 bytes), as FP32 arrays
// only (no byte array, whose rows a tensor copy could not tile).  Every level
// also gets fc: the i face's j cross term (g12), the j face's i and k cross
// terms (g21, g23) and the k face's j cross term (g32), each weight with its
// own two code bits (face_coded): on levels with those terms (terrain) the
// general face form adds them to F_i, F_j, F_k; elsewhere they are zero.  All
// six cross terms take their regime from face_regime.
// ---------------------------------------------------------------------------
// A cross weight with its own two code bits in its low mantissa bits.
__device__ __forceinline__ float face_coded(double w, unsigned code) {
  return __int_as_float((__float_as_int((float)w) & ~3) | (int)code);
}
// The regime of a cross term whose pairs lie beside the face at +1 / -1
// along another axis: up / dn are the nvert sums of the pairs there,
// at_hi / at_lo the non-periodic walls, first whether the cell is at index
// 1 of that axis (the backward difference is never taken there, periodic or
// not), as in poisson.c:1184-1231 and the same tests for every face and
// cross term.  Returns the weight factor (0.25 centred, 0.5 one-sided, 0
// none) and sets the code bits.
__device__ __forceinline__ double face_regime(double up, double dn, bool at_hi, bool at_lo, bool first,
                                              unsigned& code) {
  const double THR = VFS_THR;
  code = 0;
  if (at_hi || up > THR) {
    if (dn < THR && !first) {
      code = 1u;  // backward: the upper pair is the centre pair
      return 0.5;
    }
    return 0.;
  }
  if (at_lo || dn > THR) {
    if (up < THR) {
      code = 2u;  // forward: the lower pair is the centre pair
      return 0.5;
    }
    return 0.;
  }
  return 0.25;
}

__global__ void k_face_operator(Dims d, const double* __restrict__ g, const double* __restrict__ nvert,
                                const double* __restrict__ aj, float2* __restrict__ fi, float2* __restrict__ fk,
                                float* __restrict__ fj, float* __restrict__ faj, float4* __restrict__ fc) {
  const size_t N = ncell(d);
  const int mx = d.mx, my = d.my, mz = d.mz, ip = d.ip, jp = d.jp, kp = d.kp;
  const double *g11 = g, *g13 = g + 2 * N, *g22 = g + 4 * N, *g31 = g + 6 * N, *g33 = g + 8 * N;
  const double *g12 = g + N, *g21 = g + 3 * N, *g23 = g + 5 * N, *g32 = g + 7 * N;
  const double THR = VFS_THR;
  GRID_LOOP(d) {
    DECOMP(d, i, j, k);
    float2 vi = make_float2(0.f, 0.f), vk = make_float2(0.f, 0.f);
    float vj = 0.f;
    float4 vc = make_float4(0.f, 0.f, 0.f, 0.f);
    unsigned cb = 0;
    const bool row = interior(d, i, j, k) && !(nvert[_t] > THR);
    if (row) {
#define NV(ii, jj, kk) nvert[cidx(d, ii, jj, kk)]
      const size_t c = _t;
      if (NV(i + 1, j, k) < THR && (i != mx - 2 || ip)) {  // i+1/2 face, poisson.c:1173-1232
        unsigned qk;  // the k cross term (g13): pairs (C, E) at k+1 / k-1, code bits 0-1 of aj
        const double s = face_regime(NV(i, j, k + 1) + NV(i + 1, j, k + 1), NV(i, j, k - 1) + NV(i + 1, j, k - 1),
                                     k == mz - 2 && !kp, k == 1 && !kp, k == 1, qk);
        cb |= qk;
        vi = make_float2((float)g11[c], (float)(g13[c] * s));
        unsigned q;  // the j cross term (g12): pairs (C, E) at j+1 / j-1
        const double t = face_regime(NV(i, j + 1, k) + NV(i + 1, j + 1, k), NV(i, j - 1, k) + NV(i + 1, j - 1, k),
                                     j == my - 2 && !jp, j == 1 && !jp, j == 1, q);
        vc.x = face_coded(g12[c] * t, q);
      }
      if (NV(i, j + 1, k) < THR && (j != my - 2 || jp)) {  // j+1/2 face, poisson.c:1295-1352
        vj = (float)g22[c];
        unsigned q;  // the i cross term (g21): pairs (C, N) at i+1 / i-1
        double t = face_regime(NV(i + 1, j, k) + NV(i + 1, j + 1, k), NV(i - 1, j, k) + NV(i - 1, j + 1, k),
                               i == mx - 2 && !ip, i == 1 && !ip, i == 1, q);
        vc.y = face_coded(g21[c] * t, q);
        // the k cross term (g23): pairs (C, N) at k+1 / k-1
        t = face_regime(NV(i, j, k + 1) + NV(i, j + 1, k + 1), NV(i, j, k - 1) + NV(i, j + 1, k - 1),
                        k == mz - 2 && !kp, k == 1 && !kp, k == 1, q);
        vc.z = face_coded(g23[c] * t, q);
      }
      if (NV(i, j, k + 1) < THR && (k != mz - 2 || kp)) {                   // k+1/2 face, poisson.c:1421-1488
        unsigned qi;  // the i cross term (g31): pairs (C, T) at i+1 / i-1, code bits 2-3 of aj
        const double s = face_regime(NV(i + 1, j, k) + NV(i + 1, j, k + 1), NV(i - 1, j, k) + NV(i - 1, j, k + 1),
                                     i == mx - 2 && !ip, i == 1 && !ip, i == 1, qi);
        cb |= qi << 2;
        vk = make_float2((float)g33[c], (float)(g31[c] * s));
        unsigned q;  // the j cross term (g32): pairs (C, T) at j+1 / j-1
        const double t = face_regime(NV(i, j + 1, k) + NV(i, j + 1, k + 1), NV(i, j - 1, k) + NV(i, j - 1, k + 1),
                                     j == my - 2 && !jp, j == 1 && !jp, j == 1, q);
        vc.w = face_coded(g32[c] * t, q);
      }
#undef NV
    }
    fi[_t] = vi;
    fk[_t] = vk;
    fj[_t] = vj;
    faj[_t] = row ? __int_as_float((__float_as_int((float)aj[_t]) & ~0xF) | (int)cb) : 0.f;
    fc[_t] = vc;
  }
}

// ---------------------------------------------------------------------------
// Multigrid hierarchy.
// ---------------------------------------------------------------------------
// Coarse node coordinates = every other fine node (init.c:397-449).
__global__ void k_coarse_coords(Dims f, Dims c, int si, int sj, int sk, const double* __restrict__ cf, double* cc) {
  GRID_LOOP(c) {
    DECOMP(c, i, j, k);
    if (i >= c.mx - 1 || j >= c.my - 1 || k >= c.mz - 1) {
      cc[3 * _t] = cc[3 * _t + 1] = cc[3 * _t + 2] = 0.;
      continue;
    }
    size_t s = cidx(f, si ? i : 2 * i, sj ? j : 2 * j, sk ? k : 2 * k);
    cc[3 * _t] = cf[3 * s];
    cc[3 * _t + 1] = cf[3 * s + 1];
    cc[3 * _t + 2] = cf[3 * s + 2];
  }
}

// MyNvertRestriction part 1 (poisson.c:2046-2060): product of the children.
__global__ void k_nvert_product(Dims f, Dims c, int si, int sj, int sk, const double* __restrict__ nf, double* nc) {
  const int ia = si ? 0 : 1, ja = sj ? 0 : 1, ka = sk ? 0 : 1;
  GRID_LOOP(c) {
    DECOMP(c, i, j, k);
    double v = 0.;
    if (interior(c, i, j, k)) {
      int ih = si ? i : 2 * i, jh = sj ? j : 2 * j, kh = sk ? k : 2 * k;
      double p = nf[cidx(f, ih, jh, kh)] * nf[cidx(f, ih - ia, jh, kh)] * nf[cidx(f, ih, jh - ja, kh)] *
                 nf[cidx(f, ih, jh, kh - ka)] * nf[cidx(f, ih - ia, jh - ja, kh)] * nf[cidx(f, ih, jh - ja, kh - ka)] *
                 nf[cidx(f, ih - ia, jh, kh - ka)] * nf[cidx(f, ih - ia, jh - ja, kh - ka)];
      if (p > 0.1) v = 1.;
    }
    nc[_t] = v;
  }
}

// MyNvertRestriction part 2 (poisson.c:2084-2096): the sandwich fill updates
// nvert in place in k, j, i order.  A cell's test reads its i-1, j-1, k-1
// neighbours after and its i+1, j+1, k+1 neighbours before their own update,
// so processing the anti-diagonal planes i + j + k = s in increasing s
// reproduces the sequential result exactly.  One launch per plane.
__global__ void k_nvert_sandwich(Dims c, int s, double* nc) {
  const int ni = c.mx - 2, nj = c.my - 2;
  // enumerate (i, j) on plane s, k = s - i - j
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)ni * nj; t += (size_t)gridDim.x * blockDim.x) {
    int i = 1 + (int)(t % ni), j = 1 + (int)(t / ni);
    int k = s - i - j;
    if (k < 1 || k > c.mz - 2) continue;
    size_t q = cidx(c, i, j, k);
    if (nc[q] < 0.1) {
      if (nc[cidx(c, i + 1, j, k)] + nc[cidx(c, i - 1, j, k)] > 1.1 && nc[cidx(c, i, j + 1, k)] + nc[cidx(c, i, j - 1, k)] > 1.1 &&
          nc[cidx(c, i, j, k + 1)] + nc[cidx(c, i, j, k - 1)] > 1.1)
        nc[q] = 1.;
    }
  }
}

// Prolongation code of each fine cell (GridInterpolation, poisson.c:473-506):
// bit 7 = zero (boundary or solid fine cell), bits 0-1 ia+1, 2-3 ja+1, 4-5 ka+1.
__global__ void k_prolong_codes(Dims f, Dims c, int si, int sj, int sk, const double* __restrict__ nf,
                                const double* __restrict__ ncv, uint8_t* code) {
  GRID_LOOP(f) {
    DECOMP(f, i, j, k);
    if (!interior(f, i, j, k) || nf[_t] > 0.1) {
      code[_t] = 0x80;
      continue;
    }
    int ic, jc, kc, ia, ja, ka;
    if (si) { ic = i; ia = 0; } else { ic = (i + 1) / 2; ia = (i - 2 * ic) == 0 ? 1 : -1; if (i == 1 || i == f.mx - 2) ia = 0; }
    if (sj) { jc = j; ja = 0; } else { jc = (j + 1) / 2; ja = (j - 2 * jc) == 0 ? 1 : -1; if (j == 1 || j == f.my - 2) ja = 0; }
    if (sk) { kc = k; ka = 0; } else { kc = (k + 1) / 2; ka = (k - 2 * kc) == 0 ? 1 : -1; if (k == 1 || k == f.mz - 2) ka = 0; }
    if (ka == -1 && ncv[cidx(c, ic, jc, kc - 1)] > 0.1) ka = 0;
    else if (ka == 1 && ncv[cidx(c, ic, jc, kc + 1)] > 0.1) ka = 0;
    if (ja == -1 && ncv[cidx(c, ic, jc - 1, kc)] > 0.1) ja = 0;
    else if (ja == 1 && ncv[cidx(c, ic, jc + 1, kc)] > 0.1) ja = 0;
    if (ia == -1 && ncv[cidx(c, ic - 1, jc, kc)] > 0.1) ia = 0;
    else if (ia == 1 && ncv[cidx(c, ic + 1, jc, kc)] > 0.1) ia = 0;
    code[_t] = (uint8_t)((ia + 1) | ((ja + 1) << 2) | ((ka + 1) << 4));
  }
}

// ---------------------------------------------------------------------------
// Dense inverse of the coarsest operator.  B = A + sigma * e e^T over the
// fluid cells (e = fluid indicator; identity on non-fluid cells), so that
// B^{-1} r is the mean-zero solution of A x = r for compatible r.  With
// ccomp (labels of the level's connected fluid regions) the term is
// sigma * sum_q e_q e_q^T, one per region, so B stays nonsingular when
// bodies cut the level apart.  Unknowns
// are the interior cells packed as ((k-1)*nj + (j-1))*ni + (i-1).  Work
// matrix W = [B | I], n x 2n, row-major FP64; Gauss-Jordan with partial
// pivoting, one pivot per launch sequence.
// ---------------------------------------------------------------------------
__global__ void k_dense_build(Dims d, const double* __restrict__ mcoef, double sigma, double* W, int n,
                              const int* __restrict__ ccomp) {
  const size_t N = ncell(d);
  const int ni = d.mx - 2, nj = d.my - 2;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)n * 2 * n; t += (size_t)gridDim.x * blockDim.x) {
    int r = (int)(t / (2 * (size_t)n)), col = (int)(t % (2 * (size_t)n));
    int i = 1 + r % ni, j = 1 + (r / ni) % nj, k = 1 + r / (ni * nj);
    size_t c = cidx(d, i, j, k);
    bool fr = mcoef[c] != 0.;  // CP slot of a fluid row is nonzero
    double v = 0.;
    if (col >= n) v = (col - n == r) ? 1. : 0.;
    else {
      int i2 = 1 + col % ni, j2 = 1 + (col / ni) % nj, k2 = 1 + col / (ni * nj);
      size_t c2 = cidx(d, i2, j2, k2);
      bool fc = mcoef[c2] != 0.;
      if (!fr) v = (col == r) ? 1. : 0.;
      else {
        if (fc && (!ccomp || ccomp[c] == ccomp[c2])) v = sigma;
        // add the stencil entries whose wrapped column is c2
        int II[3] = {wrapi(i - 1, d.mx, d.ip), i, wrapi(i + 1, d.mx, d.ip)};
        int JJ[3] = {wrapi(j - 1, d.my, d.jp), j, wrapi(j + 1, d.my, d.jp)};
        int KK[3] = {wrapi(k - 1, d.mz, d.kp), k, wrapi(k + 1, d.mz, d.kp)};
#pragma unroll
        for (int m = 0; m < 19; m++)
          if (cidx(d, II[slot_di(m) + 1], JJ[slot_dj(m) + 1], KK[slot_dk(m) + 1]) == c2) v += mcoef[(size_t)m * N + c];
      }
    }
    W[t] = v;
  }
}

// Pivot search for column p (single block): writes the row index to *piv and
// the pivot value to *pval (read by the swap kernel, which overwrites W).
__global__ void k_gj_pivot(const double* W, int n, int p, int* piv, double* pval) {
  __shared__ double bv[32];
  __shared__ int bi[32];
  double best = -1.;
  int arg = p;
  for (int r = p + threadIdx.x; r < n; r += blockDim.x) {
    double v = fabs(W[(size_t)r * 2 * n + p]);
    if (v > best) { best = v; arg = r; }
  }
  for (int o = 16; o > 0; o >>= 1) {
    double ov = __shfl_down_sync(0xffffffffu, best, o);
    int oa = __shfl_down_sync(0xffffffffu, arg, o);
    if (ov > best || (ov == best && oa < arg)) { best = ov; arg = oa; }
  }
  if ((threadIdx.x & 31) == 0) { bv[threadIdx.x >> 5] = best; bi[threadIdx.x >> 5] = arg; }
  __syncthreads();
  if (threadIdx.x == 0) {
    int nw = blockDim.x >> 5;
    for (int w = 1; w < nw; w++)
      if (bv[w] > bv[0] || (bv[w] == bv[0] && bi[w] < bi[0])) { bv[0] = bv[w]; bi[0] = bi[w]; }
    *piv = bi[0];
    *pval = W[(size_t)bi[0] * 2 * n + p];
  }
}

// Swap rows p and *piv, scale row p by 1 / pivot, and save column p factors.
__global__ void k_gj_swap_scale(double* W, int n, int p, const int* piv, const double* pval) {
  const int q = *piv;
  const size_t w = 2 * (size_t)n;
  const double inv = 1. / *pval;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < w; c += (size_t)gridDim.x * blockDim.x) {
    double a = W[(size_t)p * w + c], b = W[(size_t)q * w + c];
    if (q != p) W[(size_t)q * w + c] = a;
    W[(size_t)p * w + c] = b * inv;
  }
}

__global__ void k_gj_factors(const double* W, int n, int p, double* fac) {
  const size_t w = 2 * (size_t)n;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) fac[r] = (r == p) ? 0. : W[(size_t)r * w + p];
}

__global__ void k_gj_eliminate(double* W, int n, int p, const double* fac) {
  const size_t w = 2 * (size_t)n;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)n * w; t += (size_t)gridDim.x * blockDim.x) {
    int r = (int)(t / w);
    size_t c = t % w;
    double f = fac[r];
    if (f != 0.) W[t] -= f * W[(size_t)p * w + c];
  }
}

// Copy the right half of W (the inverse) into Binv (FP64) and Binv32.
__global__ void k_gj_extract(const double* W, int n, double* B, float* B32) {
  const size_t w = 2 * (size_t)n;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < (size_t)n * n; t += (size_t)gridDim.x * blockDim.x) {
    size_t r = t / n, c = t % n;
    double v = W[r * w + n + c];
    B[t] = v;
    B32[t] = (float)v;
  }
}

// ---------------------------------------------------------------------------
// Host launchers.
// ---------------------------------------------------------------------------
static inline int nblk(size_t n, int bs = 256) {
  size_t b = (n + bs - 1) / bs;
  if (b > 152 * 32) b = 152 * 32;
  return (int)(b ? b : 1);
}

int launch_form_metrics(const Dims& d, const double* coor, double* M, double* tmp, cudaStream_t s) {
  const size_t N = ncell(d);
  VFS_CUDA_OK(cudaMemsetAsync(M, 0, sizeof(double) * N * MP_TOTAL, s));
  VFS_CUDA_OK(cudaMemsetAsync(tmp, 0, sizeof(double) * N * 9, s));
  k_metrics_cells<<<nblk(N), 256, 0, s>>>(d, coor, M, tmp); ++g_launches;
  k_metrics_centred<<<nblk(N), 256, 0, s>>>(d, coor, M, tmp); ++g_launches;
  for (int a = 0; a < 3; a++) k_metrics_mirror<<<nblk(N), 256, 0, s>>>(d, M, a); ++g_launches;
  k_metrics_faces<<<nblk(N), 256, 0, s>>>(d, coor, M); ++g_launches;
  return (int)cudaGetLastError();
}

int launch_face_operator(const Dims& d, const double* g, const double* nvert, const double* aj, float2* fi, float2* fk,
                         float* fj, float* faj, float4* fc, cudaStream_t s) {
  k_face_operator<<<nblk(ncell(d)), 256, 0, s>>>(d, g, nvert, aj, fi, fk, fj, faj, fc); ++g_launches;
  return (int)cudaGetLastError();
}

int launch_gtensor(const Dims& d, const double* M, double* g, cudaStream_t s) {
  k_gtensor<<<nblk(ncell(d)), 256, 0, s>>>(d, M, g); ++g_launches;
  return (int)cudaGetLastError();
}

int launch_assemble(const Dims& d, const double* g, const double* nvert, const double* aj, double* coef, double* mcoef,
                    float* mcoef32, unsigned* mask, cudaStream_t s) {
  VFS_CUDA_OK(cudaMemsetAsync(mask, 0, sizeof(unsigned), s));
  k_assemble<<<nblk(ncell(d), 128), 128, 0, s>>>(d, g, nvert, aj, coef, mcoef, mcoef32, mask); ++g_launches;
  return (int)cudaGetLastError();
}

int launch_coarsen(const Dims& f, const Dims& c, int si, int sj, int sk, const double* coor_f, const double* nv_f,
                   double* coor_c, double* nv_c, cudaStream_t s) {
  k_coarse_coords<<<nblk(ncell(c)), 256, 0, s>>>(f, c, si, sj, sk, coor_f, coor_c); ++g_launches;
  k_nvert_product<<<nblk(ncell(c)), 256, 0, s>>>(f, c, si, sj, sk, nv_f, nv_c); ++g_launches;
  const int smax = (c.mx - 2) + (c.my - 2) + (c.mz - 2);
  const size_t plane = (size_t)(c.mx - 2) * (c.my - 2);
  for (int sd = 3; sd <= smax; sd++) k_nvert_sandwich<<<nblk(plane), 256, 0, s>>>(c, sd, nv_c); ++g_launches;
  return (int)cudaGetLastError();
}

int launch_prolong_codes(const Dims& f, const Dims& c, int si, int sj, int sk, const double* nv_f, const double* nv_c,
                         uint8_t* code, cudaStream_t s) {
  k_prolong_codes<<<nblk(ncell(f)), 256, 0, s>>>(f, c, si, sj, sk, nv_f, nv_c, code); ++g_launches;
  return (int)cudaGetLastError();
}

// fac: n doubles; piv: 1 int; pval: 1 double (device scratch).
int launch_dense_inverse(const Dims& d, const double* mcoef, double sigma, double* W, double* fac, int* piv, double* pval,
                         double* Binv, float* Binv32, int n, cudaStream_t s, const int* ccomp) {
  const size_t w = 2 * (size_t)n;
  k_dense_build<<<nblk((size_t)n * w), 256, 0, s>>>(d, mcoef, sigma, W, n, ccomp); ++g_launches;
  for (int p = 0; p < n; p++) {
    k_gj_pivot<<<1, 256, 0, s>>>(W, n, p, piv, pval); ++g_launches;
    k_gj_swap_scale<<<nblk(w), 256, 0, s>>>(W, n, p, piv, pval); ++g_launches;
    k_gj_factors<<<nblk(n), 256, 0, s>>>(W, n, p, fac); ++g_launches;
    k_gj_eliminate<<<nblk((size_t)n * w), 256, 0, s>>>(W, n, p, fac); ++g_launches;
  }
  k_gj_extract<<<nblk((size_t)n * n), 256, 0, s>>>(W, n, Binv, Binv32); ++g_launches;
  return (int)cudaGetLastError();
}

}  // namespace vfs
