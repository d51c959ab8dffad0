/*
 * vfs_oracle.c -- CPU FP64 restatement of the VFS pressure-projection step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU library in
 * vfs_v3p2_gb300/csrc.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference arm of bench.py may load it.  The product path
 * never links or calls it.
 *
 * PINNED TO THE REFERENCE'S OWN CODE.  The reference cannot be built as a
 * program here (its hot path links PETSc 3.2-p7, HYPRE and MPI, none of
 * which exist in this image: variables.h:4-18, makefile:1-53), and it ships
 * no tests or golden data.  Its path functions are compiled unmodified from
 * their sources instead, against single-rank stand-ins of the library calls
 * they make (oracle/ref.mk, oracle/ref_stub/, oracle/ref_harness.cpp), and
 * tests/test_ref_oracle.py checks this restatement against them bit for bit:
 * FormMetrics, setup_lidx2 + PoissonLHSNew (every matrix entry),
 * VolumeFlux, PoissonRHS2_hypre / PoissonRHS2, Convert_Phi2_Phi,
 * UpdatePressure, Projection + Contra2Cart, Divergence, MyNvertRestriction,
 * MyRestriction and MyInterpolation (with semi-coarsening).  The committed
 * fixtures tests/golden/golden_small.npz hold the reference's outputs, so
 * the same check runs where its sources are absent.  The solve itself is
 * HYPRE's (absent): the converged solution of the same assembled system is
 * what is compared.  Known-answer tests derived from the discretisation
 * (tests/test_oracle.py) cover it besides.
 *
 * Array conventions follow the reference's PETSc DMDA arrays exactly:
 *   - extents mx = ni+2, my = nj+2, mz = nk+2 (one ghost/boundary cell per
 *     side, init.c:157 creates the DMDA with IM+1 points where IM = ni+1
 *     grid nodes);
 *   - scalar fields are double[mz][my][mx], i fastest;
 *   - vector fields (Cmpnts, variables.h:37-39) are double[mz][my][mx][3];
 *   - node coordinates use the same [mz][my][mx][3] array, nodes 0..ni valid
 *     (init.c:340-380 fills i < IM only).
 * Periodicity: i_periodic / j_periodic / k_periodic as in the reference
 * (index 0 is the image of mx-2 and mx-1 the image of 1).  The DMDA-periodic
 * ii/jj/kk variants are not restated.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
  int mx, my, mz;
  int ip, jp, kp;
} orc_dims;

/* Stencil slots, same numbering as poisson.c:956-974. */
enum { CP = 0, EP, WP, NP, SP, TP, BP, NE, SE, NW, SW, TN, BN, TS, BS, TE, BE, TW, BW, NSTENCIL };
static const int SDI[19] = {0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, 1, -1, -1};
static const int SDJ[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 1, 1, -1, -1, 0, 0, 0, 0};
static const int SDK[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1};

static const double THR = 0.1; /* poisson_threshold, poisson.c:16 */

#define ID(d, i, j, k) ((((size_t)(k)) * (d)->my + (j)) * (d)->mx + (i))

/* Metrics pack: offsets (in units of N = mx*my*mz doubles). */
enum {
  M_CSI = 0, M_ETA = 3, M_ZET = 6, M_AJ = 9,
  M_ICSI = 10, M_IETA = 13, M_IZET = 16, M_IAJ = 19,
  M_JCSI = 20, M_JETA = 23, M_JZET = 26, M_JAJ = 29,
  M_KCSI = 30, M_KETA = 33, M_KZET = 36, M_KAJ = 39,
  M_CENT = 40, M_TOTAL = 43
};

int orc_metrics_size(void) { return M_TOTAL; }
int orc_stencil_dx(int m) { return SDI[m]; }
int orc_stencil_dy(int m) { return SDJ[m]; }
int orc_stencil_dz(int m) { return SDK[m]; }

/* Periodic wrap of one index (poisson.c:1114-1130): 0 -> m-2, m-1 -> 1. */
static inline int wrapi(int i, int m, int per) {
  if (per) {
    if (i == 0) return m - 2;
    if (i == m - 1) return 1;
  }
  return i;
}

/* ------------------------------------------------------------------------- */
/* FormMetrics, NEWMETRIC branch (metrics.c:4-1004).                          */
/* ------------------------------------------------------------------------- */
typedef struct { double x, y, z; } vec3;

static inline vec3 ld3(const double* a, size_t c) { vec3 v = {a[3 * c], a[3 * c + 1], a[3 * c + 2]}; return v; }
static inline void st3(double* a, size_t c, vec3 v) { a[3 * c] = v.x; a[3 * c + 1] = v.y; a[3 * c + 2] = v.z; }

/* The three contravariant base vectors and 1/J from the 9 derivatives
 * (metrics.c:690-710: icsi/ieta/izet/iaj and the same for j and k). */
static void face_metric(double dxdc, double dydc, double dzdc, double dxde, double dyde, double dzde,
                        double dxdz, double dydz, double dzdz, vec3* csi, vec3* eta, vec3* zet, double* aj) {
  csi->x = dyde * dzdz - dzde * dydz;
  csi->y = -dxde * dzdz + dzde * dxdz;
  csi->z = dxde * dydz - dyde * dxdz;
  eta->x = dydz * dzdc - dzdz * dydc;
  eta->y = -dxdz * dzdc + dzdz * dxdc;
  eta->z = dxdz * dydc - dydz * dxdc;
  zet->x = dydc * dzde - dzdc * dyde;
  zet->y = -dxdc * dzde + dzdc * dxde;
  zet->z = dxdc * dyde - dydc * dxde;
  double a = dxdc * (dyde * dzdz - dzde * dydz) - dydc * (dxde * dzdz - dzde * dxdz) + dzdc * (dxde * dydz - dyde * dxdz);
  *aj = 1. / a;
}

void orc_form_metrics(const orc_dims* d, const double* coor, double* M) {
  const int mx = d->mx, my = d->my, mz = d->mz;
  const size_t N = (size_t)mx * my * mz;
  memset(M, 0, sizeof(double) * N * M_TOTAL);
  double *csi = M + N * M_CSI, *eta = M + N * M_ETA, *zet = M + N * M_ZET, *aj = M + N * M_AJ;
  double *icsi = M + N * M_ICSI, *ieta = M + N * M_IETA, *izet = M + N * M_IZET, *iaj = M + N * M_IAJ;
  double *jcsi = M + N * M_JCSI, *jeta = M + N * M_JETA, *jzet = M + N * M_JZET, *jaj = M + N * M_JAJ;
  double *kcsi = M + N * M_KCSI, *keta = M + N * M_KETA, *kzet = M + N * M_KZET, *kaj = M + N * M_KAJ;
  double* cent = M + N * M_CENT;
  double* tmp = (double*)calloc(N * 9, sizeof(double));
  double *csit = tmp, *etat = tmp + 3 * N, *zett = tmp + 6 * N;
#define C(i, j, k) ld3(coor, ID(d, i, j, k))
  /* cell centres, metrics.c:80-103 */
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        vec3 a = C(i, j, k), b = C(i, j - 1, k), c = C(i, j, k - 1), e = C(i, j - 1, k - 1);
        vec3 f = C(i - 1, j, k), g = C(i - 1, j - 1, k), h = C(i - 1, j, k - 1), q = C(i - 1, j - 1, k - 1);
        vec3 r;
        r.x = 0.125 * (a.x + b.x + c.x + e.x + f.x + g.x + h.x + q.x);
        r.y = 0.125 * (a.y + b.y + c.y + e.y + f.y + g.y + h.y + q.y);
        r.z = 0.125 * (a.z + b.z + c.z + e.z + f.z + g.z + h.z + q.z);
        st3(cent, ID(d, i, j, k), r);
      }
  /* half-face normals, metrics.c:190-277 */
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 0; i < mx - 1; i++) {
        vec3 p00 = C(i, j, k), p10 = C(i, j - 1, k), p01 = C(i, j, k - 1), p11 = C(i, j - 1, k - 1);
        double dxde = 0.5 * (p00.x + p01.x - p10.x - p11.x);
        double dyde = 0.5 * (p00.y + p01.y - p10.y - p11.y);
        double dzde = 0.5 * (p00.z + p01.z - p10.z - p11.z);
        double dxdz = 0.5 * (p10.x + p00.x - p11.x - p01.x);
        double dydz = 0.5 * (p10.y + p00.y - p11.y - p01.y);
        double dzdz = 0.5 * (p10.z + p00.z - p11.z - p01.z);
        vec3 r = {dyde * dzdz - dzde * dydz, -dxde * dzdz + dzde * dxdz, dxde * dydz - dyde * dxdz};
        st3(csit, ID(d, i, j, k), r);
      }
  for (int k = 1; k < mz - 1; k++)
    for (int j = 0; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        vec3 a = C(i, j, k), b = C(i, j, k - 1), c = C(i - 1, j, k), e = C(i - 1, j, k - 1);
        double dxdc = 0.5 * (a.x + b.x - c.x - e.x);
        double dydc = 0.5 * (a.y + b.y - c.y - e.y);
        double dzdc = 0.5 * (a.z + b.z - c.z - e.z);
        double dxdz = 0.5 * (a.x + c.x - b.x - e.x);
        double dydz = 0.5 * (a.y + c.y - b.y - e.y);
        double dzdz = 0.5 * (a.z + c.z - b.z - e.z);
        vec3 r = {dydz * dzdc - dzdz * dydc, -dxdz * dzdc + dzdz * dxdc, dxdz * dydc - dydz * dxdc};
        st3(etat, ID(d, i, j, k), r);
      }
  for (int k = 0; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        vec3 a = C(i, j, k), b = C(i, j - 1, k), c = C(i - 1, j, k), e = C(i - 1, j - 1, k);
        double dxdc = 0.5 * (a.x + b.x - c.x - e.x);
        double dydc = 0.5 * (a.y + b.y - c.y - e.y);
        double dzdc = 0.5 * (a.z + b.z - c.z - e.z);
        double dxde = 0.5 * (a.x + c.x - b.x - e.x);
        double dyde = 0.5 * (a.y + c.y - b.y - e.y);
        double dzde = 0.5 * (a.z + c.z - b.z - e.z);
        vec3 r = {dydc * dzde - dzdc * dyde, -dxdc * dzde + dzdc * dxde, dxdc * dyde - dydc * dxde};
        st3(zett, ID(d, i, j, k), r);
      }
  /* averaged cell-centred normals, metrics.c:291-297 */
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        size_t c = ID(d, i, j, k);
        vec3 a = ld3(csit, c), b = ld3(csit, ID(d, i - 1, j, k));
        vec3 r = {0.5 * a.x + 0.5 * b.x, 0.5 * a.y + 0.5 * b.y, 0.5 * a.z + 0.5 * b.z};
        st3(csi, c, r);
        a = ld3(etat, c); b = ld3(etat, ID(d, i, j - 1, k));
        r.x = 0.5 * a.x + 0.5 * b.x; r.y = 0.5 * a.y + 0.5 * b.y; r.z = 0.5 * a.z + 0.5 * b.z;
        st3(eta, c, r);
        a = ld3(zett, c); b = ld3(zett, ID(d, i, j, k - 1));
        r.x = 0.5 * a.x + 0.5 * b.x; r.y = 0.5 * a.y + 0.5 * b.y; r.z = 0.5 * a.z + 0.5 * b.z;
        st3(zet, c, r);
      }
  /* cell Jacobian, metrics.c:304-371 */
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        vec3 c000 = C(i, j, k), c010 = C(i, j - 1, k), c001 = C(i, j, k - 1), c011 = C(i, j - 1, k - 1);
        vec3 c100 = C(i - 1, j, k), c110 = C(i - 1, j - 1, k), c101 = C(i - 1, j, k - 1), c111 = C(i - 1, j - 1, k - 1);
        double dxdc = 0.25 * (c000.x + c010.x + c001.x + c011.x - c100.x - c110.x - c101.x - c111.x);
        double dydc = 0.25 * (c000.y + c010.y + c001.y + c011.y - c100.y - c110.y - c101.y - c111.y);
        double dzdc = 0.25 * (c000.z + c010.z + c001.z + c011.z - c100.z - c110.z - c101.z - c111.z);
        double dxde = 0.25 * (c000.x + c100.x + c001.x + c101.x - c010.x - c110.x - c011.x - c111.x);
        double dyde = 0.25 * (c000.y + c100.y + c001.y + c101.y - c010.y - c110.y - c011.y - c111.y);
        double dzde = 0.25 * (c000.z + c100.z + c001.z + c101.z - c010.z - c110.z - c011.z - c111.z);
        double dxdz = 0.25 * (c000.x + c010.x + c100.x + c110.x - c001.x - c011.x - c101.x - c111.x);
        double dydz = 0.25 * (c000.y + c010.y + c100.y + c110.y - c001.y - c011.y - c101.y - c111.y);
        double dzdz = 0.25 * (c000.z + c010.z + c100.z + c110.z - c001.z - c011.z - c101.z - c111.z);
        double a = dxdc * (dyde * dzdz - dzde * dydz) - dydc * (dxde * dzdz - dzde * dxdz) + dzdc * (dxde * dydz - dyde * dxdz);
        aj[ID(d, i, j, k)] = 1. / a;
      }
  /* mirror copies on the boundary planes, metrics.c:373-453 (same order) */
  for (int k = 0; k < mz; k++)
    for (int j = 0; j < my; j++) {
      size_t a = ID(d, 0, j, k), b = ID(d, 1, j, k);
      st3(csi, a, ld3(csi, b)); st3(eta, a, ld3(eta, b)); st3(zet, a, ld3(zet, b)); aj[a] = aj[b];
      a = ID(d, mx - 1, j, k); b = ID(d, mx - 2, j, k);
      st3(csi, a, ld3(csi, b)); st3(eta, a, ld3(eta, b)); st3(zet, a, ld3(zet, b)); aj[a] = aj[b];
    }
  for (int k = 0; k < mz; k++)
    for (int i = 0; i < mx; i++) {
      size_t a = ID(d, i, 0, k), b = ID(d, i, 1, k);
      st3(csi, a, ld3(csi, b)); st3(eta, a, ld3(eta, b)); st3(zet, a, ld3(zet, b)); aj[a] = aj[b];
      a = ID(d, i, my - 1, k); b = ID(d, i, my - 2, k);
      st3(csi, a, ld3(csi, b)); st3(eta, a, ld3(eta, b)); st3(zet, a, ld3(zet, b)); aj[a] = aj[b];
    }
  for (int j = 0; j < my; j++)
    for (int i = 0; i < mx; i++) {
      size_t a = ID(d, i, j, 0), b = ID(d, i, j, 1);
      st3(csi, a, ld3(csi, b)); st3(eta, a, ld3(eta, b)); st3(zet, a, ld3(zet, b)); aj[a] = aj[b];
      a = ID(d, i, j, mz - 1); b = ID(d, i, j, mz - 2);
      st3(csi, a, ld3(csi, b)); st3(eta, a, ld3(eta, b)); st3(zet, a, ld3(zet, b)); aj[a] = aj[b];
    }
  /* The periodic ghost copies of metrics.c:470-510 act on the local vectors
   * only, and their one reader (the face-metric fallbacks at metrics.c:713-720,
   * 835-842, 993-1000) is commented out; the final scatter of the global
   * vectors (metrics.c:1212-1244) then restores the mirror values on every
   * boundary plane (a periodic axis has one rank, init.c:144-146, so its ghost
   * planes are owned points).  The mirror copies above are therefore final. */
  /* i-face metrics from x-face centres, metrics.c:592-723 */
  double* cx = tmp; /* reuse: face centres */
  memset(tmp, 0, sizeof(double) * N * 9);
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 0; i < mx - 1; i++) {
        vec3 a = C(i, j, k), b = C(i, j, k - 1), c = C(i, j - 1, k), e = C(i, j - 1, k - 1);
        vec3 r = {(a.x + b.x + c.x + e.x) * 0.25, (a.y + b.y + c.y + e.y) * 0.25, (a.z + b.z + c.z + e.z) * 0.25};
        st3(cx, ID(d, i, j, k), r);
      }
#define CX(i, j, k) ld3(cx, ID(d, i, j, k))
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 0; i < mx - 1; i++) {
        vec3 dc, de, dz, p, m;
        if (i == 0) {
          p = CX(i + 1, j, k); m = CX(i, j, k);
          dc.x = p.x - m.x; dc.y = p.y - m.y; dc.z = p.z - m.z;
        } else if (i == mx - 2) {
          if (d->ip) {
            vec3 a = CX(1, j, k), b = CX(0, j, k), c = CX(i, j, k), e = CX(i - 1, j, k);
            dc.x = (a.x - b.x + c.x - e.x) * 0.5; dc.y = (a.y - b.y + c.y - e.y) * 0.5; dc.z = (a.z - b.z + c.z - e.z) * 0.5;
          } else {
            p = CX(i, j, k); m = CX(i - 1, j, k);
            dc.x = p.x - m.x; dc.y = p.y - m.y; dc.z = p.z - m.z;
          }
        } else {
          p = CX(i + 1, j, k); m = CX(i - 1, j, k);
          dc.x = (p.x - m.x) * 0.5; dc.y = (p.y - m.y) * 0.5; dc.z = (p.z - m.z) * 0.5;
        }
        if (j == 1) { p = CX(i, j + 1, k); m = CX(i, j, k); de.x = p.x - m.x; de.y = p.y - m.y; de.z = p.z - m.z; }
        else if (j == my - 2) { p = CX(i, j, k); m = CX(i, j - 1, k); de.x = p.x - m.x; de.y = p.y - m.y; de.z = p.z - m.z; }
        else { p = CX(i, j + 1, k); m = CX(i, j - 1, k); de.x = (p.x - m.x) * 0.5; de.y = (p.y - m.y) * 0.5; de.z = (p.z - m.z) * 0.5; }
        if (k == 1) { p = CX(i, j, k + 1); m = CX(i, j, k); dz.x = p.x - m.x; dz.y = p.y - m.y; dz.z = p.z - m.z; }
        else if (k == mz - 2) { p = CX(i, j, k); m = CX(i, j, k - 1); dz.x = p.x - m.x; dz.y = p.y - m.y; dz.z = p.z - m.z; }
        else { p = CX(i, j, k + 1); m = CX(i, j, k - 1); dz.x = (p.x - m.x) * 0.5; dz.y = (p.y - m.y) * 0.5; dz.z = (p.z - m.z) * 0.5; }
        vec3 a, b, c; double J;
        face_metric(dc.x, dc.y, dc.z, de.x, de.y, de.z, dz.x, dz.y, dz.z, &a, &b, &c, &J);
        size_t t = ID(d, i, j, k);
        st3(icsi, t, a); st3(ieta, t, b); st3(izet, t, c); iaj[t] = J;
      }
  /* j-face metrics, metrics.c:731-822 */
  memset(tmp, 0, sizeof(double) * N * 3);
  for (int k = 1; k < mz - 1; k++)
    for (int j = 0; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        vec3 a = C(i, j, k), b = C(i, j, k - 1), c = C(i - 1, j, k), e = C(i - 1, j, k - 1);
        vec3 r = {(a.x + b.x + c.x + e.x) * 0.25, (a.y + b.y + c.y + e.y) * 0.25, (a.z + b.z + c.z + e.z) * 0.25};
        st3(cx, ID(d, i, j, k), r);
      }
  for (int k = 1; k < mz - 1; k++)
    for (int j = 0; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        vec3 dc, de, dz, p, m;
        if (i == 1) { p = CX(i + 1, j, k); m = CX(i, j, k); dc.x = p.x - m.x; dc.y = p.y - m.y; dc.z = p.z - m.z; }
        else if (i == mx - 2) { p = CX(i, j, k); m = CX(i - 1, j, k); dc.x = p.x - m.x; dc.y = p.y - m.y; dc.z = p.z - m.z; }
        else { p = CX(i + 1, j, k); m = CX(i - 1, j, k); dc.x = (p.x - m.x) * 0.5; dc.y = (p.y - m.y) * 0.5; dc.z = (p.z - m.z) * 0.5; }
        if (j == 0) { p = CX(i, j + 1, k); m = CX(i, j, k); de.x = p.x - m.x; de.y = p.y - m.y; de.z = p.z - m.z; }
        else if (j == my - 2) {
          if (d->jp) {
            vec3 a = CX(i, 1, k), b = CX(i, 0, k), c = CX(i, j, k), e = CX(i, j - 1, k);
            de.x = (a.x - b.x + c.x - e.x) * 0.5; de.y = (a.y - b.y + c.y - e.y) * 0.5; de.z = (a.z - b.z + c.z - e.z) * 0.5;
          } else { p = CX(i, j, k); m = CX(i, j - 1, k); de.x = p.x - m.x; de.y = p.y - m.y; de.z = p.z - m.z; }
        } else { p = CX(i, j + 1, k); m = CX(i, j - 1, k); de.x = (p.x - m.x) * 0.5; de.y = (p.y - m.y) * 0.5; de.z = (p.z - m.z) * 0.5; }
        if (k == 1) { p = CX(i, j, k + 1); m = CX(i, j, k); dz.x = p.x - m.x; dz.y = p.y - m.y; dz.z = p.z - m.z; }
        else if (k == mz - 2) { p = CX(i, j, k); m = CX(i, j, k - 1); dz.x = p.x - m.x; dz.y = p.y - m.y; dz.z = p.z - m.z; }
        else { p = CX(i, j, k + 1); m = CX(i, j, k - 1); dz.x = (p.x - m.x) * 0.5; dz.y = (p.y - m.y) * 0.5; dz.z = (p.z - m.z) * 0.5; }
        vec3 a, b, c; double J;
        face_metric(dc.x, dc.y, dc.z, de.x, de.y, de.z, dz.x, dz.y, dz.z, &a, &b, &c, &J);
        size_t t = ID(d, i, j, k);
        st3(jcsi, t, a); st3(jeta, t, b); st3(jzet, t, c); jaj[t] = J;
      }
  /* k-face metrics, metrics.c:840-960 */
  memset(tmp, 0, sizeof(double) * N * 3);
  for (int k = 0; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        vec3 a = C(i, j, k), b = C(i, j - 1, k), c = C(i - 1, j, k), e = C(i - 1, j - 1, k);
        vec3 r = {(a.x + b.x + c.x + e.x) * 0.25, (a.y + b.y + c.y + e.y) * 0.25, (a.z + b.z + c.z + e.z) * 0.25};
        st3(cx, ID(d, i, j, k), r);
      }
  for (int k = 0; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        vec3 dc, de, dz, p, m;
        if (i == 1) { p = CX(i + 1, j, k); m = CX(i, j, k); dc.x = p.x - m.x; dc.y = p.y - m.y; dc.z = p.z - m.z; }
        else if (i == mx - 2) { p = CX(i, j, k); m = CX(i - 1, j, k); dc.x = p.x - m.x; dc.y = p.y - m.y; dc.z = p.z - m.z; }
        else { p = CX(i + 1, j, k); m = CX(i - 1, j, k); dc.x = (p.x - m.x) * 0.5; dc.y = (p.y - m.y) * 0.5; dc.z = (p.z - m.z) * 0.5; }
        if (j == 1) { p = CX(i, j + 1, k); m = CX(i, j, k); de.x = p.x - m.x; de.y = p.y - m.y; de.z = p.z - m.z; }
        else if (j == my - 2) { p = CX(i, j, k); m = CX(i, j - 1, k); de.x = p.x - m.x; de.y = p.y - m.y; de.z = p.z - m.z; }
        else { p = CX(i, j + 1, k); m = CX(i, j - 1, k); de.x = (p.x - m.x) * 0.5; de.y = (p.y - m.y) * 0.5; de.z = (p.z - m.z) * 0.5; }
        if (k == 0) { p = CX(i, j, k + 1); m = CX(i, j, k); dz.x = p.x - m.x; dz.y = p.y - m.y; dz.z = p.z - m.z; }
        else if (k == mz - 2) {
          if (d->kp) {
            vec3 a = CX(i, j, 1), b = CX(i, j, 0), c = CX(i, j, k), e = CX(i, j, k - 1);
            dz.x = (a.x - b.x + c.x - e.x) * 0.5; dz.y = (a.y - b.y + c.y - e.y) * 0.5; dz.z = (a.z - b.z + c.z - e.z) * 0.5;
          } else { p = CX(i, j, k); m = CX(i, j, k - 1); dz.x = p.x - m.x; dz.y = p.y - m.y; dz.z = p.z - m.z; }
        } else { p = CX(i, j, k + 1); m = CX(i, j, k - 1); dz.x = (p.x - m.x) * 0.5; dz.y = (p.y - m.y) * 0.5; dz.z = (p.z - m.z) * 0.5; }
        vec3 a, b, c; double J;
        face_metric(dc.x, dc.y, dc.z, de.x, de.y, de.z, dz.x, dz.y, dz.z, &a, &b, &c, &J);
        size_t t = ID(d, i, j, k);
        st3(kcsi, t, a); st3(keta, t, b); st3(kzet, t, c); kaj[t] = J;
      }
#undef CX
#undef C
  free(tmp);
}

/* ------------------------------------------------------------------------- */
/* g tensor, poisson.c:1105-1141 (9 face coefficients, periodic-wrapped).     */
/* ------------------------------------------------------------------------- */
void orc_gtensor(const orc_dims* d, const double* M, double* g) {
  const size_t N = (size_t)d->mx * d->my * d->mz;
  const double *icsi = M + N * M_ICSI, *ieta = M + N * M_IETA, *izet = M + N * M_IZET, *iaj = M + N * M_IAJ;
  const double *jcsi = M + N * M_JCSI, *jeta = M + N * M_JETA, *jzet = M + N * M_JZET, *jaj = M + N * M_JAJ;
  const double *kcsi = M + N * M_KCSI, *keta = M + N * M_KETA, *kzet = M + N * M_KZET, *kaj = M + N * M_KAJ;
  for (int k = 0; k < d->mz; k++)
    for (int j = 0; j < d->my; j++)
      for (int i = 0; i < d->mx; i++) {
        int a = wrapi(i, d->mx, d->ip), b = wrapi(j, d->my, d->jp), c = wrapi(k, d->mz, d->kp);
        size_t s = ID(d, a, b, c), t = ID(d, i, j, k);
        vec3 ic = ld3(icsi, s), ie = ld3(ieta, s), iz = ld3(izet, s);
        vec3 jc = ld3(jcsi, s), je = ld3(jeta, s), jz = ld3(jzet, s);
        vec3 kc = ld3(kcsi, s), ke = ld3(keta, s), kz = ld3(kzet, s);
        g[0 * N + t] = (ic.x * ic.x + ic.y * ic.y + ic.z * ic.z) * iaj[s];
        g[1 * N + t] = (ie.x * ic.x + ie.y * ic.y + ie.z * ic.z) * iaj[s];
        g[2 * N + t] = (iz.x * ic.x + iz.y * ic.y + iz.z * ic.z) * iaj[s];
        g[3 * N + t] = (jc.x * je.x + jc.y * je.y + jc.z * je.z) * jaj[s];
        g[4 * N + t] = (je.x * je.x + je.y * je.y + je.z * je.z) * jaj[s];
        g[5 * N + t] = (jz.x * je.x + jz.y * je.y + jz.z * je.z) * jaj[s];
        g[6 * N + t] = (kc.x * kz.x + kc.y * kz.y + kc.z * kz.z) * kaj[s];
        g[7 * N + t] = (ke.x * kz.x + ke.y * kz.y + ke.z * kz.z) * kaj[s];
        g[8 * N + t] = (kz.x * kz.x + kz.y * kz.y + kz.z * kz.z) * kaj[s];
      }
}

/* ------------------------------------------------------------------------- */
/* Fluid-only numbering, setup_lidx2 (poisson.c:187-334): gid >= 0 for fluid  */
/* interior cells ((int)nvert <= 0.1), -1 elsewhere; periodic ghosts take the */
/* gid of their partner.  Returns the number of fluid cells.                  */
/* ------------------------------------------------------------------------- */
int orc_gid(const orc_dims* d, const double* nvert, int* gid) {
  const size_t N = (size_t)d->mx * d->my * d->mz;
  for (size_t c = 0; c < N; c++) gid[c] = -1;
  int n = 0;
  for (int k = 1; k < d->mz - 1; k++)
    for (int j = 1; j < d->my - 1; j++)
      for (int i = 1; i < d->mx - 1; i++)
        if (!((int)nvert[ID(d, i, j, k)] > THR)) gid[ID(d, i, j, k)] = n++;
  for (int k = 0; k < d->mz; k++)
    for (int j = 0; j < d->my; j++)
      for (int i = 0; i < d->mx; i++) {
        int a = wrapi(i, d->mx, d->ip), b = wrapi(j, d->my, d->jp), c = wrapi(k, d->mz, d->kp);
        if (a != i || b != j || c != k) gid[ID(d, i, j, k)] = gid[ID(d, a, b, c)];
      }
  return n;
}

/* ------------------------------------------------------------------------- */
/* PoissonLHSNew (poisson.c:976-1630), built HYPRE body.  Writes the 19 row   */
/* entries of every fluid interior cell into coef[m*N + cell] after the drop  */
/* rule of poisson.c:1607-1616 (|v| <= 1e-10 or a column without a fluid id   */
/* is dropped, the diagonal is always kept).  Non-fluid rows are all zero.    */
/* The additions happen in the reference's order, so entries are bit-equal    */
/* to the values handed to HYPRE_IJMatrixSetValues.  levelset (r != 1) is not */
/* restated.  orc_lhs_scaled is the multigrid path's form (poisson == -1):    */
/* every entry of the row is multiplied by aj first (poisson.c:1560) and the  */
/* drop rule then applies to the scaled values.                               */
/* ------------------------------------------------------------------------- */
static void lhs_rows(const orc_dims* d, const double* g, const double* nvert, const double* aj, double* coef);
void orc_lhs(const orc_dims* d, const double* g, const double* nvert, double* coef) { lhs_rows(d, g, nvert, NULL, coef); }
void orc_lhs_scaled(const orc_dims* d, const double* g, const double* nvert, const double* aj, double* coef) {
  lhs_rows(d, g, nvert, aj, coef);
}
static void lhs_rows(const orc_dims* d, const double* g, const double* nvert, const double* aj, double* coef) {
  const int mx = d->mx, my = d->my, mz = d->mz;
  const int ip = d->ip, jp = d->jp, kp = d->kp;
  const size_t N = (size_t)mx * my * mz;
  const double *g11 = g, *g12 = g + N, *g13 = g + 2 * N, *g21 = g + 3 * N, *g22 = g + 4 * N, *g23 = g + 5 * N;
  const double *g31 = g + 6 * N, *g32 = g + 7 * N, *g33 = g + 8 * N;
  int* gid = (int*)malloc(sizeof(int) * N);
  orc_gid(d, nvert, gid);
  memset(coef, 0, sizeof(double) * N * NSTENCIL);
#define NV(ii, jj, kk) nvert[ID(d, ii, jj, kk)]
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        if (NV(i, j, k) > THR) continue;
        double vol[19];
        for (int m = 0; m < 19; m++) vol[m] = 0.;
        const double r = 1.0;
        size_t c = ID(d, i, j, k);
        /* i+1 - i, poisson.c:1173-1232 */
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
        /* i - i-1, poisson.c:1235-1292 */
        if (NV(i - 1, j, k) < THR && (i != 1 || ip)) {
          size_t w = ID(d, i - 1, j, k);
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
        /* j+1 - j, poisson.c:1295-1357 */
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
        /* j - j-1, poisson.c:1360-1417 */
        if (NV(i, j - 1, k) < THR && (j != 1 || jp)) {
          size_t s = ID(d, i, j - 1, k);
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
        /* k+1 - k, poisson.c:1421-1488 */
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
        /* k - k-1, poisson.c:1491-1558 */
        if (NV(i, j, k - 1) < THR && (k != 1 || kp)) {
          size_t b = ID(d, i, j, k - 1);
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
        if (aj)  /* poisson == -1, poisson.c:1560 */
          for (int m = 0; m < 19; m++) vol[m] *= aj[c];
        /* drop rule, poisson.c:1607-1616 */
        for (int m = 0; m < 19; m++) {
          int ni = wrapi(i + SDI[m], mx, ip), nj = wrapi(j + SDJ[m], my, jp), nk = wrapi(k + SDK[m], mz, kp);
          int col = gid[ID(d, i + SDI[m], j + SDJ[m], k + SDK[m])];
          (void)ni; (void)nj; (void)nk;
          if ((fabs(vol[m]) > 1.e-10 && col >= 0) || m == CP) coef[(size_t)m * N + c] = vol[m];
        }
      }
#undef NV
  free(gid);
}

/* Column (cell index) of stencil slot m for cell (i,j,k): periodic ghosts map
 * to their partner (the gid of a ghost is its partner's gid, poisson.c:300). */
static inline size_t nbr(const orc_dims* d, int i, int j, int k, int m) {
  return ID(d, wrapi(i + SDI[m], d->mx, d->ip), wrapi(j + SDJ[m], d->my, d->jp), wrapi(k + SDK[m], d->mz, d->kp));
}

/* y = A x over the structured layout (rows of non-fluid cells are zero). */
void orc_matvec(const orc_dims* d, const double* coef, const double* x, double* y) {
  const size_t N = (size_t)d->mx * d->my * d->mz;
  memset(y, 0, sizeof(double) * N);
#pragma omp parallel for schedule(static)
  for (int k = 1; k < d->mz - 1; k++)
    for (int j = 1; j < d->my - 1; j++)
      for (int i = 1; i < d->mx - 1; i++) {
        size_t c = ID(d, i, j, k);
        double s = 0.;
        for (int m = 0; m < 19; m++) {
          double a = coef[(size_t)m * N + c];
          if (a != 0.) s += a * x[nbr(d, i, j, k, m)];
        }
        y[c] = s;
      }
}

/* Export the operator as CSR over the compact fluid numbering. */
int orc_csr(const orc_dims* d, const double* coef, const double* nvert, int* rowptr, int* col, double* val, int* gid) {
  const size_t N = (size_t)d->mx * d->my * d->mz;
  int n = orc_gid(d, nvert, gid);
  int nnz = 0, row = 0;
  rowptr[0] = 0;
  for (int k = 1; k < d->mz - 1; k++)
    for (int j = 1; j < d->my - 1; j++)
      for (int i = 1; i < d->mx - 1; i++) {
        size_t c = ID(d, i, j, k);
        if (gid[c] < 0) continue;
        for (int m = 0; m < 19; m++) {
          double a = coef[(size_t)m * N + c];
          /* the reference writes a row only for the cells it assembles
           * (nvert <= 0.1): a numbered cell with 0.1 < nvert < 1 keeps an
           * empty row (poisson.c:1160-1163) */
          if (a != 0. || (m == CP && !(nvert[c] > THR))) {
            col[nnz] = gid[ID(d, i + SDI[m], j + SDJ[m], k + SDK[m])];
            val[nnz] = a;
            if (col[nnz] < 0) continue;
            nnz++;
          }
        }
        rowptr[++row] = nnz;
      }
  (void)n;
  return nnz;
}

/* ------------------------------------------------------------------------- */
/* Connected regions of the fluid cells (interior, nvert < 0.1) through       */
/* shared faces, periodic wrap included: label[c] = 0..K-1 in the order of    */
/* each region's first cell (cell index order), -1 on other cells; returns    */
/* K.  A grid that bodies cut apart has one constant null vector per region   */
/* (the reference's two-region case: FullyBlocked, poisson.c:1918-1998, and   */
/* the split null space of PoissonNullSpaceFunction, poisson.c:819-873).      */
/* ------------------------------------------------------------------------- */
static int uf_find(int* parent, int a) {
  while (parent[a] != a) {
    parent[a] = parent[parent[a]];
    a = parent[a];
  }
  return a;
}
static void uf_unite(int* parent, int a, int b) {
  a = uf_find(parent, a);
  b = uf_find(parent, b);
  if (a != b) {
    if (a < b) parent[b] = a;
    else parent[a] = b;
  }
}
int orc_fluid_regions(const orc_dims* d, const double* nvert, int* label) {
  const int mx = d->mx, my = d->my, mz = d->mz;
  const size_t N = (size_t)mx * my * mz;
  int* parent = (int*)malloc(N * sizeof(int));
  int* id = (int*)malloc(N * sizeof(int));
  for (size_t c = 0; c < N; c++) { parent[c] = -1; id[c] = -1; label[c] = -1; }
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        size_t c = ID(d, i, j, k);
        if (nvert[c] < 0.1) parent[c] = (int)c;
      }
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        size_t c = ID(d, i, j, k);
        if (parent[c] < 0) continue;
        int in = (i == mx - 2) ? (d->ip ? 1 : -1) : i + 1;
        int jn = (j == my - 2) ? (d->jp ? 1 : -1) : j + 1;
        int kn = (k == mz - 2) ? (d->kp ? 1 : -1) : k + 1;
        if (in > 0 && parent[ID(d, in, j, k)] >= 0) uf_unite(parent, (int)c, (int)ID(d, in, j, k));
        if (jn > 0 && parent[ID(d, i, jn, k)] >= 0) uf_unite(parent, (int)c, (int)ID(d, i, jn, k));
        if (kn > 0 && parent[ID(d, i, j, kn)] >= 0) uf_unite(parent, (int)c, (int)ID(d, i, j, kn));
      }
  int K = 0;
  for (size_t c = 0; c < N; c++) {
    if (parent[c] < 0) continue;
    int r = uf_find(parent, (int)c);
    if (id[r] < 0) id[r] = K++;
    label[c] = id[r];
  }
  free(parent);
  free(id);
  return K;
}

/* Per-region fluid mean of x subtracted from the region's fluid cells; the
 * sums run in cell loop order (k, j, i), as the single-region versions. */
static void sub_region_means(const orc_dims* d, const double* nvert, const int* label, int K, double* x) {
  double* sum = (double*)calloc((size_t)K, sizeof(double));
  long* cnt = (long*)calloc((size_t)K, sizeof(long));
  for (int k = 1; k < d->mz - 1; k++)
    for (int j = 1; j < d->my - 1; j++)
      for (int i = 1; i < d->mx - 1; i++) {
        size_t c = ID(d, i, j, k);
        if (nvert[c] < 0.1) { sum[label[c]] += x[c]; cnt[label[c]]++; }
      }
  for (int k = 1; k < d->mz - 1; k++)
    for (int j = 1; j < d->my - 1; j++)
      for (int i = 1; i < d->mx - 1; i++) {
        size_t c = ID(d, i, j, k);
        if (nvert[c] < 0.1) x[c] += -sum[label[c]] / (double)cnt[label[c]];
      }
  free(sum);
  free(cnt);
}

/* Number of fluid regions (1 without allocating when no interior cell is
 * non-fluid); fills *label (malloc'd, caller frees) when more than one. */
static int regions_of(const orc_dims* d, const double* nvert, int** label) {
  *label = NULL;
  int solid = 0;
  for (int k = 1; k < d->mz - 1 && !solid; k++)
    for (int j = 1; j < d->my - 1 && !solid; j++)
      for (int i = 1; i < d->mx - 1; i++)
        if (!(nvert[ID(d, i, j, k)] < 0.1)) { solid = 1; break; }
  if (!solid) return 1;
  int* lab = (int*)malloc((size_t)d->mx * d->my * d->mz * sizeof(int));
  int K = orc_fluid_regions(d, nvert, lab);
  if (K > 1) *label = lab;
  else free(lab);
  return K;
}

/* ------------------------------------------------------------------------- */
/* PoissonRHS2_hypre (poisson_hypre.c:342-429) + optional compatibility fix   */
/* of PoissonRHS2 (poisson.c:1879-1903): subtract the fluid-cell mean (per    */
/* connected fluid region when bodies cut the grid apart).                    */
/* ucont is AoS [mz][my][mx][3]; b is 0 on non-fluid cells.                   */
/* Returns the sum of b before the fix.                                       */
/* ------------------------------------------------------------------------- */
double orc_rhs(const orc_dims* d, const double* ucont, const double* nvert, double dt, double st, double coeff,
               int meanfix, double* b) {
  const int mx = d->mx, my = d->my, mz = d->mz;
  const size_t N = (size_t)mx * my * mz;
  memset(b, 0, sizeof(double) * N);
  double sum = 0.;
  long count = 0;
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        size_t c = ID(d, i, j, k);
        if (nvert[c] >= 0.1) continue;
        double val = 0;
        val -= ucont[3 * c + 0];
        if (i == 1 && d->ip) val += ucont[3 * ID(d, mx - 2, j, k) + 0];
        else val += ucont[3 * ID(d, i - 1, j, k) + 0];
        val -= ucont[3 * c + 1];
        if (j == 1 && d->jp) val += ucont[3 * ID(d, i, my - 2, k) + 1];
        else val += ucont[3 * ID(d, i, j - 1, k) + 1];
        val -= ucont[3 * c + 2];
        if (k == 1 && d->kp) val += ucont[3 * ID(d, i, j, mz - 2) + 2];
        else val += ucont[3 * ID(d, i, j, k - 1) + 2];
        val *= -1.0 / dt * st * coeff;
        b[c] = val;
        sum += val;
        count++;
      }
  int* label = NULL;
  const int K = (meanfix && count > 0) ? regions_of(d, nvert, &label) : 1;
  if (K > 1) {
    sub_region_means(d, nvert, label, K, b);
    free(label);
  } else if (meanfix && count > 0) {
    double v = -sum / (double)count;
    for (size_t c = 0; c < N; c++) {
      int k = (int)(c / ((size_t)mx * my)), j = (int)((c / mx) % my), i = (int)(c % mx);
      if (i == 0 || j == 0 || k == 0 || i == mx - 1 || j == my - 1 || k == mz - 1) continue;
      if (nvert[c] < 0.1) b[c] += v;
    }
  }
  return sum;
}

/* ------------------------------------------------------------------------- */
/* IB flux balance.                                                           */
/*  mode 1: VolumeFlux(user, &flux, &area, flg=0), poisson.c:2898-3240, used  */
/*          with immersed==1 (poisson_hypre.c:662).                           */
/*  mode 0: VolumeFlux(user, lUcor, ...), poisson.c:2634-2828, with           */
/*          immersed==0: the correction is applied and then every face       */
/*          between a fluid cell and a non-fluid cell is zeroed.              */
/* out[0..3] = flux, area before the correction; flux, area after.           */
/* ------------------------------------------------------------------------- */
static inline double nrm(const double* v, size_t c) { return sqrt(v[3 * c] * v[3 * c] + v[3 * c + 1] * v[3 * c + 1] + v[3 * c + 2] * v[3 * c + 2]); }

void orc_volume_flux(const orc_dims* d, int mode, double* u, const double* nvert, const double* M, double* out) {
  const int mx = d->mx, my = d->my, mz = d->mz;
  const size_t N = (size_t)mx * my * mz;
  const double *csi = M + N * M_CSI, *eta = M + N * M_ETA, *zet = M + N * M_ZET;
  const double* nv = nvert;
  double flux = 0, area = 0;
  if (mode == 1) {
    const double eps = 1.e-10, ibmval = 1.1;
    for (int k = 1; k < mz - 1; k++)
      for (int j = 1; j < my - 1; j++)
        for (int i = 1; i < mx - 1; i++) {
          size_t c = ID(d, i, j, k);
          size_t ce = ID(d, i + 1, j, k), cn = ID(d, i, j + 1, k), ct = ID(d, i, j, k + 1);
          if (nv[c] < 0.1) {
            if (nv[ce] > 0.1 && nv[ce] < ibmval && i < mx - 2) {
              if (fabs(u[3 * c]) > eps) { flux += u[3 * c]; area += nrm(csi, c); } else u[3 * c] = 0.;
            }
            if (nv[cn] > 0.1 && nv[cn] < ibmval && j < my - 2) {
              if (fabs(u[3 * c + 1]) > eps) { flux += u[3 * c + 1]; area += nrm(eta, c); } else u[3 * c + 1] = 0.;
            }
            if (nv[ct] > 0.1 && nv[ct] < ibmval && k < mz - 2) {
              if (fabs(u[3 * c + 2]) > eps) { flux += u[3 * c + 2]; area += nrm(zet, c); } else u[3 * c + 2] = 0.;
            }
          }
          if (nv[c] > 0.1 && nv[c] < ibmval) {
            if (nv[ce] < 0.1 && i < mx - 2) {
              if (fabs(u[3 * c]) > eps) { flux -= u[3 * c]; area += nrm(csi, c); } else u[3 * c] = 0.;
            }
            if (nv[cn] < 0.1 && j < my - 2) {
              if (fabs(u[3 * c + 1]) > eps) { flux -= u[3 * c + 1]; area += nrm(eta, c); } else u[3 * c + 1] = 0.;
            }
            if (nv[ct] < 0.1 && k < mz - 2) {
              if (fabs(u[3 * c + 2]) > eps) { flux -= u[3 * c + 2]; area += nrm(zet, c); } else u[3 * c + 2] = 0.;
            }
          }
        }
    out[0] = flux; out[1] = area;
    double corr = (area > 1.e-15) ? flux / area : 0.;
    for (int k = 1; k < mz - 1; k++)
      for (int j = 1; j < my - 1; j++)
        for (int i = 1; i < mx - 1; i++) {
          size_t c = ID(d, i, j, k);
          size_t ce = ID(d, i + 1, j, k), cn = ID(d, i, j + 1, k), ct = ID(d, i, j, k + 1);
          if (nv[c] < 0.1) {
            if (nv[ce] > 0.1 && nv[ce] < ibmval && i < mx - 2 && fabs(u[3 * c]) > eps) u[3 * c] -= nrm(csi, c) * corr;
            if (nv[cn] > 0.1 && nv[cn] < ibmval && j < my - 2 && fabs(u[3 * c + 1]) > eps) u[3 * c + 1] -= nrm(eta, c) * corr;
            if (nv[ct] > 0.1 && nv[ct] < ibmval && k < mz - 2 && fabs(u[3 * c + 2]) > eps) u[3 * c + 2] -= nrm(zet, c) * corr;
          }
          if (nv[c] > 0.1 && nv[c] < 1.1) {
            if (nv[ce] < 0.1 && i < mx - 2 && fabs(u[3 * c]) > eps) u[3 * c] += nrm(csi, c) * corr;
            if (nv[cn] < 0.1 && j < my - 2 && fabs(u[3 * c + 1]) > eps) u[3 * c + 1] += nrm(eta, c) * corr;
            if (nv[ct] < 0.1 && k < mz - 2 && fabs(u[3 * c + 2]) > eps) u[3 * c + 2] += nrm(zet, c) * corr;
          }
        }
    flux = 0; area = 0;
    for (int k = 1; k < mz - 1; k++)
      for (int j = 1; j < my - 1; j++)
        for (int i = 1; i < mx - 1; i++) {
          size_t c = ID(d, i, j, k);
          size_t ce = ID(d, i + 1, j, k), cn = ID(d, i, j + 1, k), ct = ID(d, i, j, k + 1);
          if (nv[c] < 0.1) {
            if (nv[ce] > 0.1 && nv[ce] < ibmval && i < mx - 2) { flux += u[3 * c]; area += nrm(csi, c); }
            if (nv[cn] > 0.1 && nv[cn] < ibmval && j < my - 2) { flux += u[3 * c + 1]; area += nrm(eta, c); }
            if (nv[ct] > 0.1 && nv[ct] < ibmval && k < mz - 2) { flux += u[3 * c + 2]; area += nrm(zet, c); }
          }
          if (nv[c] > 0.1 && nv[c] < ibmval) {
            if (nv[ce] < 0.1 && i < mx - 2) { flux -= u[3 * c]; area += nrm(csi, c); }
            if (nv[cn] < 0.1 && j < my - 2) { flux -= u[3 * c + 1]; area += nrm(eta, c); }
            if (nv[ct] < 0.1 && k < mz - 2) { flux -= u[3 * c + 2]; area += nrm(zet, c); }
          }
        }
    out[2] = flux; out[3] = area;
  } else {
    for (int pass = 0; pass < 2; pass++) {
      flux = 0; area = 0;
      for (int k = 1; k < mz - 1; k++)
        for (int j = 1; j < my - 1; j++)
          for (int i = 1; i < mx - 1; i++) {
            size_t c = ID(d, i, j, k);
            size_t ce = ID(d, i + 1, j, k), cn = ID(d, i, j + 1, k), ct = ID(d, i, j, k + 1);
            if (nv[c] < THR) {
              if (nv[ce] > THR && i <= mx - 2) { flux += u[3 * c]; area += nrm(csi, c); }
              if (nv[cn] > THR && j <= my - 2) { flux += u[3 * c + 1]; area += nrm(eta, c); }
              if (nv[ct] > THR && k <= mz - 2) { flux += u[3 * c + 2]; area += nrm(zet, c); }
            }
            if (nv[c] > THR) {
              if (nv[ce] < THR && i <= mx - 2) { flux -= u[3 * c]; area += nrm(csi, c); }
              if (nv[cn] < THR && j <= my - 2) { flux -= u[3 * c + 1]; area += nrm(eta, c); }
              if (nv[ct] < THR && k <= mz - 2) { flux -= u[3 * c + 2]; area += nrm(zet, c); }
            }
          }
      out[2 * pass] = flux; out[2 * pass + 1] = area;
      if (pass == 1) break;
      /* correction then zeroing (immersed==0), poisson.c:2726-2762 */
      for (int k = 1; k < mz - 1; k++)
        for (int j = 1; j < my - 1; j++)
          for (int i = 1; i < mx - 1; i++) {
            size_t c = ID(d, i, j, k);
            size_t ce = ID(d, i + 1, j, k), cn = ID(d, i, j + 1, k), ct = ID(d, i, j, k + 1);
            if (nv[c] < THR) {
              if (nv[ce] > THR && i <= mx - 2) u[3 * c] = 0;
              if (nv[cn] > THR && j <= my - 2) u[3 * c + 1] = 0;
              if (nv[ct] > THR && k <= mz - 2) u[3 * c + 2] = 0;
            }
            if (nv[c] > THR) {
              if (nv[ce] < THR && i <= mx - 2) u[3 * c] = 0;
              if (nv[cn] < THR && j <= my - 2) u[3 * c + 1] = 0;
              if (nv[ct] < THR && k <= mz - 2) u[3 * c + 2] = 0;
            }
          }
    }
  }
}

/* ------------------------------------------------------------------------- */
/* Solution post-processing.                                                  */
/* ------------------------------------------------------------------------- */
/* Remove_Nullspace (poisson_hypre.c:207-270): subtract the fluid-cell mean
 * (per connected fluid region when bodies cut the grid apart; then returns 0). */
double orc_remove_mean(const orc_dims* d, const double* nvert, double* phi) {
  int* label = NULL;
  const int K = regions_of(d, nvert, &label);
  if (K > 1) {
    sub_region_means(d, nvert, label, K, phi);
    free(label);
    return 0.;
  }
  double sum = 0; long cnt = 0;
  for (int k = 1; k < d->mz - 1; k++)
    for (int j = 1; j < d->my - 1; j++)
      for (int i = 1; i < d->mx - 1; i++) {
        size_t c = ID(d, i, j, k);
        if (nvert[c] < 0.1) { sum += phi[c]; cnt++; }
      }
  double v = cnt ? -sum / (double)cnt : 0.;
  for (int k = 1; k < d->mz - 1; k++)
    for (int j = 1; j < d->my - 1; j++)
      for (int i = 1; i < d->mx - 1; i++) {
        size_t c = ID(d, i, j, k);
        if (nvert[c] < 0.1) phi[c] += v;
      }
  return v;
}

/* Periodic ghost fill of a scalar (the flagged-cell loop shared by
 * Convert_Phi2_Phi, poisson.c:146-181, and UpdatePressure, :2580-2616). */
static void scalar_ghosts(const orc_dims* d, double* a) {
  for (int k = 0; k < d->mz; k++)
    for (int j = 0; j < d->my; j++)
      for (int i = 0; i < d->mx; i++) {
        int ai = wrapi(i, d->mx, d->ip), bj = wrapi(j, d->my, d->jp), ck = wrapi(k, d->mz, d->kp);
        if (ai != i || bj != j || ck != k) a[ID(d, i, j, k)] = a[ID(d, ai, bj, ck)];
      }
}

/* Convert_Phi2_Phi (poisson.c:97-185): 0 on boundary and non-fluid cells
 * ((int)nvert > 0.1), then the periodic ghost fill. */
void orc_phi_finish(const orc_dims* d, const double* nvert, double* phi) {
  for (int k = 0; k < d->mz; k++)
    for (int j = 0; j < d->my; j++)
      for (int i = 0; i < d->mx; i++) {
        size_t c = ID(d, i, j, k);
        if (i == 0 || j == 0 || k == 0 || i == d->mx - 1 || j == d->my - 1 || k == d->mz - 1 || (int)nvert[c] > THR) phi[c] = 0.;
      }
  scalar_ghosts(d, phi);
}

/* UpdatePressure (poisson.c:2522-2548 non-PRIMITIVE branch + ghost fill). */
void orc_update_pressure(const orc_dims* d, const double* nvert, const double* phi, double* p) {
  for (int k = 1; k < d->mz - 1; k++)
    for (int j = 1; j < d->my - 1; j++)
      for (int i = 1; i < d->mx - 1; i++) {
        size_t c = ID(d, i, j, k);
        if (nvert[c] < 0.1) p[c] += phi[c];
      }
  scalar_ghosts(d, p);
}

/* ------------------------------------------------------------------------- */
/* Projection (poisson.c:2202-2441), without the Contra2Cart call.            */
/* ------------------------------------------------------------------------- */
void orc_projection(const orc_dims* d, const double* M, const double* nvert, const double* phi, double dt, double st,
                    double coeff, double* u) {
  const int mx = d->mx, my = d->my, mz = d->mz, ip = d->ip, jp = d->jp, kp = d->kp;
  const size_t N = (size_t)mx * my * mz;
  const double *icsi = M + N * M_ICSI, *ieta = M + N * M_IETA, *izet = M + N * M_IZET, *iaj = M + N * M_IAJ;
  const double *jcsi = M + N * M_JCSI, *jeta = M + N * M_JETA, *jzet = M + N * M_JZET, *jaj = M + N * M_JAJ;
  const double *kcsi = M + N * M_KCSI, *keta = M + N * M_KETA, *kzet = M + N * M_KZET, *kaj = M + N * M_KAJ;
#define NV(ii, jj, kk) nvert[ID(d, ii, jj, kk)]
#define PH(ii, jj, kk) phi[ID(d, ii, jj, kk)]
  for (int k = 0; k < mz; k++)
    for (int j = 0; j < my; j++)
      for (int i = 0; i < mx; i++) {
        size_t c = ID(d, i, j, k);
        const double r1 = 1.0, r2 = 1.0, r3 = 1.0;
        double dpdc, dpde, dpdz;
        if (j > 0 && j < my - 1 && k > 0 && k < mz - 1)
          if ((i > 0 && i < mx - 2) || (ip && i == mx - 2)) {
            dpdc = PH(i + 1, j, k) - PH(i, j, k);
            if (i == mx - 2 && ip) dpdc = PH(1, j, k) - PH(i, j, k);
            dpde = 0.; dpdz = 0.;
            if ((j == my - 2 && !jp) || NV(i, j + 1, k) + NV(i + 1, j + 1, k) > THR) {
              if (NV(i, j - 1, k) + NV(i + 1, j - 1, k) < THR && (j != 1))
                dpde = (PH(i, j, k) + PH(i + 1, j, k) - PH(i, j - 1, k) - PH(i + 1, j - 1, k)) * 0.5;
            } else if ((j == 1 && !jp) || NV(i, j - 1, k) + NV(i + 1, j - 1, k) > THR) {
              if (NV(i, j + 1, k) + NV(i + 1, j + 1, k) < THR)
                dpde = (PH(i, j + 1, k) + PH(i + 1, j + 1, k) - PH(i, j, k) - PH(i + 1, j, k)) * 0.5;
            } else {
              dpde = (PH(i, j + 1, k) + PH(i + 1, j + 1, k) - PH(i, j - 1, k) - PH(i + 1, j - 1, k)) * 0.25;
            }
            if ((k == mz - 2 && !kp) || NV(i, j, k + 1) + NV(i + 1, j, k + 1) > THR) {
              if (NV(i, j, k - 1) + NV(i + 1, j, k - 1) < THR && (k != 1))
                dpdz = (PH(i, j, k) + PH(i + 1, j, k) - PH(i, j, k - 1) - PH(i + 1, j, k - 1)) * 0.5;
            } else if ((k == 1 && !kp) || NV(i, j, k - 1) + NV(i + 1, j, k - 1) > THR) {
              if (NV(i, j, k + 1) + NV(i + 1, j, k + 1) < THR)
                dpdz = (PH(i, j, k + 1) + PH(i + 1, j, k + 1) - PH(i, j, k) - PH(i + 1, j, k)) * 0.5;
            } else {
              dpdz = (PH(i, j, k + 1) + PH(i + 1, j, k + 1) - PH(i, j, k - 1) - PH(i + 1, j, k - 1)) * 0.25;
            }
            if ((NV(i, j, k) + NV(i + 1, j, k)) < THR) {
              vec3 a = ld3(icsi, c), b = ld3(ieta, c), e = ld3(izet, c);
              u[3 * c] -= (dpdc * (a.x * a.x + a.y * a.y + a.z * a.z) * iaj[c] +
                           dpde * (b.x * a.x + b.y * a.y + b.z * a.z) * iaj[c] +
                           dpdz * (e.x * a.x + e.y * a.y + e.z * a.z) * iaj[c]) * dt * st / coeff / r1;
            }
          }
        if (i > 0 && i < mx - 1 && k > 0 && k < mz - 1)
          if ((j > 0 && j < my - 2) || (jp && j == my - 2)) {
            dpdc = 0.; dpdz = 0.;
            if ((i == mx - 2 && !ip) || NV(i + 1, j, k) + NV(i + 1, j + 1, k) > THR) {
              if (NV(i - 1, j, k) + NV(i - 1, j + 1, k) < THR && (i != 1))
                dpdc = (PH(i, j, k) + PH(i, j + 1, k) - PH(i - 1, j, k) - PH(i - 1, j + 1, k)) * 0.5;
            } else if ((i == 1 && !ip) || NV(i - 1, j, k) + NV(i - 1, j + 1, k) > THR) {
              if (NV(i + 1, j, k) + NV(i + 1, j + 1, k) < THR)
                dpdc = (PH(i + 1, j, k) + PH(i + 1, j + 1, k) - PH(i, j, k) - PH(i, j + 1, k)) * 0.5;
            } else {
              dpdc = (PH(i + 1, j, k) + PH(i + 1, j + 1, k) - PH(i - 1, j, k) - PH(i - 1, j + 1, k)) * 0.25;
            }
            if (j == my - 2 && jp) dpde = PH(i, 1, k) - PH(i, j, k);
            else dpde = PH(i, j + 1, k) - PH(i, j, k);
            if ((k == mz - 2 && !kp) || NV(i, j, k + 1) + NV(i, j + 1, k + 1) > THR) {
              if (NV(i, j, k - 1) + NV(i, j + 1, k - 1) < THR && (k != 1))
                dpdz = (PH(i, j, k) + PH(i, j + 1, k) - PH(i, j, k - 1) - PH(i, j + 1, k - 1)) * 0.5;
            } else if ((k == 1 && !kp) || NV(i, j, k - 1) + NV(i, j + 1, k - 1) > THR) {
              if (NV(i, j, k + 1) + NV(i, j + 1, k + 1) < THR)
                dpdz = (PH(i, j, k + 1) + PH(i, j + 1, k + 1) - PH(i, j, k) - PH(i, j + 1, k)) * 0.5;
            } else {
              dpdz = (PH(i, j, k + 1) + PH(i, j + 1, k + 1) - PH(i, j, k - 1) - PH(i, j + 1, k - 1)) * 0.25;
            }
            if ((NV(i, j, k) + NV(i, j + 1, k)) < THR) {
              vec3 a = ld3(jcsi, c), b = ld3(jeta, c), e = ld3(jzet, c);
              u[3 * c + 1] -= (dpdc * (a.x * b.x + a.y * b.y + a.z * b.z) * jaj[c] +
                               dpde * (b.x * b.x + b.y * b.y + b.z * b.z) * jaj[c] +
                               dpdz * (e.x * b.x + e.y * b.y + e.z * b.z) * jaj[c]) * dt * st / coeff / r2;
            }
          }
        if (i > 0 && i < mx - 1 && j > 0 && j < my - 1)
          if ((k > 0 && k < mz - 2) || (kp && k == mz - 2)) {
            dpdc = 0.; dpde = 0.;
            if ((i == mx - 2 && !ip) || NV(i + 1, j, k) + NV(i + 1, j, k + 1) > THR) {
              if (NV(i - 1, j, k) + NV(i - 1, j, k + 1) < THR && (i != 1))
                dpdc = (PH(i, j, k) + PH(i, j, k + 1) - PH(i - 1, j, k) - PH(i - 1, j, k + 1)) * 0.5;
            } else if ((i == 1 && !ip) || NV(i - 1, j, k) + NV(i - 1, j, k + 1) > THR) {
              if (NV(i + 1, j, k) + NV(i + 1, j, k + 1) < THR)
                dpdc = (PH(i + 1, j, k) + PH(i + 1, j, k + 1) - PH(i, j, k) - PH(i, j, k + 1)) * 0.5;
            } else {
              dpdc = (PH(i + 1, j, k) + PH(i + 1, j, k + 1) - PH(i - 1, j, k) - PH(i - 1, j, k + 1)) * 0.25;
            }
            if ((j == my - 2 && !jp) || NV(i, j + 1, k) + NV(i, j + 1, k + 1) > THR) {
              if (NV(i, j - 1, k) + NV(i, j - 1, k + 1) < THR && (j != 1))
                dpde = (PH(i, j, k) + PH(i, j, k + 1) - PH(i, j - 1, k) - PH(i, j - 1, k + 1)) * 0.5;
            } else if ((j == 1 && !jp) || NV(i, j - 1, k) + NV(i, j - 1, k + 1) > THR) {
              if (NV(i, j + 1, k) + NV(i, j + 1, k + 1) < THR)
                dpde = (PH(i, j + 1, k) + PH(i, j + 1, k + 1) - PH(i, j, k) - PH(i, j, k + 1)) * 0.5;
            } else {
              dpde = (PH(i, j + 1, k) + PH(i, j + 1, k + 1) - PH(i, j - 1, k) - PH(i, j - 1, k + 1)) * 0.25;
            }
            if (k == mz - 2 && kp) dpdz = PH(i, j, 1) - PH(i, j, k);
            else dpdz = PH(i, j, k + 1) - PH(i, j, k);
            if ((NV(i, j, k) + NV(i, j, k + 1)) < THR) {
              vec3 a = ld3(kcsi, c), b = ld3(keta, c), e = ld3(kzet, c);
              u[3 * c + 2] -= (dpdc * (a.x * e.x + a.y * e.y + a.z * e.z) * kaj[c] +
                               dpde * (b.x * e.x + b.y * e.y + b.z * e.z) * kaj[c] +
                               dpdz * (e.x * e.x + e.y * e.y + e.z * e.z) * kaj[c]) * dt * st / coeff / r3;
            }
          }
      }
#undef PH
#undef NV
  /* periodic ghost sync of the flagged component, poisson.c:2398-2437 */
  for (int k = 0; k < mz; k++)
    for (int j = 0; j < my; j++)
      for (int i = 0; i < mx; i++) {
        int a = wrapi(i, mx, ip), b = wrapi(j, my, jp), cc = wrapi(k, mz, kp);
        size_t t = ID(d, i, j, k), s = ID(d, a, b, cc);
        if (a != i) u[3 * t] = u[3 * s];
        if (b != j) u[3 * t + 1] = u[3 * s + 1];
        if (cc != k) u[3 * t + 2] = u[3 * s + 2];
      }
}

/* Divergence (main.c:1279-1349): max |sum of face-flux differences| * aj,
 * 0 where the cell or a face neighbour has nvert, and on boundaries. */
double orc_divergence(const orc_dims* d, const double* u, const double* aj, const double* nvert, double* div) {
  double mx_ = 0.;
  const size_t N = (size_t)d->mx * d->my * d->mz;
  if (div) memset(div, 0, sizeof(double) * N);
  for (int k = 1; k < d->mz - 1; k++)
    for (int j = 1; j < d->my - 1; j++)
      for (int i = 1; i < d->mx - 1; i++) {
        size_t c = ID(d, i, j, k);
        double v = fabs((u[3 * c] - u[3 * ID(d, i - 1, j, k)] + u[3 * c + 1] - u[3 * ID(d, i, j - 1, k) + 1] +
                         u[3 * c + 2] - u[3 * ID(d, i, j, k - 1) + 2]) * aj[c]);
        if (nvert[c] + nvert[ID(d, i, j, k + 1)] + nvert[ID(d, i, j, k - 1)] + nvert[ID(d, i, j + 1, k)] +
                nvert[ID(d, i, j - 1, k)] + nvert[ID(d, i + 1, j, k)] + nvert[ID(d, i - 1, j, k)] > 0.1)
          v = 0.;
        if (div) div[c] = v;
        if (v > mx_) mx_ = v;
      }
  return mx_;
}

/* Contra2Cart (rhs.c:52-190): Cartesian velocity at fluid cell centres from
 * the averaged contravariant fluxes by Cramer's rule (rhs.c:144-183).  u must
 * carry synced periodic ghosts (as after orc_projection).  Non-fluid cells
 * keep the value already in ucat. */
void orc_contra2cart(const orc_dims* d, const double* M, const double* nvert, const double* u, double* ucat) {
  const int mx = d->mx, my = d->my, mz = d->mz;
  const size_t N = (size_t)mx * my * mz;
  const double *csi = M + N * M_CSI, *eta = M + N * M_ETA, *zet = M + N * M_ZET;
  for (int k = 1; k < mz - 1; k++)
    for (int j = 1; j < my - 1; j++)
      for (int i = 1; i < mx - 1; i++) {
        size_t c = ID(d, i, j, k);
        if (!(nvert[c] < 0.1)) continue;
        vec3 q;
        q.x = 0.5 * (u[3 * ID(d, i - 1, j, k)] + u[3 * c]);
        q.y = 0.5 * (u[3 * ID(d, i, j - 1, k) + 1] + u[3 * c + 1]);
        q.z = 0.5 * (u[3 * ID(d, i, j, k - 1) + 2] + u[3 * c + 2]);
        vec3 a = ld3(csi, c), b = ld3(eta, c), e = ld3(zet, c);
        double det = a.x * (b.y * e.z - b.z * e.y) - a.y * (b.x * e.z - b.z * e.x) + a.z * (b.x * e.y - b.y * e.x);
        double det0 = q.x * (b.y * e.z - b.z * e.y) - q.y * (a.y * e.z - a.z * e.y) + q.z * (a.y * b.z - a.z * b.y);
        double det1 = -q.x * (b.x * e.z - b.z * e.x) + q.y * (a.x * e.z - a.z * e.x) - q.z * (a.x * b.z - a.z * b.x);
        double det2 = q.x * (b.x * e.y - b.y * e.x) - q.y * (a.x * e.y - a.y * e.x) + q.z * (a.x * b.y - a.y * b.x);
        ucat[3 * c] = det0 / det;
        ucat[3 * c + 1] = det1 / det;
        ucat[3 * c + 2] = det2 / det;
      }
}

/* ========================================================================= */
/* Multigrid hierarchy and the preconditioned solve.                          */
/* ========================================================================= */

/* Coarse extents (MGDACreate, init.c:95-127): IM_c = (IM_f + 1) / 2 nodes
 * per coarsened axis, i.e. n_c = n_f / 2 cells for even n_f. */
void orc_coarse_dims(const orc_dims* f, int si, int sj, int sk, orc_dims* c) {
  *c = *f;
  if (!si) c->mx = (f->mx - 1 + 1) / 2 + 1;
  if (!sj) c->my = (f->my - 1 + 1) / 2 + 1;
  if (!sk) c->mz = (f->mz - 1 + 1) / 2 + 1;
}

/* Coarse node coordinates = every other fine node (init.c:397-449 via
 * GridRestriction, poisson.c:336-362). */
void orc_coarse_coords(const orc_dims* f, const orc_dims* c, int si, int sj, int sk, const double* cf, double* cc) {
  memset(cc, 0, sizeof(double) * 3 * (size_t)c->mx * c->my * c->mz);
  for (int k = 0; k < c->mz - 1; k++)
    for (int j = 0; j < c->my - 1; j++)
      for (int i = 0; i < c->mx - 1; i++) {
        int ih = si ? i : 2 * i, jh = sj ? j : 2 * j, kh = sk ? k : 2 * k;
        size_t t = ID(c, i, j, k), s = ID(f, ih, jh, kh);
        cc[3 * t] = cf[3 * s]; cc[3 * t + 1] = cf[3 * s + 1]; cc[3 * t + 2] = cf[3 * s + 2];
      }
}

/* MyNvertRestriction (poisson.c:2004-2106): a coarse cell is solid (>= 1) if
 * the product of its children's nvert exceeds 0.1; then fluid cells hemmed in
 * on all three axes are set to 1, updating in place in k, j, i order. */
void orc_nvert_restrict(const orc_dims* f, const orc_dims* c, int si, int sj, int sk, const double* nf, double* nc) {
  memset(nc, 0, sizeof(double) * (size_t)c->mx * c->my * c->mz);
  int ia = si ? 0 : 1, ja = sj ? 0 : 1, ka = sk ? 0 : 1;
  for (int k = 1; k < c->mz - 1; k++)
    for (int j = 1; j < c->my - 1; j++)
      for (int i = 1; i < c->mx - 1; i++) {
        int ih = si ? i : 2 * i, jh = sj ? j : 2 * j, kh = sk ? k : 2 * k;
        double p = nf[ID(f, ih, jh, kh)] * nf[ID(f, ih - ia, jh, kh)] * nf[ID(f, ih, jh - ja, kh)] *
                   nf[ID(f, ih, jh, kh - ka)] * nf[ID(f, ih - ia, jh - ja, kh)] * nf[ID(f, ih, jh - ja, kh - ka)] *
                   nf[ID(f, ih - ia, jh, kh - ka)] * nf[ID(f, ih - ia, jh - ja, kh - ka)];
        if (p > 0.1) { size_t t = ID(c, i, j, k); nc[t] = nc[t] > 1. ? nc[t] : 1.; }
      }
  for (int k = 1; k < c->mz - 1; k++)
    for (int j = 1; j < c->my - 1; j++)
      for (int i = 1; i < c->mx - 1; i++) {
        size_t t = ID(c, i, j, k);
        if (nc[t] < 0.1) {
          if (nc[ID(c, i + 1, j, k)] + nc[ID(c, i - 1, j, k)] > 1.1 && nc[ID(c, i, j + 1, k)] + nc[ID(c, i, j - 1, k)] > 1.1 &&
              nc[ID(c, i, j, k + 1)] + nc[ID(c, i, j, k - 1)] > 1.1)
            nc[t] = 1.;
        }
      }
}

/* MyRestriction (poisson.c:364-471): 8-child full weighting with the fine
 * nvert weight max(0, 1 - nvert_f); zero on coarse boundaries and solids. */
void orc_restrict(const orc_dims* f, const orc_dims* c, int si, int sj, int sk, const double* nf, const double* ncv,
                  const double* x, double* out) {
  int ia = si ? 0 : 1, ja = sj ? 0 : 1, ka = sk ? 0 : 1;
#define W(ii, jj, kk) (x[ID(f, ii, jj, kk)] * fmax(0., 1 - nf[ID(f, ii, jj, kk)]))
  for (int k = 0; k < c->mz; k++)
    for (int j = 0; j < c->my; j++)
      for (int i = 0; i < c->mx; i++) {
        size_t t = ID(c, i, j, k);
        if (k == 0 || k == c->mz - 1 || j == 0 || j == c->my - 1 || i == 0 || i == c->mx - 1) { out[t] = 0.; continue; }
        int ih = si ? i : 2 * i, jh = sj ? j : 2 * j, kh = sk ? k : 2 * k;
        out[t] = 0.125 * (W(ih, jh, kh) + W(ih - ia, jh, kh) + W(ih, jh - ja, kh) + W(ih, jh, kh - ka) +
                          W(ih - ia, jh - ja, kh) + W(ih, jh - ja, kh - ka) + W(ih - ia, jh, kh - ka) +
                          W(ih - ia, jh - ja, kh - ka));
        if (ncv[t] > 0.1) out[t] = 0.;
      }
#undef W
}

/* MyInterpolation (poisson.c:526-669) with the GridInterpolation offsets
 * (poisson.c:473-506): trilinear (27,9,9,3,9,3,3,1)/64 weights, offsets
 * dropped at the first/last interior index and next to solid coarse cells;
 * fine boundary and solid cells are zero. */
void orc_prolong(const orc_dims* f, const orc_dims* c, int si, int sj, int sk, const double* nf, const double* ncv,
                 const double* x, double* out) {
  const int mx = f->mx, my = f->my, mz = f->mz;
  for (int k = 0; k < mz; k++)
    for (int j = 0; j < my; j++)
      for (int i = 0; i < mx; i++) {
        size_t t = ID(f, i, j, k);
        if (i == 0 || i == mx - 1 || j == 0 || j == my - 1 || k == 0 || k == mz - 1 || nf[t] > 0.1) { out[t] = 0.; continue; }
        int ic, jc, kc, ia, ja, ka;
        if (si) { ic = i; ia = 0; } else { ic = (i + 1) / 2; ia = (i - 2 * ic) == 0 ? 1 : -1; if (i == 1 || i == mx - 2) ia = 0; }
        if (sj) { jc = j; ja = 0; } else { jc = (j + 1) / 2; ja = (j - 2 * jc) == 0 ? 1 : -1; if (j == 1 || j == my - 2) ja = 0; }
        if (sk) { kc = k; ka = 0; } else { kc = (k + 1) / 2; ka = (k - 2 * kc) == 0 ? 1 : -1; if (k == 1 || k == mz - 2) ka = 0; }
        if (ka == -1 && ncv[ID(c, ic, jc, kc - 1)] > 0.1) ka = 0;
        else if (ka == 1 && ncv[ID(c, ic, jc, kc + 1)] > 0.1) ka = 0;
        if (ja == -1 && ncv[ID(c, ic, jc - 1, kc)] > 0.1) ja = 0;
        else if (ja == 1 && ncv[ID(c, ic, jc + 1, kc)] > 0.1) ja = 0;
        if (ia == -1 && ncv[ID(c, ic - 1, jc, kc)] > 0.1) ia = 0;
        else if (ia == 1 && ncv[ID(c, ic + 1, jc, kc)] > 0.1) ia = 0;
#define X(ii, jj, kk) x[ID(c, ii, jj, kk)]
        out[t] = (X(ic, jc, kc) * 9 + X(ic, jc + ja, kc) * 3 + X(ic + ia, jc, kc) * 3 + X(ic + ia, jc + ja, kc)) * 3. / 64. +
                 (X(ic, jc, kc + ka) * 9 + X(ic, jc + ja, kc + ka) * 3 + X(ic + ia, jc, kc + ka) * 3 +
                  X(ic + ia, jc + ja, kc + ka)) / 64.;
#undef X
      }
}

typedef struct {
  orc_dims d;
  double *coor, *nvert, *M, *g, *coef;
  double *mcoef;     /* multigrid operator: rows scaled by aj (poisson.c:1560) */
  double *lc, *linv; /* y-line LU factors of mcoef: c'_j and 1/m_j per cell */
  double *x, *b, *r, *t;
} orc_level;

typedef struct {
  int L, si, sj, sk;
  orc_level lev[16]; /* lev[L-1] is the finest, lev[0] the coarsest */
  double omega, omega_c;
  int nu1, nu2, ncoarse;
} orc_mg;

/* Line factors of the y-line (tridiagonal SP/CP/NP) solve.  Non-fluid cells
 * are identity rows.  Couplings across a j-periodic seam stay off-line. */
static void line_factors(orc_level* L) {
  const orc_dims* d = &L->d;
  const size_t N = (size_t)d->mx * d->my * d->mz;
  for (int k = 1; k < d->mz - 1; k++)
    for (int i = 1; i < d->mx - 1; i++) {
      double cprev = 0.;
      for (int j = 1; j < d->my - 1; j++) {
        size_t c = ID(d, i, j, k);
        double a = (j > 1) ? L->mcoef[SP * N + c] : 0.;
        double b = L->mcoef[CP * N + c];
        double cc = (j < d->my - 2) ? L->mcoef[NP * N + c] : 0.;
        if (b == 0.) { a = 0.; b = 1.; cc = 0.; }
        double m = b - a * cprev;
        L->linv[c] = 1. / m;
        L->lc[c] = cc / m;
        cprev = L->lc[c];
      }
    }
}

static void level_setup(orc_level* L) {
  const size_t N = (size_t)L->d.mx * L->d.my * L->d.mz;
  L->M = (double*)calloc(N * M_TOTAL, sizeof(double));
  L->g = (double*)calloc(N * 9, sizeof(double));
  L->coef = (double*)calloc(N * NSTENCIL, sizeof(double));
  L->mcoef = (double*)calloc(N * NSTENCIL, sizeof(double));
  L->lc = (double*)calloc(N, sizeof(double));
  L->linv = (double*)calloc(N, sizeof(double));
  L->x = (double*)calloc(N, sizeof(double));
  L->b = (double*)calloc(N, sizeof(double));
  L->r = (double*)calloc(N, sizeof(double));
  L->t = (double*)calloc(N, sizeof(double));
  orc_form_metrics(&L->d, L->coor, L->M);
  orc_gtensor(&L->d, L->M, L->g);
  orc_lhs(&L->d, L->g, L->nvert, L->coef);
  orc_lhs_scaled(&L->d, L->g, L->nvert, L->M + N * M_AJ, L->mcoef);
  line_factors(L);
}

orc_mg* orc_mg_create(const orc_dims* fine, const double* coor, const double* nvert, int levels, int si, int sj, int sk) {
  if (levels < 1 || levels > 16) return NULL;
  orc_mg* mg = (orc_mg*)calloc(1, sizeof(orc_mg));
  mg->L = levels; mg->si = si; mg->sj = sj; mg->sk = sk;
  mg->omega = 0.8; mg->omega_c = 0.8; mg->nu1 = 2; mg->nu2 = 2; mg->ncoarse = 32;
  orc_level* F = &mg->lev[levels - 1];
  F->d = *fine;
  size_t N = (size_t)fine->mx * fine->my * fine->mz;
  F->coor = (double*)malloc(sizeof(double) * 3 * N); memcpy(F->coor, coor, sizeof(double) * 3 * N);
  F->nvert = (double*)malloc(sizeof(double) * N); memcpy(F->nvert, nvert, sizeof(double) * N);
  for (int l = levels - 2; l >= 0; l--) {
    orc_level *C = &mg->lev[l], *H = &mg->lev[l + 1];
    orc_coarse_dims(&H->d, si, sj, sk, &C->d);
    size_t Nc = (size_t)C->d.mx * C->d.my * C->d.mz;
    C->coor = (double*)calloc(3 * Nc, sizeof(double));
    C->nvert = (double*)calloc(Nc, sizeof(double));
    orc_coarse_coords(&H->d, &C->d, si, sj, sk, H->coor, C->coor);
    orc_nvert_restrict(&H->d, &C->d, si, sj, sk, H->nvert, C->nvert);
  }
  for (int l = 0; l < levels; l++) level_setup(&mg->lev[l]);
  return mg;
}

void orc_mg_set_params(orc_mg* mg, int nu1, int nu2, int ncoarse, double omega, double omega_c) {
  mg->nu1 = nu1; mg->nu2 = nu2; mg->ncoarse = ncoarse; mg->omega = omega; mg->omega_c = omega_c;
}

void orc_mg_destroy(orc_mg* mg) {
  if (!mg) return;
  for (int l = 0; l < mg->L; l++) {
    orc_level* L = &mg->lev[l];
    free(L->coor); free(L->nvert); free(L->M); free(L->g); free(L->coef); free(L->mcoef); free(L->lc); free(L->linv);
    free(L->x); free(L->b); free(L->r); free(L->t);
  }
  free(mg);
}

/* Accessors for the tests: dims and arrays of level l (0 = coarsest). */
void orc_mg_level_dims(const orc_mg* mg, int l, orc_dims* d) { *d = mg->lev[l].d; }
const double* orc_mg_level_array(const orc_mg* mg, int l, int which) {
  const orc_level* L = &mg->lev[l];
  switch (which) {
    case 0: return L->coor; case 1: return L->nvert; case 2: return L->M; case 3: return L->g;
    case 4: return L->coef; case 5: return L->lc; case 6: return L->linv; case 7: return L->mcoef;
  }
  return NULL;
}

/* r = b - A x on level L (unscaled operator when scaled == 0). */
static void residual_op(const orc_level* L, int scaled, const double* x, const double* b, double* r) {
  orc_matvec(&L->d, scaled ? L->mcoef : L->coef, x, r);
  const size_t N = (size_t)L->d.mx * L->d.my * L->d.mz;
  for (size_t c = 0; c < N; c++) r[c] = b[c] - r[c];
}
static void residual(const orc_level* L, const double* x, const double* b, double* r) { residual_op(L, 0, x, b, r); }

/* One damped y-line Jacobi sweep: x <- x + omega * T^{-1} (b - A x), where T
 * is the tridiagonal j-coupling of each (i,k) column. */
void orc_line_sweep(const orc_dims* d, const double* coef, const double* lc, const double* linv, const double* b,
                    double* x, double* r, double omega) {
  const size_t N = (size_t)d->mx * d->my * d->mz;
  orc_matvec(d, coef, x, r);
#pragma omp parallel for schedule(static)
  for (int k = 1; k < d->mz - 1; k++)
    for (int i = 1; i < d->mx - 1; i++) {
      double dprev = 0.;
      for (int j = 1; j < d->my - 1; j++) {
        size_t c = ID(d, i, j, k);
        double res = (coef[CP * N + c] == 0.) ? 0. : b[c] - r[c];
        double a = (j > 1 && coef[CP * N + c] != 0.) ? coef[SP * N + c] : 0.;
        double dp = (res - a * dprev) * linv[c];
        r[c] = dp;
        dprev = dp;
      }
      double xn = 0.;
      for (int j = d->my - 2; j >= 1; j--) {
        size_t c = ID(d, i, j, k);
        double v = r[c] - lc[c] * xn;
        xn = v;
        x[c] += omega * v;
      }
    }
}

static void vcycle(orc_mg* mg, int l, double* x, const double* b) {
  orc_level* L = &mg->lev[l];
  const size_t N = (size_t)L->d.mx * L->d.my * L->d.mz;
  if (l == 0) {
    for (int s = 0; s < mg->ncoarse; s++) orc_line_sweep(&L->d, L->mcoef, L->lc, L->linv, b, x, L->r, mg->omega_c);
    return;
  }
  for (int s = 0; s < mg->nu1; s++) orc_line_sweep(&L->d, L->mcoef, L->lc, L->linv, b, x, L->r, mg->omega);
  residual_op(L, 1, x, b, L->r);
  orc_level* C = &mg->lev[l - 1];
  const size_t Nc = (size_t)C->d.mx * C->d.my * C->d.mz;
  orc_restrict(&L->d, &C->d, mg->si, mg->sj, mg->sk, L->nvert, C->nvert, L->r, C->b);
  memset(C->x, 0, sizeof(double) * Nc);
  vcycle(mg, l - 1, C->x, C->b);
  orc_prolong(&L->d, &C->d, mg->si, mg->sj, mg->sk, L->nvert, C->nvert, C->x, L->t);
  for (size_t c = 0; c < N; c++) x[c] += L->t[c];
  for (int s = 0; s < mg->nu2; s++) orc_line_sweep(&L->d, L->mcoef, L->lc, L->linv, b, x, L->r, mg->omega);
}

/* z = M^{-1} v: one V-cycle of the aj-scaled hierarchy from a zero initial
 * guess, applied to aj * v, so that M approximates A^{-1} for the unscaled
 * operator A (the same solution, row scaling only). */
void orc_mg_apply(orc_mg* mg, const double* v, double* z) {
  orc_level* F = &mg->lev[mg->L - 1];
  const size_t N = (size_t)F->d.mx * F->d.my * F->d.mz;
  const double* aj = F->M + N * M_AJ;
  for (size_t c = 0; c < N; c++) F->b[c] = v[c] * aj[c];
  memset(z, 0, sizeof(double) * N);
  vcycle(mg, mg->L - 1, z, F->b);
}

void orc_mg_matvec(const orc_mg* mg, int l, const double* x, double* y) { orc_matvec(&mg->lev[l].d, mg->lev[l].mcoef, x, y); }
void orc_mg_restrict(const orc_mg* mg, int l, const double* x, double* y) {
  orc_restrict(&mg->lev[l].d, &mg->lev[l - 1].d, mg->si, mg->sj, mg->sk, mg->lev[l].nvert, mg->lev[l - 1].nvert, x, y);
}
void orc_mg_prolong(const orc_mg* mg, int l, const double* x, double* y) {
  orc_prolong(&mg->lev[l].d, &mg->lev[l - 1].d, mg->si, mg->sj, mg->sk, mg->lev[l].nvert, mg->lev[l - 1].nvert, x, y);
}
void orc_mg_smooth(const orc_mg* mg, int l, const double* b, double* x, int nsweep, double omega) {
  const orc_level* L = &mg->lev[l];
  for (int s = 0; s < nsweep; s++) orc_line_sweep(&L->d, L->mcoef, L->lc, L->linv, b, x, L->r, omega);
}

static double dot(const double* a, const double* b, size_t n) {
  double s = 0.;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (size_t c = 0; c < n; c++) s += a[c] * b[c];
  return s;
}

/* Right-preconditioned flexible GMRES(m) with CGS2 orthogonalisation, the
 * Krylov method of the reference's solve (HYPRE GMRES, poisson_hypre.c:88-95;
 * PETSc KSP gmres with PCMG, mhv_poisson.c:2166-2308) made flexible so a
 * V-cycle can precondition it.  Stops when ||r|| <= rtol * ||b|| (the
 * residual estimate of the least-squares problem) or after maxit
 * preconditioner applications.  x holds the initial guess on entry.
 * info[0] = iterations, info[1] = final true ||b - A x|| / ||b||,
 * info[2] = ||b||. */
/* orth selects the Gram-Schmidt variant of the Arnoldi step:
 *   1  classical, one pass (the reference's KSP is created with PETSc's
 *      defaults, mhv_poisson.c:2166-2178, and GMRES there orthogonalises by
 *      classical Gram-Schmidt without refinement);
 *   2  classical with one re-orthogonalisation pass (CGS2). */
int orc_fgmres_ex(orc_mg* mg, const double* b, double* x, double rtol, int maxit, int restart, int orth, double* info);
int orc_fgmres(orc_mg* mg, const double* b, double* x, double rtol, int maxit, int restart, double* info) {
  return orc_fgmres_ex(mg, b, x, rtol, maxit, restart, 2, info);
}
int orc_fgmres_ex(orc_mg* mg, const double* b, double* x, double rtol, int maxit, int restart, int orth, double* info) {
  orc_level* F = &mg->lev[mg->L - 1];
  const size_t N = (size_t)F->d.mx * F->d.my * F->d.mz;
  const int m = restart;
  double* V = (double*)calloc((size_t)(m + 1) * N, sizeof(double));
  double* Z = (double*)calloc((size_t)m * N, sizeof(double));
  double* w = (double*)calloc(N, sizeof(double));
  double* H = (double*)calloc((size_t)(m + 1) * m, sizeof(double));
  double *cs = (double*)calloc(m, sizeof(double)), *sn = (double*)calloc(m, sizeof(double));
  double *gv = (double*)calloc(m + 1, sizeof(double)), *y = (double*)calloc(m, sizeof(double));
  double* h = (double*)calloc(m + 1, sizeof(double));
  double bnorm = sqrt(dot(b, b, N));
  int it = 0, conv = 0;
  if (bnorm == 0.) { memset(x, 0, sizeof(double) * N); conv = 1; }
  while (!conv && it < maxit) {
    residual(F, x, b, V);
    double beta = sqrt(dot(V, V, N));
    if (beta <= rtol * bnorm) { conv = 1; break; }
    for (size_t c = 0; c < N; c++) V[c] /= beta;
    memset(gv, 0, sizeof(double) * (m + 1));
    gv[0] = beta;
    int j;
    for (j = 0; j < m && it < maxit; j++, it++) {
      double* vj = V + (size_t)j * N;
      double* zj = Z + (size_t)j * N;
      orc_mg_apply(mg, vj, zj);
      orc_matvec(&F->d, F->coef, zj, w);
      for (int pass = 0; pass < (orth == 2 ? 2 : 1); pass++) {
        for (int q = 0; q <= j; q++) h[q] = dot(V + (size_t)q * N, w, N);
        for (int q = 0; q <= j; q++) {
          const double* vq = V + (size_t)q * N;
          double hq = h[q];
#pragma omp parallel for schedule(static)
          for (size_t c = 0; c < N; c++) w[c] -= hq * vq[c];
          H[q * m + j] += hq;
        }
      }
      double hn = sqrt(dot(w, w, N));
      H[(j + 1) * m + j] = hn;
      if (hn > 0.) {
        double* vn = V + (size_t)(j + 1) * N;
        for (size_t c = 0; c < N; c++) vn[c] = w[c] / hn;
      }
      for (int q = 0; q < j; q++) {
        double a = H[q * m + j], bb = H[(q + 1) * m + j];
        H[q * m + j] = cs[q] * a + sn[q] * bb;
        H[(q + 1) * m + j] = -sn[q] * a + cs[q] * bb;
      }
      double a = H[j * m + j], bb = H[(j + 1) * m + j];
      double den = sqrt(a * a + bb * bb);
      cs[j] = den > 0. ? a / den : 1.;
      sn[j] = den > 0. ? bb / den : 0.;
      H[j * m + j] = den;
      H[(j + 1) * m + j] = 0.;
      gv[j + 1] = -sn[j] * gv[j];
      gv[j] = cs[j] * gv[j];
      if (fabs(gv[j + 1]) <= rtol * bnorm || hn == 0.) { j++; it++; conv = 1; break; }
    }
    for (int q = j - 1; q >= 0; q--) {
      double s = gv[q];
      for (int p = q + 1; p < j; p++) s -= H[q * m + p] * y[p];
      y[q] = s / H[q * m + q];
    }
    for (int q = 0; q < j; q++) {
      const double* zq = Z + (size_t)q * N;
      double yq = y[q];
      for (size_t c = 0; c < N; c++) x[c] += yq * zq[c];
    }
    memset(H, 0, sizeof(double) * (size_t)(m + 1) * m);
  }
  residual(F, x, b, w);
  info[0] = it;
  info[1] = bnorm > 0. ? sqrt(dot(w, w, N)) / bnorm : 0.;
  info[2] = bnorm;
  free(V); free(Z); free(w); free(H); free(cs); free(sn); free(gv); free(y); free(h);
  return conv ? 0 : 1;
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
