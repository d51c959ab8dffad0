// ref_harness.cpp -- runs the reference's own pressure-path functions
// (compiled unmodified from the reference's sources by oracle/ref.mk, against
// the single-rank stand-ins of oracle/ref_stub/) on one grid, for checking the
// oracle restatement (oracle/vfs_oracle.c) entry by entry.
//
// TEST INFRASTRUCTURE ONLY: loaded by tests/test_ref_oracle.py and by
// tests/golden/make_golden.py; nothing of the product links it.
//
// One handle holds one UserCtx built the way MG_Initial (init.c:603-900)
// leaves a level: a DMDA over the ghosted extents with the node coordinates,
// nvert in Nvert/lNvert, and every vector the called functions read or write.
// The reference keeps its run options in globals (main.c:3-200); the handle
// sets those the path reads: periodicity (i/j/k_periodic, periodic), immersed,
// poisson = 1 and levelset = 0 (their defaults), ti = tistart = 0, and the
// directory its Divergence appends its log line to (path).
#include <string>
#include <vector>

#include "variables.h"

// Reference functions the header leaves undeclared.
PetscErrorCode PoissonLHSNew(UserCtx* user, HYPRE_IJMatrix& Ap);
void PoissonRHS2_hypre(UserCtx* user, HYPRE_IJVector& B, PetscInt i_lower);
void Remove_Nullspace(UserCtx* user, HYPRE_IJVector& B, int i_lower);
PetscErrorCode PoissonRHS2(UserCtx* user, Vec B);
PetscErrorCode MyRestriction(Mat A, Vec X, Vec F);
PetscErrorCode MyInterpolation(Mat A, Vec X, Vec F);

extern "C" {
HYPRE_IJMatrix vfs_ref_ij_new();
void vfs_ref_ij_free(HYPRE_IJMatrix m);
long long vfs_ref_ij_count(HYPRE_IJMatrix m);
void vfs_ref_ij_get(HYPRE_IJMatrix m, int* rows, int* cols, double* vals);
}

namespace {

struct RefGrid {
  UserCtx* u = nullptr;
  std::string dir;
  int immersed = 0;
  int ip = 0, jp = 0, kp = 0;
  PetscBool semi[3] = {PETSC_FALSE, PETSC_FALSE, PETSC_FALSE};  // isc, jsc, ksc of this level
};

void scalar(UserCtx* u, Vec* v) { DMCreateGlobalVector(u->da, v); }
void vector3(UserCtx* u, Vec* v) { DMCreateGlobalVector(u->fda, v); }

void set_globals(const RefGrid* g) {
  i_periodic = g->ip;
  j_periodic = g->jp;
  k_periodic = g->kp;
  ii_periodic = jj_periodic = kk_periodic = 0;
  periodic = (g->ip || g->jp || g->kp) ? 1 : 0;
  immersed = g->immersed;
  poisson = 1;
  levelset = 0;
  ti = 0;
  tistart = 0;
  snprintf(path, sizeof(path), "%s", g->dir.c_str());
}

// Scalar / Cmpnts vector contents in and out (the reference's [k][j][i]
// layout, Cmpnts as 3 consecutive doubles).
void put(Vec v, const double* src) { memcpy(vfs_ref_vec_data(v), src, sizeof(double) * vfs_ref_vec_size(v)); }
void get(Vec v, double* dst) { memcpy(dst, vfs_ref_vec_data(v), sizeof(double) * vfs_ref_vec_size(v)); }

}  // namespace

extern "C" {

// A level of mx x my x mz ghosted cells (node coordinates [mz][my][mx][3],
// nvert [mz][my][mx]); dir: an existing directory for Divergence's log.
void* vfs_ref_create(int mx, int my, int mz, int ip, int jp, int kp, const double* coor, const double* nvert,
                     int immersed_flag, double dt, double st, const char* dir) {
  RefGrid* g = new RefGrid;
  g->dir = dir ? dir : ".";
  g->immersed = immersed_flag;
  g->ip = ip;
  g->jp = jp;
  g->kp = kp;
  UserCtx* u = new UserCtx();
  g->u = u;
  set_globals(g);
  u->da = vfs_ref_dm_create(mx, my, mz, 1);
  vfs_ref_dm_set_coordinates(u->da, coor);
  DMDAGetCoordinateDA(u->da, &u->fda);
  DMDAGetLocalInfo(u->da, &u->info);
  u->dt = dt;
  u->st = st;
  u->ren = 3000.;
  for (int f = 0; f < 6; f++) u->bctype[f] = 1;
  Vec* sc[] = {&u->Nvert, &u->lNvert, &u->lNvert_o, &u->Aj, &u->lAj, &u->IAj, &u->lIAj, &u->JAj, &u->lJAj,
               &u->KAj, &u->lKAj, &u->P, &u->lP, &u->Phi, &u->lPhi, &u->lUstar};
  for (Vec* v : sc) scalar(u, v);
  Vec* ve[] = {&u->Cent, &u->lCent, &u->Csi, &u->lCsi, &u->Eta, &u->lEta, &u->Zet, &u->lZet,
               &u->ICsi, &u->lICsi, &u->IEta, &u->lIEta, &u->IZet, &u->lIZet,
               &u->JCsi, &u->lJCsi, &u->JEta, &u->lJEta, &u->JZet, &u->lJZet,
               &u->KCsi, &u->lKCsi, &u->KEta, &u->lKEta, &u->KZet, &u->lKZet,
               &u->Ucont, &u->lUcont, &u->Ucat, &u->lUcat, &u->lUcat_old, &u->GridSpace, &u->lGridSpace};
  for (Vec* v : ve) vector3(u, v);
  put(u->Nvert, nvert);
  put(u->lNvert, nvert);
  put(u->lNvert_o, nvert);
  return g;
}

void vfs_ref_destroy(void* h) {
  RefGrid* g = (RefGrid*)h;
  if (!g) return;
  // vectors and DMs are left to the process (test helper); the handle goes
  delete g;
}

// FormMetrics (metrics.c:4-1290).  Out: the 43-array pack of the oracle
// (csi eta zet aj icsi ieta izet iaj jcsi jeta jzet jaj kcsi keta kzet kaj
// cent; vectors AoS), read from the local (ghosted) vectors the operator
// and the projection use.
void vfs_ref_form_metrics(void* h, double* M) {
  RefGrid* g = (RefGrid*)h;
  set_globals(g);
  UserCtx* u = g->u;
  FormMetrics(u);
  const size_t N = (size_t)u->info.mx * u->info.my * u->info.mz;
  Vec order[] = {u->lCsi, u->lEta, u->lZet, u->lAj, u->lICsi, u->lIEta, u->lIZet, u->lIAj,
                 u->lJCsi, u->lJEta, u->lJZet, u->lJAj, u->lKCsi, u->lKEta, u->lKZet, u->lKAj, u->lCent};
  size_t off = 0;
  for (Vec v : order) {
    get(v, M + off);
    off += (size_t)vfs_ref_vec_size(v);
  }
  (void)N;
}

// setup_lidx2 + PoissonLHSNew (poisson.c:187-334, 976-1691): the entries the
// reference hands to HYPRE_IJMatrixSetValues, in (row, col) order, rows and
// columns in its compact fluid numbering.  gid (nullable): that numbering per
// cell (-1 where none).  Returns the entry count; the arrays must hold cap.
long long vfs_ref_lhs(void* h, int* rows, int* cols, double* vals, long long cap, double* gid) {
  RefGrid* g = (RefGrid*)h;
  set_globals(g);
  UserCtx* u = g->u;
  setup_lidx2(u);
  HYPRE_IJMatrix A = vfs_ref_ij_new();
  PoissonLHSNew(u, A);
  const long long n = vfs_ref_ij_count(A);
  if (n <= cap) vfs_ref_ij_get(A, rows, cols, vals);
  if (gid) get(u->Gid, gid);
  vfs_ref_ij_free(A);
  return n;
}

// VolumeFlux (the IB flux balance, poisson.c:2898-3240 with flg 0, or the
// immersed == 0 form, poisson.c:2634-2828) on ucont [mz][my][mx][3], in place;
// out[0..1] = the IB flux and area it reports.
void vfs_ref_volume_flux(void* h, double* ucont, double* out) {
  RefGrid* g = (RefGrid*)h;
  set_globals(g);
  UserCtx* u = g->u;
  put(u->Ucont, ucont);
  put(u->lUcont, ucont);
  PetscReal flux = 0., area = 0.;
  if (g->immersed == 1) VolumeFlux(u, &flux, &area, 0);
  else VolumeFlux(u, u->Ucont, &flux, &area);
  DMGlobalToLocalBegin(u->fda, u->Ucont, INSERT_VALUES, u->lUcont);
  DMGlobalToLocalEnd(u->fda, u->Ucont, INSERT_VALUES, u->lUcont);
  get(u->lUcont, ucont);
  out[0] = flux;
  out[1] = area;
}

// PoissonRHS2_hypre (poisson_hypre.c:272-477) of ucont: b by compact fluid
// index (setup_lidx2 must have run: vfs_ref_lhs).  Returns the fluid count.
int vfs_ref_rhs(void* h, const double* ucont, double* b, int cap) {
  RefGrid* g = (RefGrid*)h;
  set_globals(g);
  UserCtx* u = g->u;
  put(u->Ucont, ucont);
  put(u->lUcont, ucont);
  HYPRE_IJVector B = (HYPRE_IJVector)vfs_ref_ij_new();
  PoissonRHS2_hypre(u, B, u->p_global_begin);
  const int n = u->reduced_p_size;
  std::vector<int> idx(n > 0 ? n : 1);
  for (int q = 0; q < n; q++) idx[q] = q;
  if (n <= cap) HYPRE_IJVectorGetValues(B, n, idx.data(), b);
  vfs_ref_ij_free((HYPRE_IJMatrix)B);
  return n;
}

// Remove_Nullspace (poisson_hypre.c:207-270) of the compact solution phi2
// (in place, by compact fluid index).
void vfs_ref_remove_nullspace(void* h, double* phi2) {
  RefGrid* g = (RefGrid*)h;
  set_globals(g);
  UserCtx* u = g->u;
  const int n = u->reduced_p_size;
  HYPRE_IJVector B = (HYPRE_IJVector)vfs_ref_ij_new();
  std::vector<int> idx(n > 0 ? n : 1);
  for (int q = 0; q < n; q++) idx[q] = q;
  HYPRE_IJVectorSetValues(B, n, idx.data(), phi2);
  Remove_Nullspace(u, B, u->p_global_begin);
  HYPRE_IJVectorGetValues(B, n, idx.data(), phi2);
  vfs_ref_ij_free((HYPRE_IJMatrix)B);
}

// Convert_Phi2_Phi (poisson.c:97-185): the compact solution phi2 (by fluid
// index) into the structured phi with its periodic ghosts (out [mz][my][mx]).
void vfs_ref_phi2_to_phi(void* h, const double* phi2, double* phi) {
  RefGrid* g = (RefGrid*)h;
  set_globals(g);
  UserCtx* u = g->u;
  memcpy(vfs_ref_vec_data(u->Phi2), phi2, sizeof(double) * vfs_ref_vec_size(u->Phi2));
  Convert_Phi2_Phi(u);
  get(u->Phi, phi);  // its periodic ghosts are filled in the global vector
}

// UpdatePressure + Projection (poisson.c:2473-2632, 2122-2470, the latter
// ending in Contra2Cart, rhs.c:50) for the structured phi: p and ucont in
// place, ucat out ([mz][my][mx][3]).
void vfs_ref_update_and_project(void* h, const double* phi, double* p, double* ucont, double* ucat) {
  RefGrid* g = (RefGrid*)h;
  set_globals(g);
  UserCtx* u = g->u;
  put(u->Phi, phi);
  put(u->lPhi, phi);
  put(u->P, p);
  put(u->lP, p);
  put(u->Ucont, ucont);
  put(u->lUcont, ucont);
  UpdatePressure(u);
  Projection(u);
  get(u->P, p);
  // the global fluxes: the state the reference keeps and writes out (its
  // Contra2Cart also copies whole ghost cells into the local vector)
  get(u->Ucont, ucont);
  if (ucat) get(u->lUcat, ucat);
}

// PoissonRHS2 (poisson.c:1789-1915): the right-hand side with the
// compatibility fix (minus the fluid mean), b by compact fluid index.
int vfs_ref_rhs2(void* h, const double* ucont, double* b, int cap) {
  RefGrid* g = (RefGrid*)h;
  set_globals(g);
  UserCtx* u = g->u;
  put(u->Ucont, ucont);
  put(u->lUcont, ucont);
  const int n = u->reduced_p_size;
  Vec B;
  VecCreateMPI(PETSC_COMM_WORLD, n, n, &B);
  PoissonRHS2(u, B);
  if (n <= cap) memcpy(b, vfs_ref_vec_data(B), sizeof(double) * n);
  VecDestroy(&B);
  return n;
}

// Two multigrid levels, as MG_Initial links them (init.c:603-617): the
// coarse level's user_f / da_f point at the fine one, the fine level's
// user_c / da_c at the coarse one, and both carry the semi-coarsening flags
// (isc, jsc, ksc, -mg_*_semi).  thislevel: the coarse level's index (the
// finest level is the highest).
void vfs_ref_link(void* fine, void* coarse, int si, int sj, int sk, int coarse_level) {
  RefGrid *f = (RefGrid*)fine, *c = (RefGrid*)coarse;
  for (RefGrid* g : {f, c}) {
    g->semi[0] = si ? PETSC_TRUE : PETSC_FALSE;
    g->semi[1] = sj ? PETSC_TRUE : PETSC_FALSE;
    g->semi[2] = sk ? PETSC_TRUE : PETSC_FALSE;
    g->u->isc = &g->semi[0];
    g->u->jsc = &g->semi[1];
    g->u->ksc = &g->semi[2];
  }
  c->u->user_f = f->u;
  c->u->da_f = &f->u->da;
  f->u->user_c = c->u;
  f->u->da_c = &c->u->da;
  f->u->lNvert_c = &c->u->lNvert;
  c->u->thislevel = coarse_level;
  f->u->thislevel = coarse_level + 1;
}

// MyNvertRestriction (poisson.c:2004-2106) of the linked fine level's nvert
// onto the coarse level; out: the coarse level's nvert.
void vfs_ref_nvert_restrict(void* fine, void* coarse, double* nvc) {
  RefGrid *f = (RefGrid*)fine, *c = (RefGrid*)coarse;
  set_globals(c);
  MyNvertRestriction(f->u, c->u);
  get(c->u->lNvert, nvc);
}

// MyRestriction (poisson.c:364-471): the fine vector xf restricted to the
// linked coarse level (its shell matrix's context is the coarse UserCtx).
void vfs_ref_restrict(void* coarse, const double* xf, double* fc) {
  RefGrid* c = (RefGrid*)coarse;
  set_globals(c);
  UserCtx* f = c->u->user_f;
  Vec X, F;
  DMCreateGlobalVector(f->da, &X);
  DMCreateGlobalVector(c->u->da, &F);
  put(X, xf);
  Mat A = vfs_ref_shell(c->u);
  MyRestriction(A, X, F);
  get(F, fc);
  VecDestroy(&X);
  VecDestroy(&F);
  vfs_ref_shell_free(A);
}

// MyInterpolation (poisson.c:526-669): the coarse vector xc interpolated to
// the linked fine level (context: the fine UserCtx).
void vfs_ref_interpolate(void* fine, const double* xc, double* ff) {
  RefGrid* f = (RefGrid*)fine;
  set_globals(f);
  UserCtx* c = f->u->user_c;
  Vec X, F;
  DMCreateGlobalVector(c->da, &X);
  DMCreateGlobalVector(f->u->da, &F);
  put(X, xc);
  Mat A = vfs_ref_shell(f->u);
  MyInterpolation(A, X, F);
  get(F, ff);
  VecDestroy(&X);
  VecDestroy(&F);
  vfs_ref_shell_free(A);
}

// Divergence (main.c:1244-1390) of ucont: the maximum it finds (it prints it
// and appends it to <dir>/Converge_dU).
double vfs_ref_divergence(void* h, const double* ucont) {
  RefGrid* g = (RefGrid*)h;
  set_globals(g);
  UserCtx* u = g->u;
  put(u->Ucont, ucont);
  put(u->lUcont, ucont);
  Divergence(u);
  return vfs_ref_last_max;
}

}  // extern "C"
