// Runtime of the single-rank PETSc / HYPRE / MPI stand-ins declared in
// vfs_ref_stub.h (test infrastructure: it lets the reference's own
// pressure-path sources run as a checker of the oracle restatement).
#include "vfs_ref_stub.h"

#include <execinfo.h>
#include <sys/time.h>

#include <map>
#include <vector>

struct vfs_dm {
  int mx, my, mz, dof;
  vfs_dm* cda;      // the coordinate DM (dof 3), created on demand
  vfs_vec* coords;  // node coordinates (dof 3 over the same points)
  std::vector<PetscInt> gidx;  // DMDAGetGlobalIndices
};

struct vfs_vec {
  vfs_dm* da;
  PetscInt n;  // doubles
  double* a;
};

struct vfs_obj {
  void* ctx;
};

struct vfs_hypre {
  // IJ matrix: (row, col) -> value; IJ vector: index -> value
  std::map<long long, double> entries;
};

namespace {

// Pointer tables handed out by DMDAVecGetArray, released by its Restore.
std::map<void*, std::vector<void*>> g_tables;

size_t points(const vfs_dm* d) { return (size_t)d->mx * d->my * d->mz; }

vfs_vec* new_vec(vfs_dm* d) {
  vfs_vec* v = new vfs_vec;
  v->da = d;
  v->n = (PetscInt)(points(d) * d->dof);
  v->a = (double*)calloc((size_t)v->n, sizeof(double));
  return v;
}

void need(const void* p, const char* what) {
  if (!p) {
    fprintf(stderr, "vfs_ref_stub: %s on a null object, called from:\n", what);
    void* frames[8];
    const int n = backtrace(frames, 8);
    backtrace_symbols_fd(frames, n, 2);
    abort();
  }
}

}  // namespace

int vfs_ref_unimpl(const char* name) {
  fprintf(stderr, "vfs_ref_stub: %s is not provided by the single-rank stand-in\n", name);
  abort();
  return 1;
}

int vfs_ref_malloc(size_t n, void** p) {
  *p = calloc(n ? n : 1, 1);
  return *p ? 0 : 1;
}

DM vfs_ref_dm_create(int mx, int my, int mz, int dof) {
  vfs_dm* d = new vfs_dm;
  d->mx = mx;
  d->my = my;
  d->mz = mz;
  d->dof = dof;
  d->cda = nullptr;
  d->coords = nullptr;
  return d;
}

void vfs_ref_dm_set_coordinates(DM da, const double* xyz) {
  DM cda;
  DMDAGetCoordinateDA(da, &cda);
  if (!da->coords) da->coords = new_vec(cda);
  memcpy(da->coords->a, xyz, sizeof(double) * (size_t)da->coords->n);
}

double* vfs_ref_vec_data(Vec v) { return v ? v->a : nullptr; }
PetscInt vfs_ref_vec_size(Vec v) { return v ? v->n : 0; }

PetscErrorCode DMDAGetLocalInfo(DM da, DMDALocalInfo* info) {
  need(da, "DMDAGetLocalInfo");
  memset(info, 0, sizeof(*info));
  info->dim = 3;
  info->dof = da->dof;
  info->sw = 3;
  info->mx = da->mx;
  info->my = da->my;
  info->mz = da->mz;
  info->xm = info->gxm = da->mx;
  info->ym = info->gym = da->my;
  info->zm = info->gzm = da->mz;
  info->pt = DMDA_BOUNDARY_NONE;
  info->st = DMDA_STENCIL_BOX;
  info->da = da;
  return 0;
}

// [k][j][i] tables over the vector: k rows of j-row pointers, each j-row
// pointing at its i-row of dof-sized elements.
PetscErrorCode DMDAVecGetArray(DM da, Vec v, void* array) {
  need(da, "DMDAVecGetArray (DM)");
  need(v, "DMDAVecGetArray (Vec)");
  const size_t esz = sizeof(double) * (size_t)da->dof;
  if ((size_t)v->n != points(da) * da->dof) {
    fprintf(stderr, "vfs_ref_stub: DMDAVecGetArray: vector of %d doubles on a DM of %zu x %d\n", v->n, points(da),
            da->dof);
    abort();
  }
  void** kp = (void**)malloc(sizeof(void*) * (size_t)da->mz);
  void** jp = (void**)malloc(sizeof(void*) * (size_t)da->mz * da->my);
  for (int k = 0; k < da->mz; k++) {
    for (int j = 0; j < da->my; j++)
      jp[(size_t)k * da->my + j] = (char*)v->a + ((size_t)k * da->my + j) * da->mx * esz;
    kp[k] = jp + (size_t)k * da->my;
  }
  *(void***)array = kp;
  g_tables[(void*)kp] = {(void*)kp, (void*)jp};
  return 0;
}

PetscErrorCode DMDAVecRestoreArray(DM, Vec, void* array) {
  void* kp = *(void**)array;
  auto it = g_tables.find(kp);
  if (it != g_tables.end()) {
    free(it->second[1]);
    free(it->second[0]);
    g_tables.erase(it);
  }
  *(void**)array = nullptr;
  return 0;
}

PetscErrorCode DMCreateGlobalVector(DM da, Vec* v) {
  need(da, "DMCreateGlobalVector");
  *v = new_vec(da);
  return 0;
}
PetscErrorCode DMCreateLocalVector(DM da, Vec* v) { return DMCreateGlobalVector(da, v); }
PetscErrorCode DMGetLocalVector(DM da, Vec* v) { return DMCreateGlobalVector(da, v); }
PetscErrorCode DMRestoreLocalVector(DM, Vec* v) { return VecDestroy(v); }
PetscErrorCode DMGetGlobalVector(DM da, Vec* v) { return DMCreateGlobalVector(da, v); }
PetscErrorCode DMRestoreGlobalVector(DM, Vec* v) { return VecDestroy(v); }

static PetscErrorCode scatter(Vec from, InsertMode mode, Vec to) {
  need(from, "scatter (source)");
  need(to, "scatter (target)");
  if (from == to) return 0;
  if (from->n != to->n) vfs_ref_unimpl("scatter between vectors of different sizes");
  if (mode == ADD_VALUES)
    for (PetscInt t = 0; t < from->n; t++) to->a[t] += from->a[t];
  else
    memcpy(to->a, from->a, sizeof(double) * (size_t)from->n);
  return 0;
}
PetscErrorCode DMGlobalToLocalBegin(DM, Vec g, InsertMode mode, Vec l) { return scatter(g, mode, l); }
PetscErrorCode DMGlobalToLocalEnd(DM, Vec, InsertMode, Vec) { return 0; }
PetscErrorCode DMLocalToGlobalBegin(DM, Vec l, InsertMode mode, Vec g) { return scatter(l, mode, g); }
PetscErrorCode DMLocalToGlobalEnd(DM, Vec, InsertMode, Vec) { return 0; }
PetscErrorCode DMLocalToGlobal(DM, Vec l, InsertMode mode, Vec g) { return scatter(l, mode, g); }
PetscErrorCode DMDALocalToLocalBegin(DM, Vec a, InsertMode mode, Vec b) { return scatter(a, mode, b); }
PetscErrorCode DMDALocalToLocalEnd(DM, Vec, InsertMode, Vec) { return 0; }

PetscErrorCode DMDAGetCoordinateDA(DM da, DM* cda) {
  need(da, "DMDAGetCoordinateDA");
  if (!da->cda) da->cda = vfs_ref_dm_create(da->mx, da->my, da->mz, 3);
  *cda = da->cda;
  return 0;
}
PetscErrorCode DMDAGetGhostedCoordinates(DM da, Vec* c) {
  need(da, "DMDAGetGhostedCoordinates");
  need(da->coords, "DMDAGetGhostedCoordinates (no coordinates set)");
  *c = da->coords;
  return 0;
}
PetscErrorCode DMDAGetCoordinates(DM da, Vec* c) { return DMDAGetGhostedCoordinates(da, c); }
PetscErrorCode DMDAGetInfo(DM da, PetscInt* dim, PetscInt* mx, PetscInt* my, PetscInt* mz, PetscInt* m, PetscInt* n,
                           PetscInt* p, PetscInt* dof, PetscInt* s, DMDABoundaryType* bx, DMDABoundaryType* by,
                           DMDABoundaryType* bz, DMDAStencilType* st) {
  need(da, "DMDAGetInfo");
  if (dim) *dim = 3;
  if (mx) *mx = da->mx;
  if (my) *my = da->my;
  if (mz) *mz = da->mz;
  if (m) *m = 1;
  if (n) *n = 1;
  if (p) *p = 1;
  if (dof) *dof = da->dof;
  if (s) *s = 3;
  if (bx) *bx = DMDA_BOUNDARY_NONE;
  if (by) *by = DMDA_BOUNDARY_NONE;
  if (bz) *bz = DMDA_BOUNDARY_NONE;
  if (st) *st = DMDA_STENCIL_BOX;
  return 0;
}
PetscErrorCode DMDAGetGlobalIndices(DM da, PetscInt* n, PetscInt** idx) {
  need(da, "DMDAGetGlobalIndices");
  const size_t np = points(da) * (size_t)da->dof;
  if (da->gidx.size() != np) {
    da->gidx.resize(np);
    for (size_t t = 0; t < np; t++) da->gidx[t] = (PetscInt)t;
  }
  if (n) *n = (PetscInt)np;
  *idx = da->gidx.data();
  return 0;
}
Mat vfs_ref_shell(void* ctx) {
  vfs_obj* m = new vfs_obj;
  m->ctx = ctx;
  return m;
}
void vfs_ref_shell_free(Mat A) { delete A; }
PetscErrorCode MatShellGetContext(Mat A, void** ctx) {
  need(A, "MatShellGetContext");
  *ctx = A->ctx;
  return 0;
}
PetscErrorCode DMDestroy(DM* da) {
  if (da && *da) {
    if ((*da)->coords) VecDestroy(&(*da)->coords);
    if ((*da)->cda) DMDestroy(&(*da)->cda);
    delete *da;
    *da = nullptr;
  }
  return 0;
}

PetscErrorCode VecDuplicate(Vec v, Vec* w) {
  need(v, "VecDuplicate");
  vfs_vec* x = new vfs_vec;
  x->da = v->da;
  x->n = v->n;
  x->a = (double*)calloc((size_t)v->n, sizeof(double));
  *w = x;
  return 0;
}
PetscErrorCode VecDestroy(Vec* v) {
  if (v && *v) {
    free((*v)->a);
    delete *v;
    *v = nullptr;
  }
  return 0;
}
PetscErrorCode VecSet(Vec v, PetscScalar a) {
  need(v, "VecSet");
  for (PetscInt t = 0; t < v->n; t++) v->a[t] = a;
  return 0;
}
PetscErrorCode VecCopy(Vec x, Vec y) { return scatter(x, INSERT_VALUES, y); }
PetscErrorCode VecAXPY(Vec y, PetscScalar a, Vec x) {
  need(x, "VecAXPY");
  need(y, "VecAXPY");
  for (PetscInt t = 0; t < y->n; t++) y->a[t] += a * x->a[t];
  return 0;
}
PetscErrorCode VecWAXPY(Vec w, PetscScalar a, Vec x, Vec y) {
  need(w, "VecWAXPY");
  for (PetscInt t = 0; t < w->n; t++) w->a[t] = a * x->a[t] + y->a[t];
  return 0;
}
PetscErrorCode VecShift(Vec v, PetscScalar a) {
  need(v, "VecShift");
  for (PetscInt t = 0; t < v->n; t++) v->a[t] += a;
  return 0;
}
PetscErrorCode VecScale(Vec v, PetscScalar a) {
  need(v, "VecScale");
  for (PetscInt t = 0; t < v->n; t++) v->a[t] *= a;
  return 0;
}
// Sums in index order (one rank: PETSc's local loop order).
PetscErrorCode VecSum(Vec v, PetscScalar* s) {
  need(v, "VecSum");
  double acc = 0.;
  for (PetscInt t = 0; t < v->n; t++) acc += v->a[t];
  *s = acc;
  return 0;
}
PetscInt vfs_ref_last_max_at = -1;
PetscReal vfs_ref_last_max = 0.;
PetscErrorCode VecMax(Vec v, PetscInt* p, PetscReal* m) {
  need(v, "VecMax");
  PetscInt at = 0;
  double best = v->n ? v->a[0] : -HUGE_VAL;
  for (PetscInt t = 1; t < v->n; t++)
    if (v->a[t] > best) best = v->a[t], at = t;
  if (p) *p = at;
  *m = best;
  vfs_ref_last_max_at = at;
  vfs_ref_last_max = best;
  return 0;
}
PetscErrorCode VecMin(Vec v, PetscInt* p, PetscReal* m) {
  need(v, "VecMin");
  PetscInt at = 0;
  double best = v->n ? v->a[0] : HUGE_VAL;
  for (PetscInt t = 1; t < v->n; t++)
    if (v->a[t] < best) best = v->a[t], at = t;
  if (p) *p = at;
  *m = best;
  return 0;
}
PetscErrorCode VecNorm(Vec v, NormType type, PetscReal* n) {
  need(v, "VecNorm");
  double acc = 0.;
  for (PetscInt t = 0; t < v->n; t++) {
    const double a = fabs(v->a[t]);
    if (type == NORM_1) acc += a;
    else if (type == NORM_INFINITY) acc = a > acc ? a : acc;
    else acc += a * a;
  }
  *n = (type == NORM_2 || type == NORM_FROBENIUS) ? sqrt(acc) : acc;
  return 0;
}
PetscErrorCode VecGetArray(Vec v, PetscScalar** a) {
  need(v, "VecGetArray");
  *a = v->a;
  return 0;
}
PetscErrorCode VecRestoreArray(Vec, PetscScalar** a) {
  *a = nullptr;
  return 0;
}
PetscErrorCode VecGetSize(Vec v, PetscInt* n) {
  need(v, "VecGetSize");
  *n = v->n;
  return 0;
}
PetscErrorCode VecGetLocalSize(Vec v, PetscInt* n) { return VecGetSize(v, n); }
PetscErrorCode VecSetValue(Vec v, PetscInt i, PetscScalar a, InsertMode mode) {
  need(v, "VecSetValue");
  if (mode == ADD_VALUES) v->a[i] += a;
  else v->a[i] = a;
  return 0;
}
PetscErrorCode VecCreateMPI(MPI_Comm, PetscInt nlocal, PetscInt, Vec* v) {
  vfs_vec* x = new vfs_vec;
  x->da = nullptr;
  x->n = nlocal;
  x->a = (double*)calloc((size_t)(nlocal > 0 ? nlocal : 1), sizeof(double));
  *v = x;
  return 0;
}
PetscErrorCode VecCreateSeq(MPI_Comm c, PetscInt n, Vec* v) { return VecCreateMPI(c, n, n, v); }
PetscErrorCode VecAssemblyBegin(Vec) { return 0; }
PetscErrorCode VecAssemblyEnd(Vec) { return 0; }

// Output of the checked code goes to stderr only when VFS_REF_VERBOSE is set.
static bool verbose() {
  static int v = -1;
  if (v < 0) v = getenv("VFS_REF_VERBOSE") ? 1 : 0;
  return v == 1;
}
PetscErrorCode PetscPrintf(MPI_Comm, const char* fmt, ...) {
  if (!verbose()) return 0;
  va_list ap;
  va_start(ap, fmt);
  vfprintf(stderr, fmt, ap);
  va_end(ap);
  return 0;
}
PetscErrorCode PetscFPrintf(MPI_Comm, FILE* f, const char* fmt, ...) {
  if (!verbose() || !f) return 0;
  va_list ap;
  va_start(ap, fmt);
  vfprintf(f, fmt, ap);
  va_end(ap);
  return 0;
}
PetscErrorCode PetscGetTime(PetscLogDouble* t) {
  struct timeval tv;
  gettimeofday(&tv, nullptr);
  *t = tv.tv_sec + 1e-6 * tv.tv_usec;
  return 0;
}
PetscErrorCode PetscBarrier(PetscObject) { return 0; }
PetscErrorCode PetscOptionsGetInt(const char*, const char*, PetscInt*, PetscBool* set) {
  if (set) *set = PETSC_FALSE;
  return 0;
}
PetscErrorCode PetscOptionsGetReal(const char*, const char*, PetscReal*, PetscBool* set) {
  if (set) *set = PETSC_FALSE;
  return 0;
}
PetscErrorCode PetscOptionsGetBool(const char*, const char*, PetscBool*, PetscBool* set) {
  if (set) *set = PETSC_FALSE;
  return 0;
}
PetscErrorCode PetscOptionsGetString(const char*, const char*, char*, size_t, PetscBool* set) {
  if (set) *set = PETSC_FALSE;
  return 0;
}
PetscErrorCode PetscOptionsHasName(const char*, const char*, PetscBool* set) {
  if (set) *set = PETSC_FALSE;
  return 0;
}

static size_t type_size(MPI_Datatype t) {
  switch (t) {
    case MPI_INT: return sizeof(int);
    case MPI_DOUBLE: return sizeof(double);
    case MPI_CHAR: return 1;
    case MPI_FLOAT: return sizeof(float);
    case MPI_LONG: return sizeof(long);
    default: vfs_ref_unimpl("MPI datatype");
  }
  return 0;
}
int MPI_Comm_rank(MPI_Comm, int* r) {
  *r = 0;
  return 0;
}
int MPI_Comm_size(MPI_Comm, int* n) {
  *n = 1;
  return 0;
}
int MPI_Barrier(MPI_Comm) { return 0; }
int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return 0; }
int MPI_Allreduce(const void* in, void* out, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
  if (in != out) memmove(out, in, type_size(t) * (size_t)n);
  return 0;
}
int MPI_Reduce(const void* in, void* out, int n, MPI_Datatype t, MPI_Op op, int, MPI_Comm c) {
  return MPI_Allreduce(in, out, n, t, op, c);
}

static long long key(int row, int col) { return ((long long)row << 32) | (unsigned)col; }
int HYPRE_IJMatrixSetValues(HYPRE_IJMatrix A, int nrows, int* ncols, const int* rows, const int* cols,
                            const double* vals) {
  need(A, "HYPRE_IJMatrixSetValues");
  int q = 0;
  for (int r = 0; r < nrows; r++)
    for (int c = 0; c < ncols[r]; c++, q++) A->entries[key(rows[r], cols[q])] = vals[q];
  return 0;
}
int HYPRE_IJMatrixAddToValues(HYPRE_IJMatrix A, int nrows, int* ncols, const int* rows, const int* cols,
                              const double* vals) {
  need(A, "HYPRE_IJMatrixAddToValues");
  int q = 0;
  for (int r = 0; r < nrows; r++)
    for (int c = 0; c < ncols[r]; c++, q++) A->entries[key(rows[r], cols[q])] += vals[q];
  return 0;
}
int HYPRE_IJVectorSetValues(HYPRE_IJVector v, int n, const int* idx, const double* vals) {
  need(v, "HYPRE_IJVectorSetValues");
  for (int q = 0; q < n; q++) v->entries[idx[q]] = vals[q];
  return 0;
}
int HYPRE_IJVectorAddToValues(HYPRE_IJVector v, int n, const int* idx, const double* vals) {
  need(v, "HYPRE_IJVectorAddToValues");
  for (int q = 0; q < n; q++) v->entries[idx[q]] += vals[q];
  return 0;
}
int HYPRE_IJVectorGetValues(HYPRE_IJVector v, int n, const int* idx, double* vals) {
  need(v, "HYPRE_IJVectorGetValues");
  for (int q = 0; q < n; q++) {
    auto it = v->entries.find(idx[q]);
    vals[q] = it == v->entries.end() ? 0. : it->second;
  }
  return 0;
}
int HYPRE_IJMatrixAssemble(HYPRE_IJMatrix) { return 0; }
int HYPRE_IJVectorAssemble(HYPRE_IJVector) { return 0; }
int HYPRE_BoomerAMGSolve(HYPRE_Solver, HYPRE_ParCSRMatrix, HYPRE_ParVector, HYPRE_ParVector) {
  return vfs_ref_unimpl("HYPRE_BoomerAMGSolve");
}
int HYPRE_BoomerAMGSetup(HYPRE_Solver, HYPRE_ParCSRMatrix, HYPRE_ParVector, HYPRE_ParVector) {
  return vfs_ref_unimpl("HYPRE_BoomerAMGSetup");
}

// Harness access to IJ objects.
extern "C" {
HYPRE_IJMatrix vfs_ref_ij_new() { return new vfs_hypre; }
void vfs_ref_ij_free(HYPRE_IJMatrix m) { delete m; }
long long vfs_ref_ij_count(HYPRE_IJMatrix m) { return (long long)m->entries.size(); }
// entries in (row, col) order
void vfs_ref_ij_get(HYPRE_IJMatrix m, int* rows, int* cols, double* vals) {
  long long q = 0;
  for (const auto& e : m->entries) {
    rows[q] = (int)(e.first >> 32);
    cols[q] = (int)(unsigned)(e.first & 0xffffffffu);
    vals[q] = e.second;
    q++;
  }
}
}
