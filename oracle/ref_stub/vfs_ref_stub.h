/*
 * vfs_ref_stub.h -- single-process stand-ins for the PETSc 3.2, HYPRE and MPI
 * calls that the reference's pressure-projection sources make, so that those
 * sources compile unmodified (oracle/ref.mk) and run on one rank.
 *
 * TEST INFRASTRUCTURE ONLY: it exists to build the reference's own code as a
 * checker of the oracle restatement (tests/test_ref_oracle.py).  Nothing of the
 * product links it.
 *
 * Model.  One MPI rank owns the whole grid.  A DM describes a structured grid
 * of mx x my x mz points with dof values per point (1 for scalars, 3 for
 * Cmpnts); its local (ghosted) and global vectors have the same extent and
 * layout (a non-periodic DMDA on one rank has no ghost points outside the
 * domain), element (i, j, k) at ((k my) + j) mx + i.  DMDAVecGetArray hands
 * out [k][j][i] pointer tables over a vector's storage, as PETSc does.
 * Global-to-local and local-to-global scatters are copies.  Reductions over
 * MPI_COMM_WORLD return the local value.  A HYPRE IJ matrix or vector records
 * the entries set into it.  Calls that the checked path does not reach abort
 * with their name when called (vfs_ref_unimpl).
 */
#ifndef VFS_REF_STUB_H
#define VFS_REF_STUB_H

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ---- scalar types ---- */
typedef int PetscErrorCode;
typedef int PetscInt;
typedef int PetscMPIInt;
typedef double PetscReal;
typedef double PetscScalar;
typedef double PetscLogDouble;
typedef enum { PETSC_FALSE = 0, PETSC_TRUE = 1 } PetscBool;
typedef PetscBool PetscTruth;

/* ---- opaque objects ---- */
struct vfs_dm;
struct vfs_vec;
struct vfs_obj;
typedef struct vfs_dm* DM;
typedef struct vfs_vec* Vec;
typedef struct vfs_obj* Mat;
typedef struct vfs_obj* KSP;
typedef struct vfs_obj* PC;
typedef struct vfs_obj* SNES;
typedef struct vfs_obj* IS;
typedef struct vfs_obj* AO;
typedef struct vfs_obj* MatNullSpace;
typedef struct vfs_obj* PetscViewer;
typedef struct vfs_obj* VecScatter;
typedef struct vfs_obj* PetscRandom;
typedef struct vfs_obj* PetscObject;
typedef const char* KSPType;
typedef const char* PCType;
typedef const char* MatType;
typedef const char* PetscViewerType;
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

typedef enum { NOT_SET_VALUES = 0, INSERT_VALUES, ADD_VALUES, MAX_VALUES } InsertMode;
typedef enum { SCATTER_FORWARD = 0, SCATTER_REVERSE = 1 } ScatterMode;
typedef enum { NORM_1 = 0, NORM_2 = 1, NORM_FROBENIUS = 2, NORM_INFINITY = 3, NORM_1_AND_2 = 4 } NormType;
typedef enum { FILE_MODE_READ = 0, FILE_MODE_WRITE, FILE_MODE_APPEND } PetscFileMode;
typedef enum { DMDA_BOUNDARY_NONE = 0, DMDA_BOUNDARY_GHOSTED, DMDA_BOUNDARY_MIRROR, DMDA_BOUNDARY_PERIODIC } DMDABoundaryType;
typedef enum { DMDA_STENCIL_STAR = 0, DMDA_STENCIL_BOX } DMDAStencilType;
typedef enum { MAT_FLUSH_ASSEMBLY = 1, MAT_FINAL_ASSEMBLY = 0 } MatAssemblyType;
typedef enum { SAME_NONZERO_PATTERN = 0, DIFFERENT_NONZERO_PATTERN, SAME_PRECONDITIONER, SUBSET_NONZERO_PATTERN } MatStructure;
typedef enum { PC_MG_MULTIPLICATIVE = 0, PC_MG_ADDITIVE, PC_MG_FULL, PC_MG_KASKADE } PCMGType;
typedef enum { PC_MG_CYCLE_V = 1, PC_MG_CYCLE_W = 2 } PCMGCycleType;
typedef enum { KSP_NORM_NONE = 0, KSP_NORM_PRECONDITIONED, KSP_NORM_UNPRECONDITIONED, KSP_NORM_NATURAL } KSPNormType;
typedef enum { KSP_CONVERGED_ITERATING = 0 } KSPConvergedReason;
typedef enum { MAT_NEW_NONZERO_ALLOCATION_ERR = 0, MAT_KEEP_NONZERO_PATTERN, MAT_IGNORE_ZERO_ENTRIES } MatOption;

typedef struct {
  PetscInt dim, dof, sw;
  PetscInt mx, my, mz;     /* global extents */
  PetscInt xs, ys, zs;     /* owned start */
  PetscInt xm, ym, zm;     /* owned extent */
  PetscInt gxs, gys, gzs;  /* ghosted start */
  PetscInt gxm, gym, gzm;  /* ghosted extent */
  DMDABoundaryType pt;
  DMDAStencilType st;
  DM da;
} DMDALocalInfo;

#define PETSC_NULL 0
#define PETSC_NULL_INTEGER 0
#define PETSC_DECIDE (-1)
#define PETSC_DETERMINE (-1)
#define PETSC_DEFAULT (-2)
#define PETSC_COMM_WORLD 0
#define PETSC_COMM_SELF 1
#define MPI_COMM_WORLD 0
#define MPI_COMM_SELF 1
#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_CHAR 3
#define MPI_FLOAT 4
#define MPI_LONG 5
#define MPIU_REAL MPI_DOUBLE
#define MPIU_SCALAR MPI_DOUBLE
#define MPIU_INT MPI_INT
#define MPI_SUM 1
#define MPIU_SUM MPI_SUM
#define MPIU_MAX MPI_MAX
#define MPI_MAX 2
#define MPI_MIN 3
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define PETSC_VIEWER_STDOUT_WORLD ((PetscViewer)0)
#define PETSC_VIEWER_STDOUT_SELF ((PetscViewer)0)
#define PETSC_VIEWER_BINARY "binary"
#define PETSCVIEWERBINARY "binary"
#define PETSC_MAX_PATH_LEN 4096
#define KSPGMRES "gmres"
#define KSPCG "cg"
#define KSPRICHARDSON "richardson"
#define KSPPREONLY "preonly"
#define KSPBCGS "bcgs"
#define KSPFGMRES "fgmres"
#define PCMG "mg"
#define PCBJACOBI "bjacobi"
#define PCJACOBI "jacobi"
#define PCILU "ilu"
#define PCNONE "none"
#define PCSOR "sor"
#define PCLU "lu"
#define PCHYPRE "hypre"
#define PCASM "asm"
#define MATSHELL "shell"
#define MATMPIAIJ "mpiaij"
#define MATAIJ "aij"
#define MATSEQAIJ "seqaij"
#define MATMPIBAIJ "mpibaij"
#define SNESKSPONLY "ksponly"
#define MATOP_MULT 0
#define MATOP_MULT_ADD 1
#define MATOP_MULT_TRANSPOSE 2

#define PetscMax(a, b) (((a) < (b)) ? (b) : (a))
#define PetscMin(a, b) (((a) < (b)) ? (a) : (b))
#define PetscAbsScalar(a) fabs(a)
#define PetscAbsReal(a) fabs(a)
#define PetscSqrtScalar(a) sqrt(a)
#define PetscRealPart(a) (a)
#define CHKERRQ(e) ((void)(e))
#define CHKERRABORT(c, e) ((void)(e))
#define CHKMEMQ
#define PetscFunctionBegin
#define PetscFunctionReturn(v) return (v)
#define SETERRQ(c, n, s) return (n)
#define SETERRQ1(c, n, s, a) return (n)
#define PetscMalloc(n, p) vfs_ref_malloc((size_t)(n), (void**)(p))
#define PetscFree(p) (free(p), (p) = 0, 0)
#define PetscMemzero(p, n) (memset((p), 0, (size_t)(n)), 0)
#define PetscMemcpy(a, b, n) (memcpy((a), (b), (size_t)(n)), 0)

/* ---- hypre ---- */
struct vfs_hypre;
typedef struct vfs_hypre* HYPRE_IJMatrix;
typedef struct vfs_hypre* HYPRE_IJVector;
typedef struct vfs_obj* HYPRE_Solver;
typedef struct vfs_obj* HYPRE_ParCSRMatrix;
typedef struct vfs_obj* HYPRE_ParVector;
typedef struct vfs_obj* HYPRE_Matrix;
typedef struct vfs_obj* HYPRE_Vector;
typedef int HYPRE_Int;
typedef double HYPRE_Real;
typedef int (*HYPRE_PtrToSolverFcn)(HYPRE_Solver, HYPRE_Matrix, HYPRE_Vector, HYPRE_Vector);
#define HYPRE_PARCSR 5555

/* ---- runtime of the stand-ins (vfs_ref_stub.cpp) ---- */
int vfs_ref_unimpl(const char* name);
int vfs_ref_malloc(size_t n, void** p);

/* grids and vectors */
DM vfs_ref_dm_create(int mx, int my, int mz, int dof);
void vfs_ref_dm_set_coordinates(DM da, const double* xyz);
double* vfs_ref_vec_data(Vec v);
/* the location and value of the last VecMax (the reference prints, and does
 * not return, the maximum it finds, e.g. in Divergence) */
extern PetscInt vfs_ref_last_max_at;
extern PetscReal vfs_ref_last_max;
PetscInt vfs_ref_vec_size(Vec v);

PetscErrorCode DMDAGetLocalInfo(DM da, DMDALocalInfo* info);
PetscErrorCode DMDAVecGetArray(DM da, Vec v, void* array);
PetscErrorCode DMDAVecRestoreArray(DM da, Vec v, void* array);
PetscErrorCode DMCreateGlobalVector(DM da, Vec* v);
PetscErrorCode DMCreateLocalVector(DM da, Vec* v);
PetscErrorCode DMGetLocalVector(DM da, Vec* v);
PetscErrorCode DMRestoreLocalVector(DM da, Vec* v);
PetscErrorCode DMGetGlobalVector(DM da, Vec* v);
PetscErrorCode DMRestoreGlobalVector(DM da, Vec* v);
PetscErrorCode DMGlobalToLocalBegin(DM da, Vec g, InsertMode mode, Vec l);
PetscErrorCode DMGlobalToLocalEnd(DM da, Vec g, InsertMode mode, Vec l);
PetscErrorCode DMLocalToGlobalBegin(DM da, Vec l, InsertMode mode, Vec g);
PetscErrorCode DMLocalToGlobalEnd(DM da, Vec l, InsertMode mode, Vec g);
PetscErrorCode DMLocalToGlobal(DM da, Vec l, InsertMode mode, Vec g);
PetscErrorCode DMDALocalToLocalBegin(DM da, Vec a, InsertMode mode, Vec b);
PetscErrorCode DMDALocalToLocalEnd(DM da, Vec a, InsertMode mode, Vec b);
PetscErrorCode DMDAGetCoordinateDA(DM da, DM* cda);
PetscErrorCode DMDAGetGhostedCoordinates(DM da, Vec* c);
PetscErrorCode DMDAGetCoordinates(DM da, Vec* c);
PetscErrorCode DMDAGetInfo(DM da, PetscInt* dim, PetscInt* mx, PetscInt* my, PetscInt* mz, PetscInt* m, PetscInt* n,
                           PetscInt* p, PetscInt* dof, PetscInt* s, DMDABoundaryType* bx, DMDABoundaryType* by,
                           DMDABoundaryType* bz, DMDAStencilType* st);
PetscErrorCode DMDestroy(DM* da);
/* a shell matrix is its context pointer (vfs_ref_shell makes one) */
Mat vfs_ref_shell(void* ctx);
void vfs_ref_shell_free(Mat A);
PetscErrorCode MatShellGetContext(Mat A, void** ctx);
/* one rank: a point's global (PETSc) index is its local index */
PetscErrorCode DMDAGetGlobalIndices(DM da, PetscInt* n, PetscInt** idx);

PetscErrorCode VecDuplicate(Vec v, Vec* w);
PetscErrorCode VecDestroy(Vec* v);
PetscErrorCode VecSet(Vec v, PetscScalar a);
PetscErrorCode VecCopy(Vec x, Vec y);
PetscErrorCode VecAXPY(Vec y, PetscScalar a, Vec x);
PetscErrorCode VecWAXPY(Vec w, PetscScalar a, Vec x, Vec y);
PetscErrorCode VecShift(Vec v, PetscScalar a);
PetscErrorCode VecScale(Vec v, PetscScalar a);
PetscErrorCode VecSum(Vec v, PetscScalar* s);
PetscErrorCode VecMax(Vec v, PetscInt* p, PetscReal* m);
PetscErrorCode VecMin(Vec v, PetscInt* p, PetscReal* m);
PetscErrorCode VecNorm(Vec v, NormType t, PetscReal* n);
PetscErrorCode VecGetArray(Vec v, PetscScalar** a);
PetscErrorCode VecRestoreArray(Vec v, PetscScalar** a);
PetscErrorCode VecGetSize(Vec v, PetscInt* n);
PetscErrorCode VecGetLocalSize(Vec v, PetscInt* n);
PetscErrorCode VecSetValue(Vec v, PetscInt i, PetscScalar a, InsertMode mode);
PetscErrorCode VecCreateMPI(MPI_Comm c, PetscInt nlocal, PetscInt nglobal, Vec* v);
PetscErrorCode VecCreateSeq(MPI_Comm c, PetscInt n, Vec* v);
PetscErrorCode VecAssemblyBegin(Vec v);
PetscErrorCode VecAssemblyEnd(Vec v);

PetscErrorCode PetscPrintf(MPI_Comm c, const char* fmt, ...);
PetscErrorCode PetscFPrintf(MPI_Comm c, FILE* f, const char* fmt, ...);
PetscErrorCode PetscGetTime(PetscLogDouble* t);
PetscErrorCode PetscBarrier(PetscObject o);
PetscErrorCode PetscOptionsGetInt(const char* pre, const char* name, PetscInt* v, PetscBool* set);
PetscErrorCode PetscOptionsGetReal(const char* pre, const char* name, PetscReal* v, PetscBool* set);
PetscErrorCode PetscOptionsGetBool(const char* pre, const char* name, PetscBool* v, PetscBool* set);
PetscErrorCode PetscOptionsGetString(const char* pre, const char* name, char* v, size_t len, PetscBool* set);
PetscErrorCode PetscOptionsHasName(const char* pre, const char* name, PetscBool* set);

int MPI_Comm_rank(MPI_Comm c, int* r);
int MPI_Comm_size(MPI_Comm c, int* n);
int MPI_Barrier(MPI_Comm c);
int MPI_Bcast(void* buf, int n, MPI_Datatype t, int root, MPI_Comm c);
int MPI_Allreduce(const void* in, void* out, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c);
int MPI_Reduce(const void* in, void* out, int n, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c);

int HYPRE_IJMatrixSetValues(HYPRE_IJMatrix A, int nrows, int* ncols, const int* rows, const int* cols,
                            const double* vals);
int HYPRE_IJMatrixAddToValues(HYPRE_IJMatrix A, int nrows, int* ncols, const int* rows, const int* cols,
                              const double* vals);
int HYPRE_IJVectorSetValues(HYPRE_IJVector v, int n, const int* idx, const double* vals);
int HYPRE_IJVectorAddToValues(HYPRE_IJVector v, int n, const int* idx, const double* vals);
int HYPRE_IJVectorGetValues(HYPRE_IJVector v, int n, const int* idx, double* vals);
int HYPRE_IJMatrixAssemble(HYPRE_IJMatrix A);
int HYPRE_IJVectorAssemble(HYPRE_IJVector v);
int HYPRE_BoomerAMGSolve(HYPRE_Solver s, HYPRE_ParCSRMatrix A, HYPRE_ParVector b, HYPRE_ParVector x);
int HYPRE_BoomerAMGSetup(HYPRE_Solver s, HYPRE_ParCSRMatrix A, HYPRE_ParVector b, HYPRE_ParVector x);

/* Every other call of the library surface the sources name: declared with
 * any arguments, aborts with its name if the checked path ever calls it. */
#define VFS_REF_UNIMPL(name)                                          \
  template <typename... A>                                            \
  inline int name(A&&...) {                                           \
    return vfs_ref_unimpl(#name);                                     \
  }
VFS_REF_UNIMPL(PetscInitialize)
VFS_REF_UNIMPL(PetscFinalize)
VFS_REF_UNIMPL(PetscOptionsInsertFile)
VFS_REF_UNIMPL(PetscViewerBinaryOpen)
VFS_REF_UNIMPL(PetscViewerDestroy)
VFS_REF_UNIMPL(PetscViewerCreate)
VFS_REF_UNIMPL(PetscViewerSetType)
VFS_REF_UNIMPL(PetscViewerFileSetName)
VFS_REF_UNIMPL(PetscViewerFileSetMode)
VFS_REF_UNIMPL(PetscViewerBinarySetMPIIO)
VFS_REF_UNIMPL(PetscViewerASCIIOpen)
VFS_REF_UNIMPL(PetscRandomCreate)
VFS_REF_UNIMPL(PetscRandomSetFromOptions)
VFS_REF_UNIMPL(PetscRandomDestroy)
VFS_REF_UNIMPL(VecLoad)
VFS_REF_UNIMPL(VecLoadIntoVector)
VFS_REF_UNIMPL(VecView)
VFS_REF_UNIMPL(VecCreate)
VFS_REF_UNIMPL(VecSetSizes)
VFS_REF_UNIMPL(VecSetFromOptions)
VFS_REF_UNIMPL(VecSetValues)
VFS_REF_UNIMPL(VecPointwiseMult)
VFS_REF_UNIMPL(VecPointwiseDivide)
VFS_REF_UNIMPL(VecDot)
VFS_REF_UNIMPL(VecAYPX)
VFS_REF_UNIMPL(VecGetOwnershipRange)
VFS_REF_UNIMPL(VecScatterCreateToZero)
VFS_REF_UNIMPL(VecScatterCreateToAll)
VFS_REF_UNIMPL(VecScatterBegin)
VFS_REF_UNIMPL(VecScatterEnd)
VFS_REF_UNIMPL(VecScatterDestroy)
VFS_REF_UNIMPL(VecGetArray3d)
VFS_REF_UNIMPL(VecRestoreArray3d)
VFS_REF_UNIMPL(VecStrideScatter)
VFS_REF_UNIMPL(VecStrideGather)
VFS_REF_UNIMPL(DMDACreate3d)
VFS_REF_UNIMPL(DMDASetUniformCoordinates)
VFS_REF_UNIMPL(DMDACreateNaturalVector)
VFS_REF_UNIMPL(DMDAGlobalToNaturalBegin)
VFS_REF_UNIMPL(DMDAGlobalToNaturalEnd)
VFS_REF_UNIMPL(DMDAGetAO)
VFS_REF_UNIMPL(DMDAGetCorners)
VFS_REF_UNIMPL(DMDAGetGhostCorners)
VFS_REF_UNIMPL(DMDAGetProcessorSubsets)
VFS_REF_UNIMPL(DMGetMatrix)
VFS_REF_UNIMPL(DMCreateMatrix)
VFS_REF_UNIMPL(AOApplicationToPetsc)
VFS_REF_UNIMPL(AOPetscToApplication)
VFS_REF_UNIMPL(MatCreate)
VFS_REF_UNIMPL(MatSetType)
VFS_REF_UNIMPL(MatSetSizes)
VFS_REF_UNIMPL(MatSetFromOptions)
VFS_REF_UNIMPL(MatSetValues)
VFS_REF_UNIMPL(MatGetRow)
VFS_REF_UNIMPL(MatRestoreRow)
VFS_REF_UNIMPL(MatMult)
VFS_REF_UNIMPL(MatMultAdd)
VFS_REF_UNIMPL(MatMPIAIJSetPreallocation)
VFS_REF_UNIMPL(MatSeqAIJSetPreallocation)
VFS_REF_UNIMPL(MatCreateMPIAIJ)
VFS_REF_UNIMPL(MatCreateSeqAIJ)
VFS_REF_UNIMPL(MatGetOwnershipRange)
VFS_REF_UNIMPL(MatAssemblyBegin)
VFS_REF_UNIMPL(MatAssemblyEnd)
VFS_REF_UNIMPL(MatDestroy)
VFS_REF_UNIMPL(MatZeroEntries)
VFS_REF_UNIMPL(MatShellSetOperation)
VFS_REF_UNIMPL(MatCreateShell)
VFS_REF_UNIMPL(MatSetOption)
VFS_REF_UNIMPL(MatView)
VFS_REF_UNIMPL(MatNullSpaceCreate)
VFS_REF_UNIMPL(MatNullSpaceRemove)
VFS_REF_UNIMPL(MatNullSpaceDestroy)
VFS_REF_UNIMPL(MatHYPRE_IJMatrixCopy)
VFS_REF_UNIMPL(KSPCreate)
VFS_REF_UNIMPL(KSPSetType)
VFS_REF_UNIMPL(KSPSetOperators)
VFS_REF_UNIMPL(KSPSetFromOptions)
VFS_REF_UNIMPL(KSPSetOptionsPrefix)
VFS_REF_UNIMPL(KSPSetTolerances)
VFS_REF_UNIMPL(KSPSetInitialGuessNonzero)
VFS_REF_UNIMPL(KSPSetNullSpace)
VFS_REF_UNIMPL(KSPSetUp)
VFS_REF_UNIMPL(KSPSolve)
VFS_REF_UNIMPL(KSPDestroy)
VFS_REF_UNIMPL(KSPGetPC)
VFS_REF_UNIMPL(KSPGetIterationNumber)
VFS_REF_UNIMPL(KSPGetResidualNorm)
VFS_REF_UNIMPL(KSPMonitorSet)
VFS_REF_UNIMPL(KSPMonitorTrueResidualNorm)
VFS_REF_UNIMPL(KSPBuildResidual)
VFS_REF_UNIMPL(KSPGMRESSetRestart)
VFS_REF_UNIMPL(KSPSetNormType)
VFS_REF_UNIMPL(KSPGetConvergedReason)
VFS_REF_UNIMPL(PCSetType)
VFS_REF_UNIMPL(PCMGSetLevels)
VFS_REF_UNIMPL(PCMGSetType)
VFS_REF_UNIMPL(PCMGSetCycleType)
VFS_REF_UNIMPL(PCMGSetNumberSmoothUp)
VFS_REF_UNIMPL(PCMGSetNumberSmoothDown)
VFS_REF_UNIMPL(PCMGSetRestriction)
VFS_REF_UNIMPL(PCMGSetInterpolation)
VFS_REF_UNIMPL(PCMGSetInterpolate)
VFS_REF_UNIMPL(PCMGSetResidual)
VFS_REF_UNIMPL(PCMGSetRhs)
VFS_REF_UNIMPL(PCMGSetX)
VFS_REF_UNIMPL(PCMGSetR)
VFS_REF_UNIMPL(PCMGGetSmoother)
VFS_REF_UNIMPL(PCMGGetSmootherUp)
VFS_REF_UNIMPL(PCMGGetSmootherDown)
VFS_REF_UNIMPL(PCMGGetCoarseSolve)
VFS_REF_UNIMPL(PCMGDefaultResidual)
VFS_REF_UNIMPL(PCSetFromOptions)
VFS_REF_UNIMPL(PCBJacobiGetSubKSP)
VFS_REF_UNIMPL(PCFactorSetLevels)
VFS_REF_UNIMPL(SNESCreate)
VFS_REF_UNIMPL(SNESDestroy)
VFS_REF_UNIMPL(SNESSolve)
VFS_REF_UNIMPL(SNESSetFunction)
VFS_REF_UNIMPL(SNESSetJacobian)
VFS_REF_UNIMPL(SNESGetKSP)
VFS_REF_UNIMPL(SNESSetFromOptions)
VFS_REF_UNIMPL(SNESSetType)
VFS_REF_UNIMPL(SNESSetTolerances)
VFS_REF_UNIMPL(SNESGetIterationNumber)
VFS_REF_UNIMPL(SNESGetConvergedReason)
VFS_REF_UNIMPL(MatCreateSNESMF)
VFS_REF_UNIMPL(MatMFFDSetFunction)
VFS_REF_UNIMPL(ISCreateGeneral)
VFS_REF_UNIMPL(ISDestroy)
VFS_REF_UNIMPL(MPI_Send)
VFS_REF_UNIMPL(MPI_Recv)
VFS_REF_UNIMPL(MPI_Gather)
VFS_REF_UNIMPL(MPI_Scatter)
VFS_REF_UNIMPL(MPI_Allgather)
VFS_REF_UNIMPL(MPI_Gatherv)
VFS_REF_UNIMPL(MPI_Scatterv)
VFS_REF_UNIMPL(MPI_Allgatherv)
VFS_REF_UNIMPL(MPI_Wtime)
VFS_REF_UNIMPL(HYPRE_IJMatrixCreate)
VFS_REF_UNIMPL(HYPRE_IJMatrixSetObjectType)
VFS_REF_UNIMPL(HYPRE_IJMatrixInitialize)
VFS_REF_UNIMPL(HYPRE_IJMatrixGetObject)
VFS_REF_UNIMPL(HYPRE_IJMatrixDestroy)
VFS_REF_UNIMPL(HYPRE_IJMatrixSetRowSizes)
VFS_REF_UNIMPL(HYPRE_IJVectorCreate)
VFS_REF_UNIMPL(HYPRE_IJVectorSetObjectType)
VFS_REF_UNIMPL(HYPRE_IJVectorInitialize)
VFS_REF_UNIMPL(HYPRE_IJVectorGetObject)
VFS_REF_UNIMPL(HYPRE_IJVectorDestroy)
VFS_REF_UNIMPL(HYPRE_ParCSRGMRESCreate)
VFS_REF_UNIMPL(HYPRE_ParCSRGMRESSetup)
VFS_REF_UNIMPL(HYPRE_ParCSRGMRESSolve)
VFS_REF_UNIMPL(HYPRE_ParCSRGMRESDestroy)
VFS_REF_UNIMPL(HYPRE_ParCSRGMRESSetKDim)
VFS_REF_UNIMPL(HYPRE_ParCSRPCGCreate)
VFS_REF_UNIMPL(HYPRE_ParCSRPCGSetup)
VFS_REF_UNIMPL(HYPRE_ParCSRPCGSolve)
VFS_REF_UNIMPL(HYPRE_ParCSRPCGDestroy)
VFS_REF_UNIMPL(HYPRE_PCGSetTol)
VFS_REF_UNIMPL(HYPRE_PCGSetTwoNorm)
VFS_REF_UNIMPL(HYPRE_PCGSetPrintLevel)
VFS_REF_UNIMPL(HYPRE_PCGSetPrecond)
VFS_REF_UNIMPL(HYPRE_PCGSetMaxIter)
VFS_REF_UNIMPL(HYPRE_PCGSetLogging)
VFS_REF_UNIMPL(HYPRE_PCGGetNumIterations)
VFS_REF_UNIMPL(HYPRE_PCGGetFinalRelativeResidualNorm)
VFS_REF_UNIMPL(HYPRE_GMRESSetTol)
VFS_REF_UNIMPL(HYPRE_GMRESSetPrintLevel)
VFS_REF_UNIMPL(HYPRE_GMRESSetPrecond)
VFS_REF_UNIMPL(HYPRE_GMRESSetMaxIter)
VFS_REF_UNIMPL(HYPRE_GMRESSetKDim)
VFS_REF_UNIMPL(HYPRE_GMRESSetLogging)
VFS_REF_UNIMPL(HYPRE_GMRESGetNumIterations)
VFS_REF_UNIMPL(HYPRE_GMRESGetFinalRelativeResidualNorm)
VFS_REF_UNIMPL(HYPRE_BoomerAMGCreate)
VFS_REF_UNIMPL(HYPRE_BoomerAMGDestroy)
VFS_REF_UNIMPL(HYPRE_BoomerAMGSetTol)
VFS_REF_UNIMPL(HYPRE_BoomerAMGSetStrongThreshold)
VFS_REF_UNIMPL(HYPRE_BoomerAMGSetPrintLevel)
VFS_REF_UNIMPL(HYPRE_BoomerAMGSetMaxIter)
VFS_REF_UNIMPL(HYPRE_BoomerAMGSetInterpType)
VFS_REF_UNIMPL(HYPRE_BoomerAMGSetCycleType)
VFS_REF_UNIMPL(HYPRE_BoomerAMGSetCoarsenType)
VFS_REF_UNIMPL(HYPRE_BoomerAMGSetAggNumLevels)
VFS_REF_UNIMPL(HYPRE_BoomerAMGSetRelaxType)
VFS_REF_UNIMPL(HYPRE_BoomerAMGSetNumSweeps)
VFS_REF_UNIMPL(HYPRE_BoomerAMGSetMaxLevels)
VFS_REF_UNIMPL(HYPRE_BoomerAMGSetPMaxElmts)

#endif
