// Launchers of the per-step FP64 kernels (k_proj.cu) and the Krylov kernels
// (k_krylov.cu).
#pragma once

#include <cuda_runtime.h>

#include "vfs_common.cuh"

namespace vfs {

// Contravariant flux Ucont as three component arrays (SoA) on the device.
struct Ucont {
  double *x, *y, *z;
};

int partial_blocks(const Dims& d);
int launch_finish_sums(const double* parts, int nparts, int nq, double* out, cudaStream_t s);
int launch_aos2soa(size_t n, const double* aos, double* x, double* y, double* z, cudaStream_t s);
int launch_soa2aos(size_t n, const double* x, const double* y, const double* z, double* aos, cudaStream_t s);
// comp / ncomp: labels 0..ncomp-1 of the connected fluid regions (nullptr
// when the fluid is one region): the compatibility fix and the mean removal
// then act per region.  sc holds 4 doubles for launch_rhs.
int launch_rhs(const Dims& d, const Ucont& u, const double* nvert, double dt, double st, double coeff, int meanfix,
               double* b, double* parts, double* sc, cudaStream_t s, const int* comp = nullptr, int ncomp = 1);
int launch_volume_flux(const Dims& d, int mode, const Ucont& u, const double* nvert, const double* M, double* parts,
                       double* fa4, cudaStream_t s,
                       const uint8_t* nb8 = nullptr);
int launch_remove_mean(const Dims& d, const double* nvert, double* x, double* parts, double* sc, cudaStream_t s,
                       const int* comp = nullptr, int ncomp = 1);
int launch_phi_finish(const Dims& d, const double* nvert, double* phi, cudaStream_t s);
int launch_update_pressure(const Dims& d, const double* nvert, const double* phi, double* p, cudaStream_t s);
int launch_proj_dots(const Dims& d, const double* M, double* pd, cudaStream_t s);
// nb8: nvert as bytes when every value is an integer in [0, 127] (exact
// integer pair tests), else nullptr (FP64 tests).  Projects the faces of
// planes [k0, k1) (k1 < 0: mz) and syncs their periodic ghosts.  A plane
// reads phi and the metrics alone, and the ghost sync of an interior plane
// reads that plane alone, so interior slabs may go in any order; the k ghost
// planes 0 and mz-1 (filled from planes mz-2 and 1) come after all of them.
int launch_projection(const Dims& d, const double* pd, const double* M, const double* nvert, const uint8_t* nb8,
                      const double* phi, double dt, double st, double coeff, const Ucont& u, cudaStream_t s,
                      int k0 = 0, int k1 = -1);
// The same projection on face weights and cross-term codes precomputed by
// launch_proj_weights (pw [9][N], pc [N]): FMAs, no nvert tests; equal to
// the reference's operation order to rounding (<= 1e-14 relative).
int launch_proj_weights(const Dims& d, const double* pd, const double* M, const double* nvert, double* pw, uint16_t* pc,
                        cudaStream_t s);
int launch_projection_fast(const Dims& d, const double* pw, const uint16_t* pc, const double* phi, double dt, double st,
                           double coeff, const Ucont& u, cudaStream_t s, int k0 = 0, int k1 = -1);
// periodic ghost sync of the Ucont components on planes [k0, k1)
int launch_ucont_ghosts(const Dims& d, const Ucont& u, int k0, int k1, cudaStream_t s);
// minv: per-cell inverse of the metric matrix [csi; eta; zet] (9 doubles,
// row-major), from launch_inverse_metric.
int launch_contra2cart(const Dims& d, const double* minv, const double* nvert, const Ucont& u, double* ucat, cudaStream_t s);
int launch_inverse_metric(const Dims& d, const double* M, const double* nvert, double* minv, cudaStream_t s);
// Divergence check with its block partials in a static device array (no
// allocation); returns 0, 1 (argument) or 2 (CUDA) and sets *why on error.
int divergence_max_static(int device, const Dims& d, const Ucont& u, const double* aj, const double* nvert, double* out,
                          cudaStream_t s, const char** why);
int launch_masked_absmax(const Dims& d, const double* r, const double* nvert, double* parts, double* out, cudaStream_t s,
                         const uint8_t* nb8 = nullptr);
int launch_divergence(const Dims& d, const Ucont& u, const double* aj, const double* nvert, double* parts, double* out,
                      cudaStream_t s,
                      const uint8_t* nb8 = nullptr);

// ---- FGMRES device state (k_krylov.cu) ----
// One flexible GMRES(m) solve keeps all of its scalars on the device so an
// iteration is a fixed sequence of launches with no host round trip; every
// kernel returns at once when the solve has converged.
struct KrylovState {
  int m;          // restart length
  int j;          // current Arnoldi column
  int done;       // 1 once converged (or broken down)
  int epoch;      // solve round, copied to the host beside done (a stale copy is recognisable)
  int it;         // preconditioner applications so far
  int reorth;     // 1 if the second Gram-Schmidt pass is needed this column
  double rtol, atol, bnorm, beta, resid;  // converged: resid <= rtol*bnorm and (atol <= 0 or resid <= atol)
  double hn, inv_hn;
  double* H;      // (m+1) x m, column-major: H[j*(m+1) + i]
  double* cs;     // m
  double* sn;     // m
  double* g;      // m+1
  double* y;      // m
  double* h;      // m+1 dots of the current pass
  double* hacc;   // m+1 accumulated dots of the column
  double* vs;     // m+1 column scales: basis vector q is vs[q] * V_q
  int orth2;      // 1: CGS2 (columns stored normalised, vs = 1)
};

// parts must hold nblocks * (m + 2) doubles.
int krylov_nblocks(size_t n);
int launch_norm_init(KrylovState* st, const double* r, size_t n, double* parts, int is_b, cudaStream_t s);
int launch_vec_scale_first(KrylovState* st, const double* r, double* v0, size_t n, cudaStream_t s);
int launch_multidot(KrylovState* st, const double* V, int nv, const double* w, size_t n, double* parts, int pass,
                    cudaStream_t s);
int launch_gs_update(KrylovState* st, const double* V, int nv, double* w, size_t n, double* parts, int pass, cudaStream_t s);
// In the Krylov kernels nv < 0 (and vn == nullptr) mean "take the column
// count from the device state", so one iteration is a fixed launch sequence.
// second CGS pass fused with the first update (capacity <= 32); returns -1 beyond
int launch_gs_update_dots(KrylovState* st, const double* V, int nv, double* w, size_t n, double* parts, cudaStream_t s,
                          int cap = 32);
template <typename T>
int launch_cgs_update(KrylovState* st, double* V, const double* w, T* out, size_t n, double* parts, cudaStream_t s,
                      const float* dinv = nullptr);
template <typename T>
int launch_vnext_in(KrylovState* st, const double* w, double* vn, T* out, size_t n, cudaStream_t s, double* V = nullptr,
                    const float* dinv = nullptr);
// w = A z (aj-scaled FP64 operator, z in T) and Z[st->j] = z on the interior
template <typename T>
int launch_apply64_krylov(const OpView<double>& A, const T* z, T* Z, const KrylovState* st, double* w, cudaStream_t s);
int launch_arnoldi_finish(KrylovState* st, int nparts, const double* parts, cudaStream_t s);
int launch_vnext(KrylovState* st, const double* w, double* vn, size_t n, cudaStream_t s);
int launch_lsq_update(KrylovState* st, cudaStream_t s);
template <typename T>
int launch_x_update(KrylovState* st, const T* Z, size_t n, double* x, cudaStream_t s);
int launch_restart_reset(KrylovState* st, cudaStream_t s);
int launch_status_copy(const KrylovState* st, int* hst, cudaStream_t s);
int launch_norm2(const double* v, size_t n, double* parts, double* out, cudaStream_t s);

}  // namespace vfs
