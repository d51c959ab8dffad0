// Kernel launchers shared between the translation units of the library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "vfs_common.cuh"

namespace vfs {

// Metric pack offsets in units of N doubles (same order as the CPU oracle):
// csi eta zet (AoS, 3 each) aj | icsi ieta izet iaj | jcsi jeta jzet jaj |
// kcsi keta kzet kaj | cent.
enum {
  MP_CSI = 0, MP_ETA = 3, MP_ZET = 6, MP_AJ = 9,
  MP_ICSI = 10, MP_IETA = 13, MP_IZET = 16, MP_IAJ = 19,
  MP_JCSI = 20, MP_JETA = 23, MP_JZET = 26, MP_JAJ = 29,
  MP_KCSI = 30, MP_KETA = 33, MP_KZET = 36, MP_KAJ = 39,
  MP_CENT = 40, MP_TOTAL = 43
};

// ---- setup (k_setup.cu) ----
int launch_form_metrics(const Dims& d, const double* coor, double* M, double* tmp, cudaStream_t s);
int launch_gtensor(const Dims& d, const double* M, double* g, cudaStream_t s);
int launch_assemble(const Dims& d, const double* g, const double* nvert, const double* aj, double* coef, double* mcoef,
                    float* mcoef32, unsigned* mask, cudaStream_t s);
// face form of the aj-scaled operator (11-slot levels), FP32: per cell its
// +i face (g11, k-cross weight), +k face (g33, i-cross weight), +j face
// (g22), and aj with the one-sided code bits of the two cross terms in its
// four low mantissa bits; fc: the i-j and j-k cross weights of the general
// face form (OpView::ffc), zero on 11-slot levels
int launch_face_operator(const Dims& d, const double* g, const double* nvert, const double* aj, float2* fi, float2* fk,
                         float* fj, float* faj, float4* fc, cudaStream_t s);
int launch_coarsen(const Dims& f, const Dims& c, int si, int sj, int sk, const double* coor_f, const double* nv_f,
                   double* coor_c, double* nv_c, cudaStream_t s);
int launch_prolong_codes(const Dims& f, const Dims& c, int si, int sj, int sk, const double* nv_f, const double* nv_c,
                         uint8_t* code, cudaStream_t s);
// ccomp (nullable): labels of the level's connected fluid regions, one
// sigma e_q e_q^T term per region
int launch_dense_inverse(const Dims& d, const double* mcoef, double sigma, double* W, double* fac, int* piv, double* pval,
                         double* Binv, float* Binv32, int n, cudaStream_t s, const int* ccomp = nullptr);

// ---- stencils and multigrid (k_mg.cu) ----
// y = A x (FP64 accumulate; x FP64 or FP32); r = b - A x when b != nullptr.
int launch_apply64(const OpView<double>& A, const double* x, const double* b, double* y, cudaStream_t s);
int launch_apply64_xf(const OpView<double>& A, const float* x, const double* b, double* y, cudaStream_t s);
// y = A x with the FP32 face form of an 11-slot level (testing hook)
int launch_apply_face(const OpView<float>& A, const float* x, float* y, cudaStream_t s);
// multigrid operator apply in precision T (testing hook / residual)
template <typename T>
int launch_apply_mg(const OpView<T>& A, const T* x, const T* b, T* y, cudaStream_t s);
// one damped y-line Jacobi sweep: xo = xi + omega * T^{-1} (b - A xi); xi == nullptr means xi = 0;
// lf = precomputed y-line Thomas pivots 1/m_j (N of T)
// solo: this grid's solve has the GPU to itself (allows the low-occupancy
// variant on small levels)
// stage: on the face form, sweeps of levels of at least VFS_STAGE_MINCELLS
// interior cells run the kernel that stages operands this way (SweepStage:
// registers or tensor-memory copies)
template <typename T>
int launch_smooth(const OpView<T>& A, const T* lf, const T* xi, const T* b, T* xo, T omega, cudaStream_t s,
                 int cols = 0, bool solo = false, int stage = 0);
template <typename T>
int launch_line_factors(const Dims& d, const double* mcoef, T* lf, cudaStream_t s);
// FP16 diagonal-normalised copy of a level's aj-scaled operator (hidx layout), with
// optional fp32(1 / D) and fp32(D) per cell; its y-line pivots; its restriction
// weights max(0, 1 - nvert_f) D_f / D_c
// (*range |= 1 when a normalised coefficient or correction exceeds 6e4)
int launch_half_operator(const Dims& d, const double* mcoef, __half* h, float* dinv, float* dval, unsigned* range,
                         cudaStream_t s);
int launch_line_factors_half(const Dims& d, const __half* h, const double* mcoef, float* lf, cudaStream_t s);
int launch_restrict_weights_half(const Dims& f, const Dims& c, int si, int sj, int sk, const double* nvf,
                                 const double* mcf, const double* mcc, float* w, cudaStream_t s);
// fine residual r = b - A x restricted to the coarse rhs bc (MyRestriction); also zeroes xc.
// rw = the fine level's weights max(0, 1 - nvert) in T (launch_restrict_weights)
template <typename T>
int launch_residual_restrict(const OpView<T>& A, const T* x, const T* b, const T* rw, const Dims& c,
                             const double* nvc, int si, int sj, int sk, T* bc, T* xc, cudaStream_t s);
int launch_restrict_weights(size_t n, const double* nv, float* w32, double* w64, cudaStream_t s);
// plain restriction of a fine vector (testing hook)
template <typename T>
int launch_restrict(const Dims& f, const T* x, const double* nvf, const Dims& c, const double* nvc, int si, int sj, int sk,
                    T* out, cudaStream_t s);
// xf += P xc (MyInterpolation) using the prolongation codes of the fine level; add == 0 overwrites
template <typename T>
int launch_prolong(const Dims& f, const uint8_t* code, const Dims& c, const T* xc, T* xf, int add, const int* skip,
                   cudaStream_t s);
// x = Binv b over the packed interior of the coarsest level (b scaled by dsc first when dsc != nullptr)
template <typename T>
int launch_coarse_gemv(const Dims& d, const T* Binv, int n, const T* b, T* x, const T* dsc, const int* skip,
                       cudaStream_t s);
// fine-level preconditioner input: out = T(aj * v), or T(v) when aj is null; times dinv when given
template <typename T>
int launch_scale_in(const Dims& d, const double* aj, const double* v, T* out, const int* skip, cudaStream_t s,
                    const float* dinv = nullptr);

}  // namespace vfs
