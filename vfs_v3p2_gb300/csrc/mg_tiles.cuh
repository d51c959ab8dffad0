// Device bodies of the multigrid kernels, shared by the stand-alone
// kernels (k_mg.cu: one launch per sweep, restriction, prolongation and
// coarsest solve of one grid) and the grouped kernels of batched solves
// (k_group.cu: one launch per V-cycle operation for many grids): the
// stencil gathers, the face form, the y-line sweep's phases, and the tile
// bodies of the sweep, the residual restriction, the prolongation and the
// coarsest-level product, each parametrised by its tile coordinates.
#pragma once
#include <type_traits>

#include "vfs_common.cuh"

namespace vfs {


constexpr int TX = 32, TY = 8, KCHUNK = 4;
// Register budget of the stencil kernels: resident blocks per SM the
// compiler must allow (4 -> 64 registers, room for a cell's coefficient and
// neighbour loads to be in flight together).
#ifndef VFS_STENCIL_MINB
#define VFS_STENCIL_MINB 4
#endif

__host__ __forceinline__ dim3 tile_grid(const Dims& d) {
  const int ni = d.mx - 2, nj = d.my - 2, nk = d.mz - 2;
  return dim3((ni + TX - 1) / TX, (nj + TY - 1) / TY, (nk + KCHUNK - 1) / KCHUNK);
}

#define TILE_LOOP(d)                                                       \
  const int i = 1 + blockIdx.x * TX + threadIdx.x;                         \
  const int j = 1 + blockIdx.y * TY + threadIdx.y;                         \
  const bool _in = (i <= (d).mx - 2) && (j <= (d).my - 2);                 \
  const int _k0 = 1 + blockIdx.z * KCHUNK;                                 \
  const int _k1 = min(_k0 + KCHUNK, (d).mz - 1);                           \
  for (int k = _k0; k < _k1; k++)

// Slot sets known at compile time: MASK_CH holds the slots of grids whose
// metric has no i-j and no j-k cross terms (x-z skew, y stretching: the
// channel and sphere grids), MASK_ALL all 19.  A level whose nonzero slots
// fit MASK_CH runs the 11-slot instantiation.  With the set fixed at compile
// time every load of a stencil is issued before its FMAs (no per-slot
// branch), which keeps ~2 x slots loads in flight per cell.
constexpr unsigned MASK_ALL = 0x7FFFFu;
constexpr unsigned MASK_CH = (1u << CP) | (1u << EP) | (1u << WP) | (1u << NP) | (1u << SP) | (1u << TP) | (1u << BP) |
                             (1u << TE) | (1u << BE) | (1u << TW) | (1u << BW);

// sum_m coef[m] * x[nbr(m)] over the slots of MASK for interior cell (i, j, k).
// Addresses are one 32-bit cell offset plus three per-axis offsets with the
// periodic wrap folded in (i - 1 of i = 1 is mx - 2, i + 1 of i = mx - 2 is
// 1); grids stay below 2^31 cells (checked at creation).  The slot base
// coef + m N is formed in 64 bits (uniform across the block).
template <unsigned MASK, typename TC, typename TX_, typename TA>
__device__ __forceinline__ TA stencil(const Dims& d, const TC* __restrict__ coef, const TX_* __restrict__ x, int i, int j,
                                      int k) {
  const int sy = d.mx, sz = d.mx * d.my;
  const int N = sz * d.mz;
  const int c = k * sz + j * sy + i;
  const int oi[3] = {(i == 1 && d.ip) ? d.mx - 3 : -1, 0, (i == d.mx - 2 && d.ip) ? 3 - d.mx : 1};
  const int oj[3] = {((j == 1 && d.jp) ? d.my - 3 : -1) * sy, 0, ((j == d.my - 2 && d.jp) ? 3 - d.my : 1) * sy};
  const int ok[3] = {((k == 1 && d.kp) ? d.mz - 3 : -1) * sz, 0, ((k == d.mz - 2 && d.kp) ? 3 - d.mz : 1) * sz};
  TC cv[19];
  TX_ xv[19];
#pragma unroll
  for (int m = 0; m < 19; m++) {
    if (MASK & (1u << m)) {
      cv[m] = __ldg((coef + (size_t)m * N) + c);
      xv[m] = __ldg(x + (c + oi[slot_di(m) + 1] + oj[slot_dj(m) + 1] + ok[slot_dk(m) + 1]));
    }
  }
  TA s = TA(0);
#pragma unroll
  for (int m = 0; m < 19; m++)
    if (MASK & (1u << m)) s = fma((TA)cv[m], (TA)xv[m], s);
  return s;
}

// The two halves of stencil(), for kernels that gather several cells before
// summing: the MASK slots' coefficients and neighbour values (x == nullptr:
// coefficients only), then the sum in slot order.
template <unsigned MASK, typename TC, typename TX_>
__device__ __forceinline__ void stencil_gather(const Dims& d, const TC* __restrict__ coef, const TX_* __restrict__ x,
                                               int i, int j, int k, TC* cv, TX_* xv) {
  const int sy = d.mx, sz = d.mx * d.my;
  const int N = sz * d.mz;
  const int c = k * sz + j * sy + i;
  const int oi[3] = {(i == 1 && d.ip) ? d.mx - 3 : -1, 0, (i == d.mx - 2 && d.ip) ? 3 - d.mx : 1};
  const int oj[3] = {((j == 1 && d.jp) ? d.my - 3 : -1) * sy, 0, ((j == d.my - 2 && d.jp) ? 3 - d.my : 1) * sy};
  const int ok[3] = {((k == 1 && d.kp) ? d.mz - 3 : -1) * sz, 0, ((k == d.mz - 2 && d.kp) ? 3 - d.mz : 1) * sz};
#pragma unroll
  for (int m = 0; m < 19; m++) {
    if (MASK & (1u << m)) {
      cv[m] = __ldg((coef + (size_t)m * N) + c);
      xv[m] = x ? __ldg(x + (c + oi[slot_di(m) + 1] + oj[slot_dj(m) + 1] + ok[slot_dk(m) + 1])) : TX_(0);
    }
  }
}
template <unsigned MASK, typename TA, typename TC, typename TX_>
__device__ __forceinline__ TA stencil_dot(const TC* cv, const TX_* xv) {
  TA s = TA(0);
#pragma unroll
  for (int m = 0; m < 19; m++)
    if (MASK & (1u << m)) s = fma((TA)cv[m], to_acc<TA>(xv[m]), s);
  return s;
}

// stencil_gather for the FP16 operator (hidx layout; x as in stencil_gather).
template <unsigned MASK, typename TX_>
__device__ __forceinline__ void stencil_gather_h(const Dims& d, const __half* __restrict__ h, const TX_* __restrict__ x,
                                                 int i, int j, int k, __half* cv, TX_* xv) {
  const int sy = d.mx, sz = d.mx * d.my;
  const int c = k * sz + j * sy + i;
  const size_t hs = hslot(d), hc = hidx(d, i, j, k);
  const int oi[3] = {(i == 1 && d.ip) ? d.mx - 3 : -1, 0, (i == d.mx - 2 && d.ip) ? 3 - d.mx : 1};
  const int oj[3] = {((j == 1 && d.jp) ? d.my - 3 : -1) * sy, 0, ((j == d.my - 2 && d.jp) ? 3 - d.my : 1) * sy};
  const int ok[3] = {((k == 1 && d.kp) ? d.mz - 3 : -1) * sz, 0, ((k == d.mz - 2 && d.kp) ? 3 - d.mz : 1) * sz};
#pragma unroll
  for (int m = 0; m < 19; m++) {
    if (MASK & (1u << m)) {
      cv[m] = __ldg(h + (size_t)m * hs + hc);
      xv[m] = x ? __ldg(x + (c + oi[slot_di(m) + 1] + oj[slot_dj(m) + 1] + ok[slot_dk(m) + 1])) : TX_(0);
    }
  }
}
template <unsigned MASK, typename TC, typename TX_>
__device__ __forceinline__ void gather(const Dims& d, const TC* __restrict__ coef, const TX_* __restrict__ x, int i,
                                       int j, int k, TC* cv, TX_* xv) {
  if constexpr (std::is_same<TC, __half>::value) stencil_gather_h<MASK>(d, coef, x, i, j, k, cv, xv);
  else stencil_gather<MASK>(d, coef, x, i, j, k, cv, xv);
}

struct FaceOp;

// Coefficient array of a view in storage type TC: the level's own (TC = T)
// or its FP16 diagonal-normalised copy (TC = __half).
template <typename TC, typename T>
__device__ __forceinline__ const TC* coef_ptr(const OpView<T>& A) {
  if constexpr (std::is_same<TC, __half>::value) return A.hcoef;
  else if constexpr (std::is_same<TC, FaceOp>::value) return nullptr;
  else return A.coef;
}

// Row sum of gathered slots in either storage: sum_m coef_m x_m in slot
// order, or for the FP16 diagonal-normalised operator x_c first and then
// the slots (the centre slot holds the row-sum correction delta).
template <unsigned MASK, typename TA, typename TC, typename TX_>
__device__ __forceinline__ TA row_dot(const TC* cv, const TX_* xv) {
  if constexpr (std::is_same<TC, __half>::value) {
    TA s = to_acc<TA>(xv[CP]);
#pragma unroll
    for (int m = 0; m < 19; m++)
      if (MASK & (1u << m)) s = fma(to_acc<TA>(cv[m]), to_acc<TA>(xv[m]), s);
    return s;
  } else {
    return stencil_dot<MASK, TA>(cv, xv);
  }
}

// Stencil at (i, j, k) clamped into the interior (columns and rows past the
// last interior one of a partial tile read the last one's data; the caller
// discards them), with every load issued before the first FMA.
template <unsigned MASK, typename TA, typename TC, typename TX_>
__device__ __forceinline__ TA stencil_clamped(const Dims& d, const TC* __restrict__ coef, const TX_* __restrict__ x,
                                              int i, int j, int k) {
  TC cv[19];
  TX_ xv[19];
  stencil_gather<MASK>(d, coef, x, min(i, d.mx - 2), min(j, d.my - 2), k, cv, xv);
  return stencil_dot<MASK, TA>(cv, xv);
}

__host__ __forceinline__ bool fits_ch(unsigned mask) { return (mask & ~MASK_CH) == 0u; }

// Storage tag of the FP32 multigrid's face form (OpView::ffi ...): the row
// is aj times the divergence of six face fluxes (k_face_operator).
struct FaceOp {};

// Row of the face-form operator at a cell from its 11 stencil values (slot
// order of the 11-slot set: C E W N S T B TE BE TW BW), its own +i, +j, +k
// faces, the -i face of its i-1 neighbour, the -j of j-1 and the -k of k-1.
// Returns aj (A x)_c; a and cn: the row's SP and NP coefficients.
struct FaceData {
  float2 fic, fiw, fkc, fkb;  // (normal, cross weight) of the +i faces of c, c-i and the +k faces of c, c-k
  float gjc, gjs, aj;
  unsigned cc, cw, cb;        // code bits of c, c-i, c-k
};
// aj of the face form with its code bits cleared, and the code bits.
__device__ __forceinline__ float face_aj(float v) { return __int_as_float(__float_as_int(v) & ~0xF); }
__device__ __forceinline__ unsigned face_code(float v) { return (unsigned)__float_as_int(v) & 0xFu; }
__device__ __forceinline__ float face_row(const FaceData& f, const float* x) {
  const float xc = x[CP], xe = x[EP], xw = x[WP], xn = x[NP], xs = x[SP], xt = x[TP], xb = x[BP];
  const float xte = x[TE], xbe = x[BE], xtw = x[TW], xbw = x[BW];
  // +i face of c: the pair (C, E) at k+1 / k / k-1
  const float ce = xc + xe, te = xt + xte, be = xb + xbe;
  const float Fic = f.fic.x * (xe - xc) + f.fic.y * (((f.cc & 1u) ? ce : te) - ((f.cc & 2u) ? ce : be));
  // +i face of c-i: the pair (W, C)
  const float wc = xw + xc, tw = xtw + xt, bw = xbw + xb;
  const float Fiw = f.fiw.x * (xc - xw) + f.fiw.y * (((f.cw & 1u) ? wc : tw) - ((f.cw & 2u) ? wc : bw));
  // +k face of c: the pair (C, T) at i+1 / i / i-1
  const float ct = xc + xt, ete = xe + xte, wtw = xw + xtw;
  const float Fkc = f.fkc.x * (xt - xc) + f.fkc.y * (((f.cc & 4u) ? ct : ete) - ((f.cc & 8u) ? ct : wtw));
  // +k face of c-k: the pair (B, C)
  const float bc = xb + xc, eb = xbe + xe, wb = xbw + xw;
  const float Fkb = f.fkb.x * (xc - xb) + f.fkb.y * (((f.cb & 4u) ? bc : eb) - ((f.cb & 8u) ? bc : wb));
  const float Fj = f.gjc * (xn - xc) - f.gjs * (xc - xs);
  return f.aj * ((Fic - Fiw) + Fj + (Fkc - Fkb));
}
// The face data and the 11 stencil values of interior cell (i, j, k), every
// load issued before any arithmetic (periodic wraps as in stencil_gather).
__device__ __forceinline__ void face_gather(const OpView<float>& A, const float* __restrict__ x, int i, int j, int k,
                                            FaceData& f, float* xv) {
  const Dims d = A.d;
  const int sy = d.mx, sz = d.mx * d.my;
  const int c = k * sz + j * sy + i;
  const int oiW = (i == 1 && d.ip) ? d.mx - 3 : -1, oiE = (i == d.mx - 2 && d.ip) ? 3 - d.mx : 1;
  const int ojS = ((j == 1 && d.jp) ? d.my - 3 : -1) * sy, ojN = ((j == d.my - 2 && d.jp) ? 3 - d.my : 1) * sy;
  const int okB = ((k == 1 && d.kp) ? d.mz - 3 : -1) * sz, okT = ((k == d.mz - 2 && d.kp) ? 3 - d.mz : 1) * sz;
  f.fic = __ldg(A.ffi + c);
  f.fiw = __ldg(A.ffi + c + oiW);
  f.fkc = __ldg(A.ffk + c);
  f.fkb = __ldg(A.ffk + c + okB);
  f.gjc = __ldg(A.ffj + c);
  f.gjs = __ldg(A.ffj + c + ojS);
  const float ajc = __ldg(A.faj + c), ajw = __ldg(A.faj + c + oiW), ajb = __ldg(A.faj + c + okB);
  xv[CP] = __ldg(x + c);
  xv[EP] = __ldg(x + c + oiE);
  xv[WP] = __ldg(x + c + oiW);
  xv[NP] = __ldg(x + c + ojN);
  xv[SP] = __ldg(x + c + ojS);
  xv[TP] = __ldg(x + c + okT);
  xv[BP] = __ldg(x + c + okB);
  xv[TE] = __ldg(x + c + okT + oiE);
  xv[BE] = __ldg(x + c + okB + oiE);
  xv[TW] = __ldg(x + c + okT + oiW);
  xv[BW] = __ldg(x + c + okB + oiW);
  f.aj = face_aj(ajc);
  f.cc = face_code(ajc);
  f.cw = face_code(ajw);
  f.cb = face_code(ajb);
}


// The general face form (levels with i-j or j-k cross terms): face_row's
// fluxes plus the four cross terms ffc holds.  A cross weight carries its own
// code in its two low mantissa bits (face_xw clears them, face_xc reads them).
__device__ __forceinline__ float face_xw(float v) { return __int_as_float(__float_as_int(v) & ~3); }
__device__ __forceinline__ unsigned face_xc(float v) { return (unsigned)__float_as_int(v) & 3u; }
struct FaceX {
  float ijc, ijw;  // j cross weight of the +i faces of c and c-i (with their codes)
  float jic, jkc;  // i and k cross weights of the +j face of c
  float jis, jks;  // the same of the +j face of c-j
  float kjc, kjb;  // j cross weight of the +k faces of c and c-k
};
// w (U - L) of a cross term: U is the pair at +1 or, one-sided, the face's
// centre pair ctr; L the pair at -1 or the centre pair.
__device__ __forceinline__ float face_cross(float w, float ctr, float up, float dn) {
  const unsigned q = face_xc(w);
  return face_xw(w) * (((q & 1u) ? ctr : up) - ((q & 2u) ? ctr : dn));
}
// Row of the general face form from the 19 stencil values: aj times the
// divergence of the six face fluxes, each with its normal term and both
// cross terms (poisson.c:1173-1558: the i+1 face's g12 and g13 pairs, the
// j+1 face's g21 and g23 pairs, the k+1 face's g31 and g32 pairs).
__device__ __forceinline__ float face_row_all(const FaceData& f, const FaceX& e, const float* x) {
  const float xc = x[CP], xe = x[EP], xw = x[WP], xn = x[NP], xs = x[SP], xt = x[TP], xb = x[BP];
  const float xte = x[TE], xbe = x[BE], xtw = x[TW], xbw = x[BW];
  const float xne = x[NE], xse = x[SE], xnw = x[NW], xsw = x[SW], xtn = x[TN], xbn = x[BN], xts = x[TS], xbs = x[BS];
  // +i face of c: the pair (C, E) at k+1 / k-1 and at j+1 / j-1
  const float ce = xc + xe, te = xt + xte, be = xb + xbe;
  const float Fic = f.fic.x * (xe - xc) + f.fic.y * (((f.cc & 1u) ? ce : te) - ((f.cc & 2u) ? ce : be)) +
                    face_cross(e.ijc, ce, xn + xne, xs + xse);
  // +i face of c-i: the pair (W, C)
  const float wc = xw + xc, tw = xtw + xt, bw = xbw + xb;
  const float Fiw = f.fiw.x * (xc - xw) + f.fiw.y * (((f.cw & 1u) ? wc : tw) - ((f.cw & 2u) ? wc : bw)) +
                    face_cross(e.ijw, wc, xnw + xn, xsw + xs);
  // +j face of c: the pair (C, N) at i+1 / i-1 and at k+1 / k-1
  const float cn = xc + xn;
  const float Fjc = f.gjc * (xn - xc) + face_cross(e.jic, cn, xe + xne, xw + xnw) + face_cross(e.jkc, cn, xt + xtn, xb + xbn);
  // +j face of c-j: the pair (S, C)
  const float sc = xs + xc;
  const float Fjs = f.gjs * (xc - xs) + face_cross(e.jis, sc, xse + xe, xsw + xw) + face_cross(e.jks, sc, xts + xt, xbs + xb);
  // +k face of c: the pair (C, T) at i+1 / i-1 and at j+1 / j-1
  const float ct = xc + xt, ete = xe + xte, wtw = xw + xtw;
  const float Fkc = f.fkc.x * (xt - xc) + f.fkc.y * (((f.cc & 4u) ? ct : ete) - ((f.cc & 8u) ? ct : wtw)) +
                    face_cross(e.kjc, ct, xn + xtn, xs + xts);
  // +k face of c-k: the pair (B, C)
  const float bc = xb + xc, eb = xbe + xe, wb = xbw + xw;
  const float Fkb = f.fkb.x * (xc - xb) + f.fkb.y * (((f.cb & 4u) ? bc : eb) - ((f.cb & 8u) ? bc : wb)) +
                    face_cross(e.kjb, bc, xbn + xn, xbs + xs);
  return f.aj * ((Fic - Fiw) + (Fjc - Fjs) + (Fkc - Fkb));
}
// The row's S and N coefficients (its j-line couplings) over aj: the
// coefficients of x_S and x_N in face_row_all's divergence -- the j faces'
// normal weights, the j cross terms of the i and k faces (the pair at j-1 or
// j+1 unless the regime takes the centre pair) and the j faces' cross terms
// whose centre pair is the pair they take.
__device__ __forceinline__ void face_row_sn(const FaceData& f, const FaceX& e, float& s, float& n) {
  auto nq1 = [](float w) { return (face_xc(w) & 1u) ? 0.f : face_xw(w); };  // upper pair at +1
  auto nq2 = [](float w) { return (face_xc(w) & 2u) ? 0.f : face_xw(w); };  // lower pair at -1
  auto ctr = [](float w) {  // the centre pair: +w as the upper pair, -w as the lower one
    const unsigned q = face_xc(w);
    return ((q & 1u) ? face_xw(w) : 0.f) - ((q & 2u) ? face_xw(w) : 0.f);
  };
  s = f.gjs - nq2(e.ijc) + nq2(e.ijw) - nq2(e.kjc) + nq2(e.kjb) - ctr(e.jis) - ctr(e.jks);
  n = f.gjc + nq1(e.ijc) - nq1(e.ijw) + nq1(e.kjc) - nq1(e.kjb) + ctr(e.jic) + ctr(e.jkc);
}
// face_gather plus the cross weights of c, c-i, c-j, c-k and the eight x
// values face_row leaves out (NE SE NW SW TN BN TS BS), periodic wraps as in
// stencil_gather.
__device__ __forceinline__ void face_gather_all(const OpView<float>& A, const float* __restrict__ x, int i, int j,
                                                int k, FaceData& f, FaceX& e, float* xv) {
  const Dims d = A.d;
  const int sy = d.mx, sz = d.mx * d.my;
  const int c = k * sz + j * sy + i;
  const int oiW = (i == 1 && d.ip) ? d.mx - 3 : -1, oiE = (i == d.mx - 2 && d.ip) ? 3 - d.mx : 1;
  const int ojS = ((j == 1 && d.jp) ? d.my - 3 : -1) * sy, ojN = ((j == d.my - 2 && d.jp) ? 3 - d.my : 1) * sy;
  const int okB = ((k == 1 && d.kp) ? d.mz - 3 : -1) * sz, okT = ((k == d.mz - 2 && d.kp) ? 3 - d.mz : 1) * sz;
  const float* __restrict__ fc = reinterpret_cast<const float*>(A.ffc);
  const float4 own = __ldg(A.ffc + c);
  e.ijw = __ldg(fc + 4 * (size_t)(c + oiW));
  e.jis = __ldg(fc + 4 * (size_t)(c + ojS) + 1);
  e.jks = __ldg(fc + 4 * (size_t)(c + ojS) + 2);
  e.kjb = __ldg(fc + 4 * (size_t)(c + okB) + 3);
  xv[NE] = __ldg(x + c + oiE + ojN);
  xv[SE] = __ldg(x + c + oiE + ojS);
  xv[NW] = __ldg(x + c + oiW + ojN);
  xv[SW] = __ldg(x + c + oiW + ojS);
  xv[TN] = __ldg(x + c + okT + ojN);
  xv[BN] = __ldg(x + c + okB + ojN);
  xv[TS] = __ldg(x + c + okT + ojS);
  xv[BS] = __ldg(x + c + okB + ojS);
  face_gather(A, x, i, j, k, f, xv);
  e.ijc = own.x;
  e.jic = own.y;
  e.jkc = own.z;
  e.kjc = own.w;
}


// ---------------------------------------------------------------------------
// Damped y-line Jacobi sweep: xo = xi + omega * T^{-1} (b - A xi), T the
// tridiagonal j-coupling (SP, CP, NP) of each (i, k) column.  T is constant
// per level, so its Thomas factors c'_j and 1/m_j are precomputed at setup
// (k_line_factors) and the per-column recurrences are one FMA (forward) and
// one FMA (backward) deep.  One block owns TW consecutive i-columns x all j
// of one k plane: phase 1 (all threads, coalesced over i) forms the residual
// and stages it with the factors in shared memory, phase 2 (one thread per
// column) runs the two substitutions, phase 3 writes xo.  Couplings across a
// j-periodic seam and to non-fluid cells stay in the residual; non-fluid
// cells have delta = 0.
// ---------------------------------------------------------------------------
#ifndef VFS_SMOOTH_NT
#define VFS_SMOOTH_NT 256  // threads per block
#endif
#ifndef VFS_SMOOTH_MINB
#define VFS_SMOOTH_MINB 4  // resident blocks per SM the register budget must allow
#endif
#ifndef VFS_SMOOTH_MINB_HALF
#define VFS_SMOOTH_MINB_HALF 3  // the same for the two-cells-per-thread FP16 sweep (more registers)
#endif
#ifndef VFS_SMOOTH_PAIR_MAXN
#define VFS_SMOOTH_PAIR_MAXN 0  // 11-slot FP16 levels up to this many cells sweep two cells per thread (measured: none faster)
#endif
#ifndef VFS_SMOOTH_U
#define VFS_SMOOTH_U 1  // cells whose loads one thread issues together in phase 1 (large levels)
#endif
#ifndef VFS_SMOOTH_U_SMALL
#define VFS_SMOOTH_U_SMALL 2  // the same on levels with fewer than two blocks per SM
#endif
#ifndef VFS_SMOOTH_TWMAX
#define VFS_SMOOTH_TWMAX 32  // columns per block
#endif
#ifndef VFS_SMOOTH_PF
#define VFS_SMOOTH_PF 1  // phase-1 rows prefetched into L2 this many iterations ahead (0: off), FP32 operator
#endif
#ifndef VFS_SMOOTH_PF_HALF
#define VFS_SMOOTH_PF_HALF 0  // the same for the FP16 operator and the face form (measured: the prefetches cost more
                              // than they save; face form 55.4 -> 78 us per finest sweep one to three row bands ahead)
#endif
#ifndef VFS_SMOOTH_MINBLK
#define VFS_SMOOTH_MINBLK 152  // automatic tile: narrow while a sweep has fewer blocks (one per SM)
#endif
#ifndef VFS_SMOOTH_TWMIN
#define VFS_SMOOTH_TWMIN 8  // automatic tile: narrowest width
#endif
#ifndef VFS_SMOOTH_U3
#define VFS_SMOOTH_U3 8  // phase-3 (write) loop unroll
#endif
#ifndef VFS_SMOOTH_CARVE
#define VFS_SMOOTH_CARVE -1  // preferred shared-memory carveout in percent (-1: the driver's choice)
#endif

// Phase 1 of the sweep on the FP16 operator, two cells per thread (see the
// caller); writes su, sp, sl of the tile.
template <unsigned MASK, typename T>
__device__ __forceinline__ void smooth_pairs(const OpView<T>& A, const T* __restrict__ lf, const T* __restrict__ xi,
                                             const T* __restrict__ b, T* su, T* sp, T* sl, int i0, int k, int TW) {
  const Dims d = A.d;
  const __half* __restrict__ h = A.hcoef;
  const int nj = d.my - 2, np = TW >> 1;
  const int sy = d.mx, sz = d.mx * d.my;
  const size_t hs = hslot(d);
  const int lastodd = d.mx - 2 - ((d.mx - 1) & 1);  // largest odd column <= mx - 2
  const int kk[3] = {(k == 1 && d.kp) ? d.mz - 2 : k - 1, k, (k == d.mz - 2 && d.kp) ? 1 : k + 1};
  // np divides the block: the thread keeps its pair p and steps rows
  const int p = threadIdx.x % np, jstep = VFS_SMOOTH_NT / np;
  const int ia = i0 + 2 * p, ib = ia + 1;
  const int ca = min(ia, d.mx - 2), cb = min(ib, d.mx - 2);
  const int la = min(ia, lastodd);  // the aligned word holding the pair (clamped)
  const int cL = (ca == 1 && d.ip) ? d.mx - 2 : ca - 1;
  const int cR = (cb == d.mx - 2 && d.ip) ? 1 : cb + 1;
  const bool sep = ca < cb;  // two distinct cells (else b is the clamped copy of a)
  const size_t hrow1 = hidx(d, la, 1, k);
  const int hp = hpitch(d);
  for (int jl = threadIdx.x / np; jl < nj; jl += jstep) {
    const int j = 1 + jl;
    const int jm = (j == 1 && d.jp) ? nj : j - 1, jp1 = (j == nj && d.jp) ? 1 : j + 1;
    const size_t hrow = hrow1 + (size_t)jl * hp;
    __half2 cw[19];
    T xL[3][3], xA[3][3], xB[3][3], xR[3][3];  // [dk + 1][dj + 1]
#pragma unroll
    for (int m = 0; m < 19; m++)
      if ((MASK & (1u << m)) && (xi || m == SP || m == NP)) cw[m] = __ldg((const __half2*)(h + (size_t)m * hs + hrow));
    if (xi) {
#pragma unroll
      for (int dk = -1; dk <= 1; dk++)
#pragma unroll
        for (int dj = -1; dj <= 1; dj++) {
          bool any = false, side = false;
#pragma unroll
          for (int m = 0; m < 19; m++)
            if ((MASK & (1u << m)) && slot_dj(m) == dj && slot_dk(m) == dk) {
              any = true;
              if (slot_di(m) != 0) side = true;
            }
          if (!any) continue;
          const int row = kk[dk + 1] * sz + (dj < 0 ? jm : (dj > 0 ? jp1 : j)) * sy;
          xA[dk + 1][dj + 1] = __ldg(xi + row + ca);
          xB[dk + 1][dj + 1] = __ldg(xi + row + cb);
          if (side) {
            xL[dk + 1][dj + 1] = __ldg(xi + row + cL);
            xR[dk + 1][dj + 1] = __ldg(xi + row + cR);
          }
        }
    }
    const int ra = k * sz + j * sy + ca, rb = k * sz + j * sy + cb;
    const T bba = __ldg(b + ra), bbb = __ldg(b + rb), iva = __ldg(lf + ra), ivb = __ldg(lf + rb);
#pragma unroll
    for (int e = 0; e < 2; e++) {
      __half cv[19];
      T xv[19];
#pragma unroll
      for (int m = 0; m < 19; m++) {
        if (!(MASK & (1u << m))) continue;
        if (xi || m == SP || m == NP) cv[m] = e == 0 ? __low2half(cw[m]) : __high2half(cw[m]);
        if (!xi) continue;
        const int di = slot_di(m), dj = slot_dj(m) + 1, dk = slot_dk(m) + 1;
        if (e == 0) xv[m] = di < 0 ? xL[dk][dj] : (di > 0 ? (sep ? xB[dk][dj] : xR[dk][dj]) : xA[dk][dj]);
        else xv[m] = di < 0 ? (sep ? xA[dk][dj] : xL[dk][dj]) : (di > 0 ? xR[dk][dj] : xB[dk][dj]);
      }
      const int il = 2 * p + e;
      const bool live = i0 + il <= d.mx - 2;
      const T ax = xi ? row_dot<MASK, T>(cv, xv) : T(0);
      const T a = jl > 0 ? to_acc<T>(cv[SP]) : T(0), cn = jl < nj - 1 ? to_acc<T>(cv[NP]) : T(0);
      const T bb = e == 0 ? bba : bbb, inv = e == 0 ? iva : ivb;
      const int idx = jl * TW + il;
      su[idx] = live ? (bb - ax) * inv : T(0);
      sp[idx] = live ? a * inv : T(0);
      sl[idx] = live ? cn * inv : T(0);
    }
  }
}

// Phase 2 of the sweep for column il of a tile: forward substitution
// y_j = su_j - sp_j y_{j-1}, then backward delta_j = y_j - sl_j delta_{j+1},
// both in place in su.  The operands of 8 rows are read into registers
// before their 8 dependent FMAs (the staged arrays share one buffer, so a
// plain loop would order every load after the previous row's store), which
// leaves only the FMA chain on the critical path; the arithmetic is the
// same row by row.
template <typename T>
__device__ __forceinline__ void line_solve(T* su, const T* sp, const T* sl, int nj, int TW, int il) {
  constexpr int B = 8;
  T y = T(0);
  int jl = 0;
  for (; jl + B <= nj; jl += B) {
    T a[B], r[B];
#pragma unroll
    for (int u = 0; u < B; u++) {
      a[u] = sp[(jl + u) * TW + il];
      r[u] = su[(jl + u) * TW + il];
    }
#pragma unroll
    for (int u = 0; u < B; u++) {
      y = fma(-a[u], y, r[u]);
      su[(jl + u) * TW + il] = y;
    }
  }
  for (; jl < nj; jl++) {
    y = fma(-sp[jl * TW + il], y, su[jl * TW + il]);
    su[jl * TW + il] = y;
  }
  T xn = T(0);
  jl = nj - 1;
  for (; jl - B + 1 >= 0; jl -= B) {
    T c[B], r[B];
#pragma unroll
    for (int u = 0; u < B; u++) {
      c[u] = sl[(jl - u) * TW + il];
      r[u] = su[(jl - u) * TW + il];
    }
#pragma unroll
    for (int u = 0; u < B; u++) {
      xn = fma(-c[u], xn, r[u]);
      su[(jl - u) * TW + il] = xn;
    }
  }
  for (; jl >= 0; jl--) {
    xn = fma(-sl[jl * TW + il], xn, su[jl * TW + il]);
    su[jl * TW + il] = xn;
  }
}

// Shared memory of a sweep tile: su, sp, sl (TW x nj each).
template <typename T>
__host__ __device__ inline size_t smooth_smem(int tw, int nj) {
  return (size_t)3 * tw * nj * sizeof(T);
}

// Phase 1 of the sweep on the face form (FP32): U cells per thread batch,
// every load issued before the arithmetic; writes su, sp, sl of the tile.
// From a zero guess (ZG) the residual is b and only the j faces and aj are
// read.  Non-fluid rows (aj = 0) stage zeros.
template <int U, bool ZG>
__device__ __forceinline__ void face_phase1(const OpView<float>& A, const float* __restrict__ lf,
                                            const float* __restrict__ xi, const float* __restrict__ b, float* su,
                                            float* sp, float* sl, int i0, int k, int tw) {
  const Dims d = A.d;
  const int nj = d.my - 2, sy = d.mx, sz = d.mx * d.my;
  const int okB = ((k == 1 && d.kp) ? d.mz - 3 : -1) * sz, okT = ((k == d.mz - 2 && d.kp) ? 3 - d.mz : 1) * sz;
  for (int base = threadIdx.x; base < tw * nj; base += U * VFS_SMOOTH_NT) {
    FaceData f[U];
    float xv[U][11], bb[U], inv[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int idx = min(base + u * VFS_SMOOTH_NT, tw * nj - 1);
      const int il = idx % tw, jl = idx / tw;
      const int i = min(i0 + il, d.mx - 2), j = 1 + jl;
      const int c = k * sz + j * sy + i;
      const int oiW = (i == 1 && d.ip) ? d.mx - 3 : -1, oiE = (i == d.mx - 2 && d.ip) ? 3 - d.mx : 1;
      const int ojS = ((j == 1 && d.jp) ? d.my - 3 : -1) * sy, ojN = ((j == d.my - 2 && d.jp) ? 3 - d.my : 1) * sy;
      f[u].gjc = __ldg(A.ffj + c);
      f[u].gjs = __ldg(A.ffj + c + ojS);
      f[u].aj = __ldg(A.faj + c);  // code bits still set: split below
      if (!ZG) {
        f[u].fic = __ldg(A.ffi + c);
        f[u].fiw = __ldg(A.ffi + c + oiW);
        f[u].fkc = __ldg(A.ffk + c);
        f[u].fkb = __ldg(A.ffk + c + okB);
        f[u].cw = face_code(__ldg(A.faj + c + oiW));
        f[u].cb = face_code(__ldg(A.faj + c + okB));
        xv[u][0] = __ldg(xi + c);
        xv[u][1] = __ldg(xi + c + oiE);
        xv[u][2] = __ldg(xi + c + oiW);
        xv[u][3] = __ldg(xi + c + ojN);
        xv[u][4] = __ldg(xi + c + ojS);
        xv[u][5] = __ldg(xi + c + okT);
        xv[u][6] = __ldg(xi + c + okB);
        xv[u][7] = __ldg(xi + c + okT + oiE);
        xv[u][8] = __ldg(xi + c + okB + oiE);
        xv[u][9] = __ldg(xi + c + okT + oiW);
        xv[u][10] = __ldg(xi + c + okB + oiW);
      }
      bb[u] = __ldg(b + c);
      inv[u] = __ldg(lf + c);
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int idx = base + u * VFS_SMOOTH_NT;
      if (idx >= tw * nj) break;
      const int jl = idx / tw;
      f[u].cc = face_code(f[u].aj);
      f[u].aj = face_aj(f[u].aj);
      const bool live = (i0 + idx % tw <= d.mx - 2) && f[u].aj != 0.f;
      float x11[19];  // slot-indexed view of the 11 values (TE, BE, TW, BW: the stencil slots)
      if (!ZG) {
        x11[CP] = xv[u][0]; x11[EP] = xv[u][1]; x11[WP] = xv[u][2]; x11[NP] = xv[u][3]; x11[SP] = xv[u][4];
        x11[TP] = xv[u][5]; x11[BP] = xv[u][6]; x11[TE] = xv[u][7]; x11[BE] = xv[u][8]; x11[TW] = xv[u][9];
        x11[BW] = xv[u][10];
      }
      const float ax = ZG ? 0.f : face_row(f[u], x11);
      const float a = jl > 0 ? f[u].aj * f[u].gjs : 0.f, cn = jl < nj - 1 ? f[u].aj * f[u].gjc : 0.f;
      su[idx] = live ? (bb[u] - ax) * inv[u] : 0.f;
      sp[idx] = live ? a * inv[u] : 0.f;
      sl[idx] = live ? cn * inv[u] : 0.f;
    }
  }
}

// Phase 1 on the general face form (levels with i-j or j-k cross terms):
// the residual from face_row_all and the line couplings aj times
// face_row_sn's coefficients (the cross terms add to them; the pivots 1/m are
// factored from the assembled rows).  From a zero guess only aj, the
// assembled FP32 SP and NP, b and 1/m are read.
template <int U, bool ZG>
__device__ __forceinline__ void face_phase1_all(const OpView<float>& A, const float* __restrict__ lf,
                                                const float* __restrict__ xi, const float* __restrict__ b, float* su,
                                                float* sp, float* sl, int i0, int k, int tw) {
  const Dims d = A.d;
  const int nj = d.my - 2, sy = d.mx, sz = d.mx * d.my;
  const size_t N = ncell(d);
  const float* __restrict__ csp = A.coef + (size_t)SP * N;
  const float* __restrict__ cnp = A.coef + (size_t)NP * N;
  for (int base = threadIdx.x; base < tw * nj; base += U * VFS_SMOOTH_NT) {
    FaceData f[U];
    FaceX e[U];
    float xv[U][19], bb[U], inv[U], av[U], cv[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int idx = min(base + u * VFS_SMOOTH_NT, tw * nj - 1);
      const int il = idx % tw, jl = idx / tw;
      const int i = min(i0 + il, d.mx - 2), j = 1 + jl;
      const int c = k * sz + j * sy + i;
      if (ZG) {
        f[u].aj = __ldg(A.faj + c);
        av[u] = __ldg(csp + c);
        cv[u] = __ldg(cnp + c);
      } else {
        face_gather_all(A, xi, i, j, k, f[u], e[u], xv[u]);
      }
      bb[u] = __ldg(b + c);
      inv[u] = __ldg(lf + c);
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int idx = base + u * VFS_SMOOTH_NT;
      if (idx >= tw * nj) break;
      const int jl = idx / tw;
      const float aj = face_aj(f[u].aj);
      const bool live = (i0 + idx % tw <= d.mx - 2) && aj != 0.f;
      float ax = 0.f;
      if (!ZG) {
        ax = face_row_all(f[u], e[u], xv[u]);
        face_row_sn(f[u], e[u], av[u], cv[u]);
        av[u] *= aj;
        cv[u] *= aj;
      }
      const float a = jl > 0 ? av[u] : 0.f, cn = jl < nj - 1 ? cv[u] : 0.f;
      su[idx] = live ? (bb[u] - ax) * inv[u] : 0.f;
      sp[idx] = live ? a * inv[u] : 0.f;
      sl[idx] = live ? cn * inv[u] : 0.f;
    }
  }
}

// UU: cells whose loads one thread issues together in phase 1 (2 on levels
// with fewer than two blocks per SM, where the looser register budget costs
// no occupancy and halves the serial chain of round trips).
// ZG: the zero-initial-guess sweep (xi == nullptr), its own instantiation so
// that its phase 1 (four cells a batch) leaves the others' registers alone.

// One tile of the sweep: columns i0 = 1 + bx TW .. of plane k = 1 + by,
// staged in smraw (3 TW nj values of T).
template <unsigned MASK, typename T, typename TC, bool PAIR, int UU, bool ZG>
__device__ __forceinline__ void smooth_tile(const OpView<T>& A, const T* __restrict__ lf, const T* __restrict__ xi_arg,
                                            const T* __restrict__ b, T* __restrict__ xo, T omega, int TW, int bx, int by,
                                            unsigned char* smraw) {
  const T* __restrict__ xi = ZG ? nullptr : xi_arg;
  // NRM: the FP16 diagonal-normalised operator (b is divided by D, non-fluid
  // rows have 1/m = 0 so their delta is 0 without a test)
  constexpr bool NRM = std::is_same<TC, __half>::value;
  constexpr bool FACE = std::is_same<TC, FaceOp>::value;
  constexpr int PF = (NRM || FACE) ? VFS_SMOOTH_PF_HALF : VFS_SMOOTH_PF;
  const TC* __restrict__ coef = coef_ptr<TC>(A);
  const Dims d = A.d;
  const int nj = d.my - 2;
  T* su = (T*)smraw;     // r_j / m_j, then y_j, then delta_j
  T* sp = su + TW * nj;  // a_j / m_j
  T* sl = sp + TW * nj;  // c'_j
  const int N = (int)ncell(d);
  const int i0 = 1 + bx * TW;
  const int k = 1 + by;
  constexpr int U = UU;
  // L2 prefetch of the rows a warp will stream PF iterations later: the
  // loads in flight are bounded by registers (4 bytes each), the prefetches
  // are not, so they keep more of HBM's latency-bandwidth product busy.  One
  // lane per 128-byte line: the 11 coefficient slots' (or MASK's) row, b, 1/m
  // and the x rows of planes k-1, k, k+1 (a row of TW floats starting at i0
  // spans two lines).  Every prefetched line lies inside its array: the
  // element offset is clamped to [0, N - 32].  (FP32 operator only: the FP16
  // one measured faster without.)
  auto prefetch_row = [&](int jrow) {
    if (PF <= 0 || jrow > d.my - 2) return;
    const int lane = threadIdx.x & 31;
    const int q = lane >> 1;  // stream index
    constexpr int NS = __builtin_popcount(MASK);
    int m = -1;
    for (int s = 0, n = 0; s < 19; s++)
      if (MASK & (1u << s)) {
        if (n == q) m = s;
        n++;
      }
    const char* base = nullptr;
    size_t es = sizeof(T);
    int shift = 0;
    if (m >= 0) {
      if constexpr (NRM) return;  // hidx layout: not this row arithmetic
      base = (const char*)(coef + (size_t)m * N);
      es = sizeof(TC);
    } else if (q == NS) base = (const char*)b;
    else if (q == NS + 1) base = (const char*)lf;
    else if (xi && q <= NS + 4) {
      base = (const char*)xi;
      shift = (q == NS + 3) ? -d.mx * d.my : (q == NS + 4) ? d.mx * d.my : 0;
    }
    if (!base) return;
    int e = k * d.mx * d.my + jrow * d.mx + i0 + shift + (lane & 1) * 32;
    e = max(0, min(e, N - 32));
    asm volatile("prefetch.global.L2 [%0];" ::"l"(base + (size_t)e * es));
  };
  static_assert(!PAIR || NRM, "the two-cells-per-thread sweep reads the FP16 layout");
  if constexpr (PAIR) {
    // FP16 operator, two cells per thread: one thread takes the cell pair
    // (ia, ia + 1), ia = i0 + 2 p odd, whose coefficients of a slot are one
    // aligned word of the hidx layout; x is read once per column (L, A, B,
    // R = ia - 1 .. ia + 2, the periodic wraps and the clamp of the per-cell
    // path applied) and shared by the two cells.  Per cell the arithmetic is
    // the per-cell path's.  Chosen for the 19-slot operator and for smaller
    // 11-slot levels (half the serial loads per thread); the large 11-slot
    // levels measured faster one cell per thread at 4 blocks per SM.
    smooth_pairs<MASK, T>(A, lf, xi, b, su, sp, sl, i0, k, TW);
  } else if constexpr (FACE) {
    static_assert(sizeof(T) == 4, "the face form is FP32");
    if constexpr (MASK == MASK_CH) face_phase1<UU, ZG>(A, lf, xi, b, su, sp, sl, i0, k, TW);
    else face_phase1_all<UU, ZG>(A, lf, xi, b, su, sp, sl, i0, k, TW);
  } else {
    // Phase 1 in batches of U cells per thread: every load of the batch is
    // issued before any arithmetic (all addresses are interior cells: columns
    // past the last one are clamped onto it and discarded; non-fluid rows have
    // finite factors and are selected out).  The line factors a_j/m_j and c'_j
    // are formed from the SP and NP coefficients the stencil loads anyway; only
    // 1/m_j is stored.  With xi == nullptr (zero initial guess) the residual is
    // b and only CP, SP, NP of the stencil are loaded, four cells a batch
    // (few registers a cell: the serial chain of round trips is a quarter).
    // TW divides the block: a thread keeps its column (il) and steps rows by
    // jstep; its cell and coefficient offsets advance by one row pitch.
    const int il = threadIdx.x % TW, jl0 = threadIdx.x / TW, jstep = VFS_SMOOTH_NT / TW;
    const int ic = min(i0 + il, d.mx - 2);
    const bool col_in = i0 + il <= d.mx - 2;
    const int c1 = k * d.mx * d.my + d.mx + ic;  // cell (ic, 1, k)
    size_t cstride, cc1;                          // coefficient slot stride and (ic, 1, k) offset
    int crow;                                     // coefficient row pitch
    if constexpr (NRM) {
      cstride = hslot(d);
      cc1 = hidx(d, ic, 1, k);
      crow = hpitch(d);
    } else {
      cstride = (size_t)N;
      cc1 = (size_t)c1;
      crow = d.mx;
    }
    if constexpr (ZG) {
      constexpr int U0 = 4;
      for (int jb = jl0; jb < nj; jb += U0 * jstep) {
        TC ccp[U0], csp[U0], cnp[U0];
        T bb[U0], inv[U0];
  #pragma unroll
        for (int u = 0; u < U0; u++) {
          const int jl = min(jb + u * jstep, nj - 1);
          const int c = c1 + jl * d.mx;
          const size_t cc = cc1 + (size_t)jl * crow;
          if constexpr (!NRM) ccp[u] = __ldg(coef + cc);
          csp[u] = __ldg(coef + (size_t)SP * cstride + cc);
          cnp[u] = __ldg(coef + (size_t)NP * cstride + cc);
          bb[u] = __ldg(b + c);
          inv[u] = __ldg(lf + c);
        }
  #pragma unroll
        for (int u = 0; u < U0; u++) {
          const int jl = jb + u * jstep;
          if (jl >= nj) break;
          const int idx = jl * TW + il;
          const bool live = col_in && (NRM || to_acc<T>(ccp[u]) != T(0));
          const T a = jl > 0 ? to_acc<T>(csp[u]) : T(0), cn = jl < nj - 1 ? to_acc<T>(cnp[u]) : T(0);
          su[idx] = live ? (bb[u] - T(0)) * inv[u] : T(0);
          sp[idx] = live ? a * inv[u] : T(0);
          sl[idx] = live ? cn * inv[u] : T(0);
        }
      }
    } else
    if constexpr (sizeof(T) == 8) {
      // FP64: the thread's column, i / k offsets and base addresses
      // hoisted (fewer integer instructions, measured faster); FP32 keeps
      // the per-cell index arithmetic, whose registers the 64-register
      // budget rather spends on loads in flight (measured faster there).
    {
      // x offsets of the stencil's i and k neighbours (periodic seams
      // folded in) are fixed for the thread; the j ones depend on the row
      const int sz = d.mx * d.my;
      const int oi[3] = {(ic == 1 && d.ip) ? d.mx - 3 : -1, 0, (ic == d.mx - 2 && d.ip) ? 3 - d.mx : 1};
      const int ok[3] = {((k == 1 && d.kp) ? d.mz - 3 : -1) * sz, 0, ((k == d.mz - 2 && d.kp) ? 3 - d.mz : 1) * sz};
    for (int jb = jl0; jb < nj; jb += U * jstep) {
      if (PF > 0 && sizeof(T) == 4 && TW == 32) prefetch_row(1 + jb + PF * U * jstep);
      TC cv[U][19];
      T xv[U][19], bb[U], inv[U];
  #pragma unroll
      for (int u = 0; u < U; u++) {
        const int jl = min(jb + u * jstep, nj - 1);
        const int j = 1 + jl;
        const int c = c1 + jl * d.mx;
        const size_t cc = cc1 + (size_t)jl * crow;
        const int oj[3] = {((j == 1 && d.jp) ? d.my - 3 : -1) * d.mx, 0, ((j == d.my - 2 && d.jp) ? 3 - d.my : 1) * d.mx};
  #pragma unroll
        for (int m = 0; m < 19; m++) {
          if (MASK & (1u << m)) {
            cv[u][m] = __ldg(coef + (size_t)m * cstride + cc);
            xv[u][m] = __ldg(xi + (c + oi[slot_di(m) + 1] + oj[slot_dj(m) + 1] + ok[slot_dk(m) + 1]));
          }
        }
        bb[u] = __ldg(b + c);
        inv[u] = __ldg(lf + c);
      }
  #pragma unroll
      for (int u = 0; u < U; u++) {
        const int jl = jb + u * jstep;
        if (jl >= nj) break;
        const int idx = jl * TW + il;
        const bool live = col_in && (NRM || to_acc<T>(cv[u][CP]) != T(0));
        const T ax = row_dot<MASK, T>(cv[u], xv[u]);
        const T a = jl > 0 ? to_acc<T>(cv[u][SP]) : T(0), cn = jl < nj - 1 ? to_acc<T>(cv[u][NP]) : T(0);
        su[idx] = live ? (bb[u] - ax) * inv[u] : T(0);
        sp[idx] = live ? a * inv[u] : T(0);
        sl[idx] = live ? cn * inv[u] : T(0);
      }
    }
    }
    } else {
    for (int base = threadIdx.x; base < TW * nj; base += U * VFS_SMOOTH_NT) {
      if (PF > 0 && sizeof(T) == 4 && TW == 32) prefetch_row(1 + (base + PF * U * VFS_SMOOTH_NT) / TW);
      TC cv[U][19];
      T xv[U][19], bb[U], inv[U];
  #pragma unroll
      for (int u = 0; u < U; u++) {
        const int idx = min(base + u * VFS_SMOOTH_NT, TW * nj - 1);
        const int il = idx % TW, jl = idx / TW;
        const int i = min(i0 + il, d.mx - 2), j = 1 + jl;
        const int c = k * d.mx * d.my + j * d.mx + i;
        if (xi) {
          gather<MASK>(d, coef, xi, i, j, k, cv[u], xv[u]);
        } else if constexpr (NRM) {
          const size_t hc = hidx(d, i, j, k), hs = hslot(d);
          cv[u][SP] = __ldg(coef + (size_t)SP * hs + hc);
          cv[u][NP] = __ldg(coef + (size_t)NP * hs + hc);
        } else {
          cv[u][CP] = __ldg(coef + c);
          cv[u][SP] = __ldg((coef + (size_t)SP * N) + c);
          cv[u][NP] = __ldg((coef + (size_t)NP * N) + c);
        }
        bb[u] = __ldg(b + c);
        inv[u] = __ldg(lf + c);
      }
  #pragma unroll
      for (int u = 0; u < U; u++) {
        const int idx = base + u * VFS_SMOOTH_NT;
        if (idx >= TW * nj) break;
        const int jl = idx / TW;
        const bool live = (i0 + idx % TW <= d.mx - 2) && (NRM || to_acc<T>(cv[u][CP]) != T(0));
        const T ax = xi ? row_dot<MASK, T>(cv[u], xv[u]) : T(0);
        const T a = jl > 0 ? to_acc<T>(cv[u][SP]) : T(0), cn = jl < nj - 1 ? to_acc<T>(cv[u][NP]) : T(0);
        su[idx] = live ? (bb[u] - ax) * inv[u] : T(0);
        sp[idx] = live ? a * inv[u] : T(0);
        sl[idx] = live ? cn * inv[u] : T(0);
      }
    }
    }
  }
  __syncthreads();
  if (threadIdx.x < TW) line_solve<T>(su, sp, sl, nj, TW, threadIdx.x);
  __syncthreads();
  // Phase 3, unrolled so that the old values of several cells are loaded
  // together (columns past the last one are clamped and not stored).
  constexpr int U3 = VFS_SMOOTH_U3;
#pragma unroll U3
  for (int idx = threadIdx.x; idx < TW * nj; idx += VFS_SMOOTH_NT) {
    const int il = idx % TW, jl = idx / TW;
    const int i = min(i0 + il, d.mx - 2), j = 1 + jl;
    const int c = k * d.mx * d.my + j * d.mx + i;
    const T x0 = xi ? __ldg(xi + c) : T(0);
    const T v = x0 + omega * su[idx];
    if (i0 + il <= d.mx - 2) xo[c] = v;
  }
}

// ---------------------------------------------------------------------------
// The face-form sweep with warp-row neighbours (x != 0).  A warp's 32 lanes
// hold 32 consecutive columns of one row (i0 - 1 .. i0 + 30): lanes 1..30
// are the tile's cells, lanes 0 and 31 their -i and +i halo.  Every lane
// loads x of planes k, k + 1, k - 1, its +i face and aj; a cell's E, W, TE,
// TW, BE, BW values, its -i face and the code bits of its i - 1 neighbour
// are its neighbour lanes' (warp shuffles), so a cell keeps 17 loaded values
// in registers instead of 24, and VFS_SMOOTH_W_U cells' loads fit in flight
// per thread at the register budget of four blocks per SM.  The halo lanes
// carry the periodic wrap (lane 0 of the first tile holds column mx - 2,
// the lane past the last interior column holds column 1).  Inputs and
// arithmetic per cell are face_phase1's, so results are bit for bit the
// one-cell-per-thread sweep's.  Tiles are VFS_SMOOTH_W_TW = 30 columns
// wide; the line arrays keep 32 columns (the halo lanes' stay zero).
// ---------------------------------------------------------------------------
#ifndef VFS_SMOOTH_W_U
#define VFS_SMOOTH_W_U 2  // rows (cells) whose loads one thread issues together
#endif
#ifndef VFS_SMOOTH_W_MINB
#define VFS_SMOOTH_W_MINB 4  // resident blocks per SM its register budget allows (4: 64 registers)
#endif
constexpr int SMOOTH_W_TW = 30;

template <int U>
__device__ __forceinline__ void smooth_tile_w(const OpView<float>& A, const float* __restrict__ lf,
                                              const float* __restrict__ xi, const float* __restrict__ b,
                                              float* __restrict__ xo, float omega, int bx, int by,
                                              unsigned char* smraw) {
  static_assert(VFS_SMOOTH_NT == 256, "eight warps per block");
  const Dims d = A.d;
  const int nj = d.my - 2, sy = d.mx, sz = d.mx * d.my;
  const int k = 1 + by, i0 = 1 + SMOOTH_W_TW * bx;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float* su = (float*)smraw;  // [nj][32]
  float* sp = su + 32 * nj;
  float* sl = sp + 32 * nj;
  // the lane's column, periodic wraps folded in, clamped past the ghost column
  int il = i0 - 1 + lane;
  if (d.ip && il == 0) il = d.mx - 2;
  else if (d.ip && il == d.mx - 1) il = 1;
  il = min(il, d.mx - 1);
  const bool comp = lane >= 1 && lane <= SMOOTH_W_TW && i0 - 1 + lane <= d.mx - 2;  // the lane is a cell
  const int okB = ((k == 1 && d.kp) ? d.mz - 3 : -1) * sz, okT = ((k == d.mz - 2 && d.kp) ? 3 - d.mz : 1) * sz;
  const int pk = k * sz + il;
  constexpr unsigned FULL = 0xFFFFFFFFu;
  for (int jb = warp; jb < nj; jb += 8 * U) {
    float xc[U], xn[U], xs[U], xt[U], xb[U], gjc[U], gjs[U], ajr[U], ajb[U], bb[U], inv[U];
    float2 fic[U], fkc[U], fkb[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int j = 1 + min(jb + 8 * u, nj - 1);
      const int ojS = ((j == 1 && d.jp) ? d.my - 3 : -1) * sy, ojN = ((j == d.my - 2 && d.jp) ? 3 - d.my : 1) * sy;
      const int c = pk + j * sy;
      xc[u] = __ldg(xi + c);
      xt[u] = __ldg(xi + c + okT);
      xb[u] = __ldg(xi + c + okB);
      fic[u] = __ldg(A.ffi + c);
      ajr[u] = __ldg(A.faj + c);
      xn[u] = comp ? __ldg(xi + c + ojN) : 0.f;
      xs[u] = comp ? __ldg(xi + c + ojS) : 0.f;
      fkc[u] = comp ? __ldg(A.ffk + c) : make_float2(0.f, 0.f);
      fkb[u] = comp ? __ldg(A.ffk + c + okB) : make_float2(0.f, 0.f);
      gjc[u] = comp ? __ldg(A.ffj + c) : 0.f;
      gjs[u] = comp ? __ldg(A.ffj + c + ojS) : 0.f;
      ajb[u] = comp ? __ldg(A.faj + c + okB) : 0.f;
      bb[u] = comp ? __ldg(b + c) : 0.f;
      inv[u] = comp ? __ldg(lf + c) : 0.f;
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int jl = jb + 8 * u;
      FaceData f;
      float x11[19];
      x11[CP] = xc[u];
      x11[EP] = __shfl_down_sync(FULL, xc[u], 1);
      x11[WP] = __shfl_up_sync(FULL, xc[u], 1);
      x11[NP] = xn[u];
      x11[SP] = xs[u];
      x11[TP] = xt[u];
      x11[BP] = xb[u];
      x11[TE] = __shfl_down_sync(FULL, xt[u], 1);
      x11[TW] = __shfl_up_sync(FULL, xt[u], 1);
      x11[BE] = __shfl_down_sync(FULL, xb[u], 1);
      x11[BW] = __shfl_up_sync(FULL, xb[u], 1);
      f.fic = fic[u];
      f.fiw.x = __shfl_up_sync(FULL, fic[u].x, 1);
      f.fiw.y = __shfl_up_sync(FULL, fic[u].y, 1);
      const float ajw = __shfl_up_sync(FULL, ajr[u], 1);
      if (jl >= nj) continue;  // warp-uniform
      f.fkc = fkc[u];
      f.fkb = fkb[u];
      f.gjc = gjc[u];
      f.gjs = gjs[u];
      f.aj = face_aj(ajr[u]);
      f.cc = face_code(ajr[u]);
      f.cw = face_code(ajw);
      f.cb = face_code(ajb[u]);
      const bool live = comp && f.aj != 0.f;
      const float ax = face_row(f, x11);
      const float a = jl > 0 ? f.aj * f.gjs : 0.f, cn = jl < nj - 1 ? f.aj * f.gjc : 0.f;
      const int idx = jl * 32 + lane;
      su[idx] = live ? (bb[u] - ax) * inv[u] : 0.f;
      sp[idx] = live ? a * inv[u] : 0.f;
      sl[idx] = live ? cn * inv[u] : 0.f;
    }
  }
  __syncthreads();
  if (threadIdx.x < 32) line_solve<float>(su, sp, sl, nj, 32, threadIdx.x);
  __syncthreads();
  constexpr int U3 = VFS_SMOOTH_U3;
#pragma unroll U3
  for (int idx = threadIdx.x; idx < 32 * nj; idx += VFS_SMOOTH_NT) {
    const int l = idx & 31, jl = idx >> 5;
    const int i = min(i0 - 1 + l, d.mx - 2);
    const int c = k * sz + (1 + jl) * sy + i;
    const float v = __ldg(xi + c) + omega * su[idx];
    if (l >= 1 && l <= SMOOTH_W_TW && i0 - 1 + l <= d.mx - 2) xo[c] = v;
  }
}

// Columns per block: the requested tile (0 = automatic), narrowed while
// three staged line arrays exceed 48 KB or the tile is twice the width of
// the level; automatically also narrowed (down to 8) while the sweep has
// fewer than VFS_SMOOTH_MINBLK blocks (one per SM), so small levels keep
// the machine busy -- when the grid solves alone (narrow): in a batch or
// under serving other grids' kernels fill the machine, and the full-width
// tiles (and their warp-row kernel) measured faster (64-grid batch: 806-830
// -> 877-883 solves/s mixed, 428 -> 443 FP64).
template <typename T>
inline int smooth_tw(int ni, int nj, int nk, int cols, bool narrow = true) {
  int tw = cols > 0 ? cols : VFS_SMOOTH_TWMAX;
  while (tw > 4 && (size_t)3 * tw * nj * sizeof(T) > 48 * 1024) tw >>= 1;
  while (tw > 4 && tw / 2 >= ni) tw >>= 1;
  if (cols == 0 && narrow)
    while (tw > VFS_SMOOTH_TWMIN && (size_t)((ni + tw - 1) / tw) * nk < VFS_SMOOTH_MINBLK) tw >>= 1;
  return tw;
}
#ifndef VFS_SMOOTH_NARROW_SHARED
#define VFS_SMOOTH_NARROW_SHARED 0  // 1: narrow for parallelism also when other grids share the GPU
#endif


// One tile of the residual restriction (see k_resrestrict_tiled): coarse
// cells (1 + 32 bx .., 1 + 4 by .., 1 + bz); sr: 2 x 8 x 64 values of T.
template <unsigned MASK, typename T, typename TC>
__device__ __forceinline__ void resrestrict_tile(const OpView<T>& A, const T* __restrict__ x, const T* __restrict__ b,
                                                 const T* __restrict__ rw, const Dims& c, const double* __restrict__ nvc,
                                                 T* __restrict__ bc, T* __restrict__ xc, int bx, int by, int bz,
                                                 T (*sr)[8][64]) {
  const TC* __restrict__ coef = coef_ptr<TC>(A);
  const Dims f = A.d;
  const int ci0 = 1 + bx * 32, cj0 = 1 + by * 4, ck = 1 + bz;
  const int fi0 = 2 * ci0 - 1, fj0 = 2 * cj0 - 1, fk0 = 2 * ck - 1;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const int ii = tx + 32 * (q & 1), kk = q >> 1;
    const int fi = fi0 + ii, fj = fj0 + ty, fk = fk0 + kk;
    // loads unconditional and clamped into the interior, the nvert weight
    // and the tile edge applied by select (no load waits on another)
    const int fic = min(fi, f.mx - 2), fjc = min(fj, f.my - 2);
    const size_t fc = cidx(f, fic, fjc, fk);
    const T w = rw[fc];
    const T bv = b[fc];
    T ax = T(0);
    if (x) {
      if constexpr (std::is_same<TC, FaceOp>::value) {
        FaceData fd;
        float xv[19];
        if constexpr (MASK == MASK_CH) {
          face_gather(A, x, fic, fjc, fk, fd, xv);
          ax = face_row(fd, xv);
        } else {
          FaceX fe;
          face_gather_all(A, x, fic, fjc, fk, fd, fe, xv);
          ax = face_row_all(fd, fe, xv);
        }
      } else {
        TC cv[19];
        T xv[19];
        gather<MASK>(f, coef, x, fic, fjc, fk, cv, xv);
        ax = row_dot<MASK, T>(cv, xv);
      }
    }
    const T rr = (bv - ax) * w;
    sr[kk][ty][ii] = (w != T(0) && fi <= f.mx - 2 && fj <= f.my - 2) ? rr : T(0);
  }
  __syncthreads();
  if (threadIdx.x < 128) {
    const int cx = threadIdx.x & 31, cy = threadIdx.x >> 5;
    const int ci = ci0 + cx, cj = cj0 + cy;
    if (ci <= c.mx - 2 && cj <= c.my - 2) {
      const size_t q = cidx(c, ci, cj, ck);
      T acc = T(0);
      if (!(nvc[q] > 0.1)) {
        // children (ih, jh, kh) - {0, 1} in MyRestriction's order
        const int ih = 2 * cx + 1, jh = 2 * cy + 1;
        acc = (sr[1][jh][ih] + sr[1][jh][ih - 1] + sr[1][jh - 1][ih] + sr[0][jh][ih] + sr[1][jh - 1][ih - 1] +
               sr[0][jh - 1][ih] + sr[0][jh][ih - 1] + sr[0][jh - 1][ih - 1]) * T(0.125);
      }
      bc[q] = acc;
      xc[q] = T(0);
    }
  }
}


// One tile of the prolongation (see k_prolong): fine columns
// (1 + TX bx + tx, 1 + TY by + ty), planes 1 + KCHUNK bz ...
template <typename T>
__device__ __forceinline__ void prolong_tile(const Dims& f, const uint8_t* __restrict__ code, const Dims& c,
                                             const T* __restrict__ xc, T* __restrict__ xf, int add, int si, int sj,
                                             int sk, int bx, int by, int bz, int tx, int ty) {
  // A thread owns KCHUNK cells of one (i, j) column: their codes (and old
  // values) are loaded first, then all coarse values, so no load waits on
  // another cell's.  Every candidate coarse index lies within the coarse
  // level's ghost frame whatever the code, so the no-correction code (bit 7)
  // is applied by select; columns and planes past the tile edge are clamped
  // and not stored.
  const int i = 1 + bx * TX + tx;
  const int j = 1 + by * TY + ty;
  const bool in = (i <= f.mx - 2) && (j <= f.my - 2);
  const int i1 = min(i, f.mx - 2), j1 = min(j, f.my - 2);
  const int k0 = 1 + bz * KCHUNK;
  uint8_t cd[KCHUNK];
  T xo[KCHUNK];
#pragma unroll
  for (int u = 0; u < KCHUNK; u++) {
    const size_t q = cidx(f, i1, j1, min(k0 + u, f.mz - 2));
    cd[u] = code[q];
    xo[u] = add ? xf[q] : T(0);
  }
  const int ic = si ? i1 : (i1 + 1) / 2, jc = sj ? j1 : (j1 + 1) / 2;
#pragma unroll
  for (int u = 0; u < KCHUNK; u++) {
    const int k = min(k0 + u, f.mz - 2);
    const int kc = sk ? k : (k + 1) / 2;
    const int ia = (cd[u] & 3) - 1, ja = ((cd[u] >> 2) & 3) - 1, ka = ((cd[u] >> 4) & 3) - 1;
#define X(a, b, cc) xc[cidx(c, a, b, cc)]
    const T v = (X(ic, jc, kc) * T(9) + X(ic, jc + ja, kc) * T(3) + X(ic + ia, jc, kc) * T(3) + X(ic + ia, jc + ja, kc)) *
                    (T(3) / T(64)) +
                (X(ic, jc, kc + ka) * T(9) + X(ic, jc + ja, kc + ka) * T(3) + X(ic + ia, jc, kc + ka) * T(3) +
                 X(ic + ia, jc + ja, kc + ka)) / T(64);
#undef X
    const T vv = (cd[u] & 0x80) ? T(0) : v;
    if (in && k0 + u <= f.mz - 2) xf[cidx(f, i1, j1, k)] = add ? xo[u] + vv : vv;
  }
}

// Rows 8 rb .. 8 rb + 7 of x = Binv (D b) over the packed interior (one warp
// per row), b staged in sb (n values of T, 16-byte aligned); dsc nullable.
// When n is a multiple of a 16-byte vector, a lane reads its row entries and
// b in 16-byte vectors (entries 4q .. 4q + 3 of FP32, lanes striding by 32
// vectors) and adds them in that order; otherwise one entry at a time.
template <typename T>
__device__ __forceinline__ void gemv_tile(const Dims& d, const T* __restrict__ Binv, int n, const T* __restrict__ b,
                                          T* __restrict__ x, const T* __restrict__ dsc, int rb, T* sb) {
  const int ni = d.mx - 2, nj = d.my - 2;
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    const int i = 1 + r % ni, j = 1 + (r / ni) % nj, k = 1 + r / (ni * nj);
    const size_t c = cidx(d, i, j, k);
    sb[r] = dsc ? b[c] * dsc[c] : b[c];
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row = rb * 8 + warp;
  if (row >= n) return;
  const T* Br = Binv + (size_t)row * n;
  T s = T(0);
  constexpr int V = 16 / (int)sizeof(T);
  if (n % V == 0) {
    using VT = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
    const VT* Bv = reinterpret_cast<const VT*>(Br);
    const VT* sv = reinterpret_cast<const VT*>(sb);
#pragma unroll 4
    for (int q = lane; q < n / V; q += 32) {
      const VT a = __ldg(Bv + q), c = sv[q];
      if constexpr (sizeof(T) == 4) {
        s = fma(a.x, c.x, s);
        s = fma(a.y, c.y, s);
        s = fma(a.z, c.z, s);
        s = fma(a.w, c.w, s);
      } else {
        s = fma(a.x, c.x, s);
        s = fma(a.y, c.y, s);
      }
    }
  } else {
    for (int col = lane; col < n; col += 32) s = fma(Br[col], sb[col], s);
  }
  s = warp_sum(s);
  if (lane == 0) {
    const int i = 1 + row % ni, j = 1 + (row / ni) % nj, k = 1 + row / (ni * nj);
    x[cidx(d, i, j, k)] = s;
  }
}

}  // namespace vfs
