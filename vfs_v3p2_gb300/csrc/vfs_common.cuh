// Shared definitions of the GB300 pressure-projection kernels.
//
// Layout.  Every field uses the reference's PETSc DMDA array layout
// (variables.h:305-383): extents mx = ni + 2, my = nj + 2, mz = nk + 2 with one
// ghost/boundary cell per side, cell (i, j, k) at ((k * my) + j) * mx + i, i
// fastest.  Scalars are one array; the contravariant flux Ucont is kept on the
// device as three SoA arrays (x, y, z components) so that a stencil reads only
// the component it needs; host transfers convert from/to the reference's AoS
// Cmpnts layout.  The 19-point operator is stored as 19 SoA coefficient
// arrays [slot][cell] in the slot order of poisson.c:956-974.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <atomic>

#define VFS_THR 0.1  // poisson_threshold, poisson.c:16

namespace vfs {

// Number of kernels this library has launched (all contexts).
extern std::atomic<unsigned long long> g_launches;

enum Slot { CP = 0, EP, WP, NP, SP, TP, BP, NE, SE, NW, SW, TN, BN, TS, BS, TE, BE, TW, BW, NSLOT };

struct Dims {
  int mx, my, mz;  // ghosted extents
  int ip, jp, kp;  // i/j/k periodic (index 0 mirrors m-2, m-1 mirrors 1)
};

__host__ __device__ __forceinline__ size_t cidx(const Dims& d, int i, int j, int k) {
  return ((size_t)k * d.my + j) * d.mx + i;
}
__host__ __device__ __forceinline__ size_t ncell(const Dims& d) { return (size_t)d.mx * d.my * d.mz; }
__host__ __device__ __forceinline__ int wrapi(int i, int m, int per) {
  return per ? (i == 0 ? m - 2 : (i == m - 1 ? 1 : i)) : i;
}
__host__ __device__ __forceinline__ bool interior(const Dims& d, int i, int j, int k) {
  return i > 0 && j > 0 && k > 0 && i < d.mx - 1 && j < d.my - 1 && k < d.mz - 1;
}

__host__ __device__ __forceinline__ int slot_di(int m) {
  const int t[19] = {0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, 1, -1, -1};
  return t[m];
}
__host__ __device__ __forceinline__ int slot_dj(int m) {
  const int t[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 1, 1, -1, -1, 0, 0, 0, 0};
  return t[m];
}
__host__ __device__ __forceinline__ int slot_dk(int m) {
  const int t[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1};
  return t[m];
}

// Wrapped neighbour offsets of one interior cell: nb[m] = cell index of slot m.
struct Nbr {
  size_t c[19];
};
__device__ __forceinline__ void neighbours(const Dims& d, int i, int j, int k, Nbr& nb) {
  const int im = wrapi(i - 1, d.mx, d.ip), ip1 = wrapi(i + 1, d.mx, d.ip);
  const int jm = wrapi(j - 1, d.my, d.jp), jp1 = wrapi(j + 1, d.my, d.jp);
  const int km = wrapi(k - 1, d.mz, d.kp), kp1 = wrapi(k + 1, d.mz, d.kp);
  const int II[3] = {im, i, ip1}, JJ[3] = {jm, j, jp1}, KK[3] = {km, k, kp1};
#pragma unroll
  for (int m = 0; m < 19; m++) nb.c[m] = cidx(d, II[slot_di(m) + 1], JJ[slot_dj(m) + 1], KK[slot_dk(m) + 1]);
}

// Layout of a level's FP16 operator (OpView::hcoef): rows padded to
// hpitch = mx + 7 rounded up to 8 halves, element (i, j, k) of slot m at
// m * hslot + (k * my + j) * hpitch + i + 7, so that column i = 1 of every
// row starts a 16-byte line and the coefficients of the cell pair (i, i + 1),
// i odd, are one aligned 4-byte word.
__host__ __device__ __forceinline__ int hpitch(const Dims& d) { return (d.mx + 14) & ~7; }
__host__ __device__ __forceinline__ size_t hslot(const Dims& d) { return (size_t)hpitch(d) * d.my * d.mz; }
__host__ __device__ __forceinline__ size_t hidx(const Dims& d, int i, int j, int k) {
  return ((size_t)k * d.my + j) * hpitch(d) + i + 7;
}

// One multigrid level (or the outer operator) as seen by a kernel.  With
// hcoef set (FP32 multigrid only) the kernels use the level's FP16
// diagonal-normalised operator instead of coef: row c holds a_m / D_c in
// every off-diagonal slot and, in the centre slot, the FP16 correction
// delta_c that restores the row sum after rounding, so the row is
// (1 + delta_c) x_c + sum_m h_m x_m and the level's right-hand sides are
// divided by D_c.
template <typename T>
struct OpView {
  Dims d;
  const T* coef;     // [19][N]
  unsigned mask;     // bit m set if slot m is nonzero somewhere on this level
  const int* skip;   // device flag (nullable): kernels return at once when *skip != 0
  const __half* hcoef = nullptr;  // [19][hslot], FP16 diagonal-normalised (nullable)
  // face form of the FP32 multigrid operator (11-slot levels, nullable): per
  // cell the +i face (g11, k-cross weight), +k face (g33, i-cross weight), +j
  // face (g22), and aj with the cross terms' one-sided code bits in its four
  // low mantissa bits (bit 0: the i face's upper pair is the centre pair,
  // bit 1: its lower pair; bits 2, 3 the same for the k face's pairs at
  // i+1 / i-1)
  const float2* ffi = nullptr;
  const float2* ffk = nullptr;
  const float* ffj = nullptr;
  const float* faj = nullptr;
  // the general face form (levels with i-j or j-k cross terms, nullable):
  // per cell the cross weights of the i-j and j-k terms, (x) the +i face's
  // j cross term (g12), (y, z) the +j face's i and k cross terms (g21, g23),
  // (w) the +k face's j cross term (g32), each carrying its own one-sided
  // code in its two low mantissa bits (bit 0: the upper pair is the face's
  // centre pair, bit 1: the lower pair)
  const float4* ffc = nullptr;
};

__device__ __forceinline__ bool skipped(const int* f) { return f && *(volatile const int*)f; }

// ---------------------------------------------------------------------------
// Deterministic reductions: every block writes one partial; a single block
// sums the partials in index order.  Same launch shape => same bits.
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
template <typename T>
__device__ __forceinline__ T warp_max(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    T w = __shfl_down_sync(0xffffffffu, v, o);
    v = w > v ? w : v;
  }
  return v;
}
// Block sum of v (blockDim.x a multiple of 32, <= 1024); result valid in thread 0.
template <typename T>
__device__ __forceinline__ T block_sum(T v, T* sh /* >= 32 */) {
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  const int nw = blockDim.x >> 5;
  v = (threadIdx.x < nw) ? sh[threadIdx.x] : T(0);
  if (w == 0) v = warp_sum(v);
  __syncthreads();
  return v;
}
template <typename T>
__device__ __forceinline__ T block_max(T v, T* sh) {
  v = warp_max(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) sh[w] = v;
  __syncthreads();
  const int nw = blockDim.x >> 5;
  v = (threadIdx.x < nw) ? sh[threadIdx.x] : T(0);
  if (w == 0) v = warp_max(v);
  __syncthreads();
  return v;
}

// Exact binary32 -> binary64 widening on the integer pipe, without branches.
// IEEE 754 fixes the result field by field: a normal number's exponent is
// rebiased by 1023 - 127 = 896 and its 23-bit fraction becomes the top of the
// 52-bit one; zero keeps its sign; a subnormal m 2^-149 with leading bit p
// becomes exponent p - 149 with the bits below p as fraction; infinities and
// NaNs keep their fraction under exponent 2047, a NaN's with the quiet bit
// set (a conversion returns a quiet NaN).  (The
// FP64 pipe, which the hardware conversion uses, is the scarce unit of the
// FP64 Krylov kernels.)
__host__ __device__ __forceinline__ double widen(float f) {
#ifdef __CUDA_ARCH__
  const unsigned u = __float_as_uint(f);
  const int p = 31 - __clz((u & 0x007fffffu) | 1u);  // leading bit of a subnormal fraction
#else
  unsigned u;
  memcpy(&u, &f, sizeof u);
  const int p = 31 - __builtin_clz((u & 0x007fffffu) | 1u);
#endif
  const unsigned e = (u >> 23) & 0xffu, m = u & 0x007fffffu;
  const unsigned long long sgn = (unsigned long long)(u >> 31) << 63;
  const unsigned long long sub = ((unsigned long long)(p + 874) << 52) |
                                 ((unsigned long long)(m ^ (1u << p)) << (52 - p));
  const unsigned mq = (e == 0xffu && m != 0u) ? (m | 0x00400000u) : m;
  const unsigned long long nrm = ((unsigned long long)(e == 0xffu ? 2047u : e + 896u) << 52) |
                                 ((unsigned long long)mq << 29);
  const unsigned long long mag = e != 0u ? nrm : (m != 0u ? sub : 0ull);
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)(sgn | mag));
#else
  const unsigned long long bits = sgn | mag;
  double d;
  memcpy(&d, &bits, sizeof d);
  return d;
#endif
}
// Operand conversion into an accumulator type (widen() for float -> double).
template <typename TA, typename TX_>
__device__ __forceinline__ TA to_acc(TX_ v) { return (TA)v; }
template <>
__device__ __forceinline__ double to_acc<double, float>(float v) { return widen(v); }
template <>
__device__ __forceinline__ float to_acc<float, __half>(__half v) { return __half2float(v); }

}  // namespace vfs

#define VFS_CUDA_OK(expr)                      \
  do {                                         \
    cudaError_t _e = (expr);                   \
    if (_e != cudaSuccess) return (int)_e;     \
  } while (0)
