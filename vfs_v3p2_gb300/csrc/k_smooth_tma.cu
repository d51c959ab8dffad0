// The finest-level y-line sweep on the FP32 face form, fed by tensor-memory
// copies (cp.async.bulk.tensor) into a shared-memory ring.
//
// The stand-alone sweep (k_smooth) stages every load of phase 1 in
// registers, so the bytes a block keeps in flight are bounded by its
// register budget, and the memory system idles while its column solves and
// its writes run.  Here one block per SM works through the level's tiles
// (32 i-columns x all j of one k plane) in a persistent loop: a producer
// thread issues the tensor copies of the tiles' 16-row bands (x on planes
// k-1, k, k+1, the face weights, aj with the code bits, b and 1/m) into a
// ring of 3 or 4 stages, each completed by an mbarrier transaction count,
// while eight consumer warps form the residuals of the bands already landed,
// run the column solves and write x.  The producer runs ahead into the next
// tile's bands while the consumers solve and write.  The arithmetic per cell
// is the stand-alone sweep's (face_row, line_solve, the same blend), so the
// result is bit for bit k_smooth's.
//
// Layouts.  The reference's ghosted rows are mx floats long (1032 bytes at
// mx = 258), not a multiple of 16 bytes, so a 4-byte array cannot be a
// tensor whose rows are the grid's rows.  With mx and my even, two rows are
// 2 mx floats, a multiple of 16 bytes: the 4-byte arrays are described as
// tensors of "row pairs" (dim 0: 2 mx elements, dim 1: my / 2 pairs, dim 2:
// mz planes), and a band's even and odd rows are two boxes of 40 x 9 x 1
// elements: the even rows from column i0 - 1 (a multiple of 32, so the
// copy's first element is 16-byte aligned), the odd rows from element
// mx + i0 - 1 - (mx mod 4) of the pair (column i0 - 1 - (mx mod 4)).  The
// 8-byte face arrays (float2) have 16-byte row pitches as they are: boxes of
// 40 x 16 x 1 elements from column i0 - 1.  Every copy starts on a 16-byte
// boundary; elements past the array come back as zeros and are never used.
//
// Periodic seams: the cells whose i or j neighbours wrap (i = 1 or mx - 2
// with i periodic, j = 1 or my - 2 with j periodic) read their stencil from
// global memory through face_gather; k wraps select the planes copied.
//
// Every mbarrier wait is bounded (about 0.2 s of clock cycles); a wait that
// runs out records an error in *err and raises the block's abort flag, after
// which the other waits return at once and the producer issues no further
// band (so a stage whose phase did not complete is never armed again); the
// consumers carry on through the same barriers (their results are then
// garbage, and the host reports the error), so that no thread is left
// waiting on another.  Before the block exits, one thread waits again
// (bounded, whatever the flag) for the last band issued on each stage, so no
// copy is still writing the block's shared memory.  drop >= 0 (a test hook)
// leaves out the 1/m copies of the block's band number drop, so that band's
// wait runs out.
#include <cuda.h>

#include "mg_tiles.cuh"
#include "mg_stage.h"
#include "vfs_kernels.h"

namespace vfs {

constexpr int TMA_TW = 32;        // columns per tile
constexpr int TMA_R = 16;         // rows per band
constexpr int TMA_BW = 40;        // box width (elements)
constexpr int TMA_PAIRS = 9;      // row pairs per 4-byte box (18 rows)
constexpr int TMA_NCONS = 256;    // consumer threads (8 warps)
constexpr int TMA_NT = TMA_NCONS + 32;
constexpr int TMA_HALF = 1536;    // one parity of a 4-byte box (1440 bytes), padded to 128-byte multiples
constexpr int TMA_A4 = 2 * TMA_HALF;           // a 4-byte array's band: even and odd rows
constexpr int TMA_A8 = TMA_BW * TMA_R * 8;     // an 8-byte array's band (5120 bytes)
// stage: x(kb) x(k) x(kt) ffj faj faj(kb) b lf (4-byte), ffi ffk ffk(kb) (8-byte)
constexpr int TMA_STAGE = 8 * TMA_A4 + 3 * TMA_A8;
constexpr unsigned TMA_TX = 8u * 2u * (TMA_BW * TMA_PAIRS * 4u) + 3u * TMA_A8;  // bytes the copies of a stage deliver
constexpr long long TMA_WAIT = 400000000LL;  // clock cycles a wait may take (about 0.2 s)

enum { S_XB = 0, S_XC = 1, S_XT = 2, S_FJ = 3, S_AJ = 4, S_AJB = 5, S_B = 6, S_LF = 7 };

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t* b, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for the completion of the phase with the given parity; on
// running out, records the error, raises the block's abort flag and returns
// false.  Once the flag is up, later waits (abortable) return at once.
__device__ __forceinline__ bool mbar_wait(uint64_t* b, unsigned parity, int* err, int code, volatile int* abort,
                                          bool abortable = true) {
  const long long t0 = clock64();
  while (!mbar_try(b, parity)) {
    if ((abortable && *abort) || clock64() - t0 > TMA_WAIT) {
      atomicOr(err, code);
      *abort = 1;
      return false;
    }
  }
  return true;
}
__device__ __forceinline__ void tma_load3(void* dst, const CUtensorMap* map, int c0, int c1, int c2, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_u32(dst)),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void consumers_sync() { asm volatile("bar.sync 1, %0;" ::"n"(TMA_NCONS) : "memory"); }

struct TmaMaps {
  CUtensorMap x, b, lf, fj, aj;  // 4-byte arrays as row-pair tensors
  CUtensorMap fi, fk;            // 8-byte face arrays
};

__global__ void __launch_bounds__(TMA_NT, 1)
    k_smooth_tma(const __grid_constant__ TmaMaps maps, OpView<float> A, const float* __restrict__ lf,
                 const float* __restrict__ xi, const float* __restrict__ b, float* __restrict__ xo, float omega,
                 int stages, int* err, int drop) {
  if (skipped(A.skip)) return;
  extern __shared__ __align__(128) unsigned char smraw[];
  __shared__ int abort_flag, n_issued;
  volatile int* abort = &abort_flag;
  const Dims d = A.d;
  const int nj = d.my - 2, ni = d.mx - 2, nk = d.mz - 2;
  const int gx = (ni + TMA_TW - 1) / TMA_TW, ntiles = gx * nk, nb = (nj + TMA_R - 1) / TMA_R;
  const int shift = d.mx & 3;  // odd rows' copies start this many columns earlier (16-byte alignment)
  unsigned char* ring = smraw;
  float* su = (float*)(smraw + (size_t)stages * TMA_STAGE);
  float* sp = su + TMA_TW * nj;
  float* sl = sp + TMA_TW * nj;
  uint64_t* full = (uint64_t*)(sl + TMA_TW * nj);
  uint64_t* empty = full + stages;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    abort_flag = 0;
    n_issued = 0;
    for (int s = 0; s < stages; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], TMA_NCONS / 32);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  if (warp == TMA_NCONS / 32) {
    // producer: one lane issues the copies of every (tile, band) in order,
    // until the abort flag is raised
    if (lane == 0) {
      long long q = 0;
      bool stop = false;
      for (int t = blockIdx.x; t < ntiles && !stop; t += gridDim.x) {
        const int bx = t % gx, k = 1 + t / gx;
        const int kb = (k == 1 && d.kp) ? d.mz - 2 : k - 1, kt = (k == d.mz - 2 && d.kp) ? 1 : k + 1;
        const int c0 = bx * TMA_TW;  // column i0 - 1
        for (int band = 0; band < nb; band++, q++) {
          const int s = (int)(q % stages);
          const unsigned use = (unsigned)(q / stages);
          if (*abort) stop = true;
          else if (use > 0) mbar_wait(&empty[s], (use - 1) & 1, err, 1, abort);
          if (stop || *abort) {
            stop = true;
            break;
          }
          unsigned char* st = ring + (size_t)s * TMA_STAGE;
          mbar_expect_tx(&full[s], TMA_TX);
          const int pr = band * (TMA_R / 2);  // first row pair: rows 16 band, 16 band + 1 (= b0 - 1, b0)
          const int b0 = 1 + band * TMA_R;
          auto pair4 = [&](int slot, const CUtensorMap* m, int plane) {
            unsigned char* dst = st + slot * TMA_A4;
            tma_load3(dst, m, c0, pr, plane, &full[s]);                             // even rows
            tma_load3(dst + TMA_HALF, m, d.mx + c0 - shift, pr, plane, &full[s]);  // odd rows
          };
          pair4(S_XB, &maps.x, kb);
          pair4(S_XC, &maps.x, k);
          pair4(S_XT, &maps.x, kt);
          pair4(S_FJ, &maps.fj, k);
          pair4(S_AJ, &maps.aj, k);
          pair4(S_AJB, &maps.aj, kb);
          pair4(S_B, &maps.b, k);
          if (q != drop) pair4(S_LF, &maps.lf, k);
          unsigned char* e8 = st + 8 * TMA_A4;
          tma_load3(e8, &maps.fi, c0, b0, k, &full[s]);
          tma_load3(e8 + TMA_A8, &maps.fk, c0, b0, k, &full[s]);
          tma_load3(e8 + 2 * TMA_A8, &maps.fk, c0, b0, kb, &full[s]);
        }
      }
      n_issued = (int)q;  // bands whose copies were issued
    }
  } else {
    // consumers: 8 warps; a band's 16 rows x 32 columns are two cells per
    // thread, rows 1 + warp and 9 + warp of the band's staged rows, column
    // 1 + lane of the staged columns.  A cell's place in a stage is the same in
    // every band, so its byte offsets are formed once.
    const int il = lane;
    // byte offset of staged row r (0 .. 17 from the band's first row) and
    // staged column e (0 .. 39 from column i0 - 1) in a 4-byte array's slot
    auto off4 = [&](int r, int e) -> int { return (r & 1) * TMA_HALF + ((r >> 1) * TMA_BW + e + (r & 1) * shift) * 4; };
    int o4[2][5];   // per cell: C E W N S in a 4-byte slot (the same for every array and plane)
    int o8[2][2];   // per cell: 8-byte (i), (i - 1) of rows 1..16
    for (int u = 0; u < 2; u++) {
      const int r = 1 + warp + 8 * u, e = 1 + il;
      o4[u][0] = off4(r, e);
      o4[u][1] = off4(r, e + 1);
      o4[u][2] = off4(r, e - 1);
      o4[u][3] = off4(r + 1, e);
      o4[u][4] = off4(r - 1, e);
      o8[u][0] = ((r - 1) * TMA_BW + e) * 8;
      o8[u][1] = ((r - 1) * TMA_BW + e - 1) * 8;
    }
    long long q = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
      const int bx = t % gx, k = 1 + t / gx;
      const int i0 = 1 + bx * TMA_TW;
      const int i = min(i0 + il, d.mx - 2);
      const bool col_in = i0 + il <= d.mx - 2;
      for (int band = 0; band < nb; band++, q++) {
        const int s = (int)(q % stages);
        mbar_wait(&full[s], (unsigned)((q / stages) & 1), err, 2, abort);
        const unsigned char* st = ring + (size_t)s * TMA_STAGE;
        auto ld4 = [&](int slot, int off) -> float { return *(const float*)(st + slot * TMA_A4 + off); };
        auto ld8 = [&](int slot, int off) -> float2 { return *(const float2*)(st + 8 * TMA_A4 + slot * TMA_A8 + off); };
  #pragma unroll
        for (int u = 0; u < 2; u++) {
          const int jl = band * TMA_R + warp + 8 * u;  // row index within the tile (j = 1 + jl)
          if (jl >= nj) continue;
          const int j = 1 + jl;
          FaceData f;
          float x11[19];
          float bb, inv;
          const bool seam = (d.ip && (i == 1 || i == d.mx - 2)) || (d.jp && (j == 1 || j == d.my - 2));
          if (seam) {
            face_gather(A, xi, i, j, k, f, x11);
            const int c = cidx(d, i, j, k);
            bb = __ldg(b + c);
            inv = __ldg(lf + c);
          } else {
            const int oc = o4[u][0], oe = o4[u][1], ow = o4[u][2], on = o4[u][3], os = o4[u][4];
            const float ajc = ld4(S_AJ, oc), ajw = ld4(S_AJ, ow), ajb = ld4(S_AJB, oc);
            f.fic = ld8(0, o8[u][0]);
            f.fiw = ld8(0, o8[u][1]);
            f.fkc = ld8(1, o8[u][0]);
            f.fkb = ld8(2, o8[u][0]);
            f.gjc = ld4(S_FJ, oc);
            f.gjs = ld4(S_FJ, os);
            f.aj = face_aj(ajc);
            f.cc = face_code(ajc);
            f.cw = face_code(ajw);
            f.cb = face_code(ajb);
            x11[CP] = ld4(S_XC, oc);
            x11[EP] = ld4(S_XC, oe);
            x11[WP] = ld4(S_XC, ow);
            x11[NP] = ld4(S_XC, on);
            x11[SP] = ld4(S_XC, os);
            x11[TP] = ld4(S_XT, oc);
            x11[BP] = ld4(S_XB, oc);
            x11[TE] = ld4(S_XT, oe);
            x11[BE] = ld4(S_XB, oe);
            x11[TW] = ld4(S_XT, ow);
            x11[BW] = ld4(S_XB, ow);
            bb = ld4(S_B, oc);
            inv = ld4(S_LF, oc);
          }
          const bool live = col_in && f.aj != 0.f;
          const float ax = face_row(f, x11);
          const float a = jl > 0 ? f.aj * f.gjs : 0.f, cn = jl < nj - 1 ? f.aj * f.gjc : 0.f;
          const int idx = jl * TMA_TW + il;
          su[idx] = live ? (bb - ax) * inv : 0.f;
          sp[idx] = live ? a * inv : 0.f;
          sl[idx] = live ? cn * inv : 0.f;
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[s]);
      }
      consumers_sync();
      if (tid < TMA_TW) line_solve<float>(su, sp, sl, nj, TMA_TW, tid);
      consumers_sync();
      for (int idx = tid; idx < TMA_TW * nj; idx += TMA_NCONS) {
        const int jl = idx / TMA_TW, ic = min(i0 + idx % TMA_TW, d.mx - 2);
        const int c = cidx(d, ic, 1 + jl, k);
        const float v = __ldg(xi + c) + omega * su[idx];
        if (i0 + idx % TMA_TW <= d.mx - 2) xo[c] = v;
      }
      consumers_sync();  // the next tile restages su, sp, sl
    }
  }
  __syncthreads();
  // every copy issued has landed before the block exits (immediate unless a
  // wait above ran out): the last band issued on each stage
  if (tid == 0) {
    const int n = n_issued;
    for (int r = n > stages ? n - stages : 0; r < n; r++)
      mbar_wait(&full[r % stages], (unsigned)((r / stages) & 1), err, 4, abort, false);
  }
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
typedef CUresult (*EncodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiled encoder() {
  static EncodeTiled fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiled)p;
    cudaGetLastError();
  }
  return fn;
}

// A 4-byte array of the level as a tensor of row pairs, boxes of 40 x 9 x 1.
static bool map4(EncodeTiled enc, CUtensorMap* m, const void* base, const Dims& d) {
  const cuuint64_t dim[3] = {(cuuint64_t)2 * d.mx, (cuuint64_t)d.my / 2, (cuuint64_t)d.mz};
  const cuuint64_t stride[2] = {(cuuint64_t)2 * d.mx * 4, (cuuint64_t)d.mx * d.my * 4};
  const cuuint32_t box[3] = {TMA_BW, TMA_PAIRS, 1}, es[3] = {1, 1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void*>(base), dim, stride, box, es,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}
// An 8-byte array (float2) of the level, boxes of 40 x 16 x 1.
static bool map8(EncodeTiled enc, CUtensorMap* m, const void* base, const Dims& d) {
  const cuuint64_t dim[3] = {(cuuint64_t)d.mx, (cuuint64_t)d.my, (cuuint64_t)d.mz};
  const cuuint64_t stride[2] = {(cuuint64_t)d.mx * 8, (cuuint64_t)d.mx * d.my * 8};
  const cuuint32_t box[3] = {TMA_BW, TMA_R, 1}, es[3] = {1, 1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<void*>(base), dim, stride, box, es,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

__device__ int g_tma_err = 0;
static int g_tma_drop = -1;  // test hook: band whose 1/m copies are left out (-1: none)

void smooth_tma_drop(int band) { g_tma_drop = band; }

int* smooth_tma_err() {
  static int* p = nullptr;
  if (!p) {
    if (cudaGetSymbolAddress((void**)&p, g_tma_err) != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
    }
  }
  return p;
}

int smooth_tma_take_error() {
  int v = 0;
  if (cudaMemcpyFromSymbol(&v, g_tma_err, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  if (v) {
    const int z = 0;
    cudaMemcpyToSymbol(g_tma_err, &z, sizeof(int));
  }
  return v;
}

static size_t tma_smem(const Dims& d, int stages) {
  return (size_t)stages * TMA_STAGE + (size_t)3 * TMA_TW * (d.my - 2) * 4 + (size_t)2 * stages * 8;
}

int smooth_tma_stages(const Dims& d) {
  if (d.mx % 2 || d.my % 2 || d.my - 2 < 2 || !encoder()) return 0;
  for (int s = 4; s >= 2; s--)
    if (tma_smem(d, s) <= (size_t)220 * 1024) return s;
  return 0;
}

static bool aligned16(const void* p) { return ((uintptr_t)p & 15) == 0; }

int launch_smooth_tma(const OpView<float>& A, const float* lf, const float* xi, const float* b, float* xo, float omega,
                      int* err, cudaStream_t s) {
  const Dims& d = A.d;
  const int stages = smooth_tma_stages(d);
  EncodeTiled enc = encoder();
  if (!stages || !enc || !A.ffi || !xi || !err) return (int)cudaErrorInvalidValue;
  if (!aligned16(xi) || !aligned16(b) || !aligned16(lf) || !aligned16(A.ffj) || !aligned16(A.faj) ||
      !aligned16(A.ffi) || !aligned16(A.ffk))
    return (int)cudaErrorInvalidValue;
  TmaMaps m;
  if (!map4(enc, &m.x, xi, d) || !map4(enc, &m.b, b, d) || !map4(enc, &m.lf, lf, d) || !map4(enc, &m.fj, A.ffj, d) ||
      !map4(enc, &m.aj, A.faj, d) || !map8(enc, &m.fi, A.ffi, d) || !map8(enc, &m.fk, A.ffk, d))
    return (int)cudaErrorInvalidValue;
  static int nsm = 0;
  static size_t opted = 0;  // dynamic shared memory the kernel is opted in for
  if (!nsm) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  }
  const size_t smem = tma_smem(d, stages);
  if (smem > opted) {
    if (cudaFuncSetAttribute(k_smooth_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
      cudaGetLastError();
      return (int)cudaErrorInvalidValue;
    }
    opted = smem;
  }
  const int ntiles = ((d.mx - 2 + TMA_TW - 1) / TMA_TW) * (d.mz - 2);
  const int grid = std::max(1, std::min(nsm, ntiles));
  k_smooth_tma<<<grid, TMA_NT, smem, s>>>(m, A, lf, xi, b, xo, omega, stages, err, g_tma_drop);
  ++g_launches;
  return (int)cudaGetLastError();
}

}  // namespace vfs
