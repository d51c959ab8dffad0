// Grouped multigrid kernels for batched solves (mg_group.h): one launch runs
// one V-cycle operation on many grids, each block one tile of one grid's
// operation, found in the launch's work-item table.  Tiles are the
// stand-alone kernels' blocks and run their tile bodies, so results are the
// per-grid launches' bit for bit.
#include "mg_group.h"
#include "mg_tiles.cuh"
#include "vfs_kernels.h"

namespace vfs {

// The item whose block range holds this block (items ascend by start).
template <typename T>
__device__ __forceinline__ const GroupItem<T>& group_item(const GroupItem<T>* __restrict__ items, int n) {
  int lo = 0, hi = n - 1;
  const int b = blockIdx.x;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (items[mid].start <= b) lo = mid;
    else hi = mid - 1;
  }
  return items[lo];
}

template <unsigned MASK, typename T, typename TC, bool ZG>
__global__ void __launch_bounds__(VFS_SMOOTH_NT, VFS_SMOOTH_MINB) k_group_smooth(const GroupItem<T>* __restrict__ items,
                                                                                 int n) {
  const GroupItem<T>& it = group_item(items, n);
  if (skipped(it.skip)) return;
  extern __shared__ unsigned char smraw[];
  const OpView<T>& A = it.A;
  const int t = blockIdx.x - it.start;
  smooth_tile<MASK, T, TC, false, 1, ZG>(A, it.lf, it.x, it.b, it.y, it.w, it.tw, t % it.gx, t / it.gx, smraw);
}

template <unsigned MASK, typename T, typename TC>
__global__ void __launch_bounds__(256, VFS_STENCIL_MINB) k_group_restrict(const GroupItem<T>* __restrict__ items, int n) {
  const GroupItem<T>& it = group_item(items, n);
  if (skipped(it.skip)) return;
  __shared__ T sr[2][8][64];
  const OpView<T>& A = it.A;
  const int t = blockIdx.x - it.start;
  resrestrict_tile<MASK, T, TC>(A, it.x, it.b, it.rw, it.c, it.nvc, it.y, it.y2, t % it.gx, (t / it.gx) % it.gy,
                                t / (it.gx * it.gy), sr);
}

template <typename T>
__global__ void __launch_bounds__(TX* TY, VFS_STENCIL_MINB) k_group_prolong(const GroupItem<T>* __restrict__ items, int n) {
  const GroupItem<T>& it = group_item(items, n);
  if (skipped(it.skip)) return;
  const Dims f = it.A.d, c = it.c;
  // semi-coarsening flags are implied by equal extents (as launch_prolong)
  const int si = (c.mx == f.mx), sj = (c.my == f.my), sk = (c.mz == f.mz);
  const int t = blockIdx.x - it.start;
  prolong_tile<T>(f, it.pcode, c, it.x, it.y, it.add, si, sj, sk, t % it.gx, (t / it.gx) % it.gy, t / (it.gx * it.gy),
                  threadIdx.x % TX, threadIdx.x / TX);
}

template <typename T>
__global__ void __launch_bounds__(256) k_group_gemv(const GroupItem<T>* __restrict__ items, int n) {
  const GroupItem<T>& it = group_item(items, n);
  if (skipped(it.skip)) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  gemv_tile<T>(it.A.d, it.Binv, it.n, it.b, it.y, (const T*)nullptr, blockIdx.x - it.start, (T*)smraw);
}

template <typename K>
static void allow_smem(K k) {
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}

template <typename T>
int launch_group(int kind, const GroupItem<T>* items, int nitems, int nblocks, size_t smem, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    if constexpr (sizeof(T) == 4) {
      allow_smem(k_group_smooth<MASK_CH, T, FaceOp, false>);
      allow_smem(k_group_smooth<MASK_CH, T, FaceOp, true>);
    }
    allow_smem(k_group_smooth<MASK_CH, T, T, false>);
    allow_smem(k_group_smooth<MASK_CH, T, T, true>);
    allow_smem(k_group_smooth<MASK_ALL, T, T, false>);
    allow_smem(k_group_smooth<MASK_ALL, T, T, true>);
    allow_smem(k_group_gemv<T>);
    attr = true;
  }
  if (nitems <= 0 || nblocks <= 0) return (int)cudaSuccess;
  const dim3 g(nblocks), b(256);
  switch (kind) {
    case GK_SMOOTH_FACE:
    case GK_SMOOTH_FACE_ZG:
    case GK_RESTRICT_FACE:
      if constexpr (sizeof(T) == 4) {
        if (kind == GK_SMOOTH_FACE) k_group_smooth<MASK_CH, T, FaceOp, false><<<g, b, smem, s>>>(items, nitems);
        else if (kind == GK_SMOOTH_FACE_ZG) k_group_smooth<MASK_CH, T, FaceOp, true><<<g, b, smem, s>>>(items, nitems);
        else k_group_restrict<MASK_CH, T, FaceOp><<<g, b, 0, s>>>(items, nitems);
        break;
      } else {
        return (int)cudaErrorInvalidValue;  // the face form is FP32 only
      }
    case GK_SMOOTH_CH: k_group_smooth<MASK_CH, T, T, false><<<g, b, smem, s>>>(items, nitems); break;
    case GK_SMOOTH_CH_ZG: k_group_smooth<MASK_CH, T, T, true><<<g, b, smem, s>>>(items, nitems); break;
    case GK_SMOOTH_ALL: k_group_smooth<MASK_ALL, T, T, false><<<g, b, smem, s>>>(items, nitems); break;
    case GK_SMOOTH_ALL_ZG: k_group_smooth<MASK_ALL, T, T, true><<<g, b, smem, s>>>(items, nitems); break;
    case GK_RESTRICT_CH: k_group_restrict<MASK_CH, T, T><<<g, b, 0, s>>>(items, nitems); break;
    case GK_RESTRICT_ALL: k_group_restrict<MASK_ALL, T, T><<<g, b, 0, s>>>(items, nitems); break;
    case GK_PROLONG: k_group_prolong<T><<<g, b, 0, s>>>(items, nitems); break;
    case GK_GEMV: k_group_gemv<T><<<g, b, smem, s>>>(items, nitems); break;
    default: return (int)cudaErrorInvalidValue;
  }
  ++g_launches;
  return (int)cudaGetLastError();
}

template int launch_group<float>(int, const GroupItem<float>*, int, int, size_t, cudaStream_t);
template int launch_group<double>(int, const GroupItem<double>*, int, int, size_t, cudaStream_t);

}  // namespace vfs
