// Grouped multigrid launches for batched solves: the V-cycles of many grids
// run as one sequence of launches, operation i of every grid's V-cycle in
// the launch (or the few launches, one per kernel instantiation) of stage i.
// A launch carries a work-item table: one GroupItem per grid, with the
// operation's arguments on that grid and the range of the launch's blocks
// that are its tiles; a block finds its item by binary search over the
// ranges and runs the stand-alone kernel's tile body (mg_tiles.cuh) on it.
// The arithmetic per cell is the stand-alone kernels', so a grouped V-cycle
// is the per-grid one bit for bit; what changes is the number of graph
// nodes (a group's V-cycle is one chain of about 33 launches whatever the
// number of its grids).  Measured on GB300 it is slower than a graph branch
// per grid (64-grid batch: 754 against 877 solves/s): graph nodes cost about
// 1 us each, and a grouped stage waits on every grid of its group, so it is
// an option (mg_grouped), off by default.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "vfs_common.cuh"

namespace vfs {

// Kernel of a grouped launch (with its instantiation).
enum GroupKind : int {
  GK_SMOOTH_FACE = 0,     // y-line sweep, FP32 face form (11-slot levels)
  GK_SMOOTH_FACE_ZG = 1,  // the same from a zero initial guess
  GK_SMOOTH_CH = 2,       // assembled coefficients, 11-slot set
  GK_SMOOTH_CH_ZG = 3,
  GK_SMOOTH_ALL = 4,      // assembled coefficients, 19 slots
  GK_SMOOTH_ALL_ZG = 5,
  GK_RESTRICT_FACE = 6,   // residual + restriction (full coarsening), face form
  GK_RESTRICT_CH = 7,
  GK_RESTRICT_ALL = 8,
  GK_PROLONG = 9,         // prolongation (+ correction when add)
  GK_GEMV = 10,           // coarsest level: x = Binv b
  GK_COUNT = 11
};

template <typename T>
struct GroupItem {
  OpView<T> A;           // the level's operator (fine level of a restriction or prolongation)
  const T* lf;           // sweep: y-line pivots 1/m
  const T* x;            // sweep: x (null: zero guess); restriction: fine x (null: 0); prolongation: coarse correction
  const T* b;            // sweep, restriction, gemv: right-hand side
  T* y;                  // sweep: new x; restriction: coarse b; prolongation: fine x; gemv: x
  T* y2;                 // restriction: coarse x, cleared
  const T* rw;           // restriction: weights max(0, 1 - nvert)
  const double* nvc;     // restriction: coarse nvert
  const uint8_t* pcode;  // prolongation: codes
  const T* Binv;         // gemv: dense inverse over the packed interior
  Dims c;                // restriction, prolongation: coarse level
  const int* skip;       // the grid's done flag (a set flag skips its tiles)
  T w;                   // sweep: damping
  int tw;                // sweep: i-columns per tile
  int n;                 // gemv: order
  int add;               // prolongation: add to the fine x
  int gx, gy;            // the operation's tile grid (x, y extents) on this grid
  int start;             // first block of this item in the launch
};

// One grouped launch: nitems items (device array), nblocks blocks in all,
// smem bytes of dynamic shared memory per block.  Returns a cudaError_t.
template <typename T>
int launch_group(int kind, const GroupItem<T>* items, int nitems, int nblocks, size_t smem, cudaStream_t s);

}  // namespace vfs
