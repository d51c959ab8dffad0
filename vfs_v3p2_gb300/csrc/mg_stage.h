// The finest-level face-form sweep that stages its operands in shared
// memory, fed by tensor-memory copies (k_smooth_tma.cu); results are the
// register-staged sweep's bit for bit.
#pragma once

#include <cuda_runtime.h>

#include "vfs_common.cuh"

#ifndef VFS_STAGE_MINCELLS
#define VFS_STAGE_MINCELLS (1 << 20)  // smallest level (interior cells) the staged sweep takes
#endif

namespace vfs {

// Staging of the finest sweeps (vfs_solve_params::mg_stage).
enum SweepStage : int { STAGE_REGS = 0, STAGE_TMA = 1 };

// Ring stages the tensor-copy sweep runs with on a level (0: the level does
// not qualify: mx and my must be even, the tensor-map encoder available).
int smooth_tma_stages(const Dims& d);

// One sweep xo = xi + omega T^-1 (b - A xi) on the face form (xi not null);
// err: a device word that records a bounded wait that ran out.  Returns a
// cudaError_t.
int launch_smooth_tma(const OpView<float>& A, const float* lf, const float* xi, const float* b, float* xo, float omega,
                      int* err, cudaStream_t s);

// The device word of the tensor-copy sweep's waits (shared by every
// launch), and a read that clears it (synchronous; 0 when no wait ran out).
int* smooth_tma_err();
int smooth_tma_take_error();

// Test hook: later launches leave out the 1/m copies of band `band` of every
// block (-1: none), so that band's bounded wait runs out and the sweep
// reports it.
void smooth_tma_drop(int band);

}  // namespace vfs
