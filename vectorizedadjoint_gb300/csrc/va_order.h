// Longest-first work order for the persistent sweeps (va_order.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace va {

struct OrderArgs {
    int B;
    const int *steps;  // backward: accepted steps per instance (or null)
    const double *t0;  // forward: horizons t1 - t0 (used when steps is null and
    const double *t1;  //   no previous sweep's counts are valid)
    const int *prev_work;  // forward: attempts per instance of the previous forward sweep
    const int *prev_valid; //   and its flag (device int, 1 once written); may be null
    int *work;         // order_work_ints() scratch ints
    int *order;        // [B] output permutation, longest first
    const int *reuse;  // backward: the forward's order, copied instead of sorting when
                       //   that order came from counts (flag in work); may be null
};

size_t order_work_ints();
cudaError_t enqueue_order(const OrderArgs &a, cudaStream_t s);

} // namespace va
