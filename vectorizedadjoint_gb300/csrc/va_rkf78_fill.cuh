// Fehlberg 7(8) entries of a one-thread model's kernel table: float and
// double-word sweeps (the FP64 sweeps come from va_inst_rkf78_fp64.cu, built
// without FMA contraction).  Included by the va_inst_rkf78_*.cu units, which
// split the models so the library builds in parallel.
#pragma once

#include "va_kernels.cuh"
#include "va_kernels_dw.cuh"
#include "va_models.cuh"
#include "va_registry.h"

namespace va {

template <class M>
void fill_rkf78_reduced(KernelSet &k)
{
    using T = TabRKF78;
    k.fwd[2][1] = (const void *)forward_kernel<M, T, float>;
    k.bwd[2][1] = (const void *)backward_kernel<M, T, float>;
    k.bwd2[2][1] = (const void *)backward_kernel_2level<M, T, float>;
    k.fwd[2][2] = (const void *)forward_kernel_dw<M, T, true>;
    k.fwd2[2][2] = (const void *)forward_kernel_dw<M, T, false>;
    k.bwd[2][2] = (const void *)backward_kernel_dw<M, T, true>;
    k.bwd1[2][2] = (const void *)backward_kernel_dw<M, T, false>;
    k.bwd2[2][2] = (const void *)backward_kernel_2level_dw<M, T>;
    k.rs_stage[2] = stage_record_doubles(M::N, T::S);
}

} // namespace va
