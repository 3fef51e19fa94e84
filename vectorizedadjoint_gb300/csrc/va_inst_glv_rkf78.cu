// Fehlberg 7(8) float and double-word sweeps of the per-instance GLV model
// (lane groups); FP64 in va_inst_glv_rkf78_fp64.cu.
#include "va_group.cuh"
#include "va_group_dw.cuh"
#include "va_registry.h"

namespace va {

void fill_rkf78_fp64_glv5(KernelSet &k);
void fill_rkf78_fp64_glv10(KernelSet &k);

template <int NN>
static void fill(KernelSet &k)
{
    using M = ModelGLVLane<NN>;
    using T = TabRKF78;
    k.fwd[2][1] = (const void *)forward_group_kernel<M, T, float>;
    k.bwd[2][1] = (const void *)backward_group_kernel<M, T, float>;
    k.fwd[2][2] = (const void *)forward_group_dw_kernel<NN, T>;
    k.bwd[2][2] = (const void *)backward_group_dw_kernel<NN, T>;
    k.fwd2[2][2] = (const void *)forward_group_kernel<M, T, dword>;
    k.bwd1[2][2] = (const void *)backward_group_kernel<M, T, dword>;
    k.rs_stage[2] = group_stage_record_doubles(NN, T::S);
}

void fill_rkf78_glv5(KernelSet &k)
{
    fill_rkf78_fp64_glv5(k);
    fill<5>(k);
}
void fill_rkf78_glv10(KernelSet &k)
{
    fill_rkf78_fp64_glv10(k);
    fill<10>(k);
}

} // namespace va
