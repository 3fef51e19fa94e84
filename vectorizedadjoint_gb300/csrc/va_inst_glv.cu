// Generalized Lotka-Volterra kernels with a per-instance interaction matrix:
// lane groups of N threads per instance, for the compiled sizes N = 5, 10.
// Reduced-precision sweeps here; FP64 sweeps in va_inst_glv_fp64.cu.  The
// mixed_dw entries are the double-word stage-record sweeps; with stage
// records off, the double-word-stage sweeps over [t, dt, y] FP64 records.
#include "va_group.cuh"
#include "va_group_dw.cuh"
#include "va_registry.h"

namespace va {

void fill_fp64_glv5(KernelSet &k);
void fill_fp64_glv10(KernelSet &k);
void fill_rkf78_glv5(KernelSet &k);
void fill_rkf78_glv10(KernelSet &k);
void fill_2level_glv5(KernelSet &k);
void fill_2level_glv10(KernelSet &k);

template <int NN>
static KernelSet make_glv(void (*fill_fp64)(KernelSet &), void (*fill_rkf78)(KernelSet &),
                          void (*fill_fixed)(KernelSet &), void (*fill_2level)(KernelSet &))
{
    using M = ModelGLVLane<NN>;
    KernelSet k{};
    k.N = NN;
    k.P = NN + NN * NN;
    k.tpi = NN;
    fill_fp64(k);
    k.fwd[0][1] = (const void *)forward_group_kernel<M, TabDopri5, float>;
    k.fwd[1][1] = (const void *)forward_group_kernel<M, TabCK54, float>;
    k.bwd[0][1] = (const void *)backward_group_kernel<M, TabDopri5, float>;
    k.bwd[1][1] = (const void *)backward_group_kernel<M, TabCK54, float>;
    k.fwd[0][2] = (const void *)forward_group_dw_kernel<NN, TabDopri5>;
    k.fwd[1][2] = (const void *)forward_group_dw_kernel<NN, TabCK54>;
    k.bwd[0][2] = (const void *)backward_group_dw_kernel<NN, TabDopri5>;
    k.bwd[1][2] = (const void *)backward_group_dw_kernel<NN, TabCK54>;
    k.fwd2[0][2] = (const void *)forward_group_kernel<M, TabDopri5, dword>;
    k.fwd2[1][2] = (const void *)forward_group_kernel<M, TabCK54, dword>;
    k.bwd1[0][2] = (const void *)backward_group_kernel<M, TabDopri5, dword>;
    k.bwd1[1][2] = (const void *)backward_group_kernel<M, TabCK54, dword>;
    k.rs_stage[0] = group_stage_record_doubles(NN, TabDopri5::S);
    k.rs_stage[1] = group_stage_record_doubles(NN, TabCK54::S);
    k.dw_records = false; // the [t, dt, y] records of the fallback sweeps are FP64
    fill_rkf78(k);
    fill_fixed(k);
    fill_2level(k);
    return k;
}

const KernelSet *kernels_glv(int n)
{
    static const KernelSet k5 = make_glv<5>(fill_fp64_glv5, fill_rkf78_glv5, fill_fixed_glv5, fill_2level_glv5);
    static const KernelSet k10 =
        make_glv<10>(fill_fp64_glv10, fill_rkf78_glv10, fill_fixed_glv10, fill_2level_glv10);
    switch (n) {
    case 5:
        return &k5;
    case 10:
        return &k10;
    default:
        return nullptr;
    }
}

} // namespace va
