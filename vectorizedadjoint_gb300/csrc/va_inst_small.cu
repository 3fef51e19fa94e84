// Kernel tables of the one-thread-per-instance models.  This unit holds the
// reduced-precision sweeps (float stages; double-word state and stages); the
// FP64 sweeps come from va_inst_small_fp64.cu, which is built without FMA
// contraction.
#include "va_kernels.cuh"
#include "va_kernels_dw.cuh"
#include "va_models.cuh"
#include "va_registry.h"

namespace va {

void fill_fp64_vdp(KernelSet &k);
void fill_fp64_vdp_petsc(KernelSet &k);
void fill_fp64_dho(KernelSet &k);
void fill_fp64_decay(KernelSet &k);

template <class M>
static KernelSet make_set(void (*fill_fp64)(KernelSet &), void (*fill_rkf78)(KernelSet &),
                          void (*fill_fixed)(KernelSet &), void (*fill_replay)(KernelSet &))
{
    KernelSet k{};
    k.N = M::N;
    k.P = M::P;
    k.tpi = 1;
    fill_fp64(k);
    k.fwd[0][1] = (const void *)forward_kernel<M, TabDopri5, float>;
    k.fwd[1][1] = (const void *)forward_kernel<M, TabCK54, float>;
    k.fwd[0][2] = (const void *)forward_kernel_dw<M, TabDopri5, true>;
    k.fwd[1][2] = (const void *)forward_kernel_dw<M, TabCK54, true>;
    k.fwd2[0][2] = (const void *)forward_kernel_dw<M, TabDopri5, false>;
    k.fwd2[1][2] = (const void *)forward_kernel_dw<M, TabCK54, false>;
    k.rs_stage[0] = stage_record_doubles(M::N, TabDopri5::S);
    k.rs_stage[1] = stage_record_doubles(M::N, TabCK54::S);
    k.bwd[0][1] = (const void *)backward_kernel<M, TabDopri5, float>;
    k.bwd[1][1] = (const void *)backward_kernel<M, TabCK54, float>;
    k.bwd[0][2] = (const void *)backward_kernel_dw<M, TabDopri5, true>;
    k.bwd[1][2] = (const void *)backward_kernel_dw<M, TabCK54, true>;
    k.bwd1[0][2] = (const void *)backward_kernel_dw<M, TabDopri5, false>;
    k.bwd1[1][2] = (const void *)backward_kernel_dw<M, TabCK54, false>;
    k.bwd2[0][1] = (const void *)backward_kernel_2level<M, TabDopri5, float>;
    k.bwd2[1][1] = (const void *)backward_kernel_2level<M, TabCK54, float>;
    k.bwd2[0][2] = (const void *)backward_kernel_2level_dw<M, TabDopri5>;
    k.bwd2[1][2] = (const void *)backward_kernel_2level_dw<M, TabCK54>;
    k.dw_records = true;
    fill_rkf78(k);
    fill_fixed(k);
    fill_replay(k);
    return k;
}

const KernelSet *kernels_vdp()
{
    static const KernelSet k = make_set<ModelVdP>(fill_fp64_vdp, fill_rkf78_vdp, fill_fixed_vdp, fill_replay_vdp);
    return &k;
}
const KernelSet *kernels_vdp_petsc()
{
    static const KernelSet k = make_set<ModelVdPPetsc>(fill_fp64_vdp_petsc, fill_rkf78_vdp_petsc,
                                                          fill_fixed_vdp_petsc, fill_replay_vdp_petsc);
    return &k;
}
const KernelSet *kernels_dho()
{
    static const KernelSet k = make_set<ModelDHO>(fill_fp64_dho, fill_rkf78_dho, fill_fixed_dho, fill_replay_dho);
    return &k;
}
const KernelSet *kernels_decay()
{
    static const KernelSet k = make_set<ModelDecay>(fill_fp64_decay, fill_rkf78_decay, fill_fixed_decay,
                                                       fill_replay_decay);
    return &k;
}

} // namespace va
