// Float and double-word sweeps of the fixed-step tableaux (runge_kutta4 = 3,
// euler = 4): the one-thread models (with two-level backward) and the
// per-instance GLV lane groups.  FP64 entries in va_inst_fixed_fp64.cu.
#include "va_group.cuh"
#include "va_group_dw.cuh"
#include "va_kernels.cuh"
#include "va_kernels_dw.cuh"
#include "va_models.cuh"
#include "va_registry.h"

namespace va {

void fill_fixed_fp64_vdp(KernelSet &k);
void fill_fixed_fp64_vdp_petsc(KernelSet &k);
void fill_fixed_fp64_dho(KernelSet &k);
void fill_fixed_fp64_decay(KernelSet &k);
void fill_fixed_fp64_glv5(KernelSet &k);
void fill_fixed_fp64_glv10(KernelSet &k);

template <class M, int I, class Tab>
static void fill_one(KernelSet &k)
{
    k.fwd[I][1] = (const void *)forward_kernel<M, Tab, float>;
    k.bwd[I][1] = (const void *)backward_kernel<M, Tab, float>;
    k.bwd2[I][1] = (const void *)backward_kernel_2level<M, Tab, float>;
    k.fwd[I][2] = (const void *)forward_kernel_dw<M, Tab, true>;
    k.fwd2[I][2] = (const void *)forward_kernel_dw<M, Tab, false>;
    k.bwd[I][2] = (const void *)backward_kernel_dw<M, Tab, true>;
    k.bwd1[I][2] = (const void *)backward_kernel_dw<M, Tab, false>;
    k.bwd2[I][2] = (const void *)backward_kernel_2level_dw<M, Tab>;
    k.rs_stage[I] = stage_record_doubles(M::N, Tab::S);
}

template <class M>
static void fill(KernelSet &k)
{
    fill_one<M, 3, TabRK4>(k);
    fill_one<M, 4, TabEuler>(k);
}

template <int NN, int I, class Tab>
static void fill_group_one(KernelSet &k)
{
    using M = ModelGLVLane<NN>;
    k.fwd[I][1] = (const void *)forward_group_kernel<M, Tab, float>;
    k.bwd[I][1] = (const void *)backward_group_kernel<M, Tab, float>;
    k.fwd[I][2] = (const void *)forward_group_dw_kernel<NN, Tab>;
    k.bwd[I][2] = (const void *)backward_group_dw_kernel<NN, Tab>;
    k.fwd2[I][2] = (const void *)forward_group_kernel<M, Tab, dword>;
    k.bwd1[I][2] = (const void *)backward_group_kernel<M, Tab, dword>;
    k.rs_stage[I] = group_stage_record_doubles(NN, Tab::S);
}

void fill_fixed_vdp(KernelSet &k)
{
    fill_fixed_fp64_vdp(k);
    fill<ModelVdP>(k);
}
void fill_fixed_vdp_petsc(KernelSet &k)
{
    fill_fixed_fp64_vdp_petsc(k);
    fill<ModelVdPPetsc>(k);
}
void fill_fixed_dho(KernelSet &k)
{
    fill_fixed_fp64_dho(k);
    fill<ModelDHO>(k);
}
void fill_fixed_decay(KernelSet &k)
{
    fill_fixed_fp64_decay(k);
    fill<ModelDecay>(k);
}
void fill_fixed_glv5(KernelSet &k)
{
    fill_fixed_fp64_glv5(k);
    fill_group_one<5, 3, TabRK4>(k);
    fill_group_one<5, 4, TabEuler>(k);
}
void fill_fixed_glv10(KernelSet &k)
{
    fill_fixed_fp64_glv10(k);
    fill_group_one<10, 3, TabRK4>(k);
    fill_group_one<10, 4, TabEuler>(k);
}

} // namespace va
