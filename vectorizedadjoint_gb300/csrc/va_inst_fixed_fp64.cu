// FP64 sweeps of the fixed-step tableaux (runge_kutta4 = 3, euler = 4) for
// every one-thread and lane-group model.  Built with -fmad=false, like
// va_inst_small_fp64.cu, so they reproduce the oracle bit for bit.
#include "va_group.cuh"
#include "va_kernels.cuh"
#include "va_models.cuh"
#include "va_registry.h"

namespace va {

template <class M, int I, class Tab>
static void fill_one(KernelSet &k)
{
    k.fwd[I][0] = (const void *)forward_kernel<M, Tab, double>;
    k.bwd[I][0] = (const void *)backward_kernel<M, Tab, double>;
    k.bwd2[I][0] = (const void *)backward_kernel_2level<M, Tab, double>;
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
    k.fwd[I][0] = (const void *)forward_group_kernel<M, Tab, double>;
    k.bwd[I][0] = (const void *)backward_group_kernel<M, Tab, double>;
}

void fill_fixed_fp64_vdp(KernelSet &k) { fill<ModelVdP>(k); }
void fill_fixed_fp64_vdp_petsc(KernelSet &k) { fill<ModelVdPPetsc>(k); }
void fill_fixed_fp64_dho(KernelSet &k) { fill<ModelDHO>(k); }
void fill_fixed_fp64_decay(KernelSet &k) { fill<ModelDecay>(k); }
void fill_fixed_fp64_glv5(KernelSet &k)
{
    fill_group_one<5, 3, TabRK4>(k);
    fill_group_one<5, 4, TabEuler>(k);
}
void fill_fixed_fp64_glv10(KernelSet &k)
{
    fill_group_one<10, 3, TabRK4>(k);
    fill_group_one<10, 4, TabEuler>(k);
}

} // namespace va
