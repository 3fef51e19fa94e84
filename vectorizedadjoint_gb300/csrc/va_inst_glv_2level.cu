// Two-level backward sweeps of the per-instance GLV lane groups (N = 5, 10):
// float and double-word stages, every tableau; FP64 in
// va_inst_glv_2level_fp64.cu.
#include "va_group_2level.cuh"
#include "va_registry.h"

namespace va {

void fill_2level_fp64_glv5(KernelSet &k);
void fill_2level_fp64_glv10(KernelSet &k);

template <int NN, int I, class Tab>
static void fill_one(KernelSet &k)
{
    using M = ModelGLVLane<NN>;
    k.bwd2[I][1] = (const void *)backward_group_kernel_2level<M, Tab, float>;
    k.bwd2[I][2] = (const void *)backward_group_kernel_2level<M, Tab, dword>;
}

template <int NN>
static void fill(KernelSet &k)
{
    fill_one<NN, 0, TabDopri5>(k);
    fill_one<NN, 1, TabCK54>(k);
    fill_one<NN, 2, TabRKF78>(k);
    fill_one<NN, 3, TabRK4>(k);
    fill_one<NN, 4, TabEuler>(k);
}

void fill_2level_glv5(KernelSet &k)
{
    fill_2level_fp64_glv5(k);
    fill<5>(k);
}
void fill_2level_glv10(KernelSet &k)
{
    fill_2level_fp64_glv10(k);
    fill<10>(k);
}

} // namespace va
