// FP64 two-level backward sweeps of the per-instance GLV lane groups, built
// with -fmad=false like the forward sweeps they re-run (va_inst_glv_fp64.cu).
#include "va_group_2level.cuh"
#include "va_registry.h"

namespace va {

template <int NN>
static void fill(KernelSet &k)
{
    using M = ModelGLVLane<NN>;
    k.bwd2[0][0] = (const void *)backward_group_kernel_2level<M, TabDopri5, double>;
    k.bwd2[1][0] = (const void *)backward_group_kernel_2level<M, TabCK54, double>;
    k.bwd2[2][0] = (const void *)backward_group_kernel_2level<M, TabRKF78, double>;
    k.bwd2[3][0] = (const void *)backward_group_kernel_2level<M, TabRK4, double>;
    k.bwd2[4][0] = (const void *)backward_group_kernel_2level<M, TabEuler, double>;
}

void fill_2level_fp64_glv5(KernelSet &k) { fill<5>(k); }
void fill_2level_fp64_glv10(KernelSet &k) { fill<10>(k); }

} // namespace va
