// FP64 sweeps of the per-instance GLV model, built with -fmad=false so that
// they reproduce the CPU oracle bit for bit (see va_inst_small_fp64.cu).
#include "va_group.cuh"
#include "va_registry.h"

namespace va {

template <int NN>
static void fill(KernelSet &k)
{
    using M = ModelGLVLane<NN>;
    k.fwd[0][0] = (const void *)forward_group_kernel<M, TabDopri5, double>;
    k.fwd[1][0] = (const void *)forward_group_kernel<M, TabCK54, double>;
    k.bwd[0][0] = (const void *)backward_group_kernel<M, TabDopri5, double>;
    k.bwd[1][0] = (const void *)backward_group_kernel<M, TabCK54, double>;
}

void fill_fp64_glv5(KernelSet &k) { fill<5>(k); }
void fill_fp64_glv10(KernelSet &k) { fill<10>(k); }

} // namespace va
