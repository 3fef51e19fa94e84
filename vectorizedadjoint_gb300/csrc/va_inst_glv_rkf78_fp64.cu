// Fehlberg 7(8) FP64 sweeps of the per-instance GLV model (lane groups),
// built with -fmad=false like va_inst_glv_fp64.cu.
#include "va_group.cuh"
#include "va_registry.h"

namespace va {

template <int NN>
static void fill(KernelSet &k)
{
    using M = ModelGLVLane<NN>;
    k.fwd[2][0] = (const void *)forward_group_kernel<M, TabRKF78, double>;
    k.bwd[2][0] = (const void *)backward_group_kernel<M, TabRKF78, double>;
}

void fill_rkf78_fp64_glv5(KernelSet &k) { fill<5>(k); }
void fill_rkf78_fp64_glv10(KernelSet &k) { fill<10>(k); }

} // namespace va
