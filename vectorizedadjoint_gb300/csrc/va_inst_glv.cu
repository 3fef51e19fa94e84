// Generalized Lotka-Volterra kernels with a per-instance interaction matrix:
// lane groups of N threads per instance, for the compiled sizes N = 5, 10.
// Reduced-precision sweeps here; FP64 sweeps in va_inst_glv_fp64.cu.
#include "va_group.cuh"
#include "va_registry.h"

namespace va {

void fill_fp64_glv5(KernelSet &k);
void fill_fp64_glv10(KernelSet &k);

template <int NN>
static KernelSet make_glv(void (*fill_fp64)(KernelSet &))
{
    using M = ModelGLVLane<NN>;
    KernelSet k{};
    k.N = NN;
    k.P = NN + NN * NN;
    k.tpi = NN;
    fill_fp64(k);
    k.fwd[0][1] = (const void *)forward_group_kernel<M, TabDopri5, float>;
    k.fwd[0][2] = (const void *)forward_group_kernel<M, TabDopri5, dword>;
    k.fwd[1][1] = (const void *)forward_group_kernel<M, TabCK54, float>;
    k.fwd[1][2] = (const void *)forward_group_kernel<M, TabCK54, dword>;
    k.bwd[0][1] = (const void *)backward_group_kernel<M, TabDopri5, float>;
    k.bwd[0][2] = (const void *)backward_group_kernel<M, TabDopri5, dword>;
    k.bwd[1][1] = (const void *)backward_group_kernel<M, TabCK54, float>;
    k.bwd[1][2] = (const void *)backward_group_kernel<M, TabCK54, dword>;
    return k;
}

const KernelSet *kernels_glv(int n)
{
    static const KernelSet k5 = make_glv<5>(fill_fp64_glv5);
    static const KernelSet k10 = make_glv<10>(fill_fp64_glv10);
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
