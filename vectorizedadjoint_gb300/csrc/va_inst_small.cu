// Kernel instantiations for the one-thread-per-instance models.
#include "va_kernels.cuh"
#include "va_models.cuh"
#include "va_registry.h"

namespace va {

template <class M>
static KernelSet make_set()
{
    KernelSet k{};
    k.N = M::N;
    k.P = M::P;
    k.tpi = 1;
    k.fwd[0][0] = (const void *)forward_kernel<M, TabDopri5, double>;
    k.fwd[0][1] = (const void *)forward_kernel<M, TabDopri5, float>;
    k.fwd[1][0] = (const void *)forward_kernel<M, TabCK54, double>;
    k.fwd[1][1] = (const void *)forward_kernel<M, TabCK54, float>;
    k.fwd[0][2] = (const void *)forward_kernel<M, TabDopri5, dword>;
    k.fwd[1][2] = (const void *)forward_kernel<M, TabCK54, dword>;
    k.bwd[0][2] = (const void *)backward_kernel<M, TabDopri5, dword>;
    k.bwd[1][2] = (const void *)backward_kernel<M, TabCK54, dword>;
    k.bwd[0][0] = (const void *)backward_kernel<M, TabDopri5, double>;
    k.bwd[0][1] = (const void *)backward_kernel<M, TabDopri5, float>;
    k.bwd[1][0] = (const void *)backward_kernel<M, TabCK54, double>;
    k.bwd[1][1] = (const void *)backward_kernel<M, TabCK54, float>;
    return k;
}

const KernelSet *kernels_vdp()
{
    static const KernelSet k = make_set<ModelVdP>();
    return &k;
}
const KernelSet *kernels_vdp_petsc()
{
    static const KernelSet k = make_set<ModelVdPPetsc>();
    return &k;
}
const KernelSet *kernels_dho()
{
    static const KernelSet k = make_set<ModelDHO>();
    return &k;
}
const KernelSet *kernels_decay()
{
    static const KernelSet k = make_set<ModelDecay>();
    return &k;
}

} // namespace va
