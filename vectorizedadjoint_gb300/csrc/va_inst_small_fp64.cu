// FP64 sweeps of the one-thread-per-instance models.  Built with
// -fmad=false: every product and sum is rounded on its own, in the operation
// order of the reference's expressions, so the FP64 path reproduces the CPU
// oracle (compiled with -ffp-contract=off) bit for bit.
#include "va_kernels.cuh"
#include "va_models.cuh"
#include "va_registry.h"

namespace va {

template <class M>
static void fill(KernelSet &k)
{
    k.fwd[0][0] = (const void *)forward_kernel<M, TabDopri5, double>;
    k.fwd[1][0] = (const void *)forward_kernel<M, TabCK54, double>;
    k.bwd[0][0] = (const void *)backward_kernel<M, TabDopri5, double>;
    k.bwd[1][0] = (const void *)backward_kernel<M, TabCK54, double>;
    k.bwd2[0][0] = (const void *)backward_kernel_2level<M, TabDopri5, double>;
    k.bwd2[1][0] = (const void *)backward_kernel_2level<M, TabCK54, double>;
}

void fill_fp64_vdp(KernelSet &k) { fill<ModelVdP>(k); }
void fill_fp64_vdp_petsc(KernelSet &k) { fill<ModelVdPPetsc>(k); }
void fill_fp64_dho(KernelSet &k) { fill<ModelDHO>(k); }
void fill_fp64_decay(KernelSet &k) { fill<ModelDecay>(k); }

} // namespace va
