// Fehlberg 7(8) FP64 sweeps of the one-thread models.  Built with
// -fmad=false, like va_inst_small_fp64.cu, so they reproduce the oracle bit
// for bit.
#include "va_kernels.cuh"
#include "va_models.cuh"
#include "va_registry.h"

namespace va {

template <class M>
static void fill(KernelSet &k)
{
    k.fwd[2][0] = (const void *)forward_kernel<M, TabRKF78, double>;
    k.bwd[2][0] = (const void *)backward_kernel<M, TabRKF78, double>;
    k.bwd2[2][0] = (const void *)backward_kernel_2level<M, TabRKF78, double>;
}

void fill_rkf78_fp64_vdp(KernelSet &k) { fill<ModelVdP>(k); }
void fill_rkf78_fp64_vdp_petsc(KernelSet &k) { fill<ModelVdPPetsc>(k); }
void fill_rkf78_fp64_dho(KernelSet &k) { fill<ModelDHO>(k); }
void fill_rkf78_fp64_decay(KernelSet &k) { fill<ModelDecay>(k); }

} // namespace va
