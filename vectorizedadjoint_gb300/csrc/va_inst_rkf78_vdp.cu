// Fehlberg 7(8) kernels of the two Van der Pol forms.
#include "va_rkf78_fill.cuh"

namespace va {

void fill_rkf78_fp64_vdp(KernelSet &k);
void fill_rkf78_fp64_vdp_petsc(KernelSet &k);

void fill_rkf78_vdp(KernelSet &k)
{
    fill_rkf78_fp64_vdp(k);
    fill_rkf78_reduced<ModelVdP>(k);
}
void fill_rkf78_vdp_petsc(KernelSet &k)
{
    fill_rkf78_fp64_vdp_petsc(k);
    fill_rkf78_reduced<ModelVdPPetsc>(k);
}

} // namespace va
