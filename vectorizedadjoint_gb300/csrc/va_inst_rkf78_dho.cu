// Fehlberg 7(8) kernels of the damped oscillator and the decay model.
#include "va_rkf78_fill.cuh"

namespace va {

void fill_rkf78_fp64_dho(KernelSet &k);
void fill_rkf78_fp64_decay(KernelSet &k);

void fill_rkf78_dho(KernelSet &k)
{
    fill_rkf78_fp64_dho(k);
    fill_rkf78_reduced<ModelDHO>(k);
}
void fill_rkf78_decay(KernelSet &k)
{
    fill_rkf78_fp64_decay(k);
    fill_rkf78_reduced<ModelDecay>(k);
}

} // namespace va
