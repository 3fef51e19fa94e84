// Generalized Lotka-Volterra kernels with a per-instance interaction matrix.
#include "va_registry.h"

namespace va {

const KernelSet *kernels_glv(int n)
{
    (void)n;
    return nullptr;
}

} // namespace va
