// FP64 sweeps of the shared-matrix GLV bundle kernels, built with
// -fmad=false so that each instance reproduces the oracle bit for bit.
#include "va_bundle.cuh"
#include "va_registry.h"

namespace va {

template <int NT>
static void fill(BundleKernelSet &k)
{
    constexpr int NB = kBundleNB;
    k.fwd[0][0] = (const void *)forward_bundle_kernel<NT, NB, TabDopri5, double>;
    k.fwd[1][0] = (const void *)forward_bundle_kernel<NT, NB, TabCK54, double>;
    k.bwd[0][0] = (const void *)backward_bundle_kernel<NT, NB, TabDopri5, double>;
    k.bwd[1][0] = (const void *)backward_bundle_kernel<NT, NB, TabCK54, double>;
    k.fwd[3][0] = (const void *)forward_bundle_kernel<NT, NB, TabRK4, double>;
    k.bwd[3][0] = (const void *)backward_bundle_kernel<NT, NB, TabRK4, double>;
    k.fwd[4][0] = (const void *)forward_bundle_kernel<NT, NB, TabEuler, double>;
    k.bwd[4][0] = (const void *)backward_bundle_kernel<NT, NB, TabEuler, double>;
}

void fill_fp64_bundle64(BundleKernelSet &k) { fill<64>(k); }
void fill_fp64_bundle256(BundleKernelSet &k) { fill<256>(k); }

} // namespace va
