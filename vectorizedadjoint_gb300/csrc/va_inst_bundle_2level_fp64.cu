// FP64 two-level backward sweeps of the shared-matrix GLV bundles, built with
// -fmad=false like the forward sweeps they re-run (va_inst_bundle_fp64.cu).
#include "va_bundle_2level.cuh"
#include "va_registry.h"

namespace va {

template <int NT>
static void fill(BundleKernelSet &k)
{
    k.bwd2[0][0] = (const void *)backward_bundle_kernel_2level<NT, kBundleNB, TabDopri5, double>;
    k.bwd2[1][0] = (const void *)backward_bundle_kernel_2level<NT, kBundleNB, TabCK54, double>;
    k.bwd2[3][0] = (const void *)backward_bundle_kernel_2level<NT, kBundleNB, TabRK4, double>;
    k.bwd2[4][0] = (const void *)backward_bundle_kernel_2level<NT, kBundleNB, TabEuler, double>;
}

void fill_bundle_2level_fp64_64(BundleKernelSet &k) { fill<64>(k); }
void fill_bundle_2level_fp64_256(BundleKernelSet &k) { fill<256>(k); }

} // namespace va
