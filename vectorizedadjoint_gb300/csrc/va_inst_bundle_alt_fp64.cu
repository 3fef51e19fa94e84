// FP64 shared-matrix GLV bundles of 2 instances (the other width, for the
// autotuner), the 5(4) pairs.  Built with -fmad=false, like every FP64 unit.
#include "va_bundle.cuh"
#include "va_registry.h"

namespace va {

template <int NT>
static void fill(BundleKernelSet &k)
{
    constexpr int NB = kBundleNBdw;
    k.fwd_alt[0][0] = (const void *)forward_bundle_kernel<NT, NB, TabDopri5, double>;
    k.bwd_alt[0][0] = (const void *)backward_bundle_kernel<NT, NB, TabDopri5, double>;
    k.fwd_alt[1][0] = (const void *)forward_bundle_kernel<NT, NB, TabCK54, double>;
    k.bwd_alt[1][0] = (const void *)backward_bundle_kernel<NT, NB, TabCK54, double>;
}

void fill_bundle_alt_fp64_64(BundleKernelSet &k) { fill<64>(k); }
void fill_bundle_alt_fp64_256(BundleKernelSet &k) { fill<256>(k); }

} // namespace va
