// The other bundle width of the shared-matrix GLV sweeps, for the autotuner:
// float-stage bundles of 2 instances and double-word bundles of 4 (the
// defaults are 4 and 2), the 5(4) pairs.  FP64 bundles of 2 come from
// va_inst_bundle_alt_fp64.cu, built without FMA contraction.
#include "va_bundle.cuh"
#include "va_registry.h"

namespace va {

template <int NT, int I, class Tab>
static void fill_tab(BundleKernelSet &k)
{
    constexpr int NB = kBundleNBdw, NW = kBundleNB;
    k.fwd_alt[I][1] = (const void *)forward_bundle_kernel<NT, NB, Tab, float>;
    k.bwd_alt[I][1] = (const void *)backward_bundle_kernel<NT, NB, Tab, float>;
    k.fwd_alt[I][2] = (const void *)forward_bundle_kernel<NT, NW, Tab, dword, true>;
    k.fwd1_alt[I][2] = (const void *)forward_bundle_kernel<NT, NW, Tab, dword>;
    k.bwd_alt[I][2] = (const void *)backward_bundle_kernel<NT, NW, Tab, dword, true>;
    k.bwd1_alt[I][2] = (const void *)backward_bundle_kernel<NT, NW, Tab, dword>;
}

void fill_bundle_alt64(BundleKernelSet &k)
{
    fill_tab<64, 0, TabDopri5>(k);
    fill_tab<64, 1, TabCK54>(k);
}

void fill_bundle_alt256(BundleKernelSet &k)
{
    fill_tab<256, 0, TabDopri5>(k);
    fill_tab<256, 1, TabCK54>(k);
}

} // namespace va
