// Two-level backward sweeps of the shared-matrix GLV bundles (N = 64, 256):
// float and double-word stages; FP64 in va_inst_bundle_2level_fp64.cu.
#include "va_bundle_2level.cuh"
#include "va_registry.h"

namespace va {

void fill_bundle_2level_fp64_64(BundleKernelSet &k);
void fill_bundle_2level_fp64_256(BundleKernelSet &k);

template <int NT, int I, class Tab>
static void fill_one(BundleKernelSet &k)
{
    k.bwd2[I][1] = (const void *)backward_bundle_kernel_2level<NT, kBundleNB, Tab, float>;
    k.bwd2[I][2] = (const void *)backward_bundle_kernel_2level<NT, kBundleNBdw, Tab, dword>;
}

template <int NT>
static void fill(BundleKernelSet &k)
{
    fill_one<NT, 0, TabDopri5>(k);
    fill_one<NT, 1, TabCK54>(k);
    fill_one<NT, 3, TabRK4>(k);
    fill_one<NT, 4, TabEuler>(k);
}

void fill_bundle_2level64(BundleKernelSet &k)
{
    fill_bundle_2level_fp64_64(k);
    fill<64>(k);
}
void fill_bundle_2level256(BundleKernelSet &k)
{
    fill_bundle_2level_fp64_256(k);
    fill<256>(k);
}

} // namespace va
