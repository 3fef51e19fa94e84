// Shared-matrix GLV bundle kernels (N = 64, 256; 4 instances per CTA, 2 in
// the double-word sweeps):
// reduced-precision sweeps (double-word: with and without stage records) and
// the helper kernels.  FP64 sweeps come from
// va_inst_bundle_fp64.cu, built without FMA contraction.
#include "va_bundle.cuh"
#include "va_registry.h"

namespace va {

void fill_fp64_bundle64(BundleKernelSet &k);
void fill_fp64_bundle256(BundleKernelSet &k);

// the fixed-step tableaux (runge_kutta4, euler): tableau slot I
template <int NT, int I, class Tab>
static void fill_fixed(BundleKernelSet &k)
{
    constexpr int NB = kBundleNB, NW = kBundleNBdw;
    k.fwd[I][1] = (const void *)forward_bundle_kernel<NT, NB, Tab, float>;
    k.fwd[I][2] = (const void *)forward_bundle_kernel<NT, NW, Tab, dword, true>;
    k.fwd1[I][2] = (const void *)forward_bundle_kernel<NT, NW, Tab, dword>;
    k.bwd[I][1] = (const void *)backward_bundle_kernel<NT, NB, Tab, float>;
    k.bwd[I][2] = (const void *)backward_bundle_kernel<NT, NW, Tab, dword, true>;
    k.bwd1[I][2] = (const void *)backward_bundle_kernel<NT, NW, Tab, dword>;
    k.rs_stage[I] = bundle_stage_record_doubles(NT, Tab::S);
    k.nsv[I] = factor_stages<Tab>();
}

template <int NT>
static BundleKernelSet make_bundle(void (*fill_fp64)(BundleKernelSet &))
{
    constexpr int NB = kBundleNB, NW = kBundleNBdw;
    BundleKernelSet k{};
    k.N = NT;
    k.nb[0] = k.nb[1] = NB;
    k.nb[2] = NW;
    fill_fp64(k);
    k.fwd[0][1] = (const void *)forward_bundle_kernel<NT, NB, TabDopri5, float>;
    k.fwd[0][2] = (const void *)forward_bundle_kernel<NT, NW, TabDopri5, dword, true>;
    k.fwd1[0][2] = (const void *)forward_bundle_kernel<NT, NW, TabDopri5, dword>;
    k.fwd[1][1] = (const void *)forward_bundle_kernel<NT, NB, TabCK54, float>;
    k.fwd[1][2] = (const void *)forward_bundle_kernel<NT, NW, TabCK54, dword, true>;
    k.fwd1[1][2] = (const void *)forward_bundle_kernel<NT, NW, TabCK54, dword>;
    k.bwd[0][1] = (const void *)backward_bundle_kernel<NT, NB, TabDopri5, float>;
    k.bwd[0][2] = (const void *)backward_bundle_kernel<NT, NW, TabDopri5, dword, true>;
    k.bwd1[0][2] = (const void *)backward_bundle_kernel<NT, NW, TabDopri5, dword>;
    k.bwd[1][1] = (const void *)backward_bundle_kernel<NT, NB, TabCK54, float>;
    k.bwd[1][2] = (const void *)backward_bundle_kernel<NT, NW, TabCK54, dword, true>;
    k.bwd1[1][2] = (const void *)backward_bundle_kernel<NT, NW, TabCK54, dword>;
    k.rs_stage[0] = bundle_stage_record_doubles(NT, TabDopri5::S);
    k.rs_stage[1] = bundle_stage_record_doubles(NT, TabCK54::S);
    k.nsv[0] = factor_stages<TabDopri5>();
    k.nsv[1] = factor_stages<TabCK54>();
    fill_fixed<NT, 3, TabRK4>(k);
    fill_fixed<NT, 4, TabEuler>(k);
    const size_t sz[3] = {sizeof(double), sizeof(float), sizeof(dword)};
    k.smem_fwd[0] = bundle_fwd_smem_bytes<NT, NB, double>();
    k.smem_fwd[1] = bundle_fwd_smem_bytes<NT, NB, float>();
    k.smem_fwd[2] = bundle_fwd_smem_bytes<NT, NW, dword>();
    for (int p = 0; p < 3; p++) {
        const size_t nb = k.nb[p];
        k.smem_bwd[p] = 3 * sz[p] * (size_t)TabDopri5::S * NT * nb;
    }
    k.prepare = (const void *)prepare_A_kernel<NT>;
    k.reduce = (const void *)reduce_dA_kernel<NT>;
    if constexpr (NT == 64) {
        fill_bundle_alt64(k);
        fill_bundle_alt_fp64_64(k);
    } else {
        fill_bundle_alt256(k);
        fill_bundle_alt_fp64_256(k);
    }
    if constexpr (NT == 64)
        fill_bundle_2level64(k);
    else
        fill_bundle_2level256(k);
    for (int p = 0; p < 3; p++)
        k.smem_bwd2[p] = k.smem_bwd[p] + sizeof(double) * (NT / 32) * k.nb[p];
    k.nb_alt[0] = k.nb_alt[1] = kBundleNBdw;
    k.nb_alt[2] = kBundleNB;
    k.smem_fwd_alt[0] = bundle_fwd_smem_bytes<NT, NW, double>();
    k.smem_fwd_alt[1] = bundle_fwd_smem_bytes<NT, NW, float>();
    k.smem_fwd_alt[2] = bundle_fwd_smem_bytes<NT, NB, dword>();
    for (int p = 0; p < 3; p++) {
        const size_t nb = k.nb_alt[p];
        k.smem_bwd_alt[p] = 3 * sz[p] * (size_t)TabDopri5::S * NT * nb;
    }
    return k;
}

const BundleKernelSet *kernels_glv_shared(int n)
{
    static const BundleKernelSet k64 = make_bundle<64>(fill_fp64_bundle64);
    static const BundleKernelSet k256 = make_bundle<256>(fill_fp64_bundle256);
    switch (n) {
    case 64:
        return &k64;
    case 256:
        return &k256;
    default:
        return nullptr;
    }
}

} // namespace va
