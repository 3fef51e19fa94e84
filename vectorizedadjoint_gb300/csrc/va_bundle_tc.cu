// Cluster backward sweep of the shared-matrix GLV with tensor-core stage
// products (va_bundle_tc.cuh): digit planes of A^T, instantiations for the
// 5(4) pairs, and the launch.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "va_bundle_tc.cuh"

namespace va {

// digit planes of a matrix M (element (row i, k) = M[i][k]): per row and
// quarter of k an exponent, 6 digits per entry, in the operand blocks [row
// tile][quarter] of the cluster sweeps
__device__ __forceinline__ void bt_digits_row(double m_ik, int i, int k, uint8_t *adig, int *aexp)
{
    __shared__ float red[8];
    const dword v(m_ik);
    int e[kTcQuarters];
    tc_quarter_exponents(fabsf(v.hi), red, e);
    const int q = k / 64, mt = i / 128, row = i % 128;
    float d[kBtQA];
    split_digits<kBtQA>(v.hi, v.lo, digit_scale(e[q]), d);
    uint8_t *blk = adig + (size_t)(mt * 4 + q) * kBtABytes + (size_t)((k % 64) / 8) * (128 * 16) + (size_t)row * 16 +
                   (size_t)(k % 8) * 2;
#pragma unroll
    for (int s = 0; s < kBtQA; s++)
        *reinterpret_cast<uint16_t *>(blk + (size_t)s * kBtAPlane) = bf16_bits(d[s]);
    if (k < kTcQuarters)
        aexp[k * kBtN + i] = e[k];
}

__global__ void __launch_bounds__(256) bt_digits_A_kernel(const double *A, uint8_t *adig, int *aexp)
{
    const int i = blockIdx.x, k = threadIdx.x;
    bt_digits_row(A[(size_t)k * kBtN + i], i, k, adig, aexp); // A^T[i][k]
}

__global__ void __launch_bounds__(256) bt_digits_Af_kernel(const double *A, uint8_t *adig, int *aexp)
{
    const int i = blockIdx.x, k = threadIdx.x;
    bt_digits_row(A[(size_t)i * kBtN + k], i, k, adig, aexp); // A[i][k]
}

__global__ void __launch_bounds__(256) bt_pack_r_kernel(const double *par, double *rpk)
{
    const size_t x = (size_t)blockIdx.x * kBtN + threadIdx.x;
    rpk[x] = dw_pack(dword(par[x]));
}

namespace {

const void *bt_kernel(int tableau)
{
    switch (tableau) {
    case 0:
        return (const void *)backward_bundle_tc_kernel<TabDopri5>;
    case 1:
        return (const void *)backward_bundle_tc_kernel<TabCK54>;
    default:
        return nullptr;
    }
}

// the forward needs the FSAL pair (DOPRI5)
const void *bt_fwd_kernel(int tableau) { return tableau == 0 ? (const void *)forward_bundle_tc_kernel<TabDopri5> : nullptr; }

// the tail sweeps: double-word bundles of kTailNB instances per CTA
constexpr int kTailNB = 1;
const void *tail_fwd_kernel(int tableau)
{
    return tableau == 0 ? (const void *)forward_bundle_kernel<kBtN, kTailNB, TabDopri5, dword, true> : nullptr;
}
const void *tail_bwd_kernel(int tableau)
{
    switch (tableau) {
    case 0:
        return (const void *)backward_bundle_kernel<kBtN, kTailNB, TabDopri5, dword, true>;
    case 1:
        return (const void *)backward_bundle_kernel<kBtN, kTailNB, TabCK54, dword, true>;
    default:
        return nullptr;
    }
}
constexpr size_t kTailFwdSmem = bundle_fwd_smem_bytes<kBtN, kTailNB, dword>();
constexpr size_t kTailBwdSmem = 3 * sizeof(dword) * (size_t)TabDopri5::S * kBtN * kTailNB; // the bundle's stages

// per device: the kernels' shared-memory attribute is set and a cluster of 8
// CTAs of kBtSmem bytes fits on this GPU (clusters: how many at once)
struct BtState {
    std::once_flag once;
    bool ok = false;
    int clusters = 0;
};
BtState g_bt[64];

int bt_cluster_fits(const void *fn)
{
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBtSmem) != cudaSuccess)
        return false;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(kBtCluster);
    cfg.blockDim = dim3(kBtThreads);
    cfg.dynamicSmemBytes = kBtSmem;
    cudaLaunchAttribute attr{};
    attr.id = cudaLaunchAttributeClusterDimension;
    attr.val.clusterDim.x = kBtCluster;
    attr.val.clusterDim.y = 1;
    attr.val.clusterDim.z = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    int clusters = 0;
    return cudaOccupancyMaxActiveClusters(&clusters, fn, &cfg) == cudaSuccess ? clusters : 0;
}

void bt_setup(int dev)
{
    int clusters = 1 << 30;
    for (int tb = 0; tb < 2; tb++)
        clusters = std::min(clusters, bt_cluster_fits(bt_kernel(tb)));
    clusters = std::min(clusters, bt_cluster_fits(bt_fwd_kernel(0)));
    bool ok = clusters > 0;
    for (int tb = 0; tb < 2 && ok; tb++) {
        ok = cudaFuncSetAttribute(tail_bwd_kernel(tb), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kTailBwdSmem) == cudaSuccess;
    }
    ok = ok && cudaFuncSetAttribute(tail_fwd_kernel(0), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)kTailFwdSmem) == cudaSuccess;
    (void)cudaGetLastError(); // a refused attribute or query leaves no sticky error
    g_bt[dev].ok = ok;
    g_bt[dev].clusters = ok ? clusters : 0;
}

BtState *bt_state()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
        return nullptr;
    std::call_once(g_bt[dev].once, bt_setup, dev);
    return &g_bt[dev];
}
bool bt_ready()
{
    const BtState *st = bt_state();
    return st && st->ok;
}

// tiles of the cluster sweep and the instances [tail0, B) left to the tail
struct BtSplit {
    int tiles, tail0;
};
BtSplit bt_split(int B)
{
    const BtState *st = bt_state();
    const int tiles = (B + kBtTile - 1) / kBtTile;
    const int c = st ? st->clusters : 0;
    if (c > 0 && tiles > c && tiles % c == 1)
        return {tiles - 1, (tiles - 1) * kBtTile};
    return {tiles, B};
}

// the tail sweep over instances [tail0, B): one CTA per instance, started
// once the cluster sweep before it in the stream has all its CTAs resident
cudaError_t launch_tail(const void *fn, BundleParams bp, int B, int tail0, size_t smem, cudaStream_t s)
{
    bp.inst0 = tail0;
    bp.nb = kTailNB;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)((B - tail0 + kTailNB - 1) / kTailNB));
    cfg.blockDim = dim3(kBtN);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr{};
    attr.id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr.val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    void *args[] = {&bp};
    return cudaLaunchKernelExC(&cfg, fn, args);
}

} // namespace

bool bundle_tc_available(int tableau) { return bt_kernel(tableau) && bt_ready(); }
int bundle_tc_tiles(int B) { return bt_split(B).tiles; }
bool bundle_tc_forward_available(int tableau) { return bt_fwd_kernel(tableau) && bt_ready(); }

cudaError_t enqueue_bundle_tc_forward(const BundleParams &bp, const double *A, uint8_t *adig, int *aexp,
                                      double *rpk, unsigned *error, int tableau, cudaStream_t s)
{
    const void *fn = bt_fwd_kernel(tableau);
    if (!fn)
        return cudaErrorInvalidValue;
    bt_digits_Af_kernel<<<kBtN, 256, 0, s>>>(A, adig, aexp);
    bt_pack_r_kernel<<<bp.f.B, 256, 0, s>>>(bp.f.par, rpk);
    BundleTcParams p{};
    p.bp = bp;
    p.adig = adig;
    p.rpk = rpk;
    p.aexp = aexp;
    p.error = error;
    const BtSplit sp = bt_split(bp.f.B);
    void *args[] = {&p};
    cudaError_t e = cudaLaunchKernel(fn, dim3(sp.tiles * kBtCluster), dim3(kBtThreads), args, kBtSmem, s);
    if (e == cudaSuccess && sp.tail0 < bp.f.B)
        e = launch_tail(tail_fwd_kernel(tableau), bp, bp.f.B, sp.tail0, kTailFwdSmem, s);
    return e;
}

cudaError_t enqueue_bundle_tc_backward(const BundleParams &bp, const double *A, uint8_t *adig, int *aexp,
                                       double *rpk, unsigned *error, int tableau, cudaStream_t s)
{
    const void *fn = bt_kernel(tableau);
    if (!fn)
        return cudaErrorInvalidValue;
    bt_digits_A_kernel<<<kBtN, 256, 0, s>>>(A, adig, aexp);
    bt_pack_r_kernel<<<bp.g.B, 256, 0, s>>>(bp.g.par, rpk);
    BundleTcParams p{};
    p.bp = bp;
    p.adig = adig;
    p.rpk = rpk;
    p.aexp = aexp;
    p.error = error;
    const BtSplit sp = bt_split(bp.g.B);
    void *args[] = {&p};
    cudaError_t e = cudaLaunchKernel(fn, dim3(sp.tiles * kBtCluster), dim3(kBtThreads), args, kBtSmem, s);
    if (e == cudaSuccess && sp.tail0 < bp.g.B)
        e = launch_tail(tail_bwd_kernel(tableau), bp, bp.g.B, sp.tail0, kTailBwdSmem, s);
    return e;
}

} // namespace va
