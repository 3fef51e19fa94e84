// Cluster backward sweep of the shared-matrix GLV with tensor-core stage
// products (va_bundle_tc.cuh): digit planes of A^T, instantiations for the
// 5(4) pairs, and the launch.
#include <cuda_runtime.h>

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

// per device: the kernels' shared-memory attribute is set and a cluster of 8
// CTAs of kBtSmem bytes fits on this GPU
struct BtState {
    std::once_flag once;
    bool ok = false;
};
BtState g_bt[64];

bool bt_cluster_fits(const void *fn)
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
    return cudaOccupancyMaxActiveClusters(&clusters, fn, &cfg) == cudaSuccess && clusters > 0;
}

void bt_setup(int dev)
{
    bool ok = true;
    for (int tb = 0; tb < 2 && ok; tb++)
        ok = bt_cluster_fits(bt_kernel(tb));
    ok = ok && bt_cluster_fits(bt_fwd_kernel(0));
    (void)cudaGetLastError(); // a refused attribute or query leaves no sticky error
    g_bt[dev].ok = ok;
}

bool bt_ready()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
        return false;
    std::call_once(g_bt[dev].once, bt_setup, dev);
    return g_bt[dev].ok;
}

} // namespace

bool bundle_tc_available(int tableau) { return bt_kernel(tableau) && bt_ready(); }
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
    const int tiles = (bp.f.B + kBtTile - 1) / kBtTile;
    void *args[] = {&p};
    return cudaLaunchKernel(fn, dim3(tiles * kBtCluster), dim3(kBtThreads), args, kBtSmem, s);
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
    const int tiles = (bp.g.B + kBtTile - 1) / kBtTile;
    void *args[] = {&p};
    return cudaLaunchKernel(fn, dim3(tiles * kBtCluster), dim3(kBtThreads), args, kBtSmem, s);
}

} // namespace va
