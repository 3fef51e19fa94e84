// Kernels of the batched tensor-core products G = A^T V (va_tc_matvec.cuh)
// and their C entry point on caller data (va_probe.h: va_matT_tc).
#include <cuda_runtime.h>

#include "../../include/va.h"
#include "../../include/va_probe.h"
#include "va_tc_matvec.cuh"

namespace va {

__global__ void __launch_bounds__(256) tc_digits_A_kernel(const double *A, uint8_t *adig, int *aexp)
{
    __shared__ float red[8];
    const int i = blockIdx.x, k = threadIdx.x;
    const dword a(A[(size_t)k * kTcN + i]); // A^T[i][k]
    int e[kTcQuarters];
    tc_quarter_exponents(fabsf(a.hi), red, e);
    const int q = k / kTcKQ;
    float d[kTcQ];
    split_digits<kTcQ>(a.hi, a.lo, digit_scale(e[q]), d);
#pragma unroll
    for (int s = 0; s < kTcQ; s++)
        *reinterpret_cast<uint16_t *>(adig + tc_a_offset(i / kTcTileM, q, s, i % kTcTileM, k)) = bf16_bits(d[s]);
    if (k < kTcQuarters)
        aexp[k * kTcN + i] = e[k];
}

__global__ void __launch_bounds__(256) tc_digits_V_kernel(const double *V, int B, uint8_t *vdig, int *vexp)
{
    __shared__ float red[8];
    const int b = blockIdx.x, k = threadIdx.x;
    const dword v = b < B ? dw_unpack(V[(size_t)b * kTcN + k]) : dword(0.0f, 0.0f);
    int e[kTcQuarters];
    tc_quarter_exponents(fabsf(v.hi), red, e);
    tc_write_v_digits(vdig, b, k, v, e[k / kTcKQ]);
    if (k < kTcQuarters)
        vexp[(size_t)b * kTcQuarters + k] = e[k];
}

__global__ void __launch_bounds__(256, 1) tc_gemm_kernel(const uint8_t *adig, const int *aexp, const uint8_t *vdig,
                                                         const int *vexp, int B, double *gpart, unsigned *error)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + kTcABlock + kTcVBlock);
    uint32_t *slot = reinterpret_cast<uint32_t *>(bar + 1);
    const int t = threadIdx.x;
    if (t < 32) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                     "r"(kTcTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (t == 0) {
        mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *slot;
    // blockIdx.x = (nt * kTcQuarters + q) * kTcTilesM + mt
    const int mt = blockIdx.x % kTcTilesM, q = (blockIdx.x / kTcTilesM) % kTcQuarters;
    const int nt = blockIdx.x / (kTcTilesM * kTcQuarters);
    uint32_t phase = 0;
    const bool ok = tc_gemm_tile(adig, aexp, vdig, vexp, B, gpart, mt, nt, q, smem, bar, tmem, phase, error);
    if (!ok && t == 0) // once more (bounded) for MMAs still in flight before the memory is released
        (void)mbar_wait_bounded(bar, phase ^ 1u, error);
    __syncthreads();
    tc_fence_after();
    if (t < 32)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcTmemCols) : "memory");
}

__global__ void tc_sum_quarters_kernel(const double *gpart, int B, double *G)
{
    const size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; // b * 256 + i
    if (x >= (size_t)B * kTcN)
        return;
    dword s = dw_unpack(gpart[x]);
#pragma unroll
    for (int q = 1; q < kTcQuarters; q++)
        s += dw_unpack(gpart[(size_t)q * B * kTcN + x]);
    G[x] = dw_pack(s);
}

} // namespace va

extern "C" VA_API int32_t va_matT_tc(int32_t B, const double *A, const double *V, double *G, void *stream)
{
    using namespace va;
    if (B < 1 || !A || !V || !G)
        return VA_BAD_ARGS;
    cudaStream_t s = (cudaStream_t)stream;
    const int nt = tc_instance_tiles(B), Bpad = nt * kTcTileN;
    uint8_t *adig = nullptr, *vdig = nullptr;
    int *aexp = nullptr, *vexp = nullptr;
    double *gpart = nullptr;
    unsigned *err = nullptr;
    cudaError_t e = cudaFuncSetAttribute(tc_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem);
    if (e == cudaSuccess)
        e = cudaMalloc(&adig, kTcTilesM * kTcQuarters * kTcABlock);
    if (e == cudaSuccess)
        e = cudaMalloc(&aexp, sizeof(int) * kTcQuarters * kTcN);
    if (e == cudaSuccess)
        e = cudaMalloc(&vdig, (size_t)nt * kTcQuarters * kTcVBlock);
    if (e == cudaSuccess)
        e = cudaMalloc(&vexp, sizeof(int) * (size_t)Bpad * kTcQuarters);
    if (e == cudaSuccess)
        e = cudaMalloc(&gpart, sizeof(double) * kTcQuarters * (size_t)B * kTcN);
    if (e == cudaSuccess)
        e = cudaMalloc(&err, sizeof(unsigned));
    if (e == cudaSuccess)
        e = cudaMemsetAsync(err, 0, sizeof(unsigned), s);
    if (e == cudaSuccess) {
        tc_digits_A_kernel<<<kTcN, 256, 0, s>>>(A, adig, aexp);
        tc_digits_V_kernel<<<Bpad, 256, 0, s>>>(V, B, vdig, vexp);
        tc_gemm_kernel<<<kTcTilesM * kTcQuarters * nt, 256, kTcSmem, s>>>(adig, aexp, vdig, vexp, B, gpart, err);
        tc_sum_quarters_kernel<<<(unsigned)(((size_t)B * kTcN + 255) / 256), 256, 0, s>>>(gpart, B, G);
        e = cudaGetLastError();
    }
    unsigned herr = 0;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&herr, err, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    cudaFree(adig);
    cudaFree(aexp);
    cudaFree(vdig);
    cudaFree(vexp);
    cudaFree(gpart);
    cudaFree(err);
    if (e != cudaSuccess || herr)
        return VA_CUDA_ERROR;
    return VA_OK;
}
