// Pipe-rate probes: the arithmetic rates that bound the sweep kernels,
// measured on the GPU the library runs on.  Not part of the solver path;
// bench.py reports them beside the roofline fractions, so that the choice of
// pipe for each contraction (FP64 vector FMA, FP64 tensor-core DMMA, FP32
// FMA) rests on measured numbers of this part.
//
// Each kernel runs `iters` iterations of eight independent dependency chains
// per thread (or per warp for the MMA forms), enough to cover the pipe
// latency at full occupancy; the accumulators are written out so nothing is
// eliminated.  FLOPs: FMA = 2; one MMA of shape m x n x k = 2 m n k.
#include <cuda_runtime.h>

#include <cstdint>

#include "va.h"
#include "va_probe.h"
#include "va_tcgen05.cuh"

namespace {

constexpr int kChains = 8;

__global__ void probe_fp64_fma(int iters, double *sink)
{
    double acc[kChains];
    const double a = 1.0 + 1e-9 * threadIdx.x, b = 1e-12;
#pragma unroll
    for (int c = 0; c < kChains; c++)
        acc[c] = c;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int c = 0; c < kChains; c++)
            acc[c] = fma(acc[c], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < kChains; c++)
        s += acc[c];
    sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void probe_fp32_fma(int iters, double *sink)
{
    float acc[kChains];
    const float a = 1.0f + 1e-7f * threadIdx.x, b = 1e-9f;
#pragma unroll
    for (int c = 0; c < kChains; c++)
        acc[c] = (float)c;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int c = 0; c < kChains; c++)
            acc[c] = fmaf(acc[c], a, b);
    }
    float s = 0.0f;
#pragma unroll
    for (int c = 0; c < kChains; c++)
        s += acc[c];
    sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// FP64 tensor-core MMA, m8n8k4 (one f64 of A and of B, two of C per thread)
__global__ void probe_dmma_m8n8k4(int iters, double *sink)
{
    double c[kChains][2];
    const double a = 1.0 + 1e-9 * threadIdx.x, b = 1e-12 * (threadIdx.x + 1);
#pragma unroll
    for (int k = 0; k < kChains; k++)
        c[k][0] = c[k][1] = k;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int k = 0; k < kChains; k++)
            asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                         : "+d"(c[k][0]), "+d"(c[k][1])
                         : "d"(a), "d"(b));
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < kChains; k++)
        s += c[k][0] + c[k][1];
    sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// FP64 tensor-core MMA, m16n8k16 (eight f64 of A, four of B and of C per thread)
__global__ void probe_dmma_m16n8k16(int iters, double *sink)
{
    double c[kChains][4];
    double a[8], b[4];
#pragma unroll
    for (int i = 0; i < 8; i++)
        a[i] = 1.0 + 1e-9 * (threadIdx.x + i);
#pragma unroll
    for (int i = 0; i < 4; i++)
        b[i] = 1e-12 * (threadIdx.x + i + 1);
#pragma unroll
    for (int k = 0; k < kChains; k++)
        c[k][0] = c[k][1] = c[k][2] = c[k][3] = k;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int k = 0; k < kChains; k++)
            asm volatile("mma.sync.aligned.m16n8k16.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, "
                         "{%4,%5,%6,%7,%8,%9,%10,%11}, {%12,%13,%14,%15}, {%0,%1,%2,%3};\n"
                         : "+d"(c[k][0]), "+d"(c[k][1]), "+d"(c[k][2]), "+d"(c[k][3])
                         : "d"(a[0]), "d"(a[1]), "d"(a[2]), "d"(a[3]), "d"(a[4]), "d"(a[5]), "d"(a[6]),
                           "d"(a[7]), "d"(b[0]), "d"(b[1]), "d"(b[2]), "d"(b[3]));
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < kChains; k++)
        s += c[k][0] + c[k][1] + c[k][2] + c[k][3];
    sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// INT8 dot products with INT32 accumulation (dp4a: four multiply-adds per
// instruction and lane; counted as 8 operations)
__global__ void probe_dp4a(int iters, double *sink)
{
    int acc[kChains];
    const int a = 0x01020304 + threadIdx.x, b = 0x05060708 ^ threadIdx.x;
#pragma unroll
    for (int c = 0; c < kChains; c++)
        acc[c] = c;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int c = 0; c < kChains; c++)
            acc[c] = __dp4a(a, b, acc[c]);
    }
    int s = 0;
#pragma unroll
    for (int c = 0; c < kChains; c++)
        s += acc[c];
    sink[blockIdx.x * blockDim.x + threadIdx.x] = (double)s;
}

// tcgen05.mma kind::f16 (bf16 inputs, FP32 accumulator in tensor memory),
// M = 128, N = n, K = 16: one CTA per SM, one thread issuing `iters` MMAs
// (a multiple of 8, unrolled by 8 with the accumulator addresses computed
// beforehand) round-robin into naccs accumulators, then a commit and a
// bounded wait.  Operands: zeros in the no-swizzle K-major layout.
constexpr int kProbeTmemCols = 256;
__global__ void __launch_bounds__(128) probe_tcgen05(int n, int iters, int naccs, unsigned *error)
{
    __shared__ __align__(1024) uint8_t a_s[2 * 128 * 16]; // [kgroup 2][row 128][8 bf16]
    __shared__ __align__(1024) uint8_t b_s[2 * 256 * 16]; // [kgroup 2][row n][8 bf16]
    __shared__ uint64_t bar;
    __shared__ uint32_t tmem_slot;
    const int t = threadIdx.x;
    for (int k = t; k < (int)sizeof(a_s) / 4; k += blockDim.x)
        reinterpret_cast<uint32_t *>(a_s)[k] = 0u;
    for (int k = t; k < (int)sizeof(b_s) / 4; k += blockDim.x)
        reinterpret_cast<uint32_t *>(b_s)[k] = 0u;
    if (t < 32) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(va::smem_u32(&tmem_slot)),
                     "r"(kProbeTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (t == 0) {
        va::mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    va::tc_fence_before();
    __syncthreads();
    va::tc_fence_after();
    const uint32_t tmem = tmem_slot;
    if (t == 0) {
        const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
        const uint64_t ad = va::umma_desc(va::smem_u32(a_s), 128 * 16, 128);
        const uint64_t bd = va::umma_desc(va::smem_u32(b_s), (uint32_t)n * 16, 128);
        uint32_t acc[8];
#pragma unroll
        for (int u = 0; u < 8; u++)
            acc[u] = tmem + (uint32_t)((u % naccs) * n);
#pragma unroll
        for (int u = 0; u < 8; u++)
            va::umma_bf16(acc[u], ad, bd, idesc, u >= naccs ? 1u : 0u);
        for (int it = 8; it < iters; it += 8) {
#pragma unroll
            for (int u = 0; u < 8; u++)
                va::umma_bf16(acc[u], ad, bd, idesc, 1u);
        }
        va::umma_commit(&bar);
        if (!va::mbar_wait_bounded(&bar, 0, error)) // once more (bounded) before the tensor memory is released
            (void)va::mbar_wait_bounded(&bar, 0, error);
    }
    __syncthreads();
    va::tc_fence_after();
    if (t < 32)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kProbeTmemCols) : "memory");
}

} // namespace

// tcgen05 bf16 MMA rate at M = 128, K = 16 and the given N (16..256, a
// multiple of 16), issued round-robin into naccs independent accumulators
// (naccs * n <= 256) by ctas CTAs per SM (1 or 2): TFLOP/s (2 M N K per MMA).
extern "C" VA_API int32_t va_probe_mma_bf16(int32_t n, int32_t naccs, int32_t ctas, int32_t iters, double *tflops,
                                            double *ms_out)
{
    if (ctas < 1 || ctas > 2)
        return VA_BAD_ARGS;
    if (!tflops || iters < 8 || iters % 8 || n < 16 || n > 256 || n % 16 || naccs < 1 || naccs > 8 ||
        naccs * n > kProbeTmemCols)
        return VA_BAD_ARGS;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return VA_CUDA_ERROR;
    unsigned *err = nullptr;
    if (cudaMalloc(&err, sizeof(unsigned)) != cudaSuccess)
        return VA_CUDA_ERROR;
    cudaMemset(err, 0, sizeof(unsigned));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    probe_tcgen05<<<sms * ctas, 128>>>(n, 8 * (iters / 64 + 1), naccs, err); // warm-up
    float best = 1e30f;
    for (int rep = 0; rep < 3; rep++) {
        cudaEventRecord(e0);
        probe_tcgen05<<<sms * ctas, 128>>>(n, iters, naccs, err);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best)
            best = ms;
    }
    unsigned herr = 0;
    const cudaError_t ce = cudaMemcpy(&herr, err, sizeof(unsigned), cudaMemcpyDeviceToHost);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(err);
    if (ce != cudaSuccess || cudaGetLastError() != cudaSuccess || herr)
        return VA_CUDA_ERROR;
    *tflops = 2.0 * 128 * n * 16 * (double)iters * sms * ctas / (best * 1e-3) / 1e12;
    if (ms_out)
        *ms_out = best;
    return VA_OK;
}

extern "C" VA_API int32_t va_probe_rate(int32_t kind, int32_t iters, double *tflops, double *ms_out)
{
    if (!tflops || iters <= 0 || kind < 0 || kind > 4)
        return VA_BAD_ARGS;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return VA_CUDA_ERROR;
    const int threads = 256, blocks = sms * 8;
    double *sink = nullptr;
    if (cudaMalloc(&sink, sizeof(double) * threads * blocks) != cudaSuccess)
        return VA_CUDA_ERROR;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    auto launch = [&](int n) {
        switch (kind) {
        case 0: probe_fp64_fma<<<blocks, threads>>>(n, sink); break;
        case 1: probe_fp32_fma<<<blocks, threads>>>(n, sink); break;
        case 2: probe_dmma_m8n8k4<<<blocks, threads>>>(n, sink); break;
        case 3: probe_dmma_m16n8k16<<<blocks, threads>>>(n, sink); break;
        default: probe_dp4a<<<blocks, threads>>>(n, sink); break;
        }
    };
    launch(iters / 8 + 1); // warm-up
    float best = 1e30f;
    for (int rep = 0; rep < 3; rep++) {
        cudaEventRecord(e0);
        launch(iters);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best)
            best = ms;
    }
    const cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    if (err != cudaSuccess)
        return VA_CUDA_ERROR;
    const double ops_per_iter = kind <= 1   ? 2.0 * kChains * threads // per thread FMAs
                                : kind == 4 ? 8.0 * kChains * threads // per thread dp4a
                                            : (kind == 2 ? 2.0 * 8 * 8 * 4 : 2.0 * 16 * 8 * 16) * kChains * threads / 32;
    const double flop = ops_per_iter * blocks * (double)iters;
    *tflops = flop / (best * 1e-3) / 1e12;
    if (ms_out)
        *ms_out = best;
    return VA_OK;
}
