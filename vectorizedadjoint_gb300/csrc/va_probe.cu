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

} // namespace

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
