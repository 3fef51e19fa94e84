/*
 * va_probe.h -- arithmetic-rate probes of libva_gb300.so.
 *
 * No counterpart in the reference, which has no GPU path: these measure the
 * pipes the sweep kernels run on (FP64 vector FMA, FP32 FMA, FP64
 * tensor-core MMA) on the current device, so that the roofline fractions the
 * benchmark reports rest on this part's own rates.
 */
#ifndef VA_GB300_PROBE_H
#define VA_GB300_PROBE_H

#include <stdint.h>

#include "va.h"

#ifdef __cplusplus
extern "C" {
#endif

/* kind 0: FP64 FMA, 1: FP32 FMA, 2: FP64 MMA m8n8k4 (mma.sync), 3: FP64 MMA
 * m16n8k16 (mma.sync), 4: INT8 dot product dp4a (8 operations each).  Runs `iters` iterations of eight independent chains
 * per thread (or warp) on 8 blocks of 256 threads per SM of the current
 * device, best of three timed launches; writes TFLOP/s (FMA = 2 FLOPs) and
 * the launch time in ms (ms_out may be NULL).  Allocates a small output
 * buffer.  Returns a va_status. */
VA_API int32_t va_probe_rate(int32_t kind, int32_t iters, double *tflops, double *ms_out);

/* The bf16 tensor-core MMA rate (tcgen05.mma kind::f16, FP32 accumulation
 * in tensor memory) at M = 128, K = 16 and N = n (16..256, a multiple of 16):
 * `ctas` CTAs per SM (1 or 2), each issuing `iters` MMAs (a multiple of 8)
 * round-robin into `naccs` independent accumulators (1..8, naccs * n <= 256); TFLOP/s (2 M N K per MMA) and the launch
 * time in ms (ms_out may be NULL).  Returns a va_status (VA_CUDA_ERROR also
 * when the bounded wait gave up). */
VA_API int32_t va_probe_mma_bf16(int32_t n, int32_t naccs, int32_t ctas, int32_t iters, double *tflops,
                                 double *ms_out);

/* The tensor-core contraction the shared-matrix GLV backward sweep uses for
 * its matrix gradient, on caller data: dA[256][256] = sum_k v_k x_k^T for
 * DEVICE arrays v[K][256], x[K][256] of double-words packed in 8-byte slots
 * (float hi in the low word, lo in the high word).  Exact integer digit
 * products on tcgen05 (bf16 inputs, FP32 tensor-memory accumulators) of
 * factors split into four 8-bit digits per 64-row chunk; the truncation of
 * the digits leaves ~2^-32 of the chunk's column maxima per term.
 * Allocates scratch, synchronises `stream`.  Returns a va_status
 * (VA_CUDA_ERROR also when a bounded wait in the kernel gave up). */
VA_API int32_t va_contract_dA(int32_t K, const double *v, const double *x, double *dA, void *stream);

/* The batched tensor-core product of the shared-matrix GLV backward sweep,
 * on caller data: G[b][i] = sum_k A[k][i] V[b][k] (G = A^T V per instance)
 * for DEVICE arrays A[256][256] (FP64, row-major), V[B][256] and G[B][256]
 * (double-words packed in 8-byte slots).  Seven 8-bit digits per factor,
 * K in quarters of 64, exact digit products on tcgen05 (bf16 inputs, FP32
 * tensor-memory accumulators); the truncation leaves ~2^-56 of the
 * quarter's maxima per term.  Allocates scratch, synchronises `stream`.
 * Returns a va_status (VA_CUDA_ERROR also when a bounded wait gave up). */
VA_API int32_t va_matT_tc(int32_t B, const double *A, const double *V, double *G, void *stream);

#ifdef __cplusplus
}
#endif
#endif
