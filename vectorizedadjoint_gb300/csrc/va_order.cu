// Longest-first work order for the persistent sweeps.  A lane that takes a
// long instance late holds the whole kernel open (the tail); handing out the
// longest instances first removes most of it.  The backward sweep orders by
// the accepted-step count the forward produced.  The forward sweep orders by
// the attempt count of the handle's previous forward sweep when there is one
// (repeated solves of a batch -- optimisation loops, sensitivity sweeps --
// change step counts little between calls), else by the horizon t1 - t0.
// Only the order comes from the previous sweep: every step is computed
// again, and each instance's result does not depend on the order.  On a
// batch with one horizon (every instance to the same T) the horizon order
// is the index order, and lanes whose last instances run long idle the rest
// of their warp.  A counting sort over 4096
// buckets (descending) builds the permutation on the device, so it can sit
// inside the captured graph.  The atomics here only decide the order; each
// instance's result does not depend on it.  The backward can take the
// forward's order when that one came from step counts (the previous sweep's
// attempts, nearly the same ranking as this sweep's accepted steps): no
// second sort, and the backward then visits the checkpoint chunks in the
// order the forward allocated them (the caller decides; one-thread models).
#include <cuda_runtime.h>

#include <cstdint>

#include "va_order.h"

namespace va {

namespace {

constexpr int kBuckets = 4096;

__device__ __forceinline__ int horizon_bucket(double h)
{
    // 64 buckets per octave of t1 - t0, from 2^-32 to 2^32
    if (!(h > 0.0))
        return 0;
    const double l = log2(h);
    const int k = (int)((l + 32.0) * 64.0);
    return k < 0 ? 0 : k >= kBuckets ? kBuckets - 1 : k;
}

__device__ __forceinline__ int count_bucket(int n) { return n < kBuckets ? (n < 0 ? 0 : n) : kBuckets - 1; }

// work[2 kBuckets]: 1 when the last forward order came from step counts
constexpr int kCountedFlag = 2 * kBuckets;

// the backward reuses the forward's order when that one was count-based
__device__ __forceinline__ bool reusing(const OrderArgs &a) { return a.reuse && a.work[kCountedFlag] == 1; }

__device__ __forceinline__ int key_of(const OrderArgs &a, int b)
{
    if (a.steps)
        return count_bucket(a.steps[b]);
    if (a.prev_work && *a.prev_valid)
        return count_bucket(a.prev_work[b]);
    return horizon_bucket(a.t1[b] - a.t0[b]);
}

__global__ void order_hist(OrderArgs a)
{
    if (reusing(a))
        return;
    __shared__ int h[kBuckets];
    for (int i = threadIdx.x; i < kBuckets; i += blockDim.x)
        h[i] = 0;
    __syncthreads();
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < a.B; b += gridDim.x * blockDim.x)
        atomicAdd(&h[key_of(a, b)], 1);
    __syncthreads();
    for (int i = threadIdx.x; i < kBuckets; i += blockDim.x)
        if (h[i])
            atomicAdd(&a.work[i], h[i]);
}

// Exclusive scan from the top bucket down: offset of bucket k = number of
// instances in buckets > k.  One block of 1024 threads, 4 buckets each.
__global__ void order_scan(OrderArgs a)
{
    if (reusing(a))
        return;
    __shared__ int part[1024];
    const int t = threadIdx.x;
    int v[4], s = 0;
    for (int j = 0; j < 4; j++) {
        v[j] = a.work[kBuckets - 1 - (t * 4 + j)];
        s += v[j];
    }
    part[t] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const int x = t >= o ? part[t - o] : 0;
        __syncthreads();
        part[t] += x;
        __syncthreads();
    }
    int run = t ? part[t - 1] : 0;
    for (int j = 0; j < 4; j++) {
        a.work[kBuckets + (kBuckets - 1 - (t * 4 + j))] = run;
        run += v[j];
    }
    if (t == 0 && !a.steps) // a forward order: say whether it came from counts
        a.work[kCountedFlag] = (a.prev_work && a.prev_valid && *a.prev_valid) ? 1 : 0;
}

// Each block takes a contiguous range of instances: it counts its range per
// bucket in shared memory, reserves one slice of every bucket it touches
// with a single global atomic, then writes its instances into the slices
// (ranks from the shared-memory atomics).  One global atomic per instance
// on the few hundred buckets a batch's step counts fall into serialised on
// those counters.
__global__ void __launch_bounds__(1024) order_scatter(OrderArgs a)
{
    __shared__ int cnt[kBuckets];
    const int per = (a.B + gridDim.x - 1) / gridDim.x;
    const int lo = blockIdx.x * per, hi = min(a.B, lo + per);
    if (reusing(a)) {
        for (int b = lo + threadIdx.x; b < hi; b += blockDim.x)
            a.order[b] = a.reuse[b];
        return;
    }
    for (int i = threadIdx.x; i < kBuckets; i += blockDim.x)
        cnt[i] = 0;
    __syncthreads();
    for (int b = lo + threadIdx.x; b < hi; b += blockDim.x)
        atomicAdd(&cnt[key_of(a, b)], 1);
    __syncthreads();
    for (int i = threadIdx.x; i < kBuckets; i += blockDim.x)
        if (cnt[i])
            cnt[i] = atomicAdd(&a.work[kBuckets + i], cnt[i]); // this block's slice of bucket i
    __syncthreads();
    for (int b = lo + threadIdx.x; b < hi; b += blockDim.x)
        a.order[atomicAdd(&cnt[key_of(a, b)], 1)] = b;
}

} // namespace

size_t order_work_ints() { return 2 * kBuckets + 1; }

cudaError_t enqueue_order(const OrderArgs &a, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(a.work, 0, sizeof(int) * kBuckets, s);
    if (e != cudaSuccess)
        return e;
    const int grid = (a.B + 255) / 256 < 1024 ? (a.B + 255) / 256 : 1024;
    order_hist<<<grid, 256, 0, s>>>(a);
    order_scan<<<1, 1024, 0, s>>>(a);
    const int sgrid = (a.B + 1023) / 1024 < 256 ? (a.B + 1023) / 1024 : 256;
    order_scatter<<<sgrid, 1024, 0, s>>>(a);
    return cudaGetLastError();
}

} // namespace va
