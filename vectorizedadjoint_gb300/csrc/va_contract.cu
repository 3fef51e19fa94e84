// Kernels of the tensor-core dA contraction (va_contract.cuh): the factor-row
// offsets of each instance, the contraction on tcgen05 with tensor-memory
// accumulators, and the fixed-order sum of the CTA partials.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "../../include/va.h"
#include "../../include/va_probe.h"
#include "va_contract.cuh"
#include "va_tcgen05.cuh"
#include "va_kernels.cuh"

namespace va {

// ------------------------------------------------------------ row offsets

// k_base[b] = nsv * sum_{b' < b, OK} T_b' (the first factor row of instance
// b), k_base[B] = K.  One block; each thread a contiguous range of instances.
__global__ void __launch_bounds__(1024) factor_offsets_kernel(const int *inst_T, const int *inst_status, int B,
                                                              int nsv, int *k_base)
{
    __shared__ long long part[1024];
    const int t = threadIdx.x, per = (B + 1023) / 1024;
    const int lo = min(B, t * per), hi = min(B, lo + per);
    long long s = 0;
    for (int b = lo; b < hi; b++)
        s += inst_status[b] == ST_OK ? (long long)inst_T[b] * nsv : 0;
    part[t] = s;
    __syncthreads();
    // inclusive scan of the 1024 partial sums (Hillis-Steele)
    for (int o = 1; o < 1024; o <<= 1) {
        const long long v = t >= o ? part[t - o] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    long long run = t > 0 ? part[t - 1] : 0;
    for (int b = lo; b < hi; b++) {
        k_base[b] = (int)run;
        run += inst_status[b] == ST_OK ? (long long)inst_T[b] * nsv : 0;
    }
    if (t == 1023)
        k_base[B] = (int)part[1023];
}

// ------------------------------------------------------------ contraction

// |hi| of a packed double-word (for the exponent bound)
__device__ __forceinline__ float dw_abs_hi(double packed) { return fabsf(dw_unpack(packed).hi); }

// exponent e with |x| < 2^e for every entry whose leading word is at most m
__device__ __forceinline__ int bound_exponent(float m) { return m > 0.0f ? ilogbf(m) + 1 : -120; }

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b)
{
    const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t *>(&v);
}

// One column's 8 consecutive rows (a core-matrix row of 16 bytes) as Q digit
// planes: vals are packed double-words, e the column's exponent.
__device__ __forceinline__ void slice_row8(const double (&vals)[8], DigitScale sc, uint8_t *plane0,
                                           size_t plane_stride)
{
    float d[8][kContractQ];
#pragma unroll
    for (int r = 0; r < 8; r++) {
        const dword w = dw_unpack(vals[r]);
        split_digits(w.hi, w.lo, sc, d[r]);
    }
#pragma unroll
    for (int s = 0; s < kContractQ; s++) {
        uint4 q;
        q.x = pack_bf16x2(d[0][s], d[1][s]);
        q.y = pack_bf16x2(d[2][s], d[3][s]);
        q.z = pack_bf16x2(d[4][s], d[5][s]);
        q.w = pack_bf16x2(d[6][s], d[7][s]);
        *reinterpret_cast<uint4 *>(plane0 + s * plane_stride) = q;
    }
}

// Slices chunk c of the CTA's tile into one shared-memory stage and stores
// the column exponents (e_v[128], e_x[64]).
__device__ __forceinline__ void slice_chunk(const ContractParams &p, int c, int K, int ti, int tj, uint8_t *stage,
                                            int *ev, int *ex, float *red, const double *const *xrow)
{
    const int t = threadIdx.x;
    const int k0 = c * kContractKC;
    // v: column i = t & 127, rows 16 h .. 16 h + 15 (h = t >> 7)
    {
        const int i = t & 127, h = t >> 7;
        const double *col = p.v + (size_t)ti * kContractTileM + i;
        float m = 0.0f;
#pragma unroll
        for (int r = 0; r < 16; r++) {
            const int k = k0 + 16 * h + r;
            if (k < K)
                m = fmaxf(m, dw_abs_hi(__ldg(col + (size_t)k * kContractN)));
        }
        red[t] = m;
    }
    // x: column j = t & 63, rows 8 q .. 8 q + 7 (q = t >> 6)
    {
        const int j = t & 63, q = t >> 6;
        float m = 0.0f;
#pragma unroll
        for (int r = 0; r < 8; r++) {
            const int k = k0 + 8 * q + r;
            if (k < K)
                m = fmaxf(m, dw_abs_hi(__ldg(xrow[8 * q + r] + tj * kContractTileN + j)));
        }
        red[kContractThreads + t] = m;
    }
    __syncthreads();
    if (t < 128) {
        ev[t] = bound_exponent(fmaxf(fmaxf(red[t], red[t + 128]), fmaxf(red[t + 256], red[t + 384])));
    } else if (t < 192) {
        const int j = t - 128;
        float m = 0.0f;
#pragma unroll
        for (int q = 0; q < 8; q++)
            m = fmaxf(m, red[kContractThreads + j + 64 * q]);
        ex[j] = bound_exponent(m);
    }
    __syncthreads();
    // digits: v planes [slice][kgroup 8][row 128][8] (plane = 16 KB, kgroup = 2 KB)
    {
        const int i = t & 127, h = t >> 7;
        const double *col = p.v + (size_t)ti * kContractTileM + i;
        const DigitScale sc = digit_scale(ev[i]);
#pragma unroll
        for (int g = 0; g < 2; g++) {
            const int kg = 2 * h + g;
            double vals[8];
#pragma unroll
            for (int r = 0; r < 8; r++) {
                const int k = k0 + 8 * kg + r;
                vals[r] = k < K ? __ldg(col + (size_t)k * kContractN) : 0.0;
            }
            slice_row8(vals, sc, stage + (size_t)kg * 2048 + i * 16, (size_t)kContractKC * kContractTileM * 2);
        }
    }
    // digits: x planes [slice][kgroup 8][row 64][8] (plane = 8 KB, kgroup = 1 KB)
    {
        const int j = t & 63, q = t >> 6;
        const DigitScale sc = digit_scale(ex[j]);
        uint8_t *xs = stage + kTileVBytes;
        {
            const int kg = q;
            double vals[8];
#pragma unroll
            for (int r = 0; r < 8; r++) {
                const int k = k0 + 8 * kg + r;
                vals[r] = k < K ? __ldg(xrow[8 * kg + r] + tj * kContractTileN + j) : 0.0;
            }
            slice_row8(vals, sc, xs + (size_t)kg * 1024 + j * 16, (size_t)kContractKC * kContractTileN * 2);
        }
    }
}

// The x-row pointers of chunk c into xrow[64] (rows past K: null, never
// dereferenced), and a prefetch of the chunk's rows of the CTA's tile into
// L2 (the factor rows are read once from DRAM; the slicing loads then wait
// on L2 instead)
__device__ __forceinline__ void prefetch_chunk(const ContractParams &p, int c, int K, int ti, int tj,
                                               const double **xrow)
{
    const int t = threadIdx.x;
    // v: 64 rows of 128 doubles, 8 threads a row; x: 64 rows of 64, 4 threads a row
    const int kv = c * kContractKC + (t >> 3);
    if (kv < K)
        asm volatile("prefetch.global.L2 [%0];" ::"l"(p.v + (size_t)kv * kContractN + ti * kContractTileM +
                                                      (t & 7) * 16));
    const int kx = c * kContractKC + (t & 63);
    if (t < 256) {
        const double *base = kx < K ? p.xp[kx] : nullptr;
        if (t < 64)
            xrow[t] = base;
        if (base)
            asm volatile("prefetch.global.L2 [%0];" ::"l"(base + tj * kContractTileN + (t >> 6) * 16));
    }
}

// The 40 MMAs of one chunk: for every group g = s + t the digit pairs
// (s, t), each over the chunk's four K steps of 16, into accumulator g.
__device__ __forceinline__ void issue_chunk(uint32_t tmem_acc, const uint8_t *stage)
{
    constexpr uint32_t idesc = umma_idesc_bf16(kContractTileM, kContractTileN);
    const uint32_t vbase = smem_u32(stage), xbase = smem_u32(stage + kTileVBytes);
    constexpr uint32_t vplane = kContractKC * kContractTileM * 2, xplane = kContractKC * kContractTileN * 2;
#pragma unroll
    for (int g = 0; g < kContractQ; g++) {
        bool first = true;
#pragma unroll
        for (int s = 0; s <= g; s++) {
            const int tq = g - s;
#pragma unroll
            for (int kk = 0; kk < kContractKC / 16; kk++) {
                // K step kk covers kgroups 2kk and 2kk + 1
                const uint64_t ad = umma_desc(vbase + s * vplane + kk * 2 * 2048, 2048, 128);
                const uint64_t bd = umma_desc(xbase + tq * xplane + kk * 2 * 1024, 1024, 128);
                umma_bf16(tmem_acc + g * kContractTileN, ad, bd, idesc, first ? 0u : 1u);
                first = false;
            }
        }
    }
}

// Folds one chunk's group sums into the double-word accumulators of this
// thread's row and 32 columns: acc += R_g 2^(e_v + e_x - 8(g + 2)).
__device__ __forceinline__ void fold_chunk(uint32_t tmem_row, const int *ev, const int *ex, int row, int col0,
                                           float (&ah)[kContractFoldCols], float (&al)[kContractFoldCols])
{
    constexpr int C = kContractFoldCols;
    // R_g 2^(esum - 8g) = (R_g 2^(-8g)) 2^esum: two exact multiplications by
    // normal powers of two when -102 <= esum <= 103 (|R_g| < 2^24, so every
    // product is a normal float); ldexpf for columns outside that range
    int esum[C];
    float p2[C];
    bool fast = true;
#pragma unroll
    for (int c = 0; c < C; c++) {
        esum[c] = ev[row] + ex[col0 + c] - 16;
        fast = fast && esum[c] >= -102 && esum[c] <= 103;
        p2[c] = pow2f(min(max(esum[c], -102), 103));
    }
#pragma unroll 1
    for (int g = 0; g < kContractQ; g++) {
        float R[C];
        tmem_ld16(tmem_row + g * kContractTileN, R);
        const float sg = pow2f(-8 * g);
#pragma unroll
        for (int c = 0; c < C; c++) {
            const float v = fast ? (R[c] * sg) * p2[c] : ldexpf(R[c], esum[c] - 8 * g); // exact
            // double-word accumulation: (ah, al) += v
            const float s = ah[c] + v;
            const float bb = s - ah[c];
            const float e = (ah[c] - (s - bb)) + (v - bb);
            const float lo = al[c] + e;
            ah[c] = s + lo;
            al[c] = lo - (ah[c] - s);
        }
    }
}

// grid = tiles x splits, kContractThreads threads, kContractSmem dynamic shared memory
__global__ void __launch_bounds__(kContractThreads, 1) contract_kernel(ContractParams p)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *stages[2] = {smem, smem + kStageBytes};
    uint64_t *done = reinterpret_cast<uint64_t *>(smem + 2 * kStageBytes); // [2]
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 2);
    __shared__ int ev_s[2][kContractTileM], ex_s[2][kContractTileN];
    __shared__ float red[2 * kContractThreads];
    __shared__ const double *xrow_s[2][kContractKC]; // x-row pointers of the chunk in each stage

    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const int tile = blockIdx.x % kContractTiles, split = blockIdx.x / kContractTiles;
    const int ti = tile / (kContractN / kContractTileN), tj = tile % (kContractN / kContractTileN);
    const int K = *p.k_total;
    const int nc = (K + kContractKC - 1) / kContractKC;
    const int c0 = (int)((long long)split * nc / p.splits), c1 = (int)((long long)(split + 1) * nc / p.splits);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(tmem_slot))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (t == 0) {
        mbar_init(&done[0], 1);
        mbar_init(&done[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    // this thread's accumulator row and columns: warp w reads tensor-memory
    // lanes 32 (w % 4) .. +31, columns 16 (w / 4) .. +15 of each group
    const int row = 32 * (warp & 3) + lane, col0 = kContractFoldCols * (warp >> 2);
    const uint32_t lane_addr = (uint32_t)(32 * (warp & 3)) << 16;
    float ah[kContractFoldCols], al[kContractFoldCols];
#pragma unroll
    for (int c = 0; c < kContractFoldCols; c++)
        ah[c] = al[c] = 0.0f;

    // ok stays uniform across the block (a bounded wait that gave up on any
    // thread stops the work of all of them at the next barrier)
    bool ok = true;
    int issued = 0, waited = 0; // chunks committed / chunks whose commit was awaited
    const int n = c1 - c0;
    if (n > 0)
        prefetch_chunk(p, c0, K, ti, tj, xrow_s[0]);
    __syncthreads();
    for (int idx = 0; idx < n; idx++) {
        const int st = idx & 1;
        if (ok) {
            slice_chunk(p, c0 + idx, K, ti, tj, stages[st], ev_s[st], ex_s[st], red, xrow_s[st]);
            if (idx + 1 < n)
                prefetch_chunk(p, c0 + idx + 1, K, ti, tj, xrow_s[st ^ 1]);
        }
        // the digit planes, written by this CTA's threads, feed the tensor core
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        tc_fence_before();
        __syncthreads();
        if (ok) {
            if (t == 0) {
                tc_fence_after();
                issue_chunk(tmem + st * kContractQ * kContractTileN, stages[st]);
                umma_commit(&done[st]);
            }
            issued = idx + 1;
        }
        if (idx > 0 && ok) {
            // the previous chunk's group sums
            const int pst = st ^ 1;
            const bool w = mbar_wait_bounded(&done[pst], ((idx - 1) >> 1) & 1, p.error);
            ok = __syncthreads_and(w) != 0;
            if (ok) {
                waited = idx;
                tc_fence_after();
                fold_chunk(tmem + lane_addr + pst * kContractQ * kContractTileN + col0, ev_s[pst], ex_s[pst], row,
                           col0, ah, al);
            }
            tc_fence_before();
        }
        __syncthreads();
    }
    if (ok && issued == n && n > 0) {
        const int idx = n - 1, st = idx & 1;
        const bool w = mbar_wait_bounded(&done[st], (idx >> 1) & 1, p.error);
        ok = __syncthreads_and(w) != 0;
        if (ok) {
            waited = n;
            tc_fence_after();
            fold_chunk(tmem + lane_addr + st * kContractQ * kContractTileN + col0, ev_s[st], ex_s[st], row, col0,
                       ah, al);
        }
    }
    // after an error: wait (bounded) for the MMAs still in flight before the
    // tensor memory is released
    for (int c = waited; c < issued; c++)
        (void)mbar_wait_bounded(&done[c & 1], (c >> 1) & 1, p.error);
    // partial[split][j][i] (transposed, as the fixed-order reduction reads it)
    const int i = ti * kContractTileM + row;
#pragma unroll
    for (int c = 0; c < kContractFoldCols; c++) {
        const int j = tj * kContractTileN + col0 + c;
        p.partials[((size_t)split * kContractN + j) * kContractN + i] = (double)ah[c] + (double)al[c];
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
}

// x_k pointers of a dense [K][256] factor matrix (the diagnostic entry point)
__global__ void dense_rows_kernel(const double *x, int K, const double **xp)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < K)
        xp[k] = x + (size_t)k * kContractN;
}

// dA[i][j] = sum over splits, in split order, of partial[split][j][i]; NaN
// everywhere when a wait of the contraction gave up
__global__ void reduce_partials_kernel(const double *part, int nparts, const unsigned *error, double *dA)
{
    constexpr int NT = kContractN;
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; // k = j * NT + i
    if (k >= (size_t)NT * NT)
        return;
    double s = 0.0;
    for (int c = 0; c < nparts; c++)
        s += part[(size_t)c * NT * NT + k];
    if (*error)
        s = __longlong_as_double(0x7ff8000000000000ll);
    const size_t j = k / NT, i = k % NT;
    dA[i * NT + j] = s;
}

int contract_splits(int sm_count) { return std::max(1, sm_count / kContractTiles); }

cudaError_t enqueue_factor_offsets(const int *inst_T, const int *inst_status, int B, int nsv, int *k_base,
                                   cudaStream_t s)
{
    factor_offsets_kernel<<<1, 1024, 0, s>>>(inst_T, inst_status, B, nsv, k_base);
    return cudaGetLastError();
}

cudaError_t contract_prepare()
{
    return cudaFuncSetAttribute(contract_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kContractSmem);
}

cudaError_t enqueue_contract(const ContractParams &p, double *dA, cudaStream_t s)
{
    contract_kernel<<<kContractTiles * p.splits, kContractThreads, kContractSmem, s>>>(p);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return e;
    constexpr int NN = kContractN * kContractN;
    reduce_partials_kernel<<<(NN + 255) / 256, 256, 0, s>>>(p.partials, p.splits, p.error, dA);
    return cudaGetLastError();
}

} // namespace va

extern "C" VA_API int32_t va_contract_dA(int32_t K, const double *v, const double *x, double *dA, void *stream)
{
    if (K < 0 || !v || !x || !dA)
        return VA_BAD_ARGS;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return VA_CUDA_ERROR;
    cudaStream_t s = (cudaStream_t)stream;
    const int splits = va::contract_splits(sms);
    const double **xp = nullptr;
    int *k_total = nullptr;
    unsigned *err = nullptr;
    double *part = nullptr;
    const size_t nn = (size_t)va::kContractN * va::kContractN;
    int32_t st = VA_OK;
    if (cudaMalloc(&xp, sizeof(double *) * (size_t)std::max(K, 1)) != cudaSuccess ||
        cudaMalloc(&k_total, sizeof(int)) != cudaSuccess || cudaMalloc(&err, sizeof(unsigned)) != cudaSuccess ||
        cudaMalloc(&part, sizeof(double) * nn * splits) != cudaSuccess)
        st = VA_CUDA_ERROR;
    if (st == VA_OK) {
        va::dense_rows_kernel<<<(K + 255) / 256 + 1, 256, 0, s>>>(x, K, xp);
        cudaMemcpyAsync(k_total, &K, sizeof(int), cudaMemcpyHostToDevice, s);
        cudaMemsetAsync(err, 0, sizeof(unsigned), s);
        va::ContractParams p{};
        p.v = v;
        p.xp = xp;
        p.k_total = k_total;
        p.partials = part;
        p.splits = splits;
        p.error = err;
        if (va::contract_prepare() != cudaSuccess || va::enqueue_contract(p, dA, s) != cudaSuccess)
            st = VA_CUDA_ERROR;
        unsigned e = 0;
        if (cudaMemcpyAsync(&e, err, sizeof(unsigned), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            st = VA_CUDA_ERROR;
        else if (e)
            st = VA_CUDA_ERROR;
    }
    cudaFree(xp);
    cudaFree(k_total);
    cudaFree(err);
    cudaFree(part);
    return st;
}
