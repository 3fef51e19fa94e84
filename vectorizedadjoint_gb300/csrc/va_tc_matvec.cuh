// Batched products G = A^T V on the tensor cores for the shared-matrix GLV
// (N = 256): G[b][i] = sum_k A[k][i] V[b][k] for every instance b of the
// batch at once, V and G double-words.  The backward sweep needs one such
// product per stage (A^T (Kbar . X_m)); with all instances in lockstep it is
// a 256 x 256 x B matrix product, a shape the MMA runs at full width.
//
// Error-free splitting as in va_contract.cuh (Ozaki, Ogita, Oishi, Rump
// 2012), here with Q = 7 digits of 8 bits (56 bits, past the 48 of a
// double-word) and the K dimension in quarters of 64:
//   - A^T[i][k]: per row i and quarter q a power of two 2^eA bounds the
//     quarter's entries; 7 digits per entry (digit planes of A^T, made once
//     per matrix by tc_digits_A_kernel);
//   - V[b][k]: per instance b and quarter q a power of two 2^eV; 7 digits;
//   - the digit pairs (s, t) with s + t = g < 7 (28 of 49) go to
//     tcgen05.mma kind::f16 (bf16 digits, exact; FP32 accumulation in tensor
//     memory): per quarter, |d_0| <= 256, |d_s| <= 128, so a pair's 64-term
//     sum is below 2^22 and a group's (at most 7 pairs, one of them (0,0))
//     below 2^24 -- every group sum R_g is an exact integer;
//   - G_q[b][i] = sum_g R_g 2^(eA + eV - 8(g + 2)), a power-of-two scaling,
//     accumulated as a double-word; the four quarters' partials are added
//     by the caller.
// Error: the digits' truncation, ~2^-56 of the quarter's maxima per term.
//
// A CTA computes one (row tile of 128, instance tile of 64, quarter) block:
// the operands are laid out in global memory exactly as the MMA reads them
// from shared memory (no-swizzle K-major canonical layout, core matrices of
// 8 rows x 16 bytes) and copied in with 16-byte loads:
//   A block: [digit 7][kgroup 8][row 128][8 k] bf16 (16 KB per digit)
//   V block: [digit 7][kgroup 8][col 64][8 k]  bf16 (8 KB per digit)
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "va_contract.cuh"
#include "va_dword.cuh"
#include "va_tcgen05.cuh"

namespace va {

constexpr int kTcN = 256;                     // matrix order
constexpr int kTcQ = 7;                       // digits
constexpr int kTcKQ = 64;                     // K entries per quarter
constexpr int kTcQuarters = kTcN / kTcKQ;     // 4
constexpr int kTcTileM = 128, kTcTileN = 64;  // MMA M (rows of A^T), N (instances)
constexpr int kTcTilesM = kTcN / kTcTileM;    // 2
constexpr int kTcGroups = kTcQ;               // digit-pair groups g = 0 .. 6
constexpr size_t kTcAPlane = (size_t)kTcKQ * kTcTileM * 2; // 16 KB
constexpr size_t kTcABlock = kTcQ * kTcAPlane;             // 112 KB
constexpr size_t kTcVPlane = (size_t)kTcKQ * kTcTileN * 2; // 8 KB
constexpr size_t kTcVBlock = kTcQ * kTcVPlane;             // 56 KB
constexpr int kTcTmemCols = 512;                           // 7 groups x 64 columns, rounded up
constexpr size_t kTcSmem = kTcABlock + kTcVBlock + 256;    // operands + barrier

__host__ __device__ constexpr int tc_instance_tiles(int B) { return (B + kTcTileN - 1) / kTcTileN; }

// byte offset of digit s of entry (row, k) in the A blocks [tile m][quarter q]
__host__ __device__ constexpr size_t tc_a_offset(int row_tile, int q, int s, int row, int k)
{
    return ((size_t)(row_tile * kTcQuarters + q)) * kTcABlock + (size_t)s * kTcAPlane +
           (size_t)((k % kTcKQ) / 8) * (kTcTileM * 16) + (size_t)row * 16 + (size_t)(k % 8) * 2;
}
// byte offset of digit s of entry (instance col, k) in the V blocks [tile n][quarter q]
__host__ __device__ constexpr size_t tc_v_offset(int col_tile, int q, int s, int col, int k)
{
    return ((size_t)(col_tile * kTcQuarters + q)) * kTcVBlock + (size_t)s * kTcVPlane +
           (size_t)((k % kTcKQ) / 8) * (kTcTileN * 16) + (size_t)col * 16 + (size_t)(k % 8) * 2;
}

__device__ __forceinline__ uint16_t bf16_bits(float v) // exact for the digits (|v| <= 256, integers)
{
    return (uint16_t)(__float_as_uint(v) >> 16);
}

// exponent e with |x| < 2^e for every entry whose leading word is at most m
__host__ __device__ __forceinline__ int tc_bound_exponent(float m)
{
#ifdef __CUDA_ARCH__
    return m > 0.0f ? ilogbf(m) + 1 : -120;
#else
    return m > 0.0f ? std::ilogb(m) + 1 : -120;
#endif
}

// Digit planes of A^T and the exponents eA[q][i]: one block per row i of
// A^T (column i of A), 256 threads (k); A row-major FP64.
__global__ void __launch_bounds__(256) tc_digits_A_kernel(const double *A, uint8_t *adig, int *aexp);

// Digit planes of V (double-words packed in 8-byte slots, V[b][256]) and
// eV[b][q]: one block per instance of the padded batch, 256 threads (k);
// instances past B get zero digits (their tile columns contribute nothing).
__global__ void __launch_bounds__(256) tc_digits_V_kernel(const double *V, int B, uint8_t *vdig, int *vexp);

// One block of 256 threads per (row tile, instance tile, quarter):
// gpart[q][b][i] = sum_k A^T[i][k] V[b][k] over the quarter's k (packed
// double-words), for b < B.  error: set when a bounded wait gave up.
__global__ void __launch_bounds__(256, 1) tc_gemm_kernel(const uint8_t *adig, const int *aexp, const uint8_t *vdig,
                                                         const int *vexp, int B, double *gpart, unsigned *error);

// G[b][i] = sum of the four quarters' partials, in quarter order (packed).
__global__ void tc_sum_quarters_kernel(const double *gpart, int B, double *G);

// ------------------------------------------------------------ building blocks

// Thread k's value v of instance b, with the quarter's exponent e, as 7
// digit planes of the V blocks.
__device__ __forceinline__ void tc_write_v_digits(uint8_t *vdig, int b, int k, dword v, int e)
{
    float d[kTcQ];
    split_digits<kTcQ>(v.hi, v.lo, digit_scale(e), d);
    const int q = k / kTcKQ;
#pragma unroll
    for (int s = 0; s < kTcQ; s++)
        *reinterpret_cast<uint16_t *>(vdig + tc_v_offset(b / kTcTileN, q, s, b % kTcTileN, k)) = bf16_bits(d[s]);
}

// Block-wide maxima of |x| over each quarter of the 256 threads (thread k
// holds x), returned to every thread as the quarter exponents e[4].
__device__ __forceinline__ void tc_quarter_exponents(float ax, float *red /* [8] */, int (&e)[kTcQuarters])
{
    const int k = threadIdx.x, lane = k & 31, w = k >> 5;
    float m = ax;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0)
        red[w] = m;
    __syncthreads();
#pragma unroll
    for (int q = 0; q < kTcQuarters; q++) // a quarter = two warps
        e[q] = tc_bound_exponent(fmaxf(red[2 * q], red[2 * q + 1]));
    __syncthreads();
}

// The tile product for one CTA of 256 threads: (row tile mt, instance tile
// nt, quarter q).  smem: kTcABlock + kTcVBlock bytes (1024-aligned); bar: an
// initialised mbarrier whose next phase parity is `phase`; tmem: 448+
// allocated columns.  Returns false (and sets *error) when the wait for the
// MMAs gave up; the caller then stops.
__device__ __forceinline__ bool tc_gemm_tile(const uint8_t *adig, const int *aexp, const uint8_t *vdig,
                                             const int *vexp, int B, double *gpart, int mt, int nt, int q,
                                             uint8_t *smem, uint64_t *bar, uint32_t tmem, uint32_t &phase,
                                             unsigned *error)
{
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    {
        const uint4 *ga = reinterpret_cast<const uint4 *>(adig + (size_t)(mt * kTcQuarters + q) * kTcABlock);
        const uint4 *gv = reinterpret_cast<const uint4 *>(vdig + (size_t)(nt * kTcQuarters + q) * kTcVBlock);
        uint4 *sa = reinterpret_cast<uint4 *>(smem);
        uint4 *sv = reinterpret_cast<uint4 *>(smem + kTcABlock);
#pragma unroll 4
        for (int x = t; x < (int)(kTcABlock / 16); x += 256)
            sa[x] = __ldcg(ga + x);
#pragma unroll 2
        for (int x = t; x < (int)(kTcVBlock / 16); x += 256)
            sv[x] = __ldcg(gv + x);
    }
    // the operands, written by this CTA's threads, feed the tensor core
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    if (t == 0) {
        tc_fence_after();
        constexpr uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTcTileN >> 3) << 17) |
                                   ((uint32_t)(kTcTileM >> 4) << 24);
        const uint32_t abase = smem_u32(smem), vbase = smem_u32(smem + kTcABlock);
#pragma unroll
        for (int g = 0; g < kTcGroups; g++) {
            bool first = true;
#pragma unroll
            for (int s = 0; s <= g; s++) {
#pragma unroll
                for (int kk = 0; kk < kTcKQ / 16; kk++) {
                    // K step kk covers kgroups 2kk and 2kk + 1
                    const uint64_t ad =
                        umma_desc(abase + (uint32_t)(s * kTcAPlane) + kk * 2 * (kTcTileM * 16), kTcTileM * 16, 128);
                    const uint64_t bd = umma_desc(vbase + (uint32_t)((g - s) * kTcVPlane) + kk * 2 * (kTcTileN * 16),
                                                  kTcTileN * 16, 128);
                    umma_bf16(tmem + (uint32_t)(g * kTcTileN), ad, bd, idesc, first ? 0u : 1u);
                    first = false;
                }
            }
        }
        umma_commit(bar);
    }
    const bool w = mbar_wait_bounded(bar, phase, error);
    phase ^= 1u;
    const bool ok = __syncthreads_and(w) != 0;
    tc_fence_after();
    if (ok) {
        // this thread's accumulator row and 32 instance columns
        const int row = 32 * (warp & 3) + lane, col0 = 32 * (warp >> 2);
        const uint32_t taddr = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)col0;
        const int i = mt * kTcTileM + row;
        const int ea = aexp[q * kTcN + i];
        float ah[32], al[32];
        int esum[32];
#pragma unroll
        for (int c = 0; c < 32; c++) {
            ah[c] = al[c] = 0.0f;
            esum[c] = ea + vexp[(size_t)(nt * kTcTileN + col0 + c) * kTcQuarters + q] - 16;
        }
#pragma unroll 1
        for (int g = 0; g < kTcGroups; g++) {
            float R[32];
            tmem_ld32(taddr + (uint32_t)(g * kTcTileN), R);
#pragma unroll
            for (int c = 0; c < 32; c++) {
                const float v = ldexpf(R[c], esum[c] - 8 * g); // exact: a power-of-two scaling
                const float s = ah[c] + v;
                const float bb = s - ah[c];
                const float e = (ah[c] - (s - bb)) + (v - bb);
                const float lo = al[c] + e;
                ah[c] = s + lo;
                al[c] = lo - (ah[c] - s);
            }
        }
#pragma unroll
        for (int c = 0; c < 32; c++) {
            const int b = nt * kTcTileN + col0 + c;
            if (b < B)
                gpart[((size_t)q * B + b) * kTcN + i] = dw_pack(dword(ah[c], al[c]));
        }
    }
    // the tensor memory is read before the next tile's MMAs write it
    tc_fence_before();
    __syncthreads();
    return ok;
}

} // namespace va
