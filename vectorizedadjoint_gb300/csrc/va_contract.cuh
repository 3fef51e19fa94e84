// Tensor-core contraction of the shared-matrix GLV gradient
//   dA = sum_k v_k x_k^T,   v_k, x_k in R^256,  k over every (instance,
//   accepted step, stage) of the batch
// (the reference's mu += J_alpha^T Kbar of back_prop_step,
// detail/backpropagation.hpp:147-152, whose A-block is sum_m (Kbar_m . X_m)
// X_m^T per step, summed here over the whole batch at once).
//
// The backward sweep writes, per (instance, step, stage), the row v_k
// (double-words packed in 8-byte slots) and a pointer to x_k, the stage
// point its forward stage record already holds, instead of updating an
// N x N partial every step; this file turns them into dA on the tensor pipe
// with an error-free splitting of the factors (the scheme of Ozaki, Ogita,
// Oishi and Rump 2012, "Error-free transformations of matrix multiplication
// by using fast routines of matrix multiplication and its applications"):
//
//  1. Chunks of KC = 64 consecutive rows.  For every chunk and every column
//     i of v (j of x) a power of two 2^e bounds the chunk's entries; each
//     value is written as Q = 4 signed integer digits,
//       v_ki = 2^e sum_{s<Q} d_s 2^(-8(s+1)) + r,   |d_0| <= 256, |d_s| <= 128,
//     |r| <= 2^(e - 8Q - 1): every digit is exact in bf16.
//  2. For each digit pair (s, t) with s + t = g < Q the products d_s d_t are
//     exact in FP32 (<= 2^16) and their sum over the chunk's 64 rows and the
//     <= Q pairs of a group stays below 2^24: tcgen05.mma (kind::f16, bf16
//     inputs, FP32 accumulation in tensor memory) computes every group sum
//     R_g EXACTLY.  (Pairs with s + t >= Q are dropped: the only truncation.)
//  3. dA_ij += 2^(eV_i + eX_j) sum_g 2^(-8(g+2)) R_g,ij, a power-of-two scaling
//     of an exact integer, accumulated as a double-word (~48 bits) in
//     registers; per-CTA partials over disjoint chunk ranges are added in a
//     fixed order afterwards.
//
// The error is the truncation of each factor after Q digits and of the digit
// pairs beyond the kept groups, ~2^-32 of the product of the chunk's column
// maxima per term: dA carries a relative error of ~1e-10..1e-8 against an
// exact sum (depending on how much the magnitudes vary within a chunk),
// against ~1e-13 for the fused double-word update it replaces.
//
// A CTA owns one 128 x 64 tile of dA (M = 128 rows of v, N = 64 columns of x)
// and a contiguous range of chunks.  Per chunk its 256 threads read the raw
// rows, find the exponents and write the digit planes into shared memory in
// the no-swizzle K-major canonical layout of the MMA operands (core matrices
// of 8 rows x 16 bytes; 128 bytes between row groups, one kgroup plane
// between the two core matrices of a 16-deep K step):
//   V: [slice 4][kgroup 8][row 128][8 k]  bf16  (64 KB)
//   X: [slice 4][kgroup 8][row 64][8 k]   bf16  (32 KB)
// one thread issues the 40 MMAs of the chunk (10 digit pairs x 4 K steps of
// 16) into one of two sets of four tensor-memory accumulators, and while
// they run the threads slice the next chunk and fold the previous chunk's
// accumulators into their double-word sums.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "va_dword.cuh"

namespace va {

constexpr int kContractN = 256;      // matrix order (GLV-256)
constexpr int kContractKC = 64;      // rows per chunk
constexpr int kContractQ = 4;        // digits per factor
constexpr int kContractTileM = 128;  // rows of v per CTA tile (tcgen05 M)
constexpr int kContractTileN = 64;   // columns of x per CTA tile (tcgen05 N)
constexpr int kContractTiles = (kContractN / kContractTileM) * (kContractN / kContractTileN); // 8
constexpr int kContractThreads = 512;  // 16 warps: 4 lane quadrants x 4 column groups of the fold
constexpr int kContractFoldCols = kContractTileN / (kContractThreads / 128); // 16 columns per thread
constexpr size_t kTileVBytes = (size_t)kContractQ * kContractKC * kContractTileM * 2;       // 64 KB
constexpr size_t kTileXBytes = (size_t)kContractQ * kContractKC * kContractTileN * 2;       // 32 KB
constexpr size_t kStageBytes = kTileVBytes + kTileXBytes;
// two stages, barriers, and 16 KB of slack: every operand read of an MMA
// (16 row groups x 2 K core matrices from its start address) stays inside
// the allocation whichever of the descriptor's two strides steps along K
constexpr size_t kContractSmem = 2 * kStageBytes + 1024 + 16384;

struct ContractParams {
    const double *v;          // [K][256] packed double-words
    const double *const *xp;  // [K] -> x_k[256] (packed double-words, in a stage record)
    const int *k_total;       // device: number of valid rows K
    double *partials;         // [splits][256][256], transposed: [j][i]
    int splits;               // CTAs per output tile
    unsigned *error;          // set to 1 when a wait gave up (bounded waits)
};

// 2^k as a float for -126 <= k <= 127 (a normal power of two)
__host__ __device__ __forceinline__ float pow2f(int k)
{
    union {
        unsigned u;
        float f;
    } c;
    c.u = (unsigned)(k + 127) << 23;
    return c.f;
}

// The digit scale 2^(8 - e) of a column as two normal powers of two
// (s1 s2 = 2^(8-e); s2 = 1 unless 8 - e > 127, i.e. a column maximum below
// 2^-119): multiplying by them is x 2^(8-e) rounded once, as ldexpf.
struct DigitScale {
    float s1, s2;
};
__host__ __device__ __forceinline__ DigitScale digit_scale(int e)
{
    const int k = 8 - e, k1 = k < 127 ? k : 127;
    return {pow2f(k1), pow2f(k - k1)};
}

// Q digits of the double-word hi + lo (|hi + lo| < 2^e), rounding to
// nearest at each level: hi + lo = 2^e sum_s d_s 2^(-8(s+1)) + r,
// |d_0| <= 256, |d_s| <= 128, |r| <= 2^(e - 8Q - 1).
template <int Q>
__host__ __device__ __forceinline__ void split_digits(float hi, float lo, DigitScale sc, float (&d)[Q])
{
    // a + b = (hi + lo) 2^(8-e), |a + b| < 256; every step below is exact
    float a = hi * sc.s1 * sc.s2, b = lo * sc.s1 * sc.s2;
#pragma unroll
    for (int s = 0; s < Q; s++) {
        const float q = rintf(a);
        d[s] = q;
        const float r = a - q; // exact: q is the integer nearest a
        // renormalise r + b (two-sum), then shift one digit up
        const float sum = r + b;
        const float bb = sum - r;
        const float err = (r - (sum - bb)) + (b - bb);
        a = sum * 256.0f;
        b = err * 256.0f;
    }
}

// Entry points of va_contract.cu (CTAs per output tile for a GPU; the
// kernel's shared-memory attribute, set once before any launch or capture;
// the row offsets of each instance's factor rows; the contraction plus the
// fixed-order sum of its partials into dA[256][256], NaN if it failed).
int contract_splits(int sm_count);
cudaError_t contract_prepare();
cudaError_t enqueue_factor_offsets(const int *inst_T, const int *inst_status, int B, int nsv, int *k_base,
                                   cudaStream_t s);
cudaError_t enqueue_contract(const ContractParams &p, double *dA, cudaStream_t s);

} // namespace va
