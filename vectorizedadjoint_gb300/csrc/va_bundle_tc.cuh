// Forward and backward sweeps of the shared-matrix GLV (N = 256, double-word
// stages with stage records) with the stage products on the tensor cores:
// z = A X in the forward (below, forward_bundle_tc_kernel), A^T v in the
// backward.  The backward first:
//
// The bundle backward (va_bundle.cuh) forms g_m = Kbar_m . (r + z_m) + A^T v_m,
// v_m = Kbar_m . X_m, for every stage of every step as double-word dot
// products on the FP32 pipe: 12 FP32 operations per term, 2 instances per
// CTA.  Here a cluster of 8 CTAs carries a tile of 64 instances in lockstep
// (iteration n runs step T_b - 1 - n of every instance b of the tile; an
// instance that has finished contributes zero columns) and forms each stage's
// product for the whole tile as one 256 x 64 x 256 matrix product on tcgen05:
//
//   CTA (mt, q) of the cluster (rank 4 mt + q) owns
//     - the product block of output rows i in [128 mt, 128 mt + 128) and
//       summation index j in the quarter [64 q, 64 q + 64): D_q[i][b] =
//       sum_j A[j][i] v_j[b], an M = 128, N = 64, K = 64 product;
//     - the adjoint state (Kbar, lambda, mu) of components j in quarter q
//       of the instances b in [32 mt, 32 mt + 32).
//   Per stage:
//     1. every CTA forms v_j[b] = Kbar_m[j][b] X_m[j][b] for its components
//        and instances and writes its 7 digits (below) into the V operand
//        of its own shared memory and of its partner (1 - mt, q), which
//        multiplies the same quarter into the other row tile; cluster
//        barrier;
//     2. one thread issues the 108 MMAs of the block (27 digit pairs x 4 K
//        steps of 16), the CTA folds the 7 group accumulators into
//        double-word partials P_q[i][b] and stores each one straight into
//        the shared memory of the CTA that owns component i for instance b
//        (distributed shared memory, slot q); cluster barrier;
//     3. every CTA reads, for its components j and instances, the four
//        partials P_0..P_3[j][b] it received, g = Kbar_m (r + z_m) +
//        P_0 + P_1 + P_2 + P_3, and updates lambda, mu and the Kbar of the
//        earlier stages.
//   The operand A (6 digit planes of the CTA's 128 x 64 block, 96 KB) stays
//   in shared memory for the whole sweep; only the 57 KB of V digits change
//   per stage.  No grid-wide barrier: the clusters are independent.
//
// Error-free splitting as in va_tc_matvec.cuh (Ozaki, Ogita, Oishi, Rump
// 2012): A^T in 6 digits of 8 bits per (row, quarter) exponent, v in 7 per
// (instance, quarter) exponent, the digit pairs (s, t) with s + t <= 6 (27 of
// 42) summed exactly in FP32 tensor memory (every group sum an integer below
// 2^24), then scaled by powers of two into double-words.  Truncation: ~2^-48
// of the quarter's largest |A| |v| per term, the precision of the double-word
// dot products it replaces.
//
// The factor rows v and x pointers of the deferred dA contraction are
// written exactly as the bundle backward writes them (va_contract.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "va_bundle.cuh"
#include "va_contract.cuh"
#include "va_kernels_dw.cuh"
#include "va_tc_matvec.cuh"
#include "va_tcgen05.cuh"

namespace va {

constexpr int kBtN = 256;                 // matrix order
constexpr int kBtTile = 64;               // instances per cluster (MMA N)
constexpr int kBtThreads = 512;           // 16 warps
constexpr int kBtCluster = 8;             // 2 row tiles x 4 quarters
constexpr int kBtQA = 6, kBtQV = 7;       // digits of A^T and of v
constexpr int kBtGroups = 7;              // digit-pair groups s + t = 0 .. 6
constexpr int kBtPairs = 27;              // pairs (s < 6, t < 7, s + t <= 6)
constexpr size_t kBtAPlane = 128 * 64 * 2;           // 16 KB: [kgroup 8][row 128][8 k] bf16
constexpr size_t kBtABytes = kBtQA * kBtAPlane;      // 96 KB
// V digit plane: [kgroup 8][col 64][8 k] bf16 with kgroups 1040 bytes apart
// (16 bytes of padding shift consecutive kgroups to other banks: the 16
// threads of an instance, which write 8 kgroups, store without conflicts)
constexpr size_t kBtVKgroup = 64 * 16 + 16;
constexpr size_t kBtVPlane = 8 * kBtVKgroup;         // 8,320 bytes
constexpr size_t kBtVBytes = kBtQV * kBtVPlane;      // 58,240 bytes
// received partials: [quarter 4][instance 32][component 64] packed double-words
constexpr size_t kBtPBytes = (size_t)4 * 32 * 64 * sizeof(double); // 64 KB
constexpr size_t kBtMiscBytes = 4096; // kernel-specific arrays (error maxima, chunks, flags, instance state)
constexpr size_t kBtSmem = kBtABytes + kBtVBytes + kBtPBytes + 256 + 128 + kBtMiscBytes + 16;
constexpr int kBtTmemCols = 512;          // 7 groups x 64 columns, rounded up

struct BundleTcParams {
    BundleParams bp;      // sweep inputs and outputs (bp.g), factor rows (fac_v, fac_xp, k_base)
    const uint8_t *adig;  // [8 blocks (mt, q)][kBtABytes] digit planes of A^T
    const double *rpk;    // [B][256] the parameters r as packed double-words
    const int *aexp;      // [4][256] exponents of A^T per (quarter, row)
    unsigned *error;      // set when a bounded wait gave up
};

// ------------------------------------------------------------ cluster helpers

__device__ __forceinline__ uint32_t cluster_rank()
{
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

// all threads of every CTA of the cluster; orders every memory access before
// it (release) against every access after it (acquire) across the cluster
__device__ __forceinline__ void cluster_sync_all()
{
    asm volatile("barrier.cluster.arrive.release.aligned;\n\t"
                 "barrier.cluster.wait.acquire.aligned;" ::
                     : "memory");
}

// the shared::cluster address of this CTA's variable p in the CTA of the given rank
__device__ __forceinline__ uint32_t dsmem_addr(const void *p, uint32_t rank)
{
    uint32_t a;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(a) : "r"(smem_u32(p)), "r"(rank));
    return a;
}

__device__ __forceinline__ double2 dsmem_ld_f64x2(uint32_t a)
{
    double2 v;
    asm volatile("ld.shared::cluster.v2.f64 {%0, %1}, [%2];" : "=d"(v.x), "=d"(v.y) : "r"(a) : "memory");
    return v;
}

__device__ __forceinline__ int dsmem_ld_s32(uint32_t a)
{
    int v;
    asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(v) : "r"(a) : "memory");
    return v;
}

__device__ __forceinline__ void dsmem_st_u32x2(uint32_t a, uint32_t x, uint32_t y)
{
    asm volatile("st.shared::cluster.v2.u32 [%0], {%1, %2};" ::"r"(a), "r"(x), "r"(y) : "memory");
}

__device__ __forceinline__ void dsmem_st_f64(uint32_t a, double v)
{
    asm volatile("st.shared::cluster.f64 [%0], %1;" ::"r"(a), "d"(v) : "memory");
}

__device__ __forceinline__ void dsmem_st_s32(uint32_t a, int v)
{
    asm volatile("st.shared::cluster.s32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}

// generic-proxy writes (the digit planes) before the tensor core reads them
__device__ __forceinline__ void fence_proxy_async_all() { asm volatile("fence.proxy.async;" ::: "memory"); }

// x * 2^k for an integer-valued float x (|x| < 2^24), exact unless the
// result leaves the normal range
__device__ __forceinline__ float scale_pow2(float x, int k)
{
    return (k >= -126 && k <= 127) ? x * pow2f(k) : ldexpf(x, k);
}

// ------------------------------------------------------------------ kernels

// Digit planes of A^T for the cluster backward: one block of 256 threads (k)
// per row i of A^T (column i of A); A row-major FP64.
__global__ void __launch_bounds__(256) bt_digits_A_kernel(const double *A, uint8_t *adig, int *aexp);
// the same for A itself (the forward's z = A x): one block per row i of A
__global__ void __launch_bounds__(256) bt_digits_Af_kernel(const double *A, uint8_t *adig, int *aexp);

// r as packed double-words: one block of 256 threads per instance
__global__ void __launch_bounds__(256) bt_pack_r_kernel(const double *par, double *rpk);

// one stage's MMAs: D_g (tensor-memory columns 64 g) = sum over the pairs
// (s, g - s) and the 4 K steps of A digit s times V digit g - s.  Fully
// unrolled: every descriptor is the base descriptor plus a constant (the
// start-address field holds address / 16, and every operand lies below 256 KB)
template <int G = 0, int S = 0, int KK = 0>
__device__ __forceinline__ void bt_issue_mmas_from(uint64_t ad0, uint64_t bd0, uint32_t tmem)
{
    if constexpr (G < kBtGroups) {
        constexpr int s_lo = G - (kBtQV - 1) > 0 ? G - (kBtQV - 1) : 0;
        constexpr int s_hi = G < kBtQA - 1 ? G : kBtQA - 1;
        constexpr int s = S < s_lo ? s_lo : S;
        if constexpr (s > s_hi) {
            bt_issue_mmas_from<G + 1, 0, 0>(ad0, bd0, tmem);
        } else {
            constexpr uint64_t aoff = (uint64_t)((s * kBtAPlane + KK * 2 * (128 * 16)) >> 4);
            constexpr uint64_t boff = (uint64_t)(((G - s) * kBtVPlane + KK * 2 * kBtVKgroup) >> 4);
            constexpr uint32_t idesc = umma_idesc_bf16(128, kBtTile);
            umma_bf16_k<!(s == s_lo && KK == 0)>(tmem + (uint32_t)(G * kBtTile), ad0 + aoff, bd0 + boff, idesc);
            if constexpr (KK < 3)
                bt_issue_mmas_from<G, s, KK + 1>(ad0, bd0, tmem);
            else
                bt_issue_mmas_from<G, s + 1, 0>(ad0, bd0, tmem);
        }
    }
}

__device__ __forceinline__ void bt_issue_mmas(const uint8_t *sA, const uint8_t *sV, uint32_t tmem)
{
    // K step kk covers kgroups 2kk and 2kk + 1 (lbo: one kgroup plane)
    bt_issue_mmas_from(umma_desc(smem_u32(sA), 128 * 16, 128), umma_desc(smem_u32(sV), kBtVKgroup, 128), tmem);
}

// ------------------------------------------------------- cluster sweep context

// One CTA of a cluster sweep: its shared-memory regions, tensor memory and
// MMA barrier, and each thread's two roles -- the 4 components j0 .. j0 + 3
// of tile instance b it carries (digits in, partials out), and the row frow
// and 16 columns fc .. fc + 15 of the product block it folds.
struct BtCta {
    uint8_t *sA, *sV; // operand digit planes (A resident, V per stage)
    double *sR;       // received partials [quarter 4][instance 32][component 64]
    int *sEv, *sBad;  // exponents of V per column [64]; non-finite flags [32]
    uint8_t *misc;    // kernel-specific small arrays (kBtMiscBytes)
    uint64_t *bar;
    int t, warp, mt, q, tile;
    uint32_t tmem, phase;
    bool ok; // every MMA wait so far ended in time
    int bl, jg, b, j0;
    int ea;
    uint32_t taddr, fold_dst, voff, v_remote, ev_remote;
    const double *p_mine;
};

// Shared memory, tensor memory, the resident A block (digit block (mt, q) of
// adig) and every thread's constants.  Ends with a CTA barrier; the kernel
// then does its own set-up and one cluster barrier before any access to
// another CTA's shared memory.
__device__ __forceinline__ void bt_begin(BtCta &c, uint8_t *smem, const uint8_t *adig, const int *aexp)
{
    c.sA = smem;
    c.sV = smem + kBtABytes;
    c.sR = reinterpret_cast<double *>(smem + kBtABytes + kBtVBytes);
    c.sEv = reinterpret_cast<int *>(smem + kBtABytes + kBtVBytes + kBtPBytes);
    c.sBad = c.sEv + kBtTile;
    c.misc = reinterpret_cast<uint8_t *>(c.sBad + 32);
    c.bar = reinterpret_cast<uint64_t *>(c.misc + kBtMiscBytes);
    uint32_t *slot_tmem = reinterpret_cast<uint32_t *>(c.bar + 1);
    c.t = threadIdx.x;
    c.warp = c.t >> 5;
    const int lane = c.t & 31;
    const uint32_t rank = cluster_rank();
    c.mt = (int)(rank >> 2);
    c.q = (int)(rank & 3);
    c.tile = blockIdx.x / kBtCluster;
    if (c.warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot_tmem)),
                     "r"(kBtTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (c.t == 0) {
        mbar_init(c.bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    {
        const uint4 *ga = reinterpret_cast<const uint4 *>(adig + (size_t)(c.mt * 4 + c.q) * kBtABytes);
        uint4 *sa = reinterpret_cast<uint4 *>(c.sA);
#pragma unroll 4
        for (int x = c.t; x < (int)(kBtABytes / 16); x += kBtThreads)
            sa[x] = __ldg(ga + x);
    }
    if (c.t < 32)
        c.sBad[c.t] = 0;
    for (int x = c.t; x < (int)(kBtMiscBytes / 4); x += kBtThreads)
        reinterpret_cast<int *>(c.misc)[x] = 0;
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    c.tmem = *slot_tmem;
    c.phase = 0;
    c.ok = true;
    // carried components: instance b = 32 mt + bl, components 64 q + 4 jg + 0..3
    c.bl = c.t >> 4;
    c.jg = c.t & 15;
    c.b = 32 * c.mt + c.bl;
    c.j0 = 64 * c.q + 4 * c.jg;
    // folded element: tensor-memory lane quadrant warp & 3, 16 columns
    const int fq = c.warp & 3, fc = 16 * (c.warp >> 2);
    const int frow = 32 * fq + lane;
    c.ea = aexp[c.q * kBtN + 128 * c.mt + frow];
    c.taddr = c.tmem + ((uint32_t)(32 * fq) << 16) + (uint32_t)fc;
    // the fold's row frow is component 128 mt + frow, carried (for the
    // instances of column half fc / 32) by CTA (fc / 32, 2 mt + frow / 64):
    // slot q of its partials
    c.fold_dst = dsmem_addr(c.sR + ((size_t)c.q * 32 + (fc & 31)) * 64 + (frow & 63),
                            (uint32_t)((fc >> 5) * 4 + 2 * c.mt + (frow >> 6)));
    c.p_mine = c.sR + (size_t)c.bl * 64 + 4 * c.jg;
    // where this thread's digits go: plane offset of (column b, components
    // j0 .. j0 + 3), here and in the partner (1 - mt, q)
    const uint32_t partner = (uint32_t)((1 - c.mt) * 4 + c.q);
    c.voff = (uint32_t)((c.jg >> 1) * kBtVKgroup + c.b * 16 + (c.jg & 1) * 8);
    c.v_remote = dsmem_addr(c.sV + c.voff, partner);
    c.ev_remote = dsmem_addr(c.sEv + c.b, partner);
}

// The digits of this thread's 4 values of instance b (the exponent over the
// instance's 64 components of the quarter: its 16 threads) into the V
// operand here and in the partner.
__device__ __forceinline__ void bt_put(const BtCta &c, const dword (&v)[4])
{
    float mx = fmaxf(fmaxf(fabsf(v[0].hi), fabsf(v[1].hi)), fmaxf(fabsf(v[2].hi), fabsf(v[3].hi)));
#pragma unroll
    for (int o = 8; o > 0; o >>= 1)
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    const int ev = tc_bound_exponent(mx);
    const DigitScale sc = digit_scale(ev);
    // digit s of the four values, packed as 4 bf16 (8 bytes)
    uint32_t pk[kBtQV][2];
#pragma unroll
    for (int e = 0; e < 4; e++) {
        float d[kBtQV];
        split_digits<kBtQV>(v[e].hi, v[e].lo, sc, d);
#pragma unroll
        for (int s = 0; s < kBtQV; s++) {
            const uint32_t w = (uint32_t)bf16_bits(d[s]) << (16 * (e & 1));
            pk[s][e >> 1] = (e & 1) ? (pk[s][e >> 1] | w) : w;
        }
    }
#pragma unroll
    for (int s = 0; s < kBtQV; s++) {
        *reinterpret_cast<uint2 *>(c.sV + (size_t)s * kBtVPlane + c.voff) = make_uint2(pk[s][0], pk[s][1]);
        dsmem_st_u32x2(c.v_remote + (uint32_t)(s * kBtVPlane), pk[s][0], pk[s][1]);
    }
    if (c.jg == 0) {
        c.sEv[c.b] = ev;
        dsmem_st_s32(c.ev_remote, ev);
    }
}

// First half of a stage's product: the digits written by the generic proxy
// become visible to the tensor core, and a cluster barrier: every CTA's V
// operand and exponents are in place.
__device__ __forceinline__ void bt_product_barrier()
{
    fence_proxy_async_all();
    cluster_sync_all();
}

// Second half: the MMAs, the fold of the 7 group accumulators, every partial
// pushed to the CTA that carries its (component, instance); a cluster barrier
// after which every CTA's received partials are complete.
__device__ __forceinline__ void bt_product_rest(BtCta &c, unsigned *error)
{
    // one thread issues the MMAs and alone polls their barrier (threads
    // polling shared memory slow the tensor core's operand reads); the
    // others wait at the CTA barrier
    bool w = true;
    if (c.ok && c.t == 0) {
        tc_fence_after();
        bt_issue_mmas(c.sA, c.sV, c.tmem);
        umma_commit(c.bar);
        w = mbar_wait_bounded(c.bar, c.phase, error);
    }
    if (c.ok)
        c.phase ^= 1u;
    c.ok = __syncthreads_and(c.ok && w) != 0;
    tc_fence_after();
    // fold: S = R_0 + R_1 2^-8 + R_2 2^-16 + (R_3 2^-24 + .. + R_6 2^-48)
    // in units of group 0 (|R_g| < 2^24 integers): the tail is below 1 and
    // summed in FP32 (error < 2^-23, i.e. 2^-47 of the largest S), the head
    // with two 2Sums; then the power-of-two scaling 2^(eA + eV - 16)
    const int fc = 16 * (c.warp >> 2);
#pragma unroll 1
    for (int half = 0; half < 2; half++) {
        const int c0 = fc + 8 * half;
        const uint32_t dst = c.fold_dst + (uint32_t)(8 * half * 64 * sizeof(double));
        if (c.ok) {
            float tail[8];
            {
                float R[4][8];
                tmem_ld8_groups<4>(c.taddr + (uint32_t)(8 * half), 3, R);
#pragma unroll
                for (int k = 0; k < 8; k++)
                    tail[k] = fmaf(R[0][k], 0x1p-24f, fmaf(R[1][k], 0x1p-32f, fmaf(R[2][k], 0x1p-40f, R[3][k] * 0x1p-48f)));
            }
            float R[3][8];
            tmem_ld8_groups<3>(c.taddr + (uint32_t)(8 * half), 0, R);
#pragma unroll
            for (int k = 0; k < 8; k++) {
                float s1, e1, s2, e2, hi, lo;
                two_sum(R[0][k], R[1][k] * 0x1p-8f, s1, e1);
                two_sum(s1, R[2][k] * 0x1p-16f, s2, e2);
                two_sum(s2, (e1 + e2) + tail[k], hi, lo);
                const int sc = c.ea + c.sEv[c0 + k] - 16;
                dsmem_st_f64(dst + (uint32_t)(k * 64 * sizeof(double)), dw_pack(dword(scale_pow2(hi, sc), scale_pow2(lo, sc))));
            }
        } else {
            const double nan = __longlong_as_double(0x7ff8000000000000ll);
#pragma unroll
            for (int k = 0; k < 8; k++)
                dsmem_st_f64(dst + (uint32_t)(k * 64 * sizeof(double)), nan);
        }
    }
    tc_fence_before();
    cluster_sync_all(); // every CTA's partials delivered
}

__device__ __forceinline__ void bt_product(BtCta &c, unsigned *error)
{
    bt_product_barrier();
    bt_product_rest(c, error);
}

// The product's value for this thread's (j, b): the four received quarter
// partials added in quarter order.
__device__ __forceinline__ void bt_gather(const BtCta &c, dword (&G)[4])
{
    double2 v[4][2];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const double2 *src = reinterpret_cast<const double2 *>(c.p_mine + (size_t)k * 32 * 64);
        v[k][0] = src[0];
        v[k][1] = src[1];
    }
#pragma unroll
    for (int e = 0; e < 4; e++) {
        dword s = dw_unpack(e & 1 ? v[0][e >> 1].y : v[0][e >> 1].x);
#pragma unroll
        for (int k = 1; k < 4; k++)
            s += dw_unpack(e & 1 ? v[k][e >> 1].y : v[k][e >> 1].x);
        G[e] = s;
    }
}

// OR of the four quarter CTAs' non-finite flags for instance column bl
// (after a cluster barrier)
__device__ __forceinline__ int bt_bad(const BtCta &c)
{
    int bad = c.sBad[c.bl];
#pragma unroll
    for (int k = 0; k < 4; k++)
        if (k != c.q)
            bad |= dsmem_ld_s32(dsmem_addr(c.sBad + c.bl, (uint32_t)(c.mt * 4 + k)));
    return bad;
}

// Release of the tensor memory (after the kernel's last cluster barrier).
__device__ __forceinline__ void bt_end(BtCta &c, unsigned *error)
{
    if (!c.ok && c.t == 0) // once more (bounded) for MMAs still in flight before the memory is released
        (void)mbar_wait_bounded(c.bar, c.phase ^ 1u, error);
    __syncthreads();
    tc_fence_after();
    if (c.warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(c.tmem), "r"(kBtTmemCols)
                     : "memory");
}

// ------------------------------------------------------------ backward sweep

template <class Tab>
__global__ void __cluster_dims__(kBtCluster, 1, 1) __launch_bounds__(kBtThreads, 1)
    backward_bundle_tc_kernel(BundleTcParams p)
{
    constexpr int NS = Tab::S;
    constexpr int NSV = factor_stages<Tab>();
    constexpr int RS = bundle_stage_record_doubles(kBtN, NS);
    const AdjParams &a = p.bp.g;
    extern __shared__ __align__(1024) uint8_t smem[];
    BtCta c;
    bt_begin(c, smem, p.adig, p.aexp);
    // every CTA is resident: a dependent tail sweep may start on the idle SMs
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    int *sMaxT = reinterpret_cast<int *>(c.misc);
    const int CH = a.pool.chunk_len;

    // lockstep length of the tile: the longest instance (every CTA of the
    // cluster reads the same 64 counts and gets the same value)
    if (c.t < kBtTile) {
        const int i = c.tile * kBtTile + c.t;
        int T = 0;
        if (i < a.B && a.inst_status[i] == ST_OK)
            T = a.inst_T[i];
        atomicMax(sMaxT, T);
    }

    const int inst = c.tile * kBtTile + c.b;
    const int j0 = c.j0;
    const bool inb = inst < a.B;
    bool live = inb && a.inst_status[inst] == ST_OK;
    if (inb && !live) {
        const double nan = __longlong_as_double(0x7ff8000000000000ll);
#pragma unroll
        for (int e = 0; e < 4; e++) {
            a.dy0[(size_t)inst * kBtN + j0 + e] = nan;
            a.dpar[(size_t)inst * kBtN + j0 + e] = nan;
        }
        if (a.status_out && c.q == 0 && c.jg == 0)
            a.status_out[inst] = a.inst_status[inst];
    }
    // lambda and mu of the four components: compensated sums (each stage's
    // J^T Kbar and Kbar . X are added as they are formed)
    dacc lam[4], mu[4];
    int jstep = -1, chunk = -1, slot = 0;
    double t_next = 0.0;
#pragma unroll
    for (int e = 0; e < 4; e++) {
        lam[e] = dacc{0.0f, 0.0f};
        mu[e] = dacc{0.0f, 0.0f};
    }
    const double2 *rp = reinterpret_cast<const double2 *>(p.rpk + (size_t)(inb ? inst : 0) * kBtN + j0);
    if (live) {
        const int T = a.inst_T[inst];
        chunk = a.inst_last[inst];
        slot = T % CH;
        const double *rec = record_ptr<RS>(a.pool, chunk, slot);
        t_next = rec[0];
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int j = j0 + e;
            const double yT = to_d(dw_unpack(rec[2 + j]));
            const double l = a.cost == 0 ? 2.0 * yT : a.cost == 1 ? 1.0 : a.lambdaT[(size_t)inst * kBtN + j];
            lam[e] = dacc_of(dword(l));
        }
        jstep = T - 1;
    }
    // results of an instance whose adjoint is complete
    auto finish = [&]() {
        bool bad = false;
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int j = j0 + e;
            const double l = to_d(dacc_get(lam[e]));
            const double d = (a.mu_direct ? a.mu_direct[(size_t)inst * kBtN + j] : 0.0) + to_d(dacc_get(mu[e]));
            a.dy0[(size_t)inst * kBtN + j] = l;
            a.dpar[(size_t)inst * kBtN + j] = d;
            bad = bad || !isfinite(l) || !isfinite(d);
        }
        if (bad)
            atomicOr(&c.sBad[c.bl], 1);
    };
    if (live && jstep < 0) { // no accepted step: the seeds are the result
        finish();
        live = false;
    }
    __syncthreads();
    const int maxT = *sMaxT;
    // every CTA of the cluster has started before any distributed access
    cluster_sync_all();

    // Kbar of the step's stages as compensated sums (seed b_m h lambda plus
    // a_km h g_k of the later stages k)
    dacc Kb[NS][4];
    dword tpend[4];
    const double *srec = nullptr;
    double tn = 0.0;
    dword sh(0.0f, 0.0f);
    bool active = false;
    for (int n = 0; n <= maxT; n++) {
        if (n > 0) {
            // stage 0 of the previous step: its g, then lambda and mu
            dword G[4];
            bt_gather(c, G);
            if (active) {
#pragma unroll
                for (int e = 0; e < 4; e++)
                    dacc_add(lam[e], tpend[e] + G[e]);
                t_next = tn;
                jstep--;
                if (jstep < 0) {
                    finish();
                    live = false;
                }
            }
        }
        if (n == maxT)
            break;
        active = live && jstep >= 0;
        if (active) {
            if (slot == 0) {
                chunk = a.pool.chunk_prev[chunk];
                slot = CH - 1;
            } else {
                slot--;
            }
            srec = record_ptr<RS>(a.pool, chunk, slot);
            tn = srec[0];
            sh = dword(t_next - tn);
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const dword l = dacc_get(lam[e]);
                lam[e] = dacc_of(l);
#pragma unroll
                for (int m = 0; m < NS; m++)
                    Kb[m][e] = Tab::b(m) != 0.0 ? dacc_mul(dword(Tab::b(m)) * sh, l) : dacc{0.0f, 0.0f};
            }
        }
#pragma unroll
        for (int m = NS - 1; m >= 0; m--) {
            if (m < NS - 1) {
                // g of stage m + 1, and its share of the earlier stages' Kbar
                dword G[4];
                bt_gather(c, G);
                if (active) {
#pragma unroll
                    for (int e = 0; e < 4; e++) {
                        const dword g = tpend[e] + G[e];
                        dacc_add(lam[e], g);
                        const dword gh = g * sh;
#pragma unroll
                        for (int k = 0; k < NS - 1; k++)
                            if (k <= m && Tab::a(m + 1, k) != 0.0)
                                dacc_fma_k(Kb[k][e], Tab::a(m + 1, k), gh);
                    }
                }
            }
            // stage m: v = Kbar_m X_m (the factor row), the pending Kbar_m (r + z_m)
            dword v[4];
            if (active) {
                const double2 *xs = reinterpret_cast<const double2 *>(srec + 2 + (size_t)m * kBtN + j0);
                const double2 *zs = reinterpret_cast<const double2 *>(srec + 2 + (size_t)(NS + m) * kBtN + j0);
                const double2 x01 = __ldg(xs), x23 = __ldg(xs + 1);
                const double2 z01 = __ldg(zs), z23 = __ldg(zs + 1);
                const double xv[4] = {x01.x, x01.y, x23.x, x23.y};
                const double zv[4] = {z01.x, z01.y, z23.x, z23.y};
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const dword Km = dacc_get(Kb[m][e]);
                    v[e] = Km * dw_unpack(xv[e]);
                    dacc_add(mu[e], v[e]);
                    const double2 r2 = __ldg(rp + (e >> 1));
                    tpend[e] = Km * (dw_unpack(e & 1 ? r2.y : r2.x) + dw_unpack(zv[e]));
                }
                // the next stage's record lines into L1 while the product runs
                if (m > 0) {
                    asm volatile("prefetch.global.L1 [%0];" ::"l"(srec + 2 + (size_t)(m - 1) * kBtN + j0));
                    asm volatile("prefetch.global.L1 [%0];" ::"l"(srec + 2 + (size_t)(NS + m - 1) * kBtN + j0));
                }
                if (m < NSV) {
                    const size_t k0 = (size_t)p.bp.k_base[inst] + (size_t)jstep * NSV + m;
                    double2 *fv = reinterpret_cast<double2 *>(p.bp.fac_v + k0 * kBtN + j0);
                    fv[0] = make_double2(dw_pack(v[0]), dw_pack(v[1]));
                    fv[1] = make_double2(dw_pack(v[2]), dw_pack(v[3]));
                    if (c.q == 0 && c.jg == 0)
                        p.bp.fac_xp[k0] = srec + 2 + (size_t)m * kBtN;
                }
            } else {
#pragma unroll
                for (int e = 0; e < 4; e++)
                    v[e] = dword(0.0f, 0.0f);
            }
            bt_put(c, v);
            bt_product(c, p.error);
        }
    }
    // every partial has been read; then the instances' status from the four
    // quarters' flags (rank 4 mt + k holds quarter k of the same instances)
    cluster_sync_all();
    if (c.q == 0 && c.jg == 0 && inb && a.inst_status[inst] == ST_OK && a.status_out)
        a.status_out[inst] = bt_bad(c) ? ST_NONFINITE : ST_OK;
    cluster_sync_all(); // no CTA leaves while another reads its shared memory
    bt_end(c, p.error);
}

// ------------------------------------------------------------- forward sweep

// The forward sweep of the same tile in lockstep (DOPRI5: FSAL, controlled):
// iteration n is one attempt of every instance that has not finished, each
// with its own t, dt and odeint controller decision.  Per attempt the six
// products z_m = A X_m (stages 2 .. 6 and f(y_new)) run as in the backward,
// with A's digit planes (not A^T's).  What needs the whole instance crosses
// the 4 quarter CTAs (mt, 0..3) that carry its components:
//   - the error ratio: each CTA's maximum over its 64 components, exchanged
//     through distributed shared memory (a cluster barrier), then the same
//     controller decision in each of them (one thread per instance; its 16
//     threads take the result by shuffle);
//   - checkpoint chunks: CTA (mt, 0) allocates an instance's next chunk when
//     its current one fills and hands it to the other three (read at the
//     next top of step, many cluster barriers later);
//   - the end: non-finite flags of y(T) gathered by CTA (mt, 0), which
//     writes the instance's counters and status.
// Every accepted step writes the same stage record as the bundle forward
// [t, dt, X_0 .. X_5, z_0 .. z_5]; each CTA its 64 components.  The
// arithmetic per component is the bundle forward's double-word arithmetic;
// the error ratio is formed in double-words (|e| / tol by double-word
// division) instead of FP64.
// Per-instance state of the forward's 32 instances of a CTA, in shared
// memory: the FP64 controller and the top-of-step logic run in warp 0, one
// lane per instance (in the instance's own threads every FP64 instruction
// would issue in 16 warps: the FP64 pipe, 1/64 of FP32 on this GPU, was the
// forward's bound).
struct BtFwdInst {
    double t[32], t1[32], dt[32];
    double *rec[32];   // the current step's record
    float2 sdt[32];    // dt as a double-word
    int count[32], rej[32], fails[32], status[32], chunk[32], slot[32];
    int mode[32];      // kFwd* flags of this iteration
};
constexpr int kFwdAttempt = 1, kFwdTopRecord = 2, kFwdFinished = 4, kFwdAccepted = 8, kFwdDone = 16, kFwdAtTop = 32;

template <class Tab>
__global__ void __cluster_dims__(kBtCluster, 1, 1) __launch_bounds__(kBtThreads, 1)
    forward_bundle_tc_kernel(BundleTcParams p)
{
    static_assert(Tab::FSAL && !Tab::FIXED, "controlled FSAL pairs");
    constexpr int NS = Tab::S;
    constexpr int RS = bundle_stage_record_doubles(kBtN, NS);
    const FwdParams &a = p.bp.f;
    extern __shared__ __align__(1024) uint8_t smem[];
    BtCta c;
    bt_begin(c, smem, p.adig, p.aexp);
    // every CTA is resident: a dependent tail sweep may start on the idle SMs
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    double *sErr = reinterpret_cast<double *>(c.misc);    // [4 quarters][32 instances] error-ratio maxima
    int *sChunk = reinterpret_cast<int *>(c.misc + 1024); // [32] next checkpoint chunk
    int *sAct = sChunk + 32;                              // [8] CTAs with an attempt this iteration
    BtFwdInst &S = *reinterpret_cast<BtFwdInst *>(c.misc + 1280);
    const int CH = a.pool.chunk_len;
    const int j0 = c.j0;
    const int inst = c.tile * kBtTile + c.b;
    const bool inb = inst < a.B;
    const int lane = c.t & 31;
    const bool ctl = c.warp == 0; // warp 0: lane L runs instance column L
    const int cinst = c.tile * kBtTile + 32 * c.mt + lane;
    const bool cinb = ctl && cinst < a.B;

    dword ys[4], z0[4], K[NS][4];
    const double2 *rp = reinterpret_cast<const double2 *>(p.rpk + (size_t)(inb ? inst : 0) * kBtN + j0);
    auto rv = [&](int e) -> dword {
        const double2 r2 = __ldg(rp + (e >> 1));
        return dw_unpack(e & 1 ? r2.y : r2.x);
    };
    if (inb) {
        const double2 *y2 = reinterpret_cast<const double2 *>(a.y0 + (size_t)inst * kBtN + j0);
        const double2 y01 = y2[0], y23 = y2[1];
        ys[0] = dword(y01.x);
        ys[1] = dword(y01.y);
        ys[2] = dword(y23.x);
        ys[3] = dword(y23.y);
    } else {
#pragma unroll
        for (int e = 0; e < 4; e++)
            ys[e] = dword(0.0f, 0.0f);
    }
    if (ctl) {
        S.t[lane] = cinb ? a.t0[cinst] : 0.0;
        S.t1[lane] = cinb ? a.t1[cinst] : 0.0;
        S.dt[lane] = a.dt0;
        S.count[lane] = S.rej[lane] = S.fails[lane] = 0;
        S.status[lane] = ST_OK;
        S.chunk[lane] = -1;
        S.slot[lane] = 0;
        S.mode[lane] = cinb ? kFwdAtTop : kFwdDone;
        S.rec[lane] = nullptr;
    }
    const dword datol(a.atol), drtol(a.rtol);
    // every CTA of the cluster has started before any distributed access
    cluster_sync_all();

    // the instance's next chunk, from CTA (mt, 0) to the four quarter CTAs
    // (warp 0, lane = instance column)
    auto alloc_chunk = [&](int prev) {
        int ch = (int)atomicAdd(&a.ctl->pool_next, 1u);
        if (ch >= a.pool.n_chunks) {
            ch = -1;
            atomicOr(&a.ctl->pool_fail, 1u);
        } else {
            a.pool.chunk_prev[ch] = prev;
        }
#pragma unroll
        for (int k = 0; k < 4; k++)
            dsmem_st_s32(dsmem_addr(sChunk + lane, (uint32_t)(c.mt * 4 + k)), ch);
    };
    if (c.q == 0 && cinb)
        alloc_chunk(-1);
    // k_1 = f(y_0)
    bt_put(c, ys);
    bt_product(c, p.error); // (its barriers also deliver the first chunks)
    {
        dword G[4];
        bt_gather(c, G);
#pragma unroll
        for (int e = 0; e < 4; e++) {
            z0[e] = G[e];
            K[0][e] = ys[e] * (rv(e) + G[e]);
        }
    }
    if (cinb) {
        S.chunk[lane] = sChunk[lane];
        if (S.chunk[lane] < 0)
            S.status[lane] = ST_CKPT_BUDGET;
    }

    for (;;) {
        // top of step (warp 0): loop test, record, end clamp of the instances
        // whose last attempt was accepted (or at the start)
        if (ctl) {
            int mode = S.mode[lane] & (kFwdDone | kFwdAtTop);
            if (!(mode & kFwdDone) && (mode & kFwdAtTop)) {
                double t = S.t[lane], t1 = S.t1[lane], dt = S.dt[lane];
                int status = S.status[lane], chunk = S.chunk[lane], slot = S.slot[lane];
                const bool end = !(t1 - t > kDblEps);
                bool fin = status != ST_OK;
                if (!fin && !end && S.count[lane] >= a.max_steps) {
                    status = ST_MAX_STEPS;
                    fin = true;
                }
                if (!fin && slot == CH) {
                    chunk = sChunk[lane];
                    slot = 0;
                    if (chunk < 0) {
                        status = ST_CKPT_BUDGET;
                        fin = true;
                    }
                }
                if (!fin) {
                    double *rec = record_ptr<RS>(a.pool, chunk, slot);
                    if (c.q == 0)
                        *reinterpret_cast<double2 *>(rec) = make_double2(t, dt);
                    S.rec[lane] = rec;
                    mode |= kFwdTopRecord;
                    slot++;
                    if (slot == CH && !end && c.q == 0)
                        alloc_chunk(chunk);
                    fin = end;
                }
                if (fin) {
                    mode = (mode | kFwdDone | kFwdFinished) & ~kFwdAtTop;
                } else {
                    if ((t + dt) - t1 > kDblEps)
                        dt = t1 - t;
                    S.fails[lane] = 0;
                    mode &= ~kFwdAtTop;
                }
                S.dt[lane] = dt;
                S.status[lane] = status;
                S.chunk[lane] = chunk;
                S.slot[lane] = slot;
            }
            if (!(mode & kFwdDone)) {
                mode |= kFwdAttempt;
                const dword d(S.dt[lane]);
                S.sdt[lane] = make_float2(d.hi, d.lo);
            }
            S.mode[lane] = mode;
            // whether any instance of the tile attempts: this CTA's flag to all
            // eight (read after the first stage's cluster barrier)
            const int mine = __any_sync(0xffffffffu, (mode & kFwdAttempt) != 0);
            if (lane < kBtCluster)
                dsmem_st_s32(dsmem_addr(sAct + 4 * c.mt + c.q, (uint32_t)lane), mine);
        }
        __syncthreads();
        const int mode = S.mode[c.bl];
        const bool attempt = (mode & kFwdAttempt) != 0;
        double *rec = S.rec[c.bl];
        if (mode & kFwdTopRecord) {
            double2 *x0 = reinterpret_cast<double2 *>(rec + 2 + j0);
            double2 *zz = reinterpret_cast<double2 *>(rec + 2 + (size_t)NS * kBtN + j0);
            x0[0] = make_double2(dw_pack(ys[0]), dw_pack(ys[1]));
            x0[1] = make_double2(dw_pack(ys[2]), dw_pack(ys[3]));
            zz[0] = make_double2(dw_pack(z0[0]), dw_pack(z0[1]));
            zz[1] = make_double2(dw_pack(z0[2]), dw_pack(z0[3]));
        }
        if (mode & kFwdFinished) {
            // y(T) of this thread's components and their finiteness
            const bool moved = S.count[c.bl] > 0;
            bool bad = false;
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const double y = moved ? to_d(ys[e]) : a.y0[(size_t)inst * kBtN + j0 + e];
                if (a.yT)
                    a.yT[(size_t)inst * kBtN + j0 + e] = y;
                bad = bad || !isfinite(y);
            }
            if (bad)
                atomicOr(&c.sBad[c.bl], 1);
        }
        const dword sdt(S.sdt[c.bl].x, S.sdt[c.bl].y);
        bool stop = false;
        // stages 2 .. s: X_m = y + dt sum_{j<m} a_mj K_j, K_m = X_m (r + A X_m)
#pragma unroll
        for (int m = 1; m < NS; m++) {
            dword X[4];
#pragma unroll
            for (int e = 0; e < 4; e++) {
                if (attempt) {
                    // compensated sum of the tableau row, then y + dt s
                    dacc acc{0.0f, 0.0f};
                    bool first = true;
#pragma unroll
                    for (int j = 0; j < NS - 1; j++)
                        if (j < m && Tab::a(m, j) != 0.0) {
                            if (first)
                                acc = dacc_mul_k(Tab::a(m, j), K[j][e]);
                            else
                                dacc_fma_k(acc, Tab::a(m, j), K[j][e]);
                            first = false;
                        }
                    X[e] = axpy_dw(ys[e], sdt, acc);
                } else {
                    X[e] = dword(0.0f, 0.0f);
                }
            }
            bt_put(c, X);
            bt_product_barrier();
            if (m == 1) {
                int any = 0;
#pragma unroll
                for (int k = 0; k < kBtCluster; k++)
                    any |= sAct[k];
                if (!any) { // every CTA of the cluster reads the same flags
                    stop = true;
                    break;
                }
            }
            bt_product_rest(c, p.error);
            dword G[4];
            bt_gather(c, G);
#pragma unroll
            for (int e = 0; e < 4; e++)
                K[m][e] = X[e] * (rv(e) + G[e]);
            if (attempt) {
                // every attempt rewrites the step's stage values: the accepted one is the last
                double2 *xm = reinterpret_cast<double2 *>(rec + 2 + (size_t)m * kBtN + j0);
                double2 *zm = reinterpret_cast<double2 *>(rec + 2 + (size_t)(NS + m) * kBtN + j0);
                xm[0] = make_double2(dw_pack(X[0]), dw_pack(X[1]));
                xm[1] = make_double2(dw_pack(X[2]), dw_pack(X[3]));
                zm[0] = make_double2(dw_pack(G[0]), dw_pack(G[1]));
                zm[1] = make_double2(dw_pack(G[2]), dw_pack(G[3]));
            }
        }
        if (stop)
            break;
        // y_new = y + dt sum_j b_j K_j and f(y_new)
        dword yn[4], zn[4], kn[4];
#pragma unroll
        for (int e = 0; e < 4; e++) {
            if (attempt) {
                dacc acc{0.0f, 0.0f};
                bool first = true;
#pragma unroll
                for (int j = 0; j < NS; j++)
                    if (Tab::b(j) != 0.0) {
                        if (first)
                            acc = dacc_mul_k(Tab::b(j), K[j][e]);
                        else
                            dacc_fma_k(acc, Tab::b(j), K[j][e]);
                        first = false;
                    }
                yn[e] = axpy_dw(ys[e], sdt, acc);
            } else {
                yn[e] = dword(0.0f, 0.0f);
            }
        }
        bt_put(c, yn);
        bt_product(c, p.error);
        {
            dword G[4];
            bt_gather(c, G);
#pragma unroll
            for (int e = 0; e < 4; e++) {
                zn[e] = G[e];
                kn[e] = yn[e] * (rv(e) + G[e]);
            }
        }
        // error ratio |dt sum_j e_j K_j| / (atol + rtol (|y| + |dt| |K_1|)),
        // its maximum over the instance's components (a NaN ratio makes it
        // NaN, as in the bundle forward)
        dword rmax(0.0f, 0.0f);
        bool nanr = false;
        if (attempt) {
#pragma unroll
            for (int e = 0; e < 4; e++) {
                dacc acc{0.0f, 0.0f};
#pragma unroll
                for (int j = 0; j < NS; j++)
                    if (Tab::e(j) != 0.0)
                        dacc_fma_k(acc, Tab::e(j), K[j][e]);
                dacc_fma_k(acc, Tab::E_NEW, kn[e]);
                const dword tol = datol + drtol * (dabs(ys[e]) + dabs(sdt) * dabs(K[0][e]));
                const dword ratio = dabs(dacc_get(acc) * sdt) / tol;
                if (ratio.hi != ratio.hi)
                    nanr = true;
                else if (dw_greater(ratio, rmax))
                    rmax = ratio;
            }
        }
#pragma unroll
        for (int o = 8; o > 0; o >>= 1) {
            const dword other(__shfl_xor_sync(0xffffffffu, rmax.hi, o), __shfl_xor_sync(0xffffffffu, rmax.lo, o));
            if (dw_greater(other, rmax))
                rmax = other;
        }
        nanr = ((__ballot_sync(0xffffffffu, nanr) >> (lane & 16)) & 0xffffu) != 0;
        if (c.jg == 0) {
            // (a NaN stays NaN through the conversion)
            const double ep = nanr ? __longlong_as_double(0x7ff8000000000000ll) : to_d(rmax);
#pragma unroll
            for (int k = 0; k < 4; k++)
                dsmem_st_f64(dsmem_addr(sErr + c.q * 32 + c.bl, (uint32_t)(c.mt * 4 + k)), ep);
        }
        cluster_sync_all();
        // the controller (odeint's try_step), warp 0
        if (ctl) {
            int md = S.mode[lane];
            if (md & kFwdAttempt) {
                double err = 0.0;
                bool nan = false;
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const double x = sErr[32 * k + lane];
                    nan = nan || x != x;
                    err = fmax(err, x);
                }
                double t = S.t[lane], dt = S.dt[lane];
                int status = S.status[lane];
                if (nan) {
                    status = ST_NONFINITE;
                    md |= kFwdAtTop;
                } else {
                    bool ok;
                    if (err > 1.0) {
                        dt = decrease_step<Tab, dword>(dt, err, a.step_pow, nullptr);
                        S.rej[lane]++;
                        ok = false;
                    } else {
                        t = t + dt;
                        dt = increase_step<Tab, dword>(dt, err, a.step_pow, nullptr);
                        md |= kFwdAccepted;
                        ok = true;
                    }
                    if (S.fails[lane] >= a.max_fail) {
                        status = ST_MAX_REJECTS;
                        md |= kFwdAtTop;
                    } else {
                        S.fails[lane]++;
                        if (ok) {
                            S.count[lane]++;
                            md |= kFwdAtTop;
                        } else if (!(dt > 0.0) || !isfinite(dt)) {
                            status = ST_NONFINITE;
                            md |= kFwdAtTop;
                        }
                    }
                }
                S.t[lane] = t;
                S.dt[lane] = dt;
                S.status[lane] = status;
            }
            S.mode[lane] = md & ~(kFwdAttempt | kFwdTopRecord | kFwdFinished);
        }
        __syncthreads();
        if (S.mode[c.bl] & kFwdAccepted) {
#pragma unroll
            for (int e = 0; e < 4; e++) {
                ys[e] = yn[e];
                K[0][e] = kn[e];
                z0[e] = zn[e];
            }
        }
        __syncthreads(); // warp 0 clears the flag at the next top of step
        if (ctl)
            S.mode[lane] &= ~kFwdAccepted;
    }
    // counters and status of the tile's instances: y(T)'s finiteness from the
    // four quarter CTAs
    cluster_sync_all();
    if (c.q == 0 && c.jg == 0 && inb) {
        int status = S.status[c.bl];
        if (bt_bad(c) && status == ST_OK)
            status = ST_NONFINITE;
        const int count = S.count[c.bl];
        a.inst_T[inst] = count;
        a.inst_last[inst] = status == ST_OK ? S.chunk[c.bl] : -1;
        a.inst_status[inst] = status;
        if (a.inst_t1)
            a.inst_t1[inst] = S.t1[c.bl];
        if (a.n_acc_out)
            a.n_acc_out[inst] = count;
        if (a.n_rej_out)
            a.n_rej_out[inst] = S.rej[c.bl];
        if (a.status_out)
            a.status_out[inst] = status;
    }
    cluster_sync_all(); // no CTA leaves while another reads its shared memory
    bt_end(c, p.error);
}

// Host side (va_bundle_tc.cu): whether the cluster sweeps can run for the
// tableau on this GPU (set up once, before any capture), and their launches:
// digit planes of A (forward) or A^T (backward) and r as double-words, then
// one cluster of 8 CTAs per tile of 64 instances.  When the tiles exceed
// the clusters the GPU holds at once by exactly one, the last tile's
// instances run instead in the double-word bundle sweeps (one instance per
// CTA) on the SMs the clusters leave idle, launched as a programmatic
// dependent of the cluster sweep (they start once its clusters are resident
// and complete after it).
bool bundle_tc_available(int tableau);
bool bundle_tc_forward_available(int tableau);
// tiles of B instances that the cluster sweeps run (the rest: the tail)
int bundle_tc_tiles(int B);
cudaError_t enqueue_bundle_tc_forward(const BundleParams &bp, const double *A, uint8_t *adig, int *aexp,
                                      double *rpk, unsigned *error, int tableau, cudaStream_t s);
cudaError_t enqueue_bundle_tc_backward(const BundleParams &bp, const double *A, uint8_t *adig, int *aexp,
                                       double *rpk, unsigned *error, int tableau, cudaStream_t s);
constexpr size_t kBtADigitBytes = 8 * kBtABytes;
constexpr size_t kBtAExpInts = 4 * kBtN;

} // namespace va
