// Backward sweep of the shared-matrix GLV (N = 256, double-word stages with
// stage records) with the stage products A^T v on the tensor cores.
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
//   in shared memory for the whole sweep; only the 56 KB of V digits change
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
constexpr size_t kBtSmem = kBtABytes + kBtVBytes + kBtPBytes + 1024;  // + exponents, flags, barrier
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

template <class Tab>
__global__ void __cluster_dims__(kBtCluster, 1, 1) __launch_bounds__(kBtThreads, 1)
    backward_bundle_tc_kernel(BundleTcParams p)
{
    constexpr int NS = Tab::S;
    constexpr int NSV = factor_stages<Tab>();
    constexpr int RS = bundle_stage_record_doubles(kBtN, NS);
    const AdjParams &a = p.bp.g;
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *sA = smem;
    uint8_t *sV = smem + kBtABytes;
    double *sR = reinterpret_cast<double *>(smem + kBtABytes + kBtVBytes);
    int *sEv = reinterpret_cast<int *>(smem + kBtABytes + kBtVBytes + kBtPBytes); // [64] exponents of v per column
    int *sBad = sEv + kBtTile;                                                     // [32] non-finite results
    int *sMaxT = sBad + 32;
    uint64_t *bar = reinterpret_cast<uint64_t *>(sMaxT + 2);
    uint32_t *slot_tmem = reinterpret_cast<uint32_t *>(bar + 1);

    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const uint32_t rank = cluster_rank();
    const int mt = (int)(rank >> 2), q = (int)(rank & 3);
    const uint32_t partner = (uint32_t)((1 - mt) * 4 + q);
    const int tile = blockIdx.x / kBtCluster;
    const int CH = a.pool.chunk_len;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot_tmem)),
                     "r"(kBtTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (t == 0) {
        mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        *sMaxT = 0;
    }
    // the A operand of this CTA's block, resident for the whole sweep
    {
        const uint4 *ga = reinterpret_cast<const uint4 *>(p.adig + (size_t)(mt * 4 + q) * kBtABytes);
        uint4 *sa = reinterpret_cast<uint4 *>(sA);
#pragma unroll 4
        for (int x = t; x < (int)(kBtABytes / 16); x += kBtThreads)
            sa[x] = __ldg(ga + x);
    }
    if (t < 32)
        sBad[t] = 0;
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *slot_tmem;

    // lockstep length of the tile: the longest instance (every CTA of the
    // cluster reads the same 64 counts and gets the same value)
    if (t < kBtTile) {
        const int inst = tile * kBtTile + t;
        int T = 0;
        if (inst < a.B && a.inst_status[inst] == ST_OK)
            T = a.inst_T[inst];
        atomicMax(sMaxT, T);
    }

    // this thread's instance (tile column b) and four components j0 .. j0 + 3
    const int bl = t >> 4, jg = t & 15;
    const int b = 32 * mt + bl;
    const int inst = tile * kBtTile + b;
    const int j0 = 64 * q + 4 * jg;
    const bool inb = inst < a.B;
    bool live = inb && a.inst_status[inst] == ST_OK;
    if (inb && !live) {
        const double nan = __longlong_as_double(0x7ff8000000000000ll);
#pragma unroll
        for (int e = 0; e < 4; e++) {
            a.dy0[(size_t)inst * kBtN + j0 + e] = nan;
            a.dpar[(size_t)inst * kBtN + j0 + e] = nan;
        }
        if (a.status_out && q == 0 && jg == 0)
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
            atomicOr(&sBad[bl], 1);
    };
    if (live && jstep < 0) { // no accepted step: the seeds are the result
        finish();
        live = false;
    }

    // fold-thread constants: tensor-memory lane quadrant and 16 columns
    const int fq = warp & 3, fc = 16 * (warp >> 2);
    const int frow = 32 * fq + lane;
    const int ea = p.aexp[q * kBtN + 128 * mt + frow];
    const uint32_t taddr = tmem + ((uint32_t)(32 * fq) << 16) + (uint32_t)fc;
    // where this thread's digits go: plane offset of (column b, components j0..j0+3)
    const uint32_t voff = (uint32_t)((jg >> 1) * kBtVKgroup + b * 16 + (jg & 1) * 8);
    const uint32_t v_remote = dsmem_addr(sV + voff, partner);
    const uint32_t ev_remote = dsmem_addr(sEv + b, partner);
    // where this thread reads its partials: rows j0 - 128 (q / 2) of column b in CTAs (q / 2, 0..3)
    // where this thread's fold results go: row frow of this CTA's row tile is
    // component j = 128 mt + frow, owned (for the instances of column half
    // fc / 32) by CTA (fc / 32, 2 mt + frow / 64), slot q of its partials
    const uint32_t fold_dst = dsmem_addr(sR + ((size_t)q * 32 + (fc & 31)) * 64 + (frow & 63),
                                         (uint32_t)((fc >> 5) * 4 + 2 * mt + (frow >> 6)));
    // the four partials of this thread's (j, b) in its own shared memory
    const double *p_mine = sR + (size_t)bl * 64 + 4 * jg;

    __syncthreads();
    const int maxT = *sMaxT;
    uint32_t phase = 0;
    bool ok = true; // the MMA waits so far
    // every CTA of the cluster has started before any distributed access
    cluster_sync_all();

    // the stage's product, folded into this CTA's partials
    auto product = [&]() {
        fence_proxy_async_all();
        cluster_sync_all(); // V digits and exponents of the whole tile are in place
        // one thread issues the MMAs and alone polls their barrier (threads
        // polling shared memory slow the tensor core's operand reads); the
        // others wait at the CTA barrier
        bool w = true;
        if (ok && t == 0) {
            tc_fence_after();
            bt_issue_mmas(sA, sV, tmem);
            umma_commit(bar);
            w = mbar_wait_bounded(bar, phase, p.error);
        }
        if (ok)
            phase ^= 1u;
        ok = __syncthreads_and(ok && w) != 0;
        tc_fence_after();
        // fold: S = R_0 + R_1 2^-8 + R_2 2^-16 + (R_3 2^-24 + .. + R_6 2^-48)
        // in units of group 0 (|R_g| < 2^24 integers): the tail is below 1 and
        // summed in FP32 (error < 2^-23, i.e. 2^-47 of the largest S), the head
        // with two 2Sums; then the power-of-two scaling 2^(eA + eV - 16)
#pragma unroll 1
        for (int half = 0; half < 2; half++) {
            const int c0 = fc + 8 * half;
            const uint32_t dst = fold_dst + (uint32_t)(8 * half * 64 * sizeof(double));
            if (ok) {
                float tail[8];
                {
                    float R[4][8];
                    tmem_ld8_groups<4>(taddr + (uint32_t)(8 * half), 3, R);
#pragma unroll
                    for (int c = 0; c < 8; c++)
                        tail[c] = fmaf(R[0][c], 0x1p-24f, fmaf(R[1][c], 0x1p-32f, fmaf(R[2][c], 0x1p-40f, R[3][c] * 0x1p-48f)));
                }
                float R[3][8];
                tmem_ld8_groups<3>(taddr + (uint32_t)(8 * half), 0, R);
#pragma unroll
                for (int c = 0; c < 8; c++) {
                    float s1, e1, s2, e2, hi, lo;
                    two_sum(R[0][c], R[1][c] * 0x1p-8f, s1, e1);
                    two_sum(s1, R[2][c] * 0x1p-16f, s2, e2);
                    two_sum(s2, (e1 + e2) + tail[c], hi, lo);
                    const int k = ea + sEv[c0 + c] - 16;
                    dsmem_st_f64(dst + (uint32_t)(c * 64 * sizeof(double)), dw_pack(dword(scale_pow2(hi, k), scale_pow2(lo, k))));
                }
            } else {
                const double nan = __longlong_as_double(0x7ff8000000000000ll);
#pragma unroll
                for (int c = 0; c < 8; c++)
                    dsmem_st_f64(dst + (uint32_t)(c * 64 * sizeof(double)), nan);
            }
        }
        tc_fence_before();
        cluster_sync_all(); // every CTA's partials delivered
    };
    // the four partials of this thread's (j, b): G = P_0 + P_1 + P_2 + P_3
    auto gather = [&](dword (&G)[4]) {
        double2 v[4][2];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const double2 *src = reinterpret_cast<const double2 *>(p_mine + (size_t)k * 32 * 64);
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
    };

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
            gather(G);
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
                gather(G);
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
                    if (q == 0 && jg == 0)
                        p.bp.fac_xp[k0] = srec + 2 + (size_t)m * kBtN;
                }
            } else {
#pragma unroll
                for (int e = 0; e < 4; e++)
                    v[e] = dword(0.0f, 0.0f);
            }
            // the column exponent over the quarter (the 16 threads of instance b)
            float mx = fmaxf(fmaxf(fabsf(v[0].hi), fabsf(v[1].hi)), fmaxf(fabsf(v[2].hi), fabsf(v[3].hi)));
#pragma unroll
            for (int o = 8; o > 0; o >>= 1)
                mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            const int ev = tc_bound_exponent(mx);
            const DigitScale sc = digit_scale(ev);
            // digit s of the four components, packed as 4 bf16 (8 bytes)
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
                *reinterpret_cast<uint2 *>(sV + (size_t)s * kBtVPlane + voff) = make_uint2(pk[s][0], pk[s][1]);
                dsmem_st_u32x2(v_remote + (uint32_t)(s * kBtVPlane), pk[s][0], pk[s][1]);
            }
            if (jg == 0) {
                sEv[b] = ev;
                dsmem_st_s32(ev_remote, ev);
            }
            product();
        }
    }
    // every partial has been read; then the instances' status from the four
    // quarters' flags (rank 4 mt + k holds quarter k of the same instances)
    cluster_sync_all();
    if (q == 0 && jg == 0 && inb && a.inst_status[inst] == ST_OK && a.status_out) {
        int bad = sBad[bl];
#pragma unroll
        for (int k = 1; k < 4; k++)
            bad |= dsmem_ld_s32(dsmem_addr(sBad + bl, (uint32_t)(mt * 4 + k)));
        a.status_out[inst] = bad ? ST_NONFINITE : ST_OK;
    }
    cluster_sync_all(); // no CTA leaves while another reads its shared memory
    if (!ok && t == 0) // once more (bounded) for MMAs still in flight before the memory is released
        (void)mbar_wait_bounded(bar, phase ^ 1u, p.error);
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kBtTmemCols) : "memory");
}

// Host side (va_bundle_tc.cu): whether the cluster sweep can run for the
// tableau on this GPU (set up once, before any capture), and its launch:
// digit planes of A^T, then one cluster of 8 CTAs per tile of 64 instances.
bool bundle_tc_available(int tableau);
cudaError_t enqueue_bundle_tc_backward(const BundleParams &bp, const double *A, uint8_t *adig, int *aexp,
                                       double *rpk, unsigned *error, int tableau, cudaStream_t s);
constexpr size_t kBtADigitBytes = 8 * kBtABytes;
constexpr size_t kBtAExpInts = 4 * kBtN;

} // namespace va
