// Bundle sweeps for generalized Lotka-Volterra with ONE interaction matrix A
// shared by the whole batch: x_i' = x_i (r_i + sum_j A_ij x_j), per-instance
// r and x0.  A CTA of N threads carries a bundle of up to NB instances in
// lockstep (each instance keeps its own t, dt and controller decisions);
// thread i owns state component i of every instance in the bundle.
//
// Per stage the bundle needs z = A x for each of its instances: thread i
// forms z_i as a dot product of row i of A (read through the transposed copy
// At so that consecutive threads read consecutive addresses; A and At stay
// resident in L2) with the stage vectors, which sit in shared memory and are
// read as broadcasts.  Sharing each A element across the NB instances of the
// bundle divides the L2 traffic by NB.  The backward sweep adds
// A^T (w . x) (read through A itself, again coalesced) and the outer
// products sum (w . x) x^T that make up dA: those accumulate, once per step,
// into a private N x N partial of the CTA in global memory, and a final
// kernel adds the partials in a fixed order -- no atomics on any result.
//
// Stage records (double-word sweeps, the default): the forward also stores,
// per accepted step, the stage points X_m and the products z_m = A X_m it
// formed, so the backward reads them instead of redoing the s matrix-vector
// products of the stage recompute -- a third of its arithmetic.  Record of
// a step: [t, dt (FP64), X_0 .. X_{s-1}, z_0 .. z_{s-1} (packed
// double-words, component i at offset i)], 24.6 KB per instance-step at
// N = 256; the sweeps with [t, dt, y] records and the recompute remain
// (stage records off, FP64 and FP32 modes).
//
// The arithmetic per component follows the reference's GLV functor
// (examples/GeneralizedLotkaVolterra/main.cpp:109-118: sum_j in ascending
// order, then x_i (r_i + sum)) and the same back_prop_step recurrence as the
// other sweeps, so the FP64 build reproduces the oracle's per-instance
// results bit for bit; dA, a sum over the batch, agrees to rounding.
#pragma once

#include "va_kernels.cuh"

namespace va {

// doubles per stage record of a bundle instance (padded to 32 bytes)
__host__ __device__ constexpr int bundle_stage_record_doubles(int nt, int s) { return (2 + 2 * s * nt + 3) & ~3; }

struct BundleParams {
    FwdParams f;          // batch, inputs (par = r[B][N]), tolerances, outputs, pool
    AdjParams g;          // seeds / gradient outputs (par = r)
    const double *A;      // [N][N] row-major (FP64 path)
    const double *At;     // [N][N] = A^T row-major
    const dword *Aw;      // double-word copies (double-word path)
    const dword *Atw;
    double *dA_part;      // [gridDim.x][N][N], transposed per CTA: [j][i] += dA_ij
    int nb;               // instances per CTA (<= NB)
    int inst0;            // the first CTA's first instance (a tail of the batch; 0: all of it)
    // deferred dA (double-word sweeps with stage records; null: the CTA
    // partials above): factor row k = k_base[b] + n nsv + m of step n, stage m
    // of instance b holds v = Kbar_m . X_m (packed double-words) and a pointer
    // to X_m in the step's stage record; the tensor-core contraction
    // (va_contract.cu) forms dA = sum_k v_k X_k^T from them
    double *fac_v;        // [K][N]
    const double **fac_xp;// [K]
    const int *k_base;    // [B + 1]
};

// stages whose factor row can be non-zero: all but a last stage of weight 0
// (the FSAL stage of Dormand-Prince, whose adjoint seed b_s h lambda is 0
// and which feeds no other stage)
template <class Tab>
__host__ __device__ constexpr int factor_stages()
{
    return Tab::S - (Tab::b(Tab::S - 1) == 0.0 ? 1 : 0);
}

// the value as a double-word (used where S is dword; other S never reach it)
template <class S>
__device__ __forceinline__ dword dword_of(S v)
{
    if constexpr (std::is_same<S, dword>::value)
        return v;
    else
        return dword(0.0f, 0.0f);
}

template <class S>
__device__ __forceinline__ S load_A(const double *A, const dword *Aw, size_t k)
{
    if constexpr (std::is_same<S, dword>::value)
        return Aw[k];
    else
        return (S)A[k];
}

// Block-wide maximum per instance of non-negative values (NaN propagates).
template <int NT, int NB>
__device__ __forceinline__ void bundle_max(double (&v)[NB], double *red /* [NT/32][NB] */)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int b = 0; b < NB; b++) {
        double x = v[b];
        bool nan = x != x;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            x = fmax(x, __shfl_xor_sync(0xffffffffu, x, o));
        nan = __any_sync(0xffffffffu, nan);
        if (lane == 0)
            red[warp * NB + b] = nan ? __longlong_as_double(0x7ff8000000000000ll) : x;
    }
    __syncthreads();
#pragma unroll
    for (int b = 0; b < NB; b++) {
        double m = 0.0;
        bool nan = false;
#pragma unroll
        for (int w = 0; w < NT / 32; w++) {
            const double x = red[w * NB + b];
            nan = nan || x != x;
            m = fmax(m, x);
        }
        v[b] = nan ? __longlong_as_double(0x7ff8000000000000ll) : m;
    }
    __syncthreads();
}

// z_b += sum_j M_ij xs[b][j], j ascending, for the NB vectors in shared
// memory (thread i).  Mt is the matrix read as Mt[j][i] (consecutive i are
// consecutive addresses).  One pass over the matrix serves all NB vectors.
// (Double-word path: the dot products run through the compensated
// accumulator dacc, ~12 FP32 operations per term.)  UNR: matrix rows in
// flight per thread (the loads come from L2; measured at N = 256 with
// bundles of 2: 16 rows suit both sweeps; 8 slowed the forward by 3%, 32
// by 12%).
template <int NT, int NB, class S, int UNR = 8>
__device__ __forceinline__ void bundle_matvec_acc(const double *Mt, const dword *Mtw,
                                                  const S *xs /* [NT][NB] */, S (&z)[NB])
{
    const int i = threadIdx.x;
    if constexpr (std::is_same<S, dword>::value) {
        dacc zc[NB];
#pragma unroll
        for (int b = 0; b < NB; b++)
            zc[b] = dacc_of(z[b]);
#pragma unroll UNR
        for (int j = 0; j < NT; j++) {
            const dword a = Mtw[(size_t)j * NT + i];
#pragma unroll
            for (int b = 0; b < NB; b++)
                dacc_fma(zc[b], a, xs[j * NB + b]);
        }
#pragma unroll
        for (int b = 0; b < NB; b++)
            z[b] = dacc_get(zc[b]);
    } else {
#pragma unroll 4
        for (int j = 0; j < NT; j++) {
            const S a = load_A<S>(Mt, Mtw, (size_t)j * NT + i);
#pragma unroll
            for (int b = 0; b < NB; b++)
                z[b] = madd(a, xs[j * NB + b], z[b]);
        }
    }
}

// cp.async of 8 bytes global -> shared (this thread's own element), and the
// waits on this thread's own groups of copies (no spin: the hardware wait)
__device__ __forceinline__ void cp_async8(void *dst, const void *src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
                 "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait()
{
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// The double-word matrix-vector products of bundle_matvec with the matrix
// rows streamed through a shared-memory ring of R rows (ring[R][NT]): thread
// i copies and then reads only column i, so R rows of lookahead cost no
// registers and need no barrier; groups of G rows per cp.async group.  The
// same operations in the same order as bundle_matvec_acc: the same bits.
constexpr int kRingRows = 16, kRingGroup = 4;
template <int NT, int NB>
__device__ __forceinline__ void bundle_matvec_dw_ring(const dword *Mtw, const dword *xs /* [NT][NB] */,
                                                      dword (&z)[NB], dword *ring /* [kRingRows][NT] */)
{
    constexpr int R = kRingRows, G = kRingGroup;
    static_assert(NT % G == 0 && R % G == 0 && R <= NT, "ring shape");
    const int i = threadIdx.x;
    dacc zc[NB];
#pragma unroll
    for (int b = 0; b < NB; b++)
        zc[b] = dacc{0.0f, 0.0f};
#pragma unroll
    for (int g = 0; g < R / G; g++) {
#pragma unroll
        for (int u = 0; u < G; u++)
            cp_async8(ring + (size_t)(g * G + u) * NT + i, Mtw + (size_t)(g * G + u) * NT + i);
        cp_async_commit();
    }
#pragma unroll 2
    for (int j0 = 0; j0 < NT; j0 += G) {
        cp_async_wait<R / G - 1>(); // rows j0 .. j0 + G - 1 have landed
#pragma unroll
        for (int u = 0; u < G; u++) {
            const int j = j0 + u;
            const dword a = ring[(size_t)(j % R) * NT + i];
#pragma unroll
            for (int b = 0; b < NB; b++)
                dacc_fma(zc[b], a, xs[j * NB + b]);
        }
        if (j0 + R < NT) {
#pragma unroll
            for (int u = 0; u < G; u++)
                cp_async8(ring + (size_t)((j0 + u) % R) * NT + i, Mtw + (size_t)(j0 + R + u) * NT + i);
        }
        cp_async_commit(); // (empty near the end: the group count stays uniform)
    }
    cp_async_wait<0>();
#pragma unroll
    for (int b = 0; b < NB; b++)
        z[b] = dacc_get(zc[b]);
}

// dynamic shared memory of forward_bundle_kernel<NT, NB, *, S>: the stage
// vectors xs[NT][NB], the reduction slots, the chunk slots and, for the
// double-word sweep, the matrix-row ring (16-byte aligned)
template <int NT, int NB, class S>
__host__ __device__ constexpr size_t bundle_fwd_smem_bytes()
{
    const size_t base = sizeof(S) * NT * NB + sizeof(double) * (NT / 32) * NB + sizeof(int) * NB;
    return std::is_same<S, dword>::value ? ((base + 15) & ~(size_t)15) + sizeof(dword) * kRingRows * NT : base;
}

template <int NT, int NB, class S, int UNR = 8>
__device__ __forceinline__ void bundle_matvec(const double *Mt, const dword *Mtw, const S *xs /* [NT][NB] */,
                                              S (&z)[NB])
{
#pragma unroll
    for (int b = 0; b < NB; b++)
        z[b] = S(0);
    bundle_matvec_acc<NT, NB, S, UNR>(Mt, Mtw, xs, z);
}

// ------------------------------------------------- per-instance arithmetic
// (shared by the forward, the backward's stage recompute and the two-level
// re-integration, so that all three form the same bits)

// stage point X_m = y + h sum_{j<m} a_mj K_j of instance b (thread i's
// component): FP64 in the oracle's order, else a stage-precision sum
template <class Tab, class S, int NB>
__device__ __forceinline__ S bundle_stage_point(int m, int b, double y, S ys, const S (&K)[Tab::S][NB], double h,
                                                S sh)
{
    constexpr int NS = Tab::S;
    if constexpr (std::is_same<S, double>::value) {
        double acc = y;
#pragma unroll
        for (int j = 0; j < NS - 1; j++)
            if (j < m)
                acc = acc + (Tab::a(m, j) * h) * K[j][b];
        return acc;
    } else {
        S acc = S(0);
#pragma unroll
        for (int j = 0; j < NS - 1; j++)
            if (j < m)
                acc = madd(S(Tab::a(m, j)), K[j][b], acc);
        return madd(acc, sh, ys);
    }
}

// y_new = y + dt sum_j b_j K_j of instance b: ynew_s in stage precision and
// ynew in FP64
template <class Tab, class S, int NB>
__device__ __forceinline__ void bundle_solution(int b, double y, S ys, const S (&K)[Tab::S][NB], double dt, S sdt,
                                                S &ynew_s, double &ynew)
{
    constexpr int NS = Tab::S;
    if constexpr (std::is_same<S, double>::value) {
        double acc = y;
#pragma unroll
        for (int j = 0; j < NS; j++)
            if (Tab::b(j) != 0.0)
                acc = acc + (Tab::b(j) * dt) * K[j][b];
        ynew = acc;
        ynew_s = acc;
    } else {
        S acc = S(0);
#pragma unroll
        for (int j = 0; j < NS; j++)
            if (Tab::b(j) != 0.0)
                acc = madd(S(Tab::b(j)), K[j][b], acc);
        ynew_s = madd(acc, sdt, ys);
        ynew = to_d(ynew_s);
    }
}

// thread i's ratio |e_i| / (atol + rtol (|y_i| + |dt| |k0_i|)) of instance b
template <class Tab, class S, int NB>
__device__ __forceinline__ double bundle_error_ratio(int b, double y, const S (&K)[Tab::S][NB], S knew, double dt,
                                                     double atol, double rtol)
{
    constexpr int NS = Tab::S;
    if constexpr (std::is_same<S, double>::value) {
        double acc = 0.0;
        bool first = true;
#pragma unroll
        for (int j = 0; j < NS; j++)
            if (Tab::e(j) != 0.0) {
                const double term = (Tab::e(j) * dt) * K[j][b];
                acc = first ? term : acc + term;
                first = false;
            }
        if constexpr (Tab::FSAL)
            acc = acc + (Tab::E_NEW * dt) * knew;
        return fabs(acc) / (atol + rtol * (1.0 * fabs(y) + fabs(dt) * fabs(K[0][b])));
    } else {
        S acc = S(0);
#pragma unroll
        for (int j = 0; j < NS; j++)
            if (Tab::e(j) != 0.0)
                acc = madd(S(Tab::e(j)), K[j][b], acc);
        if constexpr (Tab::FSAL)
            acc = madd(S(Tab::E_NEW), knew, acc);
        const double e = dt * to_d(acc);
        return fabs(e) / (atol + rtol * (1.0 * fabs(y) + fabs(dt) * fabs(to_d(K[0][b]))));
    }
}

// ------------------------------------------------------------ forward sweep

// bundles of two: two CTAs per SM (128 registers per thread); larger
// bundles: no minimum (0), the compiler's own register choice
template <int NT, int NB, class Tab, class S, bool STAGES = false>
__global__ void __launch_bounds__(NT, NB <= 2 ? 2 : 0) forward_bundle_kernel(BundleParams bp)
{
    constexpr int NS = Tab::S;
    constexpr bool ST = STAGES && std::is_same<S, dword>::value; // stage records
    constexpr int RS = ST ? bundle_stage_record_doubles(NT, NS) : record_doubles(NT);
    const FwdParams &a = bp.f;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    S *xs = reinterpret_cast<S *>(smem_raw);                               // [NT][NB]
    double *red = reinterpret_cast<double *>(smem_raw + sizeof(S) * NT * NB); // [NT/32][NB]
    int *ichunk = reinterpret_cast<int *>(red + (NT / 32) * NB);            // [NB]
    // double-word sweep: the ring that streams A's rows (bundle_matvec_dw_ring)
    dword *ring = reinterpret_cast<dword *>(
        smem_raw + ((sizeof(S) * NT * NB + sizeof(double) * (NT / 32) * NB + sizeof(int) * NB + 15) & ~(size_t)15));
    const int i = threadIdx.x;
    const int CH = a.pool.chunk_len;
    // z = A x for the bundle's vectors in xs
    auto matvec = [&](S (&z)[NB]) {
        if constexpr (std::is_same<S, dword>::value)
            bundle_matvec_dw_ring<NT, NB>(bp.Atw, xs, z, ring);
        else
            bundle_matvec<NT, NB, S, 16>(bp.At, bp.Atw, xs, z);
    };

    double y[NB], t[NB], t1[NB], dt[NB], t_start[NB];
    S ys[NB], r[NB], K[NS][NB], knew[NB];
    S z0[NB];           // ST: z_0 = A y of the current state
    double *rec_cur[NB]; // ST: the current step's record
    int count[NB], rej[NB], fails[NB], status[NB], chunk[NB], slot[NB], inst[NB];
    bool active[NB], at_top[NB];

    // instances of this CTA
#pragma unroll
    for (int b = 0; b < NB; b++) {
        inst[b] = bp.inst0 + blockIdx.x * bp.nb + b;
        active[b] = b < bp.nb && inst[b] < a.B;
        count[b] = rej[b] = fails[b] = 0;
        status[b] = ST_OK;
        at_top[b] = true;
        slot[b] = 0;
        chunk[b] = -1;
        y[b] = 0.0;
        t[b] = t1[b] = 0.0;
        dt[b] = a.dt0;
        ys[b] = S(0);
        r[b] = S(0);
        z0[b] = S(0);
        rec_cur[b] = nullptr;
        if (active[b]) {
            y[b] = a.y0[(size_t)inst[b] * NT + i];
            r[b] = from_d<S>(a.par[(size_t)inst[b] * NT + i]);
            ys[b] = from_d<S>(y[b]);
            t[b] = a.t0[inst[b]];
            t1[b] = a.t1[inst[b]];
            t_start[b] = t[b];
        }
    }
    if (i == 0) {
#pragma unroll
        for (int b = 0; b < NB; b++) {
            int c = -1;
            if (active[b]) {
                c = (int)atomicAdd(&a.ctl->pool_next, 1u);
                if (c >= a.pool.n_chunks) {
                    c = -1;
                    atomicOr(&a.ctl->pool_fail, 1u);
                } else {
                    a.pool.chunk_prev[c] = -1;
                }
            }
            ichunk[b] = c;
        }
    }
    // k_1 = f(y_0) for the bundle
#pragma unroll
    for (int b = 0; b < NB; b++)
        xs[i * NB + b] = ys[b];
    __syncthreads();
#pragma unroll
    for (int b = 0; b < NB; b++) {
        chunk[b] = ichunk[b];
        if (active[b] && chunk[b] < 0)
            status[b] = ST_CKPT_BUDGET;
    }
    {
        S z[NB];
        matvec(z);
#pragma unroll
        for (int b = 0; b < NB; b++) {
            K[0][b] = ys[b] * (r[b] + z[b]);
            z0[b] = z[b];
        }
    }
    __syncthreads();

    // whether instance b's loop has ended (fixed steps: while ((t + dt) - t1
    // <= eps), runge_kutta.hpp:54)
    auto ended = [&](int b) -> bool {
        return Tab::FIXED ? !((t[b] + dt[b]) - t1[b] <= kDblEps) : !(t1[b] - t[b] > kDblEps);
    };
    // whether the top of instance b's step stores a record: every step, or
    // every stride-th (two-level checkpointing) and the last
    auto stores = [&](int b) -> bool { return a.stride <= 1 || count[b] % a.stride == 0 || ended(b); };

    for (;;) {
        // top of step for every live instance: loop test, record, end clamp.
        // Chunk allocation needs one thread and a barrier, so it is done for
        // the whole bundle at once.
        bool need_chunk = false;
#pragma unroll
        for (int b = 0; b < NB; b++) {
            if (!active[b] || status[b] != ST_OK || !at_top[b])
                continue;
            if (ended(b)) {
                // finished: write the final record, like the single-thread sweep
                if (slot[b] == CH)
                    need_chunk = true;
                continue;
            }
            if (count[b] >= a.max_steps) {
                status[b] = ST_MAX_STEPS;
                continue;
            }
            if (slot[b] == CH && stores(b))
                need_chunk = true;
        }
        if (need_chunk) {
            if (i == 0) {
#pragma unroll
                for (int b = 0; b < NB; b++) {
                    int c = chunk[b];
                    if (active[b] && status[b] == ST_OK && at_top[b] && slot[b] == CH && stores(b)) {
                        c = (int)atomicAdd(&a.ctl->pool_next, 1u);
                        if (c >= a.pool.n_chunks) {
                            c = -1;
                            atomicOr(&a.ctl->pool_fail, 1u);
                        } else {
                            a.pool.chunk_prev[c] = chunk[b];
                        }
                    }
                    ichunk[b] = c;
                }
            }
            __syncthreads();
#pragma unroll
            for (int b = 0; b < NB; b++) {
                if (active[b] && status[b] == ST_OK && at_top[b] && slot[b] == CH && stores(b)) {
                    chunk[b] = ichunk[b];
                    slot[b] = 0;
                    if (chunk[b] < 0)
                        status[b] = ST_CKPT_BUDGET;
                }
            }
            __syncthreads();
        }
        bool any_attempt = false;
#pragma unroll
        for (int b = 0; b < NB; b++) {
            if (!active[b] || !at_top[b])
                continue;
            if (status[b] == ST_OK && stores(b)) {
                double *rec = record_ptr<RS>(a.pool, chunk[b], slot[b]);
                if (i == 0)
                    *reinterpret_cast<double2 *>(rec) = make_double2(t[b], dt[b]);
                if constexpr (ST) {
                    rec[2 + i] = dw_pack(ys[b]);
                    rec[2 + NS * NT + i] = dw_pack(z0[b]);
                    rec_cur[b] = rec;
                } else if (std::is_same<S, dword>::value && a.stride > 1) {
                    // two-level checkpoints of the double-word sweep: the
                    // exact double-word state, which a re-integration resumes
                    rec[2 + i] = dw_pack(dword_of(ys[b]));
                } else {
                    rec[2 + i] = y[b];
                }
                slot[b]++;
            }
            if (status[b] != ST_OK || ended(b)) {
                // instance done: outputs
                if (__syncthreads_or(isfinite(y[b]) ? 0 : 1) && status[b] == ST_OK)
                    status[b] = ST_NONFINITE;
                if (a.yT)
                    a.yT[(size_t)inst[b] * NT + i] = y[b];
                if (i == 0) {
                    a.inst_T[inst[b]] = count[b];
                    a.inst_last[inst[b]] = status[b] == ST_OK ? chunk[b] : -1;
                    a.inst_status[inst[b]] = status[b];
                    if (a.inst_t1)
                        a.inst_t1[inst[b]] = t1[b];
                    if (Tab::FIXED && a.inst_t0)
                        a.inst_t0[inst[b]] = t_start[b];
                    if (a.n_acc_out)
                        a.n_acc_out[inst[b]] = count[b];
                    if (a.n_rej_out)
                        a.n_rej_out[inst[b]] = rej[b];
                    if (a.status_out)
                        a.status_out[inst[b]] = status[b];
                }
                active[b] = false;
                continue;
            }
            if (!Tab::FIXED && (t[b] + dt[b]) - t1[b] > kDblEps)
                dt[b] = t1[b] - t[b];
            fails[b] = 0;
            at_top[b] = false;
        }
#pragma unroll
        for (int b = 0; b < NB; b++)
            any_attempt = any_attempt || active[b];
        if (!any_attempt)
            break;

        // one attempt for every live instance: stages 2..s
        S sdt[NB];
#pragma unroll
        for (int b = 0; b < NB; b++)
            sdt[b] = from_d<S>(dt[b]);
#pragma unroll
        for (int m = 1; m < NS; m++) {
#pragma unroll
            for (int b = 0; b < NB; b++)
                xs[i * NB + b] = bundle_stage_point<Tab, S, NB>(m, b, y[b], ys[b], K, dt[b], sdt[b]);
            __syncthreads();
            S z[NB];
            matvec(z);
#pragma unroll
            for (int b = 0; b < NB; b++) {
                const S X = xs[i * NB + b];
                K[m][b] = X * (r[b] + z[b]);
                if constexpr (ST) {
                    // every attempt rewrites the step's stage values: the
                    // accepted one is the last
                    if (active[b] && !at_top[b]) {
                        rec_cur[b][2 + m * NT + i] = dw_pack(X);
                        rec_cur[b][2 + (NS + m) * NT + i] = dw_pack(z[b]);
                    }
                }
            }
            __syncthreads();
        }
        // y_new, f(y_new), error estimate
        S ynew_s[NB];
        double ynew[NB];
#pragma unroll
        for (int b = 0; b < NB; b++) {
            bundle_solution<Tab, S, NB>(b, y[b], ys[b], K, dt[b], sdt[b], ynew_s[b], ynew[b]);
            xs[i * NB + b] = ynew_s[b];
        }
        S znew[NB];
        if constexpr (Tab::FSAL) {
            __syncthreads();
            matvec(znew);
#pragma unroll
            for (int b = 0; b < NB; b++)
                knew[b] = ynew_s[b] * (r[b] + znew[b]);
            __syncthreads();
        }
        double ratio[NB];
#pragma unroll
        for (int b = 0; b < NB; b++) {
            ratio[b] = bundle_error_ratio<Tab, S, NB>(b, y[b], K, knew[b], dt[b], a.atol, a.rtol);
            if (!active[b] || at_top[b] || Tab::FIXED)
                ratio[b] = 0.0; // (fixed steps: no error estimate, every attempt accepted)
        }
        bundle_max<NT, NB>(ratio, red);
        // controller, per instance (uniform across the CTA)
#pragma unroll
        for (int b = 0; b < NB; b++) {
            if (!active[b] || at_top[b])
                continue;
            const double err = ratio[b];
            bool ok;
            if (err != err) {
                status[b] = ST_NONFINITE;
                at_top[b] = true;
                continue;
            }
            if (err > 1.0) {
                dt[b] = decrease_step<Tab, S>(dt[b], err, a.step_pow, threadIdx.x == 0 ? &a.ctl->pow_undecided : nullptr);
                rej[b]++;
                ok = false;
            } else {
                t[b] = Tab::FIXED ? fixed_time(t_start[b], count[b] + 1, dt[b]) : t[b] + dt[b];
                dt[b] = increase_step<Tab, S>(dt[b], err, a.step_pow, threadIdx.x == 0 ? &a.ctl->pow_undecided : nullptr);
                y[b] = ynew[b];
                ys[b] = ynew_s[b];
                if constexpr (Tab::FSAL) {
                    K[0][b] = knew[b];
                    z0[b] = znew[b];
                }
                ok = true;
            }
            if (fails[b] >= a.max_fail) {
                status[b] = ST_MAX_REJECTS;
                at_top[b] = true;
                continue;
            }
            fails[b]++;
            if (ok) {
                count[b]++;
                at_top[b] = true;
            } else if (!(dt[b] > 0.0) || !isfinite(dt[b])) {
                status[b] = ST_NONFINITE;
                at_top[b] = true;
            }
        }
        if constexpr (!Tab::FSAL) {
            // non-FSAL pairs: k_1 = f(y) at the new state of accepted instances
#pragma unroll
            for (int b = 0; b < NB; b++)
                xs[i * NB + b] = ys[b];
            __syncthreads();
            S z[NB];
            matvec(z);
#pragma unroll
            for (int b = 0; b < NB; b++) {
                K[0][b] = ys[b] * (r[b] + z[b]);
                z0[b] = z[b];
            }
            __syncthreads();
        }
    }
    // launched as the programmatic dependent of a cluster sweep over the
    // batch's other instances: complete only after it (no-op otherwise)
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

// ----------------------------------------------------------- backward sweep

// One back_prop_step (detail/backpropagation.hpp:160-229) for the bundle's
// instances with step[b]: from the stage record srec[b] (ST) or the state
// y[b] (the stages recomputed), with step h[b]; lambda and mu updated, the
// matrix gradient either written as factor rows (ST with bp.fac_v) or added
// into the CTA's partial part.  j[b] is the step index (factor rows).
template <int NT, int NB, class Tab, class S, bool ST>
__device__ __forceinline__ void bundle_back_step(const BundleParams &bp, S *xall, S *vall, S *zall,
                                                 const bool (&step)[NB], const double (&y)[NB],
                                                 const double (&h)[NB], const S (&ys)[NB], const S (&sh)[NB],
                                                 const double *const (&srec)[NB], const S (&r)[NB],
                                                 const int (&inst)[NB], const int (&j)[NB], double *part,
                                                 double (&lam)[NB], double (&mu)[NB])
{
    constexpr int NS = Tab::S;
    const int i = threadIdx.x;
    if constexpr (ST) {
        // the forward's stage points and products A X_m
#pragma unroll
        for (int m = 0; m < NS; m++)
#pragma unroll
            for (int b = 0; b < NB; b++) {
                S X = S(0), z = S(0);
                if (step[b]) {
                    X = dw_unpack(__ldcs(srec[b] + 2 + m * NT + i));
                    z = dw_unpack(__ldcs(srec[b] + 2 + (NS + m) * NT + i));
                }
                xall[((size_t)m * NT + i) * NB + b] = X;
                zall[((size_t)m * NT + i) * NB + b] = z;
            }
        __syncthreads();
    }
    // recompute the stages (compute_intermediate_states)
    S K[NS][NB];
#pragma unroll
    for (int m = 0; m < NS && !ST; m++) {
#pragma unroll
        for (int b = 0; b < NB; b++)
            xall[((size_t)m * NT + i) * NB + b] = bundle_stage_point<Tab, S, NB>(m, b, y[b], ys[b], K, h[b], sh[b]);
        __syncthreads();
        S z[NB];
        bundle_matvec<NT, NB, S>(bp.At, bp.Atw, xall + (size_t)m * NT * NB, z);
#pragma unroll
        for (int b = 0; b < NB; b++) {
            zall[((size_t)m * NT + i) * NB + b] = z[b];
            K[m][b] = xall[((size_t)m * NT + i) * NB + b] * (r[b] + z[b]);
        }
    }
    // seeds and the stage loop s..1 (back_prop_step)
    S Kbar[NS][NB];
    double ybar[NB];
    S gsum[NB], vsum[NB];
#pragma unroll
    for (int b = 0; b < NB; b++) {
        ybar[b] = lam[b];
#pragma unroll
        for (int m = 0; m < NS; m++) {
            if constexpr (std::is_same<S, double>::value)
                Kbar[m][b] = (Tab::b(m) * h[b]) * lam[b];
            else
                Kbar[m][b] = (S(Tab::b(m)) * sh[b]) * from_d<S>(lam[b]);
        }
    }
#pragma unroll
    for (int m = NS - 1; m >= 0; m--) {
#pragma unroll
        for (int b = 0; b < NB; b++) {
            const S x = xall[((size_t)m * NT + i) * NB + b];
            vall[((size_t)m * NT + i) * NB + b] = step[b] ? Kbar[m][b] * x : S(0);
        }
        __syncthreads();
        // g = w (r + z), then += A_ji v_j for j ascending (the oracle's
        // order); A[j][i] is read row-major, coalesced across threads
        S g_all[NB];
#pragma unroll
        for (int b = 0; b < NB; b++)
            g_all[b] = Kbar[m][b] * (r[b] + zall[((size_t)m * NT + i) * NB + b]);
        bundle_matvec_acc<NT, NB, S, 16>(bp.A, bp.Aw, vall + (size_t)m * NT * NB, g_all);
#pragma unroll
        for (int b = 0; b < NB; b++) {
            if (!step[b])
                continue;
            const S v = vall[((size_t)m * NT + i) * NB + b];
            const S g = g_all[b];
            if constexpr (std::is_same<S, double>::value) {
                ybar[b] += g;
                mu[b] += v;
            } else {
                gsum[b] = (m == NS - 1) ? g : gsum[b] + g;
                vsum[b] = (m == NS - 1) ? v : vsum[b] + v;
            }
#pragma unroll
            for (int k = 0; k < NS - 1; k++)
                if (k < m) {
                    if constexpr (std::is_same<S, double>::value)
                        Kbar[k][b] += g * Tab::a(m, k) * h[b];
                    else
                        Kbar[k][b] = madd(g * S(Tab::a(m, k)), sh[b], Kbar[k][b]);
                }
        }
        __syncthreads();
    }
    if constexpr (ST) {
        if (bp.fac_v) {
            // deferred dA: this step's factor rows v_m (and pointers to X_m)
            constexpr int NSV = factor_stages<Tab>();
#pragma unroll
            for (int b = 0; b < NB; b++) {
                if (!step[b])
                    continue;
                const size_t k0 = (size_t)bp.k_base[inst[b]] + (size_t)j[b] * NSV;
#pragma unroll
                for (int m = 0; m < NSV; m++) {
                    bp.fac_v[(k0 + m) * NT + i] = dw_pack(vall[((size_t)m * NT + i) * NB + b]);
                    if (i == 0)
                        bp.fac_xp[k0 + m] = srec[b] + 2 + (size_t)m * NT;
                }
            }
        }
    }
    // dA partial: part[jj][i] += sum_{m,b} v_{m,b,i} x_{m,b,jj}
    if (!(ST && bp.fac_v)) {
        S vi[NS][NB];
#pragma unroll
        for (int m = 0; m < NS; m++)
#pragma unroll
            for (int b = 0; b < NB; b++)
                vi[m][b] = vall[((size_t)m * NT + i) * NB + b];
        if constexpr (std::is_same<S, dword>::value) {
            // the partial stays a double-word (packed in the 8-byte
            // slot): accumulating it in FP64 cost four FP64-pipe
            // operations per element and step.  Eight rows per
            // iteration keep eight partial loads in flight (the
            // partials of all CTAs exceed L2: DRAM latency)
#pragma unroll 8
            for (int jj = 0; jj < NT; jj++) {
                dacc acc{0.0f, 0.0f};
#pragma unroll
                for (int m = NS - 1; m >= 0; m--)
#pragma unroll
                    for (int b = 0; b < NB; b++)
                        dacc_fma(acc, vi[m][b], xall[((size_t)m * NT + jj) * NB + b]);
                double &pe = part[(size_t)jj * NT + i];
                pe = dw_pack(dw_unpack(pe) + dacc_get(acc));
            }
        } else {
            for (int jj = 0; jj < NT; jj++) {
                S acc = S(0);
#pragma unroll
                for (int m = NS - 1; m >= 0; m--)
#pragma unroll
                    for (int b = 0; b < NB; b++)
                        acc = madd(vi[m][b], xall[((size_t)m * NT + jj) * NB + b], acc);
                part[(size_t)jj * NT + i] += to_d(acc);
            }
        }
    }
#pragma unroll
    for (int b = 0; b < NB; b++) {
        if (!step[b])
            continue;
        if constexpr (std::is_same<S, double>::value) {
            lam[b] = ybar[b];
        } else {
            lam[b] += to_d(gsum[b]);
            mu[b] += to_d(vsum[b]);
        }
    }
}


// bundles of two: two CTAs per SM (128 registers per thread); larger
// bundles: no minimum (0), the compiler's own register choice
template <int NT, int NB, class Tab, class S, bool STAGES = false>
__global__ void __launch_bounds__(NT, NB <= 2 ? 2 : 0) backward_bundle_kernel(BundleParams bp)
{
    constexpr int NS = Tab::S;
    constexpr bool ST = STAGES && std::is_same<S, dword>::value; // stage records
    constexpr int RS = ST ? bundle_stage_record_doubles(NT, NS) : record_doubles(NT);
    const AdjParams &a = bp.g;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    S *xall = reinterpret_cast<S *>(smem_raw);      // [NS][NT][NB] stage points
    S *vall = xall + (size_t)NS * NT * NB;          // [NS][NT][NB] w . x per stage
    S *zall = vall + (size_t)NS * NT * NB;          // [NS][NT][NB] A x per stage
    const int i = threadIdx.x;
    const int CH = a.pool.chunk_len;

    int inst[NB], T[NB], j[NB], chunk[NB], slot[NB];
    bool live[NB];
    double lam[NB], mu[NB], t_next[NB];
    S r[NB];
#pragma unroll
    for (int b = 0; b < NB; b++) {
        inst[b] = bp.inst0 + blockIdx.x * bp.nb + b;
        live[b] = b < bp.nb && inst[b] < a.B;
        T[b] = 0;
        j[b] = -1;
        chunk[b] = -1;
        slot[b] = 0;
        lam[b] = 0.0;
        mu[b] = 0.0;
        t_next[b] = 0.0;
        r[b] = S(0);
        if (!live[b])
            continue;
        if (a.inst_status[inst[b]] != ST_OK) {
            const double nan = __longlong_as_double(0x7ff8000000000000ll);
            a.dy0[(size_t)inst[b] * NT + i] = nan;
            a.dpar[(size_t)inst[b] * NT + i] = nan;
            if (a.status_out && i == 0)
                a.status_out[inst[b]] = a.inst_status[inst[b]];
            live[b] = false;
            continue;
        }
        r[b] = from_d<S>(a.par[(size_t)inst[b] * NT + i]);
        T[b] = a.inst_T[inst[b]];
        chunk[b] = a.inst_last[inst[b]];
        slot[b] = T[b] % CH;
        const double *rec = record_ptr<RS>(a.pool, chunk[b], slot[b]);
        t_next[b] = rec[0];
        const double yT = ST ? to_d(dw_unpack(rec[2 + i])) : rec[2 + i];
        lam[b] = a.cost == 0 ? 2.0 * yT : a.cost == 1 ? 1.0 : a.lambdaT[(size_t)inst[b] * NT + i];
        j[b] = T[b] - 1;
        if (j[b] < 0) {
            // no accepted step (t0 = t1): the seeds are the result
            a.dy0[(size_t)inst[b] * NT + i] = lam[b];
            const double d = a.mu_direct ? a.mu_direct[(size_t)inst[b] * NT + i] : 0.0;
            a.dpar[(size_t)inst[b] * NT + i] = d;
            if (a.status_out && i == 0)
                a.status_out[inst[b]] = ST_OK;
        }
    }
    // this CTA's partial of dA, transposed: part[jj][i] += dA_i,jj
    double *part = bp.dA_part + (size_t)blockIdx.x * NT * NT;
    if (!(ST && bp.fac_v))
        for (int jj = 0; jj < NT; jj++)
            part[(size_t)jj * NT + i] = 0.0;

    for (;;) {
        bool any = false;
#pragma unroll
        for (int b = 0; b < NB; b++)
            any = any || (live[b] && j[b] >= 0);
        if (!any)
            break;
        bool step[NB];
        double y[NB], h[NB], tn[NB];
        S ys[NB], sh[NB];
        const double *srec[NB]; // ST: the step's stage record
#pragma unroll
        for (int b = 0; b < NB; b++) {
            step[b] = live[b] && j[b] >= 0;
            y[b] = 0.0;
            h[b] = 0.0;
            tn[b] = 0.0;
            if (step[b]) {
                if (slot[b] == 0) {
                    chunk[b] = a.pool.chunk_prev[chunk[b]];
                    slot[b] = CH - 1;
                } else {
                    slot[b]--;
                }
                const double *rec = record_ptr<RS>(a.pool, chunk[b], slot[b]);
                srec[b] = rec;
                tn[b] = rec[0];
                if constexpr (!ST)
                    y[b] = rec[2 + i];
                h[b] = t_next[b] - tn[b];
            }
            ys[b] = from_d<S>(y[b]);
            sh[b] = from_d<S>(h[b]);
        }
        bundle_back_step<NT, NB, Tab, S, ST>(bp, xall, vall, zall, step, y, h, ys, sh, srec, r, inst, j, part, lam,
                                             mu);
#pragma unroll
        for (int b = 0; b < NB; b++) {
            if (!step[b])
                continue;
            t_next[b] = tn[b];
            j[b]--;
            if (j[b] < 0) {
                a.dy0[(size_t)inst[b] * NT + i] = lam[b];
                const double d = a.mu_direct ? a.mu_direct[(size_t)inst[b] * NT + i] : 0.0;
                a.dpar[(size_t)inst[b] * NT + i] = d + mu[b];
                const bool finite = isfinite(lam[b]) && isfinite(mu[b]);
                const int all_finite = __syncthreads_and(finite ? 1 : 0);
                if (a.status_out && i == 0)
                    a.status_out[inst[b]] = all_finite ? ST_OK : ST_NONFINITE;
            }
        }
        __syncthreads();
    }
    // launched as the programmatic dependent of a cluster sweep over the
    // batch's other instances: complete only after it (no-op otherwise)
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

// dA = sum over CTAs of the transposed partials, in CTA order (FP64 sum of
// the partials; dw: the partials are packed double-words).
template <int NT>
__global__ void reduce_dA_kernel(const double *part, int nparts, int dw, double *dA)
{
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; // k = jj * NT + i
    if (k >= (size_t)NT * NT)
        return;
    double s = 0.0;
    for (int c = 0; c < nparts; c++) {
        const double v = part[(size_t)c * NT * NT + k];
        s += dw ? to_d(dw_unpack(v)) : v; // double-word sweeps keep packed partials
    }
    const size_t jj = k / NT, i = k % NT;
    dA[i * NT + jj] = s;
}

// A^T and the double-word copies of A and A^T.
template <int NT>
__global__ void prepare_A_kernel(const double *A, double *At, dword *Aw, dword *Atw)
{
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= (size_t)NT * NT)
        return;
    const size_t row = k / NT, col = k % NT;
    const double v = A[k];
    At[col * NT + row] = v;
    Aw[k] = dword(v);
    Atw[col * NT + row] = dword(v);
}

} // namespace va
