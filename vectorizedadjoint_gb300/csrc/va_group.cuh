// Lane-group sweeps: one instance is carried by a group of TPI lanes of a
// warp, lane i owning state component i (32 / TPI groups per warp; leftover
// lanes idle).  Used for models whose state and parameters do not fit one
// thread, e.g. generalized Lotka-Volterra with a per-instance N x N matrix.
// The group refills independently of the other groups of its warp.
//
// The step arithmetic is the single-thread code (attempt / back_step) run on
// each lane's own component with a per-lane model whose RHS and VJP exchange
// components inside the group with masked shuffles; the error norm is the
// group maximum of the per-component ratios (default_error_checker's max
// norm), so every control decision is uniform within the group.
#pragma once

#include "va_kernels.cuh"

namespace va {

template <int G>
struct LaneGroup {
    static constexpr int PER_WARP = 32 / G;
    int lane;     // lane in warp
    int index;    // lane in group (= state component)
    int base;     // first lane of the group
    unsigned mask;
    __device__ __forceinline__ LaneGroup()
    {
        lane = threadIdx.x & 31;
        const int g = lane / G;
        base = g * G;
        index = lane - base;
        mask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << base);
    }
    __device__ __forceinline__ bool active() const { return lane < PER_WARP * G; }
};

// Broadcast of lane `src` (absolute lane) within `mask`.
__device__ __forceinline__ double shfl(double v, int src, unsigned mask) { return __shfl_sync(mask, v, src); }
__device__ __forceinline__ float shfl(float v, int src, unsigned mask) { return __shfl_sync(mask, v, src); }
__device__ __forceinline__ int shfl(int v, int src, unsigned mask) { return __shfl_sync(mask, v, src); }
__device__ __forceinline__ dword shfl(dword v, int src, unsigned mask)
{
    return dword(__shfl_sync(mask, v.hi, src), __shfl_sync(mask, v.lo, src));
}

// Group maximum of non-negative ratios that propagates NaN (fmax would drop
// it): a gather of the G values, the same maximum on every lane.
template <int G>
__device__ __forceinline__ double group_max(double v, unsigned mask)
{
    const bool nan = v != v;
    const int base = (threadIdx.x & 31) / G * G;
    double m = 0.0;
#pragma unroll
    for (int j = 0; j < G; j++)
        m = fmax(m, __shfl_sync(mask, v, base + j));
    return __any_sync(mask, nan) ? __longlong_as_double(0x7ff8000000000000ll) : m;
}

// Generalized Lotka-Volterra x_i' = x_i (r_i + sum_j A_ij x_j) with a
// per-instance A (examples/GeneralizedLotkaVolterra/main.cpp:105-119,
// parameters r then A row-major: p[N(i+1)+j] = A_ij).  Lane i holds r_i, row
// i and column i of A; it accumulates dr_i and row i of dA.
template <int NN>
struct ModelGLVLane {
    static constexpr int TPI = NN, NTOT = NN, PTOT = NN + NN * NN;
    static constexpr int N = 1, P = 1 + 2 * NN, PG = 1 + NN;

    template <class S>
    __device__ __forceinline__ static void load_params(const double *par, int i, S (&p)[P])
    {
        p[0] = from_d<S>(par[i]);
#pragma unroll
        for (int j = 0; j < NN; j++) {
            p[1 + j] = from_d<S>(par[NN + i * NN + j]);
            p[1 + NN + j] = from_d<S>(par[NN + j * NN + i]);
        }
    }

    __device__ __forceinline__ static void store_grads(double *dpar, const double *mu_direct, int i,
                                                       const double (&g)[PG])
    {
        dpar[i] = (mu_direct ? mu_direct[i] : 0.0) + g[0];
#pragma unroll
        for (int j = 0; j < NN; j++) {
            const int k = NN + i * NN + j;
            dpar[k] = (mu_direct ? mu_direct[k] : 0.0) + g[1 + j];
        }
    }

    // f_i = x_i (r_i + sum_j A_ij x_j)
    template <class S>
    __device__ __forceinline__ static void rhs(const S *x, const S *p, S t, S *f)
    {
        (void)t;
        const LaneGroup<NN> G;
        S acc = S(0);
#pragma unroll
        for (int j = 0; j < NN; j++)
            acc = madd(p[1 + j], shfl(x[0], G.base + j, G.mask), acc);
        f[0] = x[0] * (p[0] + acc);
    }

    // gx_k = w_k s_k + sum_i A_ik w_i x_i ; gr_k = w_k x_k ; gA_kj = w_k x_k x_j
    template <class S>
    __device__ __forceinline__ static void vjp(const S *w, const S *x, const S *p, S t, S *gx, S *gp)
    {
        (void)t;
        const LaneGroup<NN> G;
        const S v = w[0] * x[0];
        S s = S(0);
#pragma unroll
        for (int j = 0; j < NN; j++) {
            const S xj = shfl(x[0], G.base + j, G.mask);
            s = madd(p[1 + j], xj, s);
            gp[1 + j] = v * xj;
        }
        S g = w[0] * (p[0] + s);
#pragma unroll
        for (int j = 0; j < NN; j++)
            g = madd(p[1 + NN + j], shfl(v, G.base + j, G.mask), g);
        gx[0] = g;
        gp[0] = v;
    }
};

// accept_state for a lane group (lane i's component): the state after an
// accepted attempt restarts, for double-word stages, from the FP64 value a
// checkpoint stores (so a two-level re-integration from that checkpoint runs
// the same bits), and f(y_new) is reused only when every lane's component
// round-trips; the decision is the group's, since f exchanges components.
template <class M, class Tab, class S>
__device__ __forceinline__ void accept_state_group(double (&y)[1], S (&ys)[1], S (&k0)[1], const double (&ynew)[1],
                                                   const S (&ynew_s)[1], const S (&knew)[1], const S (&p)[M::P],
                                                   double t, unsigned mask)
{
    bool same = true;
    if constexpr (std::is_same<S, dword>::value) {
        y[0] = to_d(ynew_s[0]);
        if ((y[0] - (double)ynew_s[0].hi) == (double)ynew_s[0].lo &&
            ynew_s[0].hi + ynew_s[0].lo == ynew_s[0].hi) {
            ys[0] = ynew_s[0];
        } else {
            ys[0] = from_d<S>(y[0]);
            same = false;
        }
        same = __all_sync(mask, same);
    } else {
        y[0] = ynew[0];
        ys[0] = ynew_s[0];
    }
    if (Tab::FSAL && same)
        k0[0] = knew[0];
    else
        M::template rhs<S>(ys, p, from_d<S>(t), k0);
}

// ------------------------------------------------------------ forward sweep

template <class M, class Tab, class S>
__global__ void __launch_bounds__(256) forward_group_kernel(FwdParams a)
{
    constexpr int G = M::TPI, NT = M::NTOT, PT = M::PTOT, P = M::P;
    constexpr int RS = record_doubles(NT);
    const LaneGroup<G> grp;
    if (!grp.active())
        return;
    const int li = grp.index, src = grp.base;
    const unsigned mask = grp.mask;
    const int CH = a.pool.chunk_len;

    int b = -1;
    double y[1], t = 0.0, t1 = 0.0, dt = 0.0, t_start = 0.0;
    S ys[1], k0[1], p[P];
    int count = 0, rej = 0, fails = 0, status = ST_OK, chunk = -1, slot = 0;
    bool at_top = true;

    auto alloc_chunk = [&]() -> int {
        int c = 0;
        if (li == 0)
            c = (int)atomicAdd(&a.ctl->pool_next, 1u);
        return shfl(c, src, mask);
    };

    auto fetch = [&]() -> bool {
        int nb = 0;
        if (li == 0)
            nb = (int)atomicAdd(&a.ctl->fwd_next, 1u);
        b = shfl(nb, src, mask);
        if (b >= a.B)
            return false;
        if (a.order)
            b = a.order[b];
        y[0] = a.y0[(size_t)b * NT + li];
        M::template load_params<S>(a.par + (size_t)b * PT, li, p);
        t = t_start = a.t0[b];
        t1 = a.t1[b];
        dt = a.dt0;
        count = rej = fails = 0;
        status = ST_OK;
        at_top = true;
        slot = 0;
        chunk = alloc_chunk();
        if (chunk >= a.pool.n_chunks) {
            status = ST_CKPT_BUDGET;
            chunk = -1;
            if (li == 0)
                atomicOr(&a.ctl->pool_fail, 1u);
        } else if (li == 0) {
            a.pool.chunk_prev[chunk] = -1;
        }
        ys[0] = from_d<S>(y[0]);
        M::template rhs<S>(ys, p, from_d<S>(t), k0);
        return true;
    };

    auto reserve = [&]() -> bool {
        if (chunk < 0)
            return false;
        if (count > 0 && slot == CH) {
            const int c = alloc_chunk();
            if (c >= a.pool.n_chunks) {
                if (li == 0)
                    atomicOr(&a.ctl->pool_fail, 1u);
                return false;
            }
            if (li == 0)
                a.pool.chunk_prev[c] = chunk;
            chunk = c;
            slot = 0;
        }
        return true;
    };

    auto write = [&]() {
        double *r = record_ptr<RS>(a.pool, chunk, slot);
        if (li == 0)
            *reinterpret_cast<double2 *>(r) = make_double2(t, dt);
        r[2 + li] = y[0];
        slot++;
    };

    auto finish = [&]() {
        if (status == ST_OK) {
            if (reserve())
                write();
            else
                status = ST_CKPT_BUDGET;
            if (__any_sync(mask, !isfinite(y[0])))
                status = ST_NONFINITE;
        }
        if (a.yT)
            a.yT[(size_t)b * NT + li] = y[0];
        if (li == 0) {
            a.inst_T[b] = count;
            a.inst_last[b] = chunk;
            a.inst_status[b] = status;
            if (a.inst_t1)
                a.inst_t1[b] = t1;
            if (Tab::FIXED && a.inst_t0)
                a.inst_t0[b] = t_start;
            note_work(a, b, count + rej);
            if (a.n_acc_out)
                a.n_acc_out[b] = count;
            if (a.n_rej_out)
                a.n_rej_out[b] = rej;
            if (a.status_out)
                a.status_out[b] = status;
        }
    };

    bool alive = fetch();
    while (alive) {
        if (status != ST_OK) {
            finish();
            alive = fetch();
            continue;
        }
        if (at_top) {
            if (Tab::FIXED ? !((t + dt) - t1 <= kDblEps) : !(t1 - t > kDblEps)) {
                finish();
                alive = fetch();
                continue;
            }
            if (count >= a.max_steps) {
                status = ST_MAX_STEPS;
                continue;
            }
            // every stride-th accepted step is checkpointed (stride <= 1: all)
            if (a.stride <= 1 || count % a.stride == 0) {
                if (!reserve()) {
                    status = ST_CKPT_BUDGET;
                    continue;
                }
                write();
            }
            if (!Tab::FIXED && (t + dt) - t1 > kDblEps)
                dt = t1 - t;
            fails = 0;
            at_top = false;
        }
        double ynew[1];
        S ynew_s[1], knew[1];
        const double err = group_max<G>(
            attempt<M, Tab, S>(y, ys, k0, p, t, dt, a.atol, a.rtol, ynew, ynew_s, knew), mask);
        bool ok;
        if (err != err) {
            status = ST_NONFINITE;
            continue;
        }
        if (err > 1.0) {
            dt = decrease_step<Tab, S>(dt, err, a.step_pow, li == 0 ? &a.ctl->pow_undecided : nullptr);
            rej++;
            ok = false;
        } else {
            if constexpr (Tab::FIXED) {
                t = fixed_time(t_start, count + 1, dt);
            } else {
                t += dt;
                dt = increase_step<Tab, S>(dt, err, a.step_pow, li == 0 ? &a.ctl->pow_undecided : nullptr);
            }
            accept_state_group<M, Tab, S>(y, ys, k0, ynew, ynew_s, knew, p, t, mask);
            ok = true;
        }
        if (fails >= a.max_fail) {
            status = ST_MAX_REJECTS;
            continue;
        }
        fails++;
        if (ok) {
            count++;
            at_top = true;
        } else if (!(dt > 0.0) || !isfinite(dt)) {
            status = ST_NONFINITE;
        }
    }
}

// ----------------------------------------------------------- backward sweep

template <class M, class Tab, class S>
__global__ void __launch_bounds__(256) backward_group_kernel(AdjParams a)
{
    constexpr int G = M::TPI, NT = M::NTOT, PT = M::PTOT, P = M::P, PG = M::PG;
    constexpr int RS = record_doubles(NT);
    const LaneGroup<G> grp;
    if (!grp.active())
        return;
    const int li = grp.index, src = grp.base;
    const unsigned mask = grp.mask;
    const int CH = a.pool.chunk_len;

    int b = -1, q = 0, j = -1, chunk = -1, slot = 0, T = 0, last = -1;
    double lam[1], mu[PG], t_next = 0.0;
    S p[P];

    auto start_seed = [&]() {
        chunk = last;
        slot = T % CH;
        const double *r = record_ptr<RS>(a.pool, chunk, slot);
        t_next = r[0];
        const double yT = r[2 + li];
        const size_t o = ((size_t)b * a.nout + q);
        lam[0] = a.cost == 0 ? 2.0 * yT : a.cost == 1 ? 1.0 : a.lambdaT[o * NT + li];
#pragma unroll
        for (int k = 0; k < PG; k++)
            mu[k] = 0.0;
        note_lambda_lane(a, b, q, T, NT, li, lam[0]);
        j = T - 1;
    };

    auto fetch = [&]() -> bool {
        for (;;) {
            int w = 0;
            if (li == 0)
                w = (int)atomicAdd(&a.ctl->adj_next, 1u);
            w = shfl(w, src, mask);
            if (w >= a.B)
                return false;
            b = a.order ? a.order[w] : w;
            const int st = a.inst_status[b];
            if (st != ST_OK) {
                const double nan = __longlong_as_double(0x7ff8000000000000ll);
                for (int qq = 0; qq < a.nout; qq++) {
                    const size_t o = ((size_t)b * a.nout + qq);
                    a.dy0[o * NT + li] = nan;
                    for (int k = li; k < PT; k += G)
                        a.dpar[o * PT + k] = nan;
                }
                if (a.status_out && li == 0)
                    a.status_out[b] = st;
                continue;
            }
            M::template load_params<S>(a.par + (size_t)b * PT, li, p);
            T = a.inst_T[b];
            last = a.inst_last[b];
            q = 0;
            start_seed();
            return true;
        }
    };

    auto finish_seed = [&]() {
        const size_t o = ((size_t)b * a.nout + q);
        a.dy0[o * NT + li] = lam[0];
        M::store_grads(a.dpar + o * PT, a.mu_direct ? a.mu_direct + o * PT : nullptr, li, mu);
        bool finite = isfinite(lam[0]);
#pragma unroll
        for (int k = 0; k < PG; k++)
            finite = finite && isfinite(mu[k]);
        const bool all_finite = __all_sync(mask, finite);
        if (a.status_out && li == 0 && (q == a.nout - 1 || !all_finite))
            a.status_out[b] = all_finite ? ST_OK : ST_NONFINITE;
    };

    bool alive = fetch();
    while (alive) {
        if (j < 0) {
            finish_seed();
            if (q + 1 < a.nout) {
                q++;
                start_seed();
            } else {
                alive = fetch();
            }
            continue;
        }
        if (slot == 0) {
            chunk = a.pool.chunk_prev[chunk];
            slot = CH - 1;
        } else {
            slot--;
        }
        const double *r = record_ptr<RS>(a.pool, chunk, slot);
        const double tn = r[0];
        double y[1] = {r[2 + li]};
        const double h = t_next - tn;
        back_step<M, Tab, S>(y, tn, h, p, lam, mu);
        note_lambda_lane(a, b, q, j, NT, li, lam[0]);
        t_next = tn;
        j--;
    }
}

} // namespace va
