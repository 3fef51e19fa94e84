// Double-word lane-group sweeps of the generalized Lotka-Volterra model with
// a per-instance interaction matrix: a group of NN lanes carries one
// instance, lane i owning x_i, r_i, row i and column i of A (the layout of
// va_group.cuh), with the design of the one-thread double-word sweeps
// (va_kernels_dw.cuh): state, stages, step size, controller, error norm,
// lambda, mu and the checkpoint records in double-word, FP64 only for t.
//
// Control decisions stay uniform within the group: the error norm is the
// group maximum of the per-lane double-word ratios (odeint's max norm over
// components), compared exactly, and every lane runs the controller on the
// same values.  Records are stage records, lane i writing its components:
//   [t_n, dt_n, y_n[0..NN), X_1[0..NN), ..., X_{s-1}[0..NN),
//    s_0[0..NN), ..., s_{s-1}[0..NN)]
// with s_m = r + A X_m the rates of the stage points, so the backward step
// reads X_m and s_m instead of recomputing them (the rates were a quarter
// of the backward's time at N = 10), and fuses each stage's VJP with the mu
// accumulation (dr_i += w_i x_i, dA_ij += w_i x_i x_j) through compensated
// accumulators.
#pragma once

#include "va_group.cuh"
#include "va_kernels_dw.cuh"

namespace va {

// doubles per lane-group stage record: t, dt, X_0 .. X_{s-1}, s_0 .. s_{s-1}
// (NN each), padded to 32 bytes
__host__ __device__ constexpr int group_stage_record_doubles(int nn, int s) { return (2 + 2 * nn * s + 3) & ~3; }

// Group maximum of non-negative double-word ratios, NaN if any lane's is.
template <int G>
__device__ __forceinline__ dword group_max_dw(dword v, unsigned mask)
{
    const bool nan = v.hi != v.hi;
    const int base = (threadIdx.x & 31) / G * G;
    dword m(0.0f, 0.0f);
#pragma unroll
    for (int j = 0; j < G; j++) {
        const dword o = shfl(v, base + j, mask);
        if (dw_greater(o, m))
            m = o;
    }
    return __any_sync(mask, nan) ? dw_nan() : m;
}

// f_i = x_i (r_i + sum_j A_ij x_j) and its VJP, per lane (p as
// ModelGLVLane::load_params: r_i, row i of A, column i of A).
template <int NN>
struct GLVLaneDw {
    static constexpr int P = 1 + 2 * NN, PG = 1 + NN;

    // f_i, and the rate rate = r_i + sum_j A_ij x_j with f_i = x_i rate
    __device__ __forceinline__ static dword rhs(dword x, const dword (&p)[P], int base, unsigned mask,
                                                dword &rate)
    {
        dacc s = dacc_of(p[0]);
#pragma unroll
        for (int j = 0; j < NN; j++)
            dacc_fma(s, p[1 + j], shfl(x, base + j, mask));
        rate = dacc_get(s);
        return x * rate;
    }
    __device__ __forceinline__ static dword rhs(dword x, const dword (&p)[P], int base, unsigned mask)
    {
        dword rate;
        return rhs(x, p, base, mask, rate);
    }

    // (J^T w)_i = w_i (r_i + sum_j A_ij x_j) + sum_k A_ki w_k x_k, returned;
    // the parameter adjoint (dr_i, dA_i.) += (v_i, v_i x_.) with v = w x,
    // added into dm
    // (the rate of x, r_i + sum_j A_ij x_j, comes from the stage record)
    __device__ __forceinline__ static dword vjp_acc(dword w, dword x, dword rate, const dword (&p)[P], int base,
                                                    unsigned mask, dacc (&dm)[PG])
    {
        const dword v = w * x;
#pragma unroll
        for (int j = 0; j < NN; j++)
            dacc_fma(dm[1 + j], v, shfl(x, base + j, mask));
        dacc_add(dm[0], v);
        dacc g = dacc_mul(w, rate);
#pragma unroll
        for (int k = 0; k < NN; k++)
            dacc_fma(g, p[1 + NN + k], shfl(v, base + k, mask));
        return dacc_get(g);
    }
};

// One attempt on lane i's component (the group runs it in lockstep):
// y_new, k_new (and its rate) and this lane's error ratio; xrec (may be
// null) receives X_m at xrec + (m - 1) NN and its rate s_m at
// xrec + (s + m - 1) NN, m = 1 .. s-1.
template <int NN, class Tab>
__device__ __forceinline__ dword attempt_glv_dw(dword y, dword k0, const dword (&p)[GLVLaneDw<NN>::P], dword dt,
                                                const DwTol &tol, int base, unsigned mask, dword &ynew,
                                                dword &knew, dword &rate_new, double *xrec)
{
    constexpr int NS = Tab::S;
    using L = GLVLaneDw<NN>;
    dword K[NS][1];
    const dword ys[1] = {y};
    K[0][0] = k0;
#pragma unroll
    for (int m = 1; m < NS; m++) {
        dword X[1];
        stage_dw<Tab, 1>(m, ys, K, dt, X);
        dword rate;
        K[m][0] = L::rhs(X[0], p, base, mask, rate);
        if (xrec) {
            xrec[(m - 1) * NN] = dw_pack(X[0]);
            xrec[(NS + m - 1) * NN] = dw_pack(rate);
        }
    }
    ynew = axpy_dw(y, dt, wsum_dw<NS>(typename BWeights::template of<Tab>(), K, 0));
    if constexpr (Tab::FIXED)
        return dword(0.0f, 0.0f); // no error estimate: every attempt is accepted
    if constexpr (Tab::FSAL)
        knew = L::rhs(ynew, p, base, mask, rate_new);
    dacc e = wsum_dw<NS>(typename EWeights::template of<Tab>(), K, 0);
    if constexpr (Tab::FSAL)
        dacc_fma_k(e, Tab::E_NEW, knew);
    const dword adt = dabs(dt);
    const dword num = dabs(dacc_get(e) * adt);
    dacc d = dacc_of(tol.atol);
    dacc_fma(d, tol.rtol, dabs(y));
    dacc_fma(d, tol.rtol * adt, dabs(k0));
    return num / dacc_get(d);
}

template <int NN, class Tab>
__global__ void __launch_bounds__(256) forward_group_dw_kernel(FwdParams a)
{
    using M = ModelGLVLane<NN>;
    using L = GLVLaneDw<NN>;
    constexpr int G = NN, PT = M::PTOT, P = L::P;
    constexpr int RS = group_stage_record_doubles(NN, Tab::S);
    const LaneGroup<G> grp;
    if (!grp.active())
        return;
    const int li = grp.index, src = grp.base;
    const unsigned mask = grp.mask;
    const int CH = a.pool.chunk_len;
    const DwTol tol{dword(a.atol), dword(a.rtol)};

    int b = -1;
    double t = 0.0, t1 = 0.0, t_start = 0.0;
    EndTests et{}; // the loop and end-clamp tests as integer comparisons
    dword y, k0, dt, p[P];
    dword rate0; // r_i + (A y)_i of the current state (stage record slot s_0)
    int count = 0, rej = 0, fails = 0, status = ST_OK, chunk = -1, slot = 0;
    bool at_top = true, to_end = false;
    double *xrec = nullptr;

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
        y = dword(a.y0[(size_t)b * NN + li]);
        M::template load_params<dword>(a.par + (size_t)b * PT, li, p);
        t = t_start = a.t0[b];
        t1 = a.t1[b];
        et = end_tests(t1);
        dt = dword(a.dt0);
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
        k0 = L::rhs(y, p, src, mask, rate0);
        return true;
    };

    auto reserve = [&]() -> bool {
        if (chunk < 0)
            return false;
        if (slot == CH) {
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

    // [t, dt, y] of the current step; the attempts add the stage values
    auto write = [&]() {
        double *r = record_ptr<RS>(a.pool, chunk, slot);
        if (li == 0)
            *reinterpret_cast<double2 *>(r) = make_double2(t, dw_pack(dt));
        r[2 + li] = dw_pack(y);
        xrec = r + 2 + NN + li;
        r[2 + Tab::S * NN + li] = dw_pack(rate0);
        slot++;
    };

    auto finish = [&]() {
        if (status == ST_OK) {
            if (reserve())
                write();
            else
                status = ST_CKPT_BUDGET;
            if (__any_sync(mask, !isfinite(y.hi)))
                status = ST_NONFINITE;
        }
        if (a.yT)
            a.yT[(size_t)b * NN + li] = to_d(y);
        if (li == 0) {
            a.inst_T[b] = count;
            a.inst_last[b] = chunk;
            a.inst_status[b] = status;
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
            if (Tab::FIXED ? !((t + a.dt0) - t1 <= kDblEps) : !end_loop(et, t, t1)) {
                finish();
                alive = fetch();
                continue;
            }
            if (count >= a.max_steps) {
                status = ST_MAX_STEPS;
                continue;
            }
            if (!reserve()) {
                status = ST_CKPT_BUDGET;
                continue;
            }
            write();
            to_end = !Tab::FIXED && end_clamp(et, t + to_d_int(dt), t1);
            if (to_end)
                dt = dword(t1 - t);
            fails = 0;
            at_top = false;
        }
        dword ynew, knew, rate_new;
        const dword err = group_max_dw<G>(attempt_glv_dw<NN, Tab>(y, k0, p, dt, tol, src, mask, ynew, knew, rate_new,
                                                                  xrec),
                                          mask);
        bool ok;
        if (err.hi != err.hi) {
            status = ST_NONFINITE;
            continue;
        }
        const bool reject = dw_greater(err, dword(1.0f, 0.0f));
        const dword dt_next = adjust_dw<Tab>(dt, err, reject); // groups of a warp may differ
        if (reject) {
            dt = dt_next;
            rej++;
            to_end = false;
            ok = false;
        } else {
            if constexpr (Tab::FIXED) {
                t = fixed_time(t_start, count + 1, a.dt0);
            } else {
                t = to_end ? t1 : t + to_d_int(dt);
                dt = dt_next;
            }
            y = ynew;
            if constexpr (Tab::FSAL) {
                k0 = knew;
                rate0 = rate_new;
            } else {
                k0 = L::rhs(y, p, src, mask, rate0);
            }
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
        } else if (!(dt.hi > 0.0f) || !isfinite(dt.hi)) {
            status = ST_NONFINITE;
        }
    }
}

template <int NN, class Tab>
__global__ void __launch_bounds__(256) backward_group_dw_kernel(AdjParams a)
{
    using M = ModelGLVLane<NN>;
    using L = GLVLaneDw<NN>;
    constexpr int G = NN, PT = M::PTOT, P = L::P, PG = L::PG, NS = Tab::S;
    constexpr int RS = group_stage_record_doubles(NN, NS);
    const LaneGroup<G> grp;
    if (!grp.active())
        return;
    const int li = grp.index, src = grp.base;
    const unsigned mask = grp.mask;
    const int CH = a.pool.chunk_len;

    int b = -1, q = 0, j = -1, chunk = -1, slot = 0, T = 0, last = -1;
    double t_next = 0.0;
    dword lam, p[P];
    dacc dm[PG];
    // this lane's part of record j (t, X_0 .. X_{s-1}, s_0 .. s_{s-1}),
    // loaded one step ahead
    double nt, nx[NS], ns[NS];

    auto step_back_load = [&]() {
        if (slot == 0) {
            chunk = a.pool.chunk_prev[chunk];
            slot = CH - 1;
        } else {
            slot--;
        }
        const double *r = record_ptr<RS>(a.pool, chunk, slot);
        nt = __ldcs(r);
#pragma unroll
        for (int m = 0; m < NS; m++) {
            nx[m] = __ldcs(r + 2 + m * NN + li);
            ns[m] = __ldcs(r + 2 + (NS + m) * NN + li);
        }
    };

    auto start_seed = [&]() {
        chunk = last;
        slot = T % CH;
        const double *r = record_ptr<RS>(a.pool, chunk, slot);
        t_next = r[0];
        const dword yT = dw_unpack(r[2 + li]);
        const size_t o = ((size_t)b * a.nout + q);
        lam = a.cost == 0 ? dword(2.0f * yT.hi, 2.0f * yT.lo)
            : a.cost == 1 ? dword(1.0f, 0.0f) : dword(a.lambdaT[o * NN + li]);
#pragma unroll
        for (int k = 0; k < PG; k++)
            dm[k] = dacc{0.0f, 0.0f};
        note_lambda_lane(a, b, q, T, NN, li, lam);
        j = T - 1;
        if (j >= 0)
            step_back_load();
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
                    a.dy0[o * NN + li] = nan;
                    for (int k = li; k < PT; k += G)
                        a.dpar[o * PT + k] = nan;
                }
                if (a.status_out && li == 0)
                    a.status_out[b] = st;
                continue;
            }
            M::template load_params<dword>(a.par + (size_t)b * PT, li, p);
            T = a.inst_T[b];
            last = a.inst_last[b];
            q = 0;
            start_seed();
            return true;
        }
    };

    auto finish_seed = [&]() {
        const size_t o = ((size_t)b * a.nout + q);
        const double l = to_d(lam);
        a.dy0[o * NN + li] = l;
        double g[PG];
#pragma unroll
        for (int k = 0; k < PG; k++)
            g[k] = to_d(dacc_get(dm[k]));
        M::store_grads(a.dpar + o * PT, a.mu_direct ? a.mu_direct + o * PT : nullptr, li, g);
        bool finite = isfinite(l);
#pragma unroll
        for (int k = 0; k < PG; k++)
            finite = finite && isfinite(g[k]);
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
        const double tn = nt;
        dword X[NS], rate[NS];
#pragma unroll
        for (int m = 0; m < NS; m++) {
            X[m] = dw_unpack(nx[m]);
            rate[m] = dw_unpack(ns[m]);
        }
        if (j > 0)
            step_back_load();
        // back_prop_step (backpropagation.hpp:160-229) on lane i's components
        const dword h = dword(t_next - tn);
        dacc Kb[NS];
#pragma unroll
        for (int m = 0; m < NS; m++) {
            if (Tab::b(m) != 0.0)
                Kb[m] = dacc_mul(dacc_get(dacc_mul_k(Tab::b(m), h)), lam);
            else
                Kb[m] = dacc{0.0f, 0.0f};
        }
        dacc dl = dacc_of(lam);
#pragma unroll
        for (int m = NS - 1; m >= 0; m--) {
            const dword gx = L::vjp_acc(dacc_get(Kb[m]), X[m], rate[m], p, src, mask, dm);
            dacc_add(dl, gx);
            if (m > 0) {
                const dword gh = gx * h;
#pragma unroll
                for (int k = 0; k < NS - 1; k++)
                    if (k < m && Tab::a(m, k) != 0.0)
                        dacc_fma_k(Kb[k], Tab::a(m, k), gh);
            }
        }
        lam = dacc_get(dl);
#pragma unroll
        for (int k = 0; k < PG; k++)
            dm[k] = dacc_of(dacc_get(dm[k]));
        note_lambda_lane(a, b, q, j, NN, li, lam);
        t_next = tn;
        j--;
    }
}

} // namespace va
