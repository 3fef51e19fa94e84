// Two-level backward sweep of the lane-group models (checkpoint stride > 1):
// the scheme of backward_kernel_2level (va_kernels.cuh) carried by a group of
// G lanes per instance, lane i owning state component i.  The forward
// (forward_group_kernel) stores every stride-th accepted step's [t, dt, y]
// plus the last; for each segment, last first, the group re-runs the forward
// controller from the segment's checkpoint -- the same attempt, step-size and
// accept code as forward_group_kernel, so the same bits -- into the group's
// scratch of (stride + 1) records, checks that it lands exactly on the next
// checkpoint, and back-steps through the segment with back_step, as
// backward_group_kernel does over an every-step store.  FP64, float stages
// and double-word stages (S = dword: the records hold the state rounded to
// FP64, and the forward itself restarts from that value after every
// accepted step, accept_state_group).
#pragma once

#include "va_group.cuh"

namespace va {

// doubles of scratch per lane group at a stride (records of the group's state)
__host__ __device__ constexpr int group_scratch_doubles(int ntot, int stride)
{
    return (stride + 1) * record_doubles(ntot);
}

template <class M, class Tab, class S>
__global__ void __launch_bounds__(256) backward_group_kernel_2level(AdjParams a)
{
    constexpr int G = M::TPI, NT = M::NTOT, PT = M::PTOT, P = M::P, PG = M::PG;
    constexpr int RS = record_doubles(NT);
    const LaneGroup<G> grp;
    if (!grp.active())
        return;
    const int li = grp.index, src = grp.base;
    const unsigned mask = grp.mask;
    const int CH = a.pool.chunk_len, SK = a.stride;
    // this group's scratch: groups numbered across the grid
    const size_t gid =
        ((size_t)blockIdx.x * blockDim.x + threadIdx.x) / 32 * LaneGroup<G>::PER_WARP + grp.lane / G;
    double *scr = a.scratch + gid * (size_t)group_scratch_doubles(NT, SK);

    int b = -1, q = 0, T = 0, R = 0, k = 0, last = -1, chunk = -1, slot = 0, L = 0, done = 0, jb = 0, fails = 0;
    int first = 0;        // step index of the segment's first record
    double t_start = 0.0; // t_0 (fixed-step tableaux)
    int phase = 0;        // 0: re-integrate segment k, 1: back-step through it
    double lam[1], mu[PG], t = 0.0, dt = 0.0, t1 = 0.0, y[1], t_end = 0.0, y_end = 0.0;
    S p[P], ys[1], k0[1];
    bool at_top = true;

    auto step_back = [&]() {
        if (slot == 0) {
            chunk = a.pool.chunk_prev[chunk];
            slot = CH - 1;
        } else {
            slot--;
        }
    };

    auto fail_instance = [&](int st) {
        const double nan = __longlong_as_double(0x7ff8000000000000ll);
        for (int qq = 0; qq < a.nout; qq++) {
            const size_t o = ((size_t)b * a.nout + qq);
            a.dy0[o * NT + li] = nan;
            for (int kk = li; kk < PT; kk += G)
                a.dpar[o * PT + kk] = nan;
        }
        if (a.status_out && li == 0)
            a.status_out[b] = st;
    };

    // Load the start of segment k (the walk is on record k + 1) and set up
    // its re-integration.
    auto begin_segment = [&]() {
        step_back();
        const double *r = record_ptr<RS>(a.pool, chunk, slot);
        t = r[0];
        dt = r[1];
        y[0] = r[2 + li];
        first = k * SK;
        L = (k == R - 2) ? T - first : SK;
        ys[0] = from_d<S>(y[0]);
        scr[0] = t; // every lane writes the same t: each later reads its own write
        scr[2 + li] = y[0];
        M::template rhs<S>(ys, p, from_d<S>(t), k0);
        done = 0;
        fails = 0;
        at_top = true;
        phase = 0;
    };

    auto start_seed = [&]() {
        chunk = last;
        slot = (R - 1) % CH;
        const double *r = record_ptr<RS>(a.pool, chunk, slot);
        t_end = r[0];
        y_end = r[2 + li];
        const size_t o = ((size_t)b * a.nout + q);
        lam[0] = a.cost == 0 ? 2.0 * y_end : a.cost == 1 ? 1.0 : a.lambdaT[o * NT + li];
#pragma unroll
        for (int kk = 0; kk < PG; kk++)
            mu[kk] = 0.0;
        note_lambda_lane(a, b, q, T, NT, li, lam[0]);
        k = R - 2;
        if (k >= 0)
            begin_segment();
    };

    auto finish_seed = [&]() {
        const size_t o = ((size_t)b * a.nout + q);
        a.dy0[o * NT + li] = lam[0];
        M::store_grads(a.dpar + o * PT, a.mu_direct ? a.mu_direct + o * PT : nullptr, li, mu);
        bool finite = isfinite(lam[0]);
#pragma unroll
        for (int kk = 0; kk < PG; kk++)
            finite = finite && isfinite(mu[kk]);
        const bool all_finite = __all_sync(mask, finite);
        if (a.status_out && li == 0 && (q == a.nout - 1 || !all_finite))
            a.status_out[b] = all_finite ? ST_OK : ST_NONFINITE;
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
                fail_instance(st);
                continue;
            }
            M::template load_params<S>(a.par + (size_t)b * PT, li, p);
            T = a.inst_T[b];
            R = (T + SK - 1) / SK + 1;
            last = a.inst_last[b];
            t1 = a.inst_t1[b];
            if constexpr (Tab::FIXED)
                t_start = a.inst_t0[b];
            q = 0;
            start_seed();
            return true;
        }
    };

    bool alive = fetch();
    while (alive) {
        if (k < 0) {
            finish_seed();
            if (q + 1 < a.nout) {
                q++;
                start_seed();
            } else {
                alive = fetch();
            }
            continue;
        }
        if (phase == 0) {
            // one attempt of the forward controller, as forward_group_kernel does
            if (at_top) {
                if (!Tab::FIXED && (t + dt) - t1 > kDblEps)
                    dt = t1 - t;
                fails = 0;
                at_top = false;
            }
            double ynew[1];
            S ynew_s[1], knew[1];
            const double err = group_max<G>(
                attempt<M, Tab, S>(y, ys, k0, p, t, dt, a.atol, a.rtol, ynew, ynew_s, knew), mask);
            if (err != err || fails >= a.max_fail) {
                fail_instance(ST_RECOMPUTE_MISMATCH);
                alive = fetch();
                continue;
            }
            fails++;
            if (err > 1.0) {
                dt = decrease_step<Tab, S>(dt, err, a.step_pow, li == 0 ? &a.ctl->pow_undecided : nullptr);
                continue;
            }
            if constexpr (Tab::FIXED) {
                t = fixed_time(t_start, first + done + 1, dt);
            } else {
                t += dt;
                dt = increase_step<Tab, S>(dt, err, a.step_pow, li == 0 ? &a.ctl->pow_undecided : nullptr);
            }
            accept_state_group<M, Tab, S>(y, ys, k0, ynew, ynew_s, knew, p, t, mask);
            at_top = true;
            done++;
            double *r = scr + (size_t)done * RS;
            r[0] = t;
            r[2 + li] = y[0];
            if (done == L) {
                // the re-integration must land exactly on the next checkpoint
                const bool same = __all_sync(mask, t == t_end && y[0] == y_end);
                if (!same) {
                    fail_instance(ST_RECOMPUTE_MISMATCH);
                    alive = fetch();
                    continue;
                }
                phase = 1;
                jb = L - 1;
                __syncwarp(mask);
            }
            continue;
        }
        // phase 1: back_step through the segment, last step first
        {
            const double *r = scr + (size_t)jb * RS;
            double yj[1] = {r[2 + li]};
            const double tn = r[0];
            const double h = scr[(size_t)(jb + 1) * RS] - tn;
            back_step<M, Tab, S>(yj, tn, h, p, lam, mu);
            note_lambda_lane(a, b, q, first + jb, NT, li, lam[0]);
            jb--;
            if (jb < 0) {
                // the segment's start becomes the next segment's end
                t_end = scr[0];
                y_end = scr[2 + li];
                k--;
                __syncwarp(mask);
                if (k >= 0)
                    begin_segment();
            }
        }
    }
}

} // namespace va
