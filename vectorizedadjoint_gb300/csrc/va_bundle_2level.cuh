// Two-level backward sweep of the shared-matrix bundles (checkpoint stride
// k > 1).  The forward (forward_bundle_kernel with stride k) stores every
// k-th accepted step's [t, dt, y] plus the last -- for the double-word sweep
// the exact double-word state, packed.  Each CTA carries a bundle of NB
// instances; every instance walks its segments last first, on its own
// schedule: phase 0 re-runs the forward controller from the segment's
// checkpoint (the same per-instance arithmetic as the forward: the
// bundle_stage_point / bundle_solution / bundle_error_ratio helpers and the
// bundle matrix-vector products) into the instance's scratch of k + 1
// [t, y] records, checks that it lands exactly on the next checkpoint, and
// phase 1 back-steps through the segment (bundle_back_step, the stages
// recomputed from y as in the every-step sweep over [t, dt, y] records).
// Per loop iteration the CTA runs one attempt for the instances in phase 0
// and one back step for those in phase 1, each a pass over A shared by the
// bundle.  The matrix gradient goes into the CTA's partial (reduced in CTA
// order afterwards); its summation order differs from the every-step
// sweep's, so dA agrees to rounding while each instance's gradients are
// equal bit for bit.  An instance whose re-integration does not land on its
// checkpoint (VA_RECOMPUTE_MISMATCH; the same code from the same bits, so
// not expected) may already have added steps into the partial: the CTA's
// partial is then set to NaN, and so is dA.
#pragma once

#include "va_bundle.cuh"

namespace va {

// doubles of two-level scratch per instance: k + 1 records of [t, -, y]
__host__ __device__ constexpr int bundle_scratch_doubles(int nt, int stride)
{
    return (stride + 1) * record_doubles(nt);
}

template <int NT, int NB, class Tab, class S>
__global__ void __launch_bounds__(NT, NB <= 2 ? 2 : 0) backward_bundle_kernel_2level(BundleParams bp)
{
    constexpr int NS = Tab::S;
    constexpr int RS = record_doubles(NT);
    constexpr bool DW = std::is_same<S, dword>::value;
    const AdjParams &a = bp.g;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    S *xall = reinterpret_cast<S *>(smem_raw);                      // [NS][NT][NB]; plane 0: attempt stages
    S *vall = xall + (size_t)NS * NT * NB;                          // [NS][NT][NB]
    S *zall = vall + (size_t)NS * NT * NB;                          // [NS][NT][NB]
    double *red = reinterpret_cast<double *>(zall + (size_t)NS * NT * NB); // [NT/32][NB]
    const int i = threadIdx.x;
    const int CH = a.pool.chunk_len, SK = a.stride;

    int inst[NB], T[NB], R[NB], k[NB], chunk[NB], slot[NB], L[NB], done[NB], jb[NB], fails[NB], first[NB];
    int phase[NB]; // 0: re-integrate segment k, 1: back-step through it
    bool live[NB], need_k0[NB], at_top[NB];
    double lam[NB], mu[NB], t[NB], dt[NB], t1[NB], t_start[NB], y[NB], t_end[NB], y_end[NB];
    S r[NB], ys[NB], K[NS][NB];
    double *scr[NB];

    // the state stored in a checkpoint record
    auto rec_state = [&](const double *rec, double &yv, S &ysv) {
        if constexpr (DW) {
            ysv = dw_unpack(rec[2 + i]);
            yv = to_d(ysv);
        } else {
            yv = rec[2 + i];
            ysv = from_d<S>(yv);
        }
    };
    auto step_back = [&](int b) {
        if (slot[b] == 0) {
            chunk[b] = a.pool.chunk_prev[chunk[b]];
            slot[b] = CH - 1;
        } else {
            slot[b]--;
        }
    };
    bool poisoned = false; // a re-integration failed after contributing to the dA partial (CTA-uniform)
    auto fail_instance = [&](int b, int st) {
        const double nan = __longlong_as_double(0x7ff8000000000000ll);
        if (st == ST_RECOMPUTE_MISMATCH)
            poisoned = true;
        a.dy0[(size_t)inst[b] * NT + i] = nan;
        a.dpar[(size_t)inst[b] * NT + i] = nan;
        if (a.status_out && i == 0)
            a.status_out[inst[b]] = st;
        live[b] = false;
    };
    // the segment ending at the walk's current record: load its checkpoint
    // (one record back) and set up the re-integration
    auto begin_segment = [&](int b) {
        step_back(b);
        const double *rec = record_ptr<RS>(a.pool, chunk[b], slot[b]);
        t[b] = rec[0];
        dt[b] = rec[1];
        rec_state(rec, y[b], ys[b]);
        first[b] = k[b] * SK;
        L[b] = (k[b] == R[b] - 2) ? T[b] - first[b] : SK;
        scr[b][0] = t[b]; // every thread writes the same t
        scr[b][2 + i] = y[b];
        done[b] = 0;
        fails[b] = 0;
        at_top[b] = true;
        need_k0[b] = true;
        phase[b] = 0;
    };
    auto finish = [&](int b) {
        a.dy0[(size_t)inst[b] * NT + i] = lam[b];
        const double d = a.mu_direct ? a.mu_direct[(size_t)inst[b] * NT + i] : 0.0;
        a.dpar[(size_t)inst[b] * NT + i] = d + mu[b];
        const bool finite = isfinite(lam[b]) && isfinite(mu[b]);
        const int all_finite = __syncthreads_and(finite ? 1 : 0);
        if (a.status_out && i == 0)
            a.status_out[inst[b]] = all_finite ? ST_OK : ST_NONFINITE;
        live[b] = false;
    };

#pragma unroll
    for (int b = 0; b < NB; b++) {
        inst[b] = blockIdx.x * bp.nb + b;
        live[b] = b < bp.nb && inst[b] < a.B;
        T[b] = R[b] = k[b] = L[b] = done[b] = jb[b] = fails[b] = first[b] = 0;
        phase[b] = 0;
        need_k0[b] = at_top[b] = false;
        chunk[b] = -1;
        slot[b] = 0;
        lam[b] = mu[b] = t[b] = dt[b] = t1[b] = t_start[b] = y[b] = t_end[b] = y_end[b] = 0.0;
        r[b] = ys[b] = S(0);
#pragma unroll
        for (int m = 0; m < NS; m++)
            K[m][b] = S(0);
        scr[b] = nullptr;
        if (!live[b])
            continue;
        if (a.inst_status[inst[b]] != ST_OK) {
            fail_instance(b, a.inst_status[inst[b]]);
            continue;
        }
        scr[b] = a.scratch + (size_t)inst[b] * bundle_scratch_doubles(NT, SK);
        r[b] = from_d<S>(a.par[(size_t)inst[b] * NT + i]);
        T[b] = a.inst_T[inst[b]];
        R[b] = (T[b] + SK - 1) / SK + 1;
        t1[b] = a.inst_t1[inst[b]];
        if constexpr (Tab::FIXED)
            t_start[b] = a.inst_t0[inst[b]];
        chunk[b] = a.inst_last[inst[b]];
        slot[b] = (R[b] - 1) % CH;
        const double *rec = record_ptr<RS>(a.pool, chunk[b], slot[b]);
        S yTs;
        t_end[b] = rec[0];
        rec_state(rec, y_end[b], yTs);
        lam[b] = a.cost == 0 ? 2.0 * y_end[b] : a.cost == 1 ? 1.0 : a.lambdaT[(size_t)inst[b] * NT + i];
        k[b] = R[b] - 2;
    }
    // this CTA's partial of dA, transposed: part[jj][i] += dA_i,jj
    double *part = bp.dA_part + (size_t)blockIdx.x * NT * NT;
    for (int jj = 0; jj < NT; jj++)
        part[(size_t)jj * NT + i] = 0.0;
#pragma unroll
    for (int b = 0; b < NB; b++) {
        if (!live[b])
            continue;
        if (k[b] >= 0)
            begin_segment(b);
        else
            finish(b); // no steps: dG/dy0 is the seed
    }

    for (;;) {
        bool any = false, any_k0 = false, any_attempt = false, any_back = false;
#pragma unroll
        for (int b = 0; b < NB; b++) {
            any = any || live[b];
            any_k0 = any_k0 || (live[b] && need_k0[b]);
            any_attempt = any_attempt || (live[b] && phase[b] == 0);
            any_back = any_back || (live[b] && phase[b] == 1);
        }
        if (!any)
            break;

        // k_1 = f(y) at the checkpoints just loaded (and after accepted
        // attempts of the non-FSAL pairs), as the forward forms it
        if (any_k0) {
#pragma unroll
            for (int b = 0; b < NB; b++)
                xall[i * NB + b] = ys[b];
            __syncthreads();
            S z[NB];
            bundle_matvec<NT, NB, S, 16>(bp.At, bp.Atw, xall, z);
#pragma unroll
            for (int b = 0; b < NB; b++)
                if (live[b] && need_k0[b]) {
                    K[0][b] = ys[b] * (r[b] + z[b]);
                    need_k0[b] = false;
                }
            __syncthreads();
        }

        // phase 0: one attempt of the forward controller per instance
        if (any_attempt) {
            bool att[NB];
            S sdt[NB];
#pragma unroll
            for (int b = 0; b < NB; b++) {
                att[b] = live[b] && phase[b] == 0;
                if (att[b] && at_top[b]) {
                    if (!Tab::FIXED && (t[b] + dt[b]) - t1[b] > kDblEps)
                        dt[b] = t1[b] - t[b];
                    fails[b] = 0;
                    at_top[b] = false;
                }
                sdt[b] = from_d<S>(dt[b]);
            }
#pragma unroll
            for (int m = 1; m < NS; m++) {
#pragma unroll
                for (int b = 0; b < NB; b++)
                    xall[i * NB + b] = bundle_stage_point<Tab, S, NB>(m, b, y[b], ys[b], K, dt[b], sdt[b]);
                __syncthreads();
                S z[NB];
                bundle_matvec<NT, NB, S, 16>(bp.At, bp.Atw, xall, z);
#pragma unroll
                for (int b = 0; b < NB; b++)
                    K[m][b] = xall[i * NB + b] * (r[b] + z[b]);
                __syncthreads();
            }
            S ynew_s[NB], knew[NB];
            double ynew[NB];
#pragma unroll
            for (int b = 0; b < NB; b++) {
                bundle_solution<Tab, S, NB>(b, y[b], ys[b], K, dt[b], sdt[b], ynew_s[b], ynew[b]);
                xall[i * NB + b] = ynew_s[b];
                knew[b] = S(0);
            }
            if constexpr (Tab::FSAL) {
                __syncthreads();
                S znew[NB];
                bundle_matvec<NT, NB, S, 16>(bp.At, bp.Atw, xall, znew);
#pragma unroll
                for (int b = 0; b < NB; b++)
                    knew[b] = ynew_s[b] * (r[b] + znew[b]);
                __syncthreads();
            }
            double ratio[NB];
#pragma unroll
            for (int b = 0; b < NB; b++) {
                ratio[b] = bundle_error_ratio<Tab, S, NB>(b, y[b], K, knew[b], dt[b], a.atol, a.rtol);
                if (!att[b] || Tab::FIXED)
                    ratio[b] = 0.0;
            }
            bundle_max<NT, NB>(ratio, red);
#pragma unroll
            for (int b = 0; b < NB; b++) {
                if (!att[b])
                    continue;
                const double err = ratio[b];
                if (err != err || fails[b] >= a.max_fail) {
                    fail_instance(b, ST_RECOMPUTE_MISMATCH);
                    continue;
                }
                fails[b]++;
                if (err > 1.0) {
                    dt[b] = decrease_step<Tab, S>(dt[b], err, a.step_pow, i == 0 ? &a.ctl->pow_undecided : nullptr);
                    continue;
                }
                t[b] = Tab::FIXED ? fixed_time(t_start[b], first[b] + done[b] + 1, dt[b]) : t[b] + dt[b];
                dt[b] = increase_step<Tab, S>(dt[b], err, a.step_pow, i == 0 ? &a.ctl->pow_undecided : nullptr);
                y[b] = ynew[b];
                ys[b] = ynew_s[b];
                if constexpr (Tab::FSAL)
                    K[0][b] = knew[b];
                else
                    need_k0[b] = true;
                at_top[b] = true;
                done[b]++;
                double *rr = scr[b] + (size_t)done[b] * RS;
                rr[0] = t[b];
                rr[2 + i] = y[b];
                if (done[b] == L[b]) {
                    // the re-integration must land exactly on the next checkpoint
                    const int same = __syncthreads_and(t[b] == t_end[b] && y[b] == y_end[b] ? 1 : 0);
                    if (!same) {
                        fail_instance(b, ST_RECOMPUTE_MISMATCH);
                        continue;
                    }
                    phase[b] = 1;
                    jb[b] = L[b] - 1;
                }
            }
            __syncthreads(); // scratch records visible to the back steps
        }

        // phase 1: one back step per instance through its segment
        if (any_back) {
            bool step[NB];
            double yv[NB], h[NB];
            S ysv[NB], sh[NB];
            const double *srec[NB];
            int jstep[NB];
#pragma unroll
            for (int b = 0; b < NB; b++) {
                step[b] = live[b] && phase[b] == 1;
                yv[b] = h[b] = 0.0;
                srec[b] = nullptr;
                jstep[b] = 0;
                if (step[b]) {
                    const double *rr = scr[b] + (size_t)jb[b] * RS;
                    srec[b] = rr;
                    yv[b] = rr[2 + i];
                    h[b] = scr[b][(size_t)(jb[b] + 1) * RS] - rr[0];
                    jstep[b] = first[b] + jb[b];
                }
                ysv[b] = from_d<S>(yv[b]);
                sh[b] = from_d<S>(h[b]);
            }
            bundle_back_step<NT, NB, Tab, S, false>(bp, xall, vall, zall, step, yv, h, ysv, sh, srec, r, inst, jstep,
                                                    part, lam, mu);
#pragma unroll
            for (int b = 0; b < NB; b++) {
                if (!step[b])
                    continue;
                jb[b]--;
                if (jb[b] < 0) {
                    // the segment's start becomes the next segment's end
                    t_end[b] = scr[b][0];
                    y_end[b] = scr[b][2 + i];
                    k[b]--;
                    __syncthreads();
                    if (k[b] >= 0)
                        begin_segment(b);
                    else
                        finish(b);
                }
            }
            __syncthreads();
        }
    }
    if (poisoned)
        for (int jj = 0; jj < NT; jj++)
            part[(size_t)jj * NT + i] = __longlong_as_double(0x7ff8000000000000ll);
}

} // namespace va
