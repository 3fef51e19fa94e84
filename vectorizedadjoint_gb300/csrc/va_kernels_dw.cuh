// Double-word sweeps of the one-thread-per-instance models.
//
// The mixed_dw variant of the forward and backward sweeps keeps FP64 for the
// time coordinate alone: the state y, the stages, the step size and its
// controller, the error norm, the adjoint (lambda, mu) and the checkpoint
// records are double-words (pairs of floats, ~48 significant bits).  On this
// part FP64 issues at 1/64 of the FP32 rate and the FP64 <-> FP32
// conversions share that narrow pipe, so a sweep that rounds its state to
// FP64 every step (to store it) and runs its controller in FP64 spends more
// of the FP64 pipe on conversions than the stages spend on the FP32 pipe.
//
// Sums of products -- the stage combinations y + dt sum_j a_mj K_j, the
// solution and error combinations, the adjoint accumulations -- go through
// the compensated accumulator dacc (va_dword.cuh): ~12 FP32 operations per
// term against ~29 for a double-word multiply followed by a double-word add,
// at the same O(u^2) accuracy.
//
// The algorithms are those of va_kernels.cuh: odeint 1.74's controlled
// stepper with its default error checker and step adjuster (forward), the
// reference's back_prop_step (lib/include/backpropagation.hpp:160-229,
// backward); only the arithmetic type differs.
//
// Stage records.  The reference's backward step recomputes the stage values
// X_m = y_n + h sum_j a_mj K_j from y_n (compute_intermediate_states,
// backpropagation.hpp:24-64) before its VJPs; that recompute is ~40% of a
// backward step here.  With 288 GB of HBM at ~7 TB/s the sweeps store them
// instead: when every step is checkpointed, the record of step n is
//   [t_n (FP64), dt_n, y_n, X_1 .. X_{s-1} (double-words)]
// (stage_record_doubles), each double-word packed into one 8-byte slot
// (dw_pack), padded to whole 32-byte sectors.  Each attempt keeps its stage
// values in registers; the accepted one writes the record, once, in 256-bit
// stores (partial-sector writes spread over the attempts cost the forward
// 11% and capped its occupancy).  The backward step reads
// X_0 = y_n .. X_{s-1} and runs only the VJPs: the adjoint differentiates
// the stages the forward computed, bit for bit.  The two-level backward
// (checkpoints every k-th step, records [t, dt, y]) keeps the stage values
// of its re-integration in the same layout in its scratch, so both modes
// give the same bits.
#pragma once

#include "va_endtests.h"
#include "va_kernels.cuh"

namespace va {

// doubles per stage record: t, dt, X_0 = y, X_1 .. X_{s-1}, padded to a
// multiple of four: every record starts on a 32-byte boundary and is moved
// with whole-sector (256-bit) loads and stores
__host__ __device__ constexpr int stage_record_doubles(int n, int s) { return (2 + n * s + 3) & ~3; }

// 256-bit global store / streaming load of four doubles (p 32-byte aligned)
__device__ __forceinline__ void st_v4(double *p, double a, double b, double c, double d)
{
    asm volatile("st.global.v4.f64 [%0], {%1, %2, %3, %4};" ::"l"(p), "d"(a), "d"(b), "d"(c), "d"(d) : "memory");
}
__device__ __forceinline__ void ld_v4_cs(const double *p, double &a, double &b, double &c, double &d)
{
    asm volatile("ld.global.cs.v4.f64 {%0, %1, %2, %3}, [%4];" : "=d"(a), "=d"(b), "=d"(c), "=d"(d) : "l"(p));
}

struct DwTol {
    dword atol, rtol;
};

__host__ __device__ __forceinline__ dword dw_nan() { return dword(f32_from_bits(0x7fc00000), 0.0f); }

// (double)f by integer operations: rebias the exponent (127 -> 1023) and
// shift the 23 fraction bits to the top of the 52; subnormals are normalised
// first, infinities and NaNs keep their fraction (payload).  The FP64 pipe's
// own conversion is as scarce as its arithmetic.  Exact, like the cast.
__device__ __forceinline__ double f2d_int(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu;
    unsigned m = u & 0x7fffffu, ed;
    if (e == 0xffu) {
        ed = 0x7ffu;
    } else if (e != 0u) {
        ed = e + 896u;
    } else if (m != 0u) {
        // m 2^-149 with the leading one at bit p: shift it to bit 23
        const unsigned sh = (unsigned)__clz((int)m) - 8u;
        m = (m << sh) & 0x7fffffu;
        ed = 897u - sh;
    } else {
        ed = 0u;
    }
    const unsigned hi = (u & 0x80000000u) | (ed << 20) | (m >> 3);
    return __hiloint2double((int)hi, (int)(m << 29));
}

// hi + lo rounded to FP64, as to_d, without FP64-pipe conversions
__device__ __forceinline__ double to_d_int(dword v) { return f2d_int(v.hi) + f2d_int(v.lo); }

// ------------------------------------------------------------- controller

// a^(-1/K) for a double-word a > 0: inv_root's FP32 iteration on the leading
// word (~1e-7), then one Newton step x + x (1 - a x^K) / K with the residual
// formed in double-word: relative error ~4e-14, the accuracy of the single
// FP64 Newton step the float-stage path takes.  a >= 1e30 returns 0, which
// the 0.2 limiter of decrease_dw turns into the factor pow would give.
template <int K>
__host__ __device__ __forceinline__ dword inv_root_dw(dword a)
{
    if (!(a.hi < 1e30f))
        return dword(0.0f, 0.0f);
    const float x = inv_root_f32<K>(a.hi);
    dword xk(x, 0.0f);
#pragma unroll
    for (int k = 1; k < K; k++)
        xk = xk * x;
    dacc r{1.0f, 0.0f};
    dacc_fma(r, -a, xk);
    const dword res = dacc_get(r);
    const float corr = fmul_rn(fmul_rn(x, res.hi), 1.0f / (float)K);
    dword z;
    fast_two_sum(x, corr, z.hi, z.lo);
    return z;
}

// inv_root_f32<KA> (first) or inv_root_f32<KB> (!first) with the same
// operations in the same order, without a branch: the powers are formed up
// to the larger order and the wanted one selected, so a warp whose lanes
// need different orders runs one evaluation instead of both.
template <int KA, int KB>
__host__ __device__ __forceinline__ float inv_root_f32_sel(float af, bool first)
{
    constexpr int KM = KA > KB ? KA : KB;
    constexpr int32_t ca = (int32_t)(((int64_t)(KA + 1) * 0x3F800000LL) / KA);
    constexpr int32_t cb = (int32_t)(((int64_t)(KB + 1) * 0x3F800000LL) / KB);
    const int32_t bits = f32_bits(af);
    float x = f32_from_bits(first ? ca - bits / KA : cb - bits / KB);
    const float rk = first ? 1.0f / (float)KA : 1.0f / (float)KB;
#pragma unroll
    for (int it = 0; it < 4; it++) {
        float pw[KM];
        pw[0] = x;
#pragma unroll
        for (int k = 1; k < KM; k++)
            pw[k] = pw[k - 1] * x;
        const float r = fmaf(-af, first ? pw[KA - 1] : pw[KB - 1], 1.0f);
        x = fmaf(x * r, rk, x);
    }
    return x;
}

// inv_root_dw<KA> (first) or inv_root_dw<KB> (!first), bit for bit, branch-free
template <int KA, int KB>
__host__ __device__ __forceinline__ dword inv_root_dw_sel(dword a, bool first)
{
    if (!(a.hi < 1e30f))
        return dword(0.0f, 0.0f);
    constexpr int KM = KA > KB ? KA : KB;
    const float x = inv_root_f32_sel<KA, KB>(a.hi, first);
    dword pw(x, 0.0f), xa = pw, xb = pw;
#pragma unroll
    for (int k = 1; k < KM; k++) {
        pw = pw * x;
        if (k == KA - 1)
            xa = pw;
        if (k == KB - 1)
            xb = pw;
    }
    dacc r{1.0f, 0.0f};
    dacc_fma(r, -a, first ? xa : xb);
    const dword res = dacc_get(r);
    const float corr = fmul_rn(fmul_rn(x, res.hi), first ? 1.0f / (float)KA : 1.0f / (float)KB);
    dword z;
    fast_two_sum(x, corr, z.hi, z.lo);
    return z;
}

// odeint default_step_adjuster::decrease_step: dt * max(0.9 err^(-1/(q-1)), 0.2)
// (fixed-step tableaux: dt unchanged; their sweeps never call it)
template <class Tab>
__host__ __device__ __forceinline__ dword decrease_dw(dword dt, dword err)
{
    if constexpr (Tab::FIXED) {
        (void)err;
        return dt;
    } else {
        const dword f = dword(9.0 / 10.0) * inv_root_dw<Tab::ERROR_ORDER - 1>(err);
        const dword lim = dword(1.0 / 5.0);
        return dt * (dw_greater(f, lim) ? f : lim);
    }
}

// odeint default_step_adjuster::increase_step:
//   if err < 0.5: dt * 0.9 max(err, 5^-p)^(-1/p)
template <class Tab>
__host__ __device__ __forceinline__ dword increase_dw(dword dt, dword err)
{
    if constexpr (Tab::FIXED)
        return dt;
    if (dw_less(err, dword(0.5))) {
        const dword fl = dword(Tab::ERR_FLOOR);
        const dword e = dw_greater(fl, err) ? fl : err;
        return dt * (dword(9.0 / 10.0) * inv_root_dw<Tab::STEPPER_ORDER>(e));
    }
    return dt;
}

// decrease_dw (reject) or increase_dw (accept), bit for bit, as one
// branch-free evaluation: the accept / reject split of a warp's lanes then
// costs one inverse root instead of two (~6% of a VdP forward attempt).
template <class Tab>
__host__ __device__ __forceinline__ dword adjust_dw(dword dt, dword err, bool reject)
{
    if constexpr (Tab::FIXED) {
        (void)err;
        (void)reject;
        return dt;
    } else {
        const dword fl = dword(Tab::ERR_FLOOR);
        const dword e = reject ? err : (dw_greater(fl, err) ? fl : err);
        const dword f = dword(9.0 / 10.0) * inv_root_dw_sel<Tab::ERROR_ORDER - 1, Tab::STEPPER_ORDER>(e, reject);
        const dword lim = dword(1.0 / 5.0);
        const dword scaled = dt * (reject ? (dw_greater(f, lim) ? f : lim) : f);
        return (reject || dw_less(err, dword(0.5))) ? scaled : dt;
    }
}

// ---------------------------------------------------------- stage algebra

// sum_j w_j K_j[i] over the nonzero compile-time weights w_j = W(j), j < J
template <int J, class W, int NS, int N>
__host__ __device__ __forceinline__ dacc wsum_dw(W w, const dword (&K)[NS][N], int i)
{
    dacc s{0.0f, 0.0f};
    bool first = true;
#pragma unroll
    for (int j = 0; j < J; j++) {
        const double c = w(j);
        if (c != 0.0) {
            if (first)
                s = dacc_mul_k(c, K[j][i]);
            else
                dacc_fma_k(s, c, K[j][i]);
            first = false;
        }
    }
    return s;
}

// y + dt s, rounded to a double-word
__host__ __device__ __forceinline__ dword axpy_dw(dword y, dword dt, dacc s)
{
    dacc r = dacc_of(y);
    dacc_fma(r, dt, dacc_get(s));
    return dacc_get(r);
}

// X_m = y + dt sum_{j<m} a_mj K_j (the order odeint's scale_sum and the
// reference's compute_intermediate_states use, backpropagation.hpp:36-45)
template <class Tab, int N>
__host__ __device__ __forceinline__ void stage_dw(int m, const dword (&y)[N], const dword (&K)[Tab::S][N],
                                                  dword dt, dword (&X)[N])
{
#pragma unroll
    for (int i = 0; i < N; i++) {
        dacc s{0.0f, 0.0f};
        bool first = true;
#pragma unroll
        for (int j = 0; j < Tab::S - 1; j++) {
            if (j < m && Tab::a(m, j) != 0.0) {
                if (first)
                    s = dacc_mul_k(Tab::a(m, j), K[j][i]);
                else
                    dacc_fma_k(s, Tab::a(m, j), K[j][i]);
                first = false;
            }
        }
        X[i] = axpy_dw(y[i], dt, s);
    }
}

struct BWeights {
    template <class Tab>
    struct of {
        __host__ __device__ constexpr double operator()(int j) const { return Tab::b(j); }
    };
};
struct EWeights {
    template <class Tab>
    struct of {
        __host__ __device__ constexpr double operator()(int j) const { return Tab::e(j); }
    };
};

// N packed double-words at r (16-byte aligned when N is even)
template <int N>
__host__ __device__ __forceinline__ void store_dw(double *r, const dword (&X)[N])
{
    if constexpr (N % 2 == 0) {
#pragma unroll
        for (int i = 0; i < N; i += 2)
            *reinterpret_cast<double2 *>(r + i) = make_double2(dw_pack(X[i]), dw_pack(X[i + 1]));
    } else {
#pragma unroll
        for (int i = 0; i < N; i++)
            r[i] = dw_pack(X[i]);
    }
}

// One attempted step from (y, k0 = f(y), t) with step dt: y_new, k_new =
// f(y_new) (FSAL pairs) and the error norm
//   max_i |dt e_i| / (atol + rtol (|y_i| + |dt| |k0_i|))
// (odeint's default_error_checker with a_x = a_dxdt = 1), NaN if any ratio is.
// sink(m, X_m) sees the stage values X_1 .. X_{s-1} as they are formed.
template <class M, class Tab, class Sink>
__host__ __device__ __forceinline__ dword attempt_dw_sink(const dword (&y)[M::N], const dword (&k0)[M::N],
                                                          const dword (&p)[M::P], dword t, dword dt,
                                                          const DwTol &tol, dword (&ynew)[M::N],
                                                          dword (&knew)[M::N], Sink &&sink)
{
    constexpr int N = M::N, NS = Tab::S;
    dword K[NS][N];
#pragma unroll
    for (int i = 0; i < N; i++)
        K[0][i] = k0[i];
#pragma unroll
    for (int m = 1; m < NS; m++) {
        dword X[N];
        stage_dw<Tab, N>(m, y, K, dt, X);
        sink(m, X);
        M::template rhs<dword>(X, p, t + dt * dword(Tab::c(m)), K[m]);
    }
#pragma unroll
    for (int i = 0; i < N; i++)
        ynew[i] = axpy_dw(y[i], dt, wsum_dw<NS>(typename BWeights::template of<Tab>(), K, i));
    if constexpr (Tab::FIXED)
        return dword(0.0f, 0.0f); // no error estimate: every attempt is accepted
    if constexpr (Tab::FSAL)
        M::template rhs<dword>(ynew, p, t + dt, knew);
    const dword adt = dabs(dt);
    const dword rdt = tol.rtol * adt;
    dword worst(0.0f, 0.0f);
    bool nan = false;
#pragma unroll
    for (int i = 0; i < N; i++) {
        dacc e = wsum_dw<NS>(typename EWeights::template of<Tab>(), K, i);
        if constexpr (Tab::FSAL)
            dacc_fma_k(e, Tab::E_NEW, knew[i]);
        const dword num = dabs(dacc_get(e) * adt);
        dacc d = dacc_of(tol.atol);
        dacc_fma(d, tol.rtol, dabs(y[i]));
        dacc_fma(d, rdt, dabs(k0[i]));
        const dword r = num / dacc_get(d);
        nan = nan || r.hi != r.hi;
        if (dw_greater(r, worst))
            worst = r;
    }
    return nan ? dw_nan() : worst;
}

// attempt_dw_sink with the stage values stored at xrec (N each; may be null)
template <class M, class Tab>
__host__ __device__ __forceinline__ dword attempt_dw(const dword (&y)[M::N], const dword (&k0)[M::N],
                                                     const dword (&p)[M::P], dword t, dword dt,
                                                     const DwTol &tol, dword (&ynew)[M::N],
                                                     dword (&knew)[M::N], double *xrec = nullptr)
{
    return attempt_dw_sink<M, Tab>(y, k0, p, t, dt, tol, ynew, knew, [&](int m, const dword (&X)[M::N]) {
        if (xrec)
            store_dw<M::N>(xrec + (m - 1) * M::N, X);
    });
}

// ----------------------------------------------------------------- records

template <int N>
__device__ __forceinline__ void write_record_dw(double *r, double t, dword dt, const dword (&y)[N])
{
    constexpr int RS = record_doubles(N);
    double v[RS];
    v[0] = t;
    v[1] = dw_pack(dt);
#pragma unroll
    for (int i = 0; i < N; i++)
        v[2 + i] = dw_pack(y[i]);
#pragma unroll
    for (int i = 2 + N; i < RS; i++)
        v[i] = 0.0;
#pragma unroll
    for (int i = 0; i < RS; i += 2)
        *reinterpret_cast<double2 *>(r + i) = make_double2(v[i], v[i + 1]);
}

template <int N>
__device__ __forceinline__ void read_record_dw(const double *r, double &t, dword &dt, dword (&y)[N])
{
    constexpr int RS = record_doubles(N);
    double v[RS];
#pragma unroll
    for (int i = 0; i < RS; i += 2) {
        double2 q = __ldcs(reinterpret_cast<const double2 *>(r + i));
        v[i] = q.x;
        v[i + 1] = q.y;
    }
    t = v[0];
    dt = dw_unpack(v[1]);
#pragma unroll
    for (int i = 0; i < N; i++)
        y[i] = dw_unpack(v[2 + i]);
}

// t_n and the stage values X_0 = y_n .. X_{S-1} of a stage record
template <int N, int S>
__device__ __forceinline__ void read_stage_record_dw(const double *r, double &t, dword (&X)[S][N])
{
    constexpr int RS = stage_record_doubles(N, S);
    double v[RS];
#pragma unroll
    for (int i = 0; i < RS; i += 2) {
        double2 q = __ldcs(reinterpret_cast<const double2 *>(r + i));
        v[i] = q.x;
        v[i + 1] = q.y;
    }
    t = v[0];
#pragma unroll
    for (int m = 0; m < S; m++)
#pragma unroll
        for (int i = 0; i < N; i++)
            X[m][i] = dw_unpack(v[2 + m * N + i]);
}

// a whole stage record [t, dt, y, X_1 .. X_{S-1}], in 256-bit stores
template <int N, int S>
__device__ __forceinline__ void write_stage_record_dw(double *r, double t, dword dt, const dword (&y)[N],
                                                      const dword (&X)[S > 1 ? S - 1 : 1][N])
{
    constexpr int RS = stage_record_doubles(N, S);
    double v[RS];
    v[0] = t;
    v[1] = dw_pack(dt);
#pragma unroll
    for (int i = 0; i < N; i++)
        v[2 + i] = dw_pack(y[i]);
#pragma unroll
    for (int m = 0; m < S - 1; m++)
#pragma unroll
        for (int i = 0; i < N; i++)
            v[2 + N + m * N + i] = dw_pack(X[m][i]);
#pragma unroll
    for (int i = 2 + N * S; i < RS; i++)
        v[i] = 0.0;
#pragma unroll
    for (int i = 0; i < RS; i += 4)
        st_v4(r + i, v[i], v[i + 1], v[i + 2], v[i + 3]);
}

__host__ __device__ __forceinline__ bool dw_same(dword x, dword y) { return x.hi == y.hi && x.lo == y.lo; }

// ------------------------------------------------------------ forward sweep

// forward_kernel with double-word state.  The end clamp and the loop test
// stay in FP64 (less_with_sign, runge_kutta.hpp:155-163); an accepted step
// that was clamped to the end lands on t1 itself.  STAGES: every step is
// checkpointed as a stage record (the stride is ignored); otherwise records
// are [t, dt, y] every stride-th step.
template <class M, class Tab, bool STAGES>
__global__ void __launch_bounds__(256) forward_kernel_dw(FwdParams a)
{
    constexpr int N = M::N, P = M::P;
    constexpr int RS = STAGES ? stage_record_doubles(N, Tab::S) : record_doubles(N);
    const int CH = a.pool.chunk_len;
    const DwTol tol{dword(a.atol), dword(a.rtol)};

    int b = -1;
    double t = 0.0, t1 = 0.0, t_start = 0.0;
    EndTests et{}; // the loop and end-clamp tests as integer comparisons
    dword y[N], k0[N], p[P], dt;
    int count = 0, rej = 0, fails = 0, status = ST_OK, chunk = -1, slot = 0;
    bool at_top = true, to_end = false;
    // STAGES: the current step's record slot and its trial step at the top;
    // the record is written once, by the accepted attempt
    double *rec = nullptr;
    dword dt_top;

    auto fetch = [&]() -> bool {
        b = (int)atomicAdd(&a.ctl->fwd_next, 1u);
        if (b >= a.B)
            return false;
        if (a.order)
            b = a.order[b];
#pragma unroll
        for (int i = 0; i < N; i++)
            y[i] = dword(a.y0[(size_t)b * N + i]);
#pragma unroll
        for (int k = 0; k < P; k++)
            p[k] = dword(a.par[(size_t)b * P + k]);
        t = t_start = a.t0[b];
        t1 = a.t1[b];
        et = end_tests(t1);
        dt = dword(a.dt0);
        count = rej = fails = 0;
        status = ST_OK;
        at_top = true;
        slot = 0;
        chunk = (int)atomicAdd(&a.ctl->pool_next, 1u);
        if (chunk >= a.pool.n_chunks) {
            status = ST_CKPT_BUDGET;
            chunk = -1;
            atomicOr(&a.ctl->pool_fail, 1u);
        } else {
            a.pool.chunk_prev[chunk] = -1;
        }
        M::template rhs<dword>(y, p, dword(t), k0);
        return true;
    };

    auto reserve = [&]() -> bool {
        if (chunk < 0)
            return false;
        if (slot == CH) {
            const int c = (int)atomicAdd(&a.ctl->pool_next, 1u);
            if (c >= a.pool.n_chunks) {
                atomicOr(&a.ctl->pool_fail, 1u);
                return false;
            }
            a.pool.chunk_prev[c] = chunk;
            chunk = c;
            slot = 0;
        }
        return true;
    };

    auto finish = [&]() {
        if (status == ST_OK) {
            if (reserve()) {
                write_record_dw<N>(record_ptr<RS>(a.pool, chunk, slot), t, dt, y);
                slot++;
            } else {
                status = ST_CKPT_BUDGET;
            }
#pragma unroll
            for (int i = 0; i < N; i++)
                if (!isfinite(y[i].hi))
                    status = ST_NONFINITE;
        }
        if (a.yT) {
#pragma unroll
            for (int i = 0; i < N; i++)
                a.yT[(size_t)b * N + i] = to_d(y[i]);
        }
        a.inst_T[b] = count;
        a.inst_last[b] = chunk;
        a.inst_status[b] = status;
        note_work(a, b, count + rej);
        if (a.inst_t1)
            a.inst_t1[b] = t1;
        if (Tab::FIXED && a.inst_t0)
            a.inst_t0[b] = t_start;
        if (a.n_acc_out)
            a.n_acc_out[b] = count;
        if (a.n_rej_out)
            a.n_rej_out[b] = rej;
        if (a.status_out)
            a.status_out[b] = status;
    };

    bool alive = fetch();
    while (alive) {
        if (status != ST_OK) {
            finish();
            alive = fetch();
            continue;
        }
        if (at_top) {
            // fixed steps: while ((t + dt) - t1 <= eps), dt the FP64 step
            if (Tab::FIXED ? !((t + a.dt0) - t1 <= kDblEps) : !end_loop(et, t, t1)) {
                finish();
                alive = fetch();
                continue;
            }
            if (count >= a.max_steps) {
                status = ST_MAX_STEPS;
                continue;
            }
            if (STAGES || a.stride <= 1 || count % a.stride == 0) {
                if (!reserve()) {
                    status = ST_CKPT_BUDGET;
                    continue;
                }
                double *r = record_ptr<RS>(a.pool, chunk, slot);
                if (STAGES) {
                    rec = r;
                    dt_top = dt;
                } else {
                    write_record_dw<N>(r, t, dt, y);
                }
                slot++;
            }
            to_end = !Tab::FIXED && end_clamp(et, t + to_d_int(dt), t1);
            if (to_end)
                dt = dword(t1 - t);
            fails = 0;
            at_top = false;
        }
        dword ynew[N], knew[N];
        constexpr int XS = Tab::S > 1 ? Tab::S - 1 : 1;
        dword xs[XS][N]; // stage values X_1 .. X_{s-1} of this attempt (STAGES)
        const dword err = attempt_dw_sink<M, Tab>(y, k0, p, dword(t), dt, tol, ynew, knew,
                                                  [&](int m, const dword (&X)[N]) {
                                                      if constexpr (STAGES) {
#pragma unroll
                                                          for (int i = 0; i < N; i++)
                                                              xs[m - 1][i] = X[i];
                                                      }
                                                  });
        bool ok;
        if (err.hi != err.hi) {
            status = ST_NONFINITE;
            continue;
        }
        const bool reject = dw_greater(err, dword(1.0f, 0.0f));
        const dword dt_next = adjust_dw<Tab>(dt, err, reject); // both branches' step, one evaluation
        if (reject) {
            dt = dt_next;
            rej++;
            to_end = false;
            ok = false;
        } else {
            if constexpr (STAGES)
                write_stage_record_dw<N, Tab::S>(rec, t, dt_top, y, xs);
            if constexpr (Tab::FIXED) {
                t = fixed_time(t_start, count + 1, a.dt0);
            } else {
                t = to_end ? t1 : t + to_d_int(dt);
                dt = dt_next;
            }
#pragma unroll
            for (int i = 0; i < N; i++)
                y[i] = ynew[i];
            if constexpr (Tab::FSAL) {
#pragma unroll
                for (int i = 0; i < N; i++)
                    k0[i] = knew[i];
            } else {
                M::template rhs<dword>(y, p, dword(t), k0);
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

// ----------------------------------------------------------- backward sweep

// back_step in double-word from the stage values X_0 = y_n .. X_{s-1} of
// step n: lambda_{n+1} -> lambda_n, mu += the step's parameter adjoint.
// Kbar_m and the lambda / mu increments are compensated accumulators,
// finished when stage m's VJP needs Kbar_m.
template <class M, class Tab>
__host__ __device__ __forceinline__ void back_step_dw_x(const dword (&X)[Tab::S][M::N], dword tn, dword h,
                                                        const dword (&p)[M::P], dword (&lam)[M::N],
                                                        dword (&mu)[M::PG])
{
    constexpr int N = M::N, PG = M::PG, NS = Tab::S;
    // seeds Kbar_m = (b_m h) lambda (:178-184)
    dacc Kb[NS][N];
#pragma unroll
    for (int m = 0; m < NS; m++) {
        if (Tab::b(m) != 0.0) {
            const dword bh = dacc_get(dacc_mul_k(Tab::b(m), h));
#pragma unroll
            for (int i = 0; i < N; i++)
                Kb[m][i] = dacc_mul(bh, lam[i]);
        } else {
#pragma unroll
            for (int i = 0; i < N; i++)
                Kb[m][i] = dacc{0.0f, 0.0f};
        }
    }
    dacc dl[N], dm[PG];
#pragma unroll
    for (int i = 0; i < N; i++)
        dl[i] = dacc_of(lam[i]);
#pragma unroll
    for (int k = 0; k < PG; k++)
        dm[k] = dacc_of(mu[k]);
    // stages s..1 (:196-224): ybar += J^T Kbar_m, Kbar_k += a_mk h J^T Kbar_m,
    // mu += J_p^T Kbar_m
#pragma unroll
    for (int m = NS - 1; m >= 0; m--) {
        dword w[N], gx[N], gp[PG];
#pragma unroll
        for (int i = 0; i < N; i++)
            w[i] = dacc_get(Kb[m][i]);
        M::template vjp<dword>(w, X[m], p, tn + h * dword(Tab::c(m)), gx, gp);
#pragma unroll
        for (int i = 0; i < N; i++) {
            dacc_add(dl[i], gx[i]);
            if (m > 0) {
                const dword g = gx[i] * h;
#pragma unroll
                for (int k = 0; k < NS - 1; k++)
                    if (k < m && Tab::a(m, k) != 0.0)
                        dacc_fma_k(Kb[k][i], Tab::a(m, k), g);
            }
        }
#pragma unroll
        for (int k = 0; k < PG; k++)
            dacc_add(dm[k], gp[k]);
    }
#pragma unroll
    for (int i = 0; i < N; i++)
        lam[i] = dacc_get(dl[i]);
#pragma unroll
    for (int k = 0; k < PG; k++)
        mu[k] = dacc_get(dm[k]);
}

// back_step_dw_x after recomputing the stage values from y_n with step h
// (compute_intermediate_states, :24-64), as the reference's backward step
// does.
template <class M, class Tab>
__host__ __device__ __forceinline__ void back_step_dw(const dword (&y)[M::N], dword tn, dword h,
                                                      const dword (&p)[M::P], dword (&lam)[M::N],
                                                      dword (&mu)[M::PG])
{
    constexpr int N = M::N, NS = Tab::S;
    // K[NS - 1] stays unset: the stages read K_j for j < m only, and the
    // VJPs need the stage values, not the last slope
    dword K[NS][N];
    dword X[NS][N];
#pragma unroll
    for (int i = 0; i < N; i++)
        X[0][i] = y[i];
#pragma unroll
    for (int m = 0; m < NS; m++) {
        if (m > 0)
            stage_dw<Tab, N>(m, y, K, h, X[m]);
        if (m < NS - 1)
            M::template rhs<dword>(X[m], p, tn + h * dword(Tab::c(m)), K[m]);
    }
    back_step_dw_x<M, Tab>(X, tn, h, p, lam, mu);
}

// cost seeds lambda_T from the last record's y_T
template <int N>
__device__ __forceinline__ void seed_lambda_dw(const AdjParams &a, size_t o, const dword (&yT)[N], dword (&lam)[N])
{
#pragma unroll
    for (int i = 0; i < N; i++) {
        if (a.cost == 0)
            lam[i] = dword(2.0f * yT[i].hi, 2.0f * yT[i].lo); // 2 y(T), exact
        else if (a.cost == 1)
            lam[i] = dword(1.0f, 0.0f);
        else
            lam[i] = dword(a.lambdaT[o * N + i]);
    }
}

template <int N, int P>
__device__ __forceinline__ void fail_outputs(const AdjParams &a, int b)
{
    for (int qq = 0; qq < a.nout; qq++) {
        const size_t o = ((size_t)b * a.nout + qq);
        for (int i = 0; i < N; i++)
            a.dy0[o * N + i] = __longlong_as_double(0x7ff8000000000000ll);
        for (int k = 0; k < P; k++)
            a.dpar[o * P + k] = __longlong_as_double(0x7ff8000000000000ll);
    }
}

// dy0 = lambda_0, dparams = mu_direct + mu (backpropagation.hpp:317-321)
template <int N, int P>
__device__ __forceinline__ void write_seed_dw(const AdjParams &a, int b, int q, const dword (&lam)[N],
                                              const dword (&mu)[P])
{
    const size_t o = ((size_t)b * a.nout + q);
    bool finite = true;
#pragma unroll
    for (int i = 0; i < N; i++) {
        const double v = to_d(lam[i]);
        a.dy0[o * N + i] = v;
        finite = finite && isfinite(v);
    }
#pragma unroll
    for (int k = 0; k < P; k++) {
        const double d = a.mu_direct ? a.mu_direct[o * P + k] : 0.0;
        const double v = d + to_d(mu[k]);
        a.dpar[o * P + k] = v;
        finite = finite && isfinite(v);
    }
    if (a.status_out && (q == a.nout - 1 || !finite))
        a.status_out[b] = finite ? ST_OK : ST_NONFINITE;
}

// Backward sweep over every-step checkpoints: the stage records of
// forward_kernel_dw<M, Tab, true> (STAGES), or [t, dt, y] records with the
// stages recomputed from y_n as the reference does.
template <class M, class Tab, bool STAGES>
__global__ void __launch_bounds__(256) backward_kernel_dw(AdjParams a)
{
    constexpr int N = M::N, P = M::P, NS = Tab::S;
    static_assert(M::PG == M::P, "parameter adjoint covers every parameter");
    constexpr int RS = STAGES ? stage_record_doubles(N, NS) : record_doubles(N);
    const int CH = a.pool.chunk_len;

    int b = -1, q = 0, j = -1, chunk = -1, slot = 0, T = 0, last = -1;
    double t_next = 0.0;
    dword lam[N], mu[P], p[P];
    // records j-1 .. j-PF, loaded PF steps ahead: their loads are in flight
    // while the VJPs of the steps before run (two steps measured no faster
    // than one)
    constexpr int PF = 1;
    double nv[PF][RS];

    // the chain link of the walk's chunk, read a few records before the walk
    // crosses into the previous chunk (the record load there does not wait
    // on a dependent load of the link)
    int prev_chunk = -1;
    // move the load walk one record back and load it into dst
    auto step_back_load = [&](double (&dst)[RS]) {
        if (slot == 0) {
            chunk = prev_chunk >= 0 ? prev_chunk : a.pool.chunk_prev[chunk];
            prev_chunk = -1;
            slot = CH - 1;
        } else {
            slot--;
        }
        if (slot == 4 || (slot < 4 && prev_chunk < 0 && slot > 0))
            prev_chunk = a.pool.chunk_prev[chunk];
        const double *r = record_ptr<RS>(a.pool, chunk, slot);
        if constexpr (STAGES) {
#pragma unroll
            for (int i = 0; i < RS; i += 4)
                ld_v4_cs(r + i, dst[i], dst[i + 1], dst[i + 2], dst[i + 3]);
        } else {
#pragma unroll
            for (int i = 0; i < RS; i += 2) {
                const double2 v = __ldcs(reinterpret_cast<const double2 *>(r + i));
                dst[i] = v.x;
                dst[i + 1] = v.y;
            }
        }
    };

    auto start_seed = [&]() {
        chunk = last;
        slot = T % a.pool.chunk_len;
        prev_chunk = -1;
        dword yTl[N], dtr;
        read_record_dw<N>(record_ptr<RS>(a.pool, chunk, slot), t_next, dtr, yTl);
        seed_lambda_dw<N>(a, (size_t)b * a.nout + q, yTl, lam);
#pragma unroll
        for (int k = 0; k < P; k++)
            mu[k] = dword(0.0f, 0.0f);
        note_lambda<N>(a, b, q, T, lam);
        j = T - 1;
#pragma unroll
        for (int d = 0; d < PF; d++)
            if (j - d >= 0)
                step_back_load(nv[d]);
    };

    auto fetch = [&]() -> bool {
        for (;;) {
            unsigned w = atomicAdd(&a.ctl->adj_next, 1u);
            if ((int)w >= a.B)
                return false;
            b = a.order ? a.order[w] : (int)w;
            const int st = a.inst_status[b];
            if (st != ST_OK) {
                fail_outputs<N, P>(a, b);
                if (a.status_out)
                    a.status_out[b] = st;
                continue;
            }
#pragma unroll
            for (int k = 0; k < P; k++)
                p[k] = dword(a.par[(size_t)b * P + k]);
            T = a.inst_T[b];
            last = a.inst_last[b];
            q = 0;
            start_seed();
            return true;
        }
    };

    bool alive = fetch();
    while (alive) {
        if (j < 0) {
            write_seed_dw<N, P>(a, b, q, lam, mu);
            if (q + 1 < a.nout) {
                q++;
                start_seed();
            } else {
                alive = fetch();
            }
            continue;
        }
        double cv[RS];
#pragma unroll
        for (int i = 0; i < RS; i++)
            cv[i] = nv[0][i];
#pragma unroll
        for (int d = 1; d < PF; d++)
#pragma unroll
            for (int i = 0; i < RS; i++)
                nv[d - 1][i] = nv[d][i];
        if (j - PF >= 0)
            step_back_load(nv[PF - 1]);
        const double tn = cv[0];
        if constexpr (STAGES) {
            dword X[NS][N];
#pragma unroll
            for (int m = 0; m < NS; m++)
#pragma unroll
                for (int i = 0; i < N; i++)
                    X[m][i] = dw_unpack(cv[2 + m * N + i]);
            back_step_dw_x<M, Tab>(X, dword(tn), dword(t_next - tn), p, lam, mu);
        } else {
            dword y[N];
#pragma unroll
            for (int i = 0; i < N; i++)
                y[i] = dw_unpack(cv[2 + i]);
            back_step_dw<M, Tab>(y, dword(tn), dword(t_next - tn), p, lam, mu);
        }
        note_lambda<N>(a, b, q, j, lam);
        t_next = tn;
        j--;
    }
}

// --------------------------------------------- backward sweep, two levels

// backward_kernel_2level with double-word state: segments re-run from their
// checkpoint's exact double-words (t, dt, y), so the re-integration
// reproduces the forward's bits and lands on the next checkpoint.  (The
// restart evaluates k_1 = f(y) afresh; the built-in models do not read t,
// so it equals the forward's FSAL value.)  The re-integration keeps stage
// records in the thread's scratch, and the back-steps read them, as the
// every-step sweep does.
template <class M, class Tab>
__global__ void __launch_bounds__(256) backward_kernel_2level_dw(AdjParams a)
{
    constexpr int N = M::N, P = M::P, NS = Tab::S;
    static_assert(M::PG == M::P, "parameter adjoint covers every parameter");
    constexpr int RS = record_doubles(N), RX = stage_record_doubles(N, NS);
    const int CH = a.pool.chunk_len, SK = a.stride;
    double *scr = a.scratch + ((size_t)blockIdx.x * blockDim.x + threadIdx.x) * (SK + 1) * RX;
    const DwTol tol{dword(a.atol), dword(a.rtol)};

    int b = -1, q = 0, T = 0, R = 0, k = 0, last = -1, chunk = -1, slot = 0, L = 0, done = 0, jb = 0, fails = 0;
    int phase = 0; // 0: re-integrate segment k, 1: back-step through it
    int first = 0; // step index of the segment's first record
    double t = 0.0, t1 = 0.0, t_end = 0.0, t_start = 0.0;
    EndTests et{};
    dword lam[N], mu[P], p[P], y[N], k0[N], y_end[N], dt;
    bool at_top = true, to_end = false;

    auto step_back = [&]() {
        if (slot == 0) {
            chunk = a.pool.chunk_prev[chunk];
            slot = CH - 1;
        } else {
            slot--;
        }
    };

    auto fail_instance = [&](int st) {
        fail_outputs<N, P>(a, b);
        if (a.status_out)
            a.status_out[b] = st;
    };

    auto begin_segment = [&]() {
        step_back();
        read_record_dw<N>(record_ptr<RS>(a.pool, chunk, slot), t, dt, y);
        first = k * SK;
        L = (k == R - 2) ? T - first : SK;
        write_record_dw<N>(scr, t, dt, y);
        M::template rhs<dword>(y, p, dword(t), k0);
        done = 0;
        fails = 0;
        at_top = true;
        phase = 0;
    };

    auto start_seed = [&]() {
        chunk = last;
        slot = (R - 1) % CH;
        dword dtr;
        read_record_dw<N>(record_ptr<RS>(a.pool, chunk, slot), t_end, dtr, y_end);
        seed_lambda_dw<N>(a, (size_t)b * a.nout + q, y_end, lam);
#pragma unroll
        for (int kk = 0; kk < P; kk++)
            mu[kk] = dword(0.0f, 0.0f);
        note_lambda<N>(a, b, q, T, lam);
        k = R - 2;
        if (k >= 0)
            begin_segment();
    };

    auto fetch = [&]() -> bool {
        for (;;) {
            unsigned w = atomicAdd(&a.ctl->adj_next, 1u);
            if ((int)w >= a.B)
                return false;
            b = a.order ? a.order[w] : (int)w;
            const int st = a.inst_status[b];
            if (st != ST_OK) {
                fail_instance(st);
                continue;
            }
#pragma unroll
            for (int kk = 0; kk < P; kk++)
                p[kk] = dword(a.par[(size_t)b * P + kk]);
            T = a.inst_T[b];
            R = (T + SK - 1) / SK + 1;
            last = a.inst_last[b];
            t1 = a.inst_t1[b];
            et = end_tests(t1);
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
            write_seed_dw<N, P>(a, b, q, lam, mu);
            if (q + 1 < a.nout) {
                q++;
                start_seed();
            } else {
                alive = fetch();
            }
            continue;
        }
        if (phase == 0) {
            // one attempt of the forward controller, as forward_kernel_dw does
            if (at_top) {
                to_end = !Tab::FIXED && end_clamp(et, t + to_d_int(dt), t1);
                if (to_end)
                    dt = dword(t1 - t);
                fails = 0;
                at_top = false;
            }
            dword ynew[N], knew[N];
            const dword err = attempt_dw<M, Tab>(y, k0, p, dword(t), dt, tol, ynew, knew,
                                                 scr + (size_t)done * RX + 2 + N);
            if (err.hi != err.hi || fails >= a.max_fail) {
                fail_instance(ST_RECOMPUTE_MISMATCH);
                alive = fetch();
                continue;
            }
            fails++;
            if (dw_greater(err, dword(1.0f, 0.0f))) {
                dt = decrease_dw<Tab>(dt, err);
                to_end = false;
                continue;
            }
            if constexpr (Tab::FIXED) {
                t = fixed_time(t_start, first + done + 1, a.dt0);
            } else {
                t = to_end ? t1 : t + to_d_int(dt);
                dt = increase_dw<Tab>(dt, err);
            }
#pragma unroll
            for (int i = 0; i < N; i++)
                y[i] = ynew[i];
            if constexpr (Tab::FSAL) {
#pragma unroll
                for (int i = 0; i < N; i++)
                    k0[i] = knew[i];
            } else {
                M::template rhs<dword>(y, p, dword(t), k0);
            }
            at_top = true;
            done++;
            write_record_dw<N>(scr + (size_t)done * RX, t, dt, y);
            if (done == L) {
                // the re-integration must land exactly on the next checkpoint
                bool same = t == t_end;
#pragma unroll
                for (int i = 0; i < N; i++)
                    same = same && dw_same(y[i], y_end[i]);
                if (!same) {
                    fail_instance(ST_RECOMPUTE_MISMATCH);
                    alive = fetch();
                    continue;
                }
                phase = 1;
                jb = L - 1;
            }
            continue;
        }
        // phase 1: back_step through the segment, last step first
        {
            dword X[NS][N], dtr;
            double tn, tn1;
            read_stage_record_dw<N, NS>(scr + (size_t)jb * RX, tn, X);
            tn1 = scr[(size_t)(jb + 1) * RX];
            back_step_dw_x<M, Tab>(X, dword(tn), dword(tn1 - tn), p, lam, mu);
            note_lambda<N>(a, b, q, first + jb, lam);
            jb--;
            if (jb < 0) {
                // the segment's start becomes the next segment's end
                read_record_dw<N>(scr, t_end, dtr, y_end);
                k--;
                if (k >= 0)
                    begin_segment();
            }
        }
    }
}

} // namespace va
