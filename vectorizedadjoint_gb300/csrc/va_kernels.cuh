// Persistent forward and backward sweeps for models whose whole state fits in
// one thread (VdP, DHO, decay): one thread owns one instance at a time and,
// when that instance is done, takes the next one from a global counter, so a
// lane never waits for the slowest instance of its warp.
//
// Forward sweep  = the reference's controlled loop
//   (lib/include/detail/runge_kutta.hpp:137-180) with odeint 1.74's
//   controlled_runge_kutta::try_step, default_error_checker and
//   default_step_adjuster run on the device.  Every accepted (t_n, dt_n, y_n)
//   is written to a chunked checkpoint pool in HBM (StateStorage.hpp:23-35).
// Backward sweep = back_prop / back_prop_step
//   (lib/include/detail/backpropagation.hpp:160-278): h_n = t_{n+1} - t_n
//   (StateStorage.hpp:22), stages recomputed from y_n, seeds b_m h lambda,
//   transposed-tableau accumulation, mu += J_p^T Kbar.
//
// S is the stage type: double (FP64 path, the reference's arithmetic order)
// or float (mixed path: stages and VJPs in FP32; t, h, y, the error norm,
// the controller and the gradient accumulators stay FP64).
#pragma once

#include <cstdint>
#include <cstring>
#include <limits>
#include <type_traits>

#include "va_dword.cuh"
#include "va_stepfactor.cuh"
#include "va_tableau.cuh"

namespace va {

enum : int32_t {
    ST_OK = 0,
    ST_MAX_REJECTS = 1,
    ST_MAX_STEPS = 2,
    ST_NONFINITE = 3,
    ST_CKPT_BUDGET = 4,
    ST_BAD_ARGS = 5,
    ST_RECOMPUTE_MISMATCH = 8,
    ST_NOT_RUN = 9
};

constexpr double kDblEps = 2.220446049250313080847e-16; // std::numeric_limits<double>::epsilon()

// Device control block, cleared before every launch.
struct Control {
    unsigned int fwd_next;  // next instance for the forward sweep
    unsigned int adj_next;  // next position in the backward work order
    unsigned int pool_next; // next free checkpoint chunk
    unsigned int pool_fail; // set when the pool ran out
    unsigned int pow_undecided; // step factors whose rounding test failed (cr_step_pow)
};

// Checkpoint pool: chunks of `chunk_len` records of `rs` doubles.
// Record layout: [t_n, dt_n (trial step at the top of step n), y_n[0..N)].
struct Pool {
    double *rec;
    int *chunk_prev;
    int n_chunks;
    int chunk_len;
};

struct FwdParams {
    int B;
    const double *y0;  // [B][N]
    const double *par; // [B][P]
    const double *t0;  // [B]
    const double *t1;  // [B]
    double atol, rtol, dt0;
    int max_steps, max_fail;
    int step_pow;    // FP64 controller: 1 = correctly rounded pow (odeint's
                     // std::pow), 0 = Newton root (cr_step_pow / inv_root)
    double *yT;      // [B][N] (may be null)
    int *n_acc_out;  // [B] (may be null)
    int *n_rej_out;  // [B] (may be null)
    int *status_out; // [B] (may be null)
    int *inst_T;     // [B] accepted steps
    int *inst_last;  // [B] last checkpoint chunk
    int *inst_status;// [B]
    double *inst_t1; // [B] end times (kept for segment re-integration; may be null)
    double *inst_t0; // [B] start times, written by the fixed-step sweeps (the
                     // two-level backward re-forms t_0 + n dt from them; may be null)
    int stride;      // store every stride-th accepted step (and the last); 1 = all
    const int *order;// [B] work order (may be null = index order)
    int *inst_work;  // [B] attempts (accepted + rejected) of this sweep, the next
                     // sweep's length estimate (may be null)
    int *work_valid; // set to 1 once inst_work holds a sweep's counts (may be null)
    Pool pool;
    Control *ctl;
};

// Record an instance's attempt count for the next forward sweep's order.
__device__ __forceinline__ void note_work(const FwdParams &a, int b, int attempts)
{
    if (a.inst_work) {
        a.inst_work[b] = attempts;
        *a.work_valid = 1;
    }
}

struct AdjParams {
    int B;
    int nout;
    const double *par;       // [B][P]
    const double *lambdaT;   // [B][nout][N]  (null when cost >= 0)
    const double *mu_direct; // [B][nout][P]  (may be null)
    int cost;                // -1 seeds from lambdaT; 0: g = sum y(T)^2; 1: g = sum y(T)
    double *dy0;             // [B][nout][N]
    double *dpar;            // [B][nout][P]
    int *status_out;         // [B] (may be null)
    const int *order;        // [B] work order (may be null = identity)
    const int *inst_T;
    const int *inst_last;
    const int *inst_status;
    Pool pool;
    Control *ctl;
    // two-level checkpointing (stride > 1): segment re-integration
    int stride;
    const double *inst_t1;   // [B]
    const double *inst_t0;   // [B] start times (fixed-step tableaux)
    double *scratch;         // per thread: (stride + 1) records
    double atol, rtol;
    double dt0;              // the step of the fixed-step tableaux
    int max_fail;
    int step_pow;            // the forward's step-factor power (FwdParams::step_pow)
    // adjoint history (may be null): lambda_n of seed q at
    // hist[((b * nout + q) * hist_cap + n) * N + i] for record n < hist_cap
    double *hist;
    int hist_cap;
};

__host__ __device__ constexpr int record_doubles(int n) { return (2 + n + 1) & ~1; }

// Stage-type helpers for the reduced-precision paths (S = float or dword).
template <class S>
__host__ __device__ __forceinline__ S from_d(double v)
{
    return S(v);
}
__host__ __device__ __forceinline__ double to_d(double v) { return v; }
__host__ __device__ __forceinline__ double to_d(float v) { return (double)v; }
__host__ __device__ __forceinline__ double to_d(dword v) { return (double)v; }

// The reference's back_prop observer (detail/backpropagation.hpp:243,250)
// sees (lambda_n, t_n) after every back step, n = T .. 0; the sweeps store
// lambda_n instead, at its record index (t_n is the forward's record).
template <int N, class V>
__device__ __forceinline__ void note_lambda(const AdjParams &a, int b, int q, int n, const V (&lam)[N])
{
    if (a.hist && n < a.hist_cap) {
        double *d = a.hist + (((size_t)b * a.nout + q) * a.hist_cap + n) * N;
#pragma unroll
        for (int i = 0; i < N; i++)
            d[i] = to_d(lam[i]);
    }
}

// the same for lane i of a lane group (component i of an NT-state)
template <class V>
__device__ __forceinline__ void note_lambda_lane(const AdjParams &a, int b, int q, int n, int NT, int li, V lam)
{
    if (a.hist && n < a.hist_cap)
        a.hist[(((size_t)b * a.nout + q) * a.hist_cap + n) * NT + li] = to_d(lam);
}

// a * b + c (for double: fused only where the translation unit contracts;
// the FP64 kernels are built without contraction)
__host__ __device__ __forceinline__ double madd(double a, double b, double c) { return a * b + c; }
__host__ __device__ __forceinline__ float madd(float a, float b, float c) { return fmaf(a, b, c); }
__host__ __device__ __forceinline__ dword madd(dword a, dword b, dword c) { return a * b + c; }
template <class S>
__host__ __device__ __forceinline__ S fromf(float v)
{
    return S(v, 0.0f);
}
template <>
__host__ __device__ __forceinline__ float fromf<float>(float v)
{
    return v;
}

// ---------------------------------------------------------------- controller

// FP64 Newton steps of the step-factor root: two on the FP64 path (the
// scheme the oracle shares), one on the reduced paths (~3e-14 relative,
// far below the error estimate's own accuracy there).
template <class S>
struct RootSteps {
    static constexpr int value = std::is_same<S, double>::value ? 2 : 1;
};

// odeint default_step_adjuster::decrease_step:
//   dt *= max(0.9 err^(-1/(q-1)), 0.2)
// (fixed-step tableaux: dt unchanged; their sweeps never call it).
// step_pow != 0 on the FP64 path: err^(-1/(q-1)) is odeint's
// pow(err, -1.0/(q-1)) correctly rounded (cr_step_pow; undecided roundings
// are counted in *undecided); else the Newton root.
template <class Tab, class S = double>
__host__ __device__ __forceinline__ double decrease_step(double dt, double err, int step_pow = 0,
                                                         unsigned int *undecided = nullptr)
{
    if constexpr (Tab::FIXED) {
        (void)err;
        (void)step_pow;
        (void)undecided;
        return dt;
    } else {
        double r;
        if (std::is_same<S, double>::value && step_pow)
            r = cr_step_pow<Tab::ERROR_ORDER - 1>(err, undecided);
        else
            r = inv_root<Tab::ERROR_ORDER - 1, RootSteps<S>::value>(err);
        double f = 9.0 / 10.0 * r;
        return dt * fmax(f, 1.0 / 5.0);
    }
}

// odeint default_step_adjuster::increase_step:
//   if err < 0.5: dt *= 0.9 max(err, 5^-p)^(-1/p)
template <class Tab, class S = double>
__host__ __device__ __forceinline__ double increase_step(double dt, double err, int step_pow = 0,
                                                         unsigned int *undecided = nullptr)
{
    if constexpr (Tab::FIXED) {
        (void)err;
        (void)step_pow;
        (void)undecided;
        return dt;
    } else {
        if (err < 0.5) {
            // 5^-p as the correctly rounded quotient (1/3125, 1/390625), what
            // pow(5.0, -p) returns
            err = fmax(Tab::ERR_FLOOR, err);
            double r;
            if (std::is_same<S, double>::value && step_pow)
                r = cr_step_pow<Tab::STEPPER_ORDER>(err, undecided);
            else
                r = inv_root<Tab::STEPPER_ORDER, RootSteps<S>::value>(err);
            dt *= 9.0 / 10.0 * r;
        }
        return dt;
    }
}

// ------------------------------------------------------------- stage algebra

__host__ __device__ __forceinline__ double hi_of(double v) { return v; }
__host__ __device__ __forceinline__ float hi_of(float v) { return v; }
__host__ __device__ __forceinline__ float hi_of(dword v) { return v.hi; }

// X_m = y + sum_{j<m} (a_mj dt) K_j, in the order odeint's scale_sum
// evaluates it (and the reference recomputes it, backpropagation.hpp:36-45).
// ys / sdt: y and dt in stage precision (unused on the FP64 path).
template <class Tab, int N, class S>
__host__ __device__ __forceinline__ void form_stage(int m, const double (&y)[N], const S (&ys)[N],
                                                   const S (&K)[Tab::S][N], double dt, S sdt, S (&X)[N])
{
    if constexpr (std::is_same<S, double>::value) {
        (void)ys;
        (void)sdt;
#pragma unroll
        for (int i = 0; i < N; i++) {
            double acc = y[i];
#pragma unroll
            for (int j = 0; j < Tab::S - 1; j++)
                if (j < m)
                    acc = acc + (Tab::a(m, j) * dt) * K[j][i];
            X[i] = acc;
        }
    } else {
        // X = y + dt * sum_{j<m} a_mj K_j  (float or double-word stages)
        (void)y;
        (void)dt;
#pragma unroll
        for (int i = 0; i < N; i++) {
            S acc = S(0);
#pragma unroll
            for (int j = 0; j < Tab::S - 1; j++)
                if (j < m)
                    acc = madd(S(Tab::a(m, j)), K[j][i], acc);
            X[i] = madd(acc, sdt, ys[i]);
        }
    }
}

// One attempted step of the embedded pair from (y, k0 = f(y), t) with step dt:
// y_new, k_new = f(y_new) (FSAL pairs) and the error norm
// max_i |err_i| / (atol + rtol (|y_i| + |dt| |k0_i|))  (default_error_checker
// with a_x = a_dxdt = 1, evaluated at the step start).
// ys is y in stage precision.  Outputs: FP64 and double-word paths give
// ynew_s (the new state in stage precision; FP64: = ynew); FP64 and float
// paths give ynew in FP64.  The double-word path leaves ynew to the caller,
// which rounds ynew_s to FP64 once per accepted step.
template <class M, class Tab, class S>
__host__ __device__ __forceinline__ double attempt_pair(const double (&y)[M::N], const S (&ys)[M::N],
                                                        const S (&k0)[M::N], const S (&p)[M::P], double t,
                                                        double dt, double atol, double rtol,
                                                        double (&ynew)[M::N], S (&ynew_s)[M::N], S (&knew)[M::N])
{
    constexpr int N = M::N, NS = Tab::S;
    S K[NS][N];
    const S sdt = std::is_same<S, double>::value ? S(dt) : from_d<S>(dt);
#pragma unroll
    for (int i = 0; i < N; i++)
        K[0][i] = k0[i];
#pragma unroll
    for (int m = 1; m < NS; m++) {
        S X[N];
        form_stage<Tab, N, S>(m, y, ys, K, dt, sdt, X);
        M::template rhs<S>(X, p, S(t + Tab::c(m) * dt), K[m]);
    }
    double e[N];
    if constexpr (std::is_same<S, double>::value) {
#pragma unroll
        for (int i = 0; i < N; i++) {
            double acc = y[i];
#pragma unroll
            for (int j = 0; j < NS; j++)
                if (Tab::b(j) != 0.0)
                    acc = acc + (Tab::b(j) * dt) * K[j][i];
            ynew[i] = acc;
            ynew_s[i] = acc;
        }
        if constexpr (Tab::FSAL)
            M::template rhs<S>(ynew, p, t + dt, knew);
#pragma unroll
        for (int i = 0; i < N; i++) {
            double acc = 0.0;
            bool first = true;
#pragma unroll
            for (int j = 0; j < NS; j++)
                if (Tab::e(j) != 0.0) {
                    double term = (Tab::e(j) * dt) * K[j][i];
                    acc = first ? term : acc + term;
                    first = false;
                }
            if constexpr (Tab::FSAL)
                acc = acc + (Tab::E_NEW * dt) * knew[i];
            e[i] = acc;
        }
    } else {
        // y_new = y + dt * sum_j b_j K_j: an FP64 update of an FP32 increment
        // (float stages) or a double-word sum (rounded to FP64 by the caller).
#pragma unroll
        for (int i = 0; i < N; i++) {
            S acc = S(0);
#pragma unroll
            for (int j = 0; j < NS; j++)
                if (Tab::b(j) != 0.0)
                    acc = madd(S(Tab::b(j)), K[j][i], acc);
            if constexpr (std::is_same<S, float>::value) {
                ynew[i] = fma(dt, (double)acc, y[i]);
                ynew_s[i] = (float)ynew[i];
            } else {
                ynew_s[i] = madd(acc, sdt, ys[i]);
            }
        }
        if constexpr (Tab::FSAL)
            M::template rhs<S>(ynew_s, p, from_d<S>(t + dt), knew);
        // error vector at full stage precision: a coarser estimate (leading
        // word only) flips accept/reject decisions near err = 1
        S eacc[N];
#pragma unroll
        for (int i = 0; i < N; i++) {
            S acc = S(0);
#pragma unroll
            for (int j = 0; j < NS; j++)
                if (Tab::e(j) != 0.0)
                    acc = madd(S(Tab::e(j)), K[j][i], acc);
            if constexpr (Tab::FSAL)
                acc = madd(S(Tab::E_NEW), knew[i], acc);
            eacc[i] = acc;
            if constexpr (!std::is_same<S, dword>::value)
                e[i] = dt * to_d(acc);
        }
        if constexpr (std::is_same<S, dword>::value) {
            // The norm in double-word arithmetic on the FP32 pipe (relative
            // error ~2^-44, the decision quality of FP64), rounded once to FP64
            // for the FP64 controller: the FP64 pipe of this part is scarce and
            // the conversions an FP64 norm needs cost more than its arithmetic.
            const dword sat = dword(atol), srt = dword(rtol);
            dword m = dword(0);
            bool nan = false;
#pragma unroll
            for (int i = 0; i < N; i++) {
                const dword num = dabs(eacc[i] * sdt);
                const dword den = sat + srt * (dabs(ys[i]) + sdt * dabs(k0[i]));
                const dword r = num / den;
                nan = nan || r.hi != r.hi;
                if (dw_greater(r, m))
                    m = r;
            }
            (void)e;
            return nan ? std::numeric_limits<double>::quiet_NaN() : to_d(m);
        }
    }
    const double adt = fabs(dt);
    if constexpr (std::is_same<S, double>::value) {
        // odeint's rel_error + norm_inf: one quotient per component, then max
        double m = 0.0;
#pragma unroll
        for (int i = 0; i < N; i++) {
            const double r = fabs(e[i]) / (atol + rtol * (1.0 * fabs(y[i]) + adt * fabs(k0[i])));
            if (r != r)
                return r;
            if (r > m)
                m = r;
        }
        return m;
    }
    // reduced paths: max-norm with one division, the largest ratio kept as a fraction
    double num = fabs(e[0]);
    double den = atol + rtol * (1.0 * fabs(y[0]) + adt * fabs(to_d(k0[0])));
#pragma unroll
    for (int i = 1; i < N; i++) {
        double ni = fabs(e[i]);
        double di = atol + rtol * (1.0 * fabs(y[i]) + adt * fabs(to_d(k0[i])));
        if (ni * den > num * di || ni != ni) {
            num = ni;
            den = di;
        }
    }
    return num / den;
}

// One step of a fixed-step tableau: the stages and
// y_new = y + sum_j (b_j dt) K_j (odeint's explicit_generic_rk::do_step, the
// same arithmetic as the embedded pairs' solution update); no error estimate.
template <class M, class Tab, class S>
__host__ __device__ __forceinline__ void step_fixed(const double (&y)[M::N], const S (&ys)[M::N],
                                                    const S (&k0)[M::N], const S (&p)[M::P], double t,
                                                    double dt, double (&ynew)[M::N], S (&ynew_s)[M::N])
{
    constexpr int N = M::N, NS = Tab::S;
    S K[NS][N];
    const S sdt = std::is_same<S, double>::value ? S(dt) : from_d<S>(dt);
#pragma unroll
    for (int i = 0; i < N; i++)
        K[0][i] = k0[i];
#pragma unroll
    for (int m = 1; m < NS; m++) {
        S X[N];
        form_stage<Tab, N, S>(m, y, ys, K, dt, sdt, X);
        M::template rhs<S>(X, p, S(t + Tab::c(m) * dt), K[m]);
    }
#pragma unroll
    for (int i = 0; i < N; i++) {
        if constexpr (std::is_same<S, double>::value) {
            double acc = y[i];
#pragma unroll
            for (int j = 0; j < NS; j++)
                if (Tab::b(j) != 0.0)
                    acc = acc + (Tab::b(j) * dt) * K[j][i];
            ynew[i] = acc;
            ynew_s[i] = acc;
        } else {
            S acc = S(0);
#pragma unroll
            for (int j = 0; j < NS; j++)
                if (Tab::b(j) != 0.0)
                    acc = madd(S(Tab::b(j)), K[j][i], acc);
            if constexpr (std::is_same<S, float>::value) {
                ynew[i] = fma(dt, (double)acc, y[i]);
                ynew_s[i] = (float)ynew[i];
            } else {
                ynew_s[i] = madd(acc, sdt, ys[i]);
            }
        }
    }
}

// attempt_pair for the embedded pairs; a fixed-step tableau's step, with
// error 0 (always accepted)
template <class M, class Tab, class S>
__host__ __device__ __forceinline__ double attempt(const double (&y)[M::N], const S (&ys)[M::N],
                                                   const S (&k0)[M::N], const S (&p)[M::P], double t,
                                                   double dt, double atol, double rtol, double (&ynew)[M::N],
                                                   S (&ynew_s)[M::N], S (&knew)[M::N])
{
    if constexpr (Tab::FIXED) {
        (void)atol;
        (void)rtol;
        (void)knew;
        step_fixed<M, Tab, S>(y, ys, k0, p, t, dt, ynew, ynew_s);
        return 0.0;
    } else {
        return attempt_pair<M, Tab, S>(y, ys, k0, p, t, dt, atol, rtol, ynew, ynew_s, knew);
    }
}

// State after an accepted attempt: y (FP64, what a checkpoint stores), its
// stage-precision copy ys and k0 = f(y).  For double-word stages ys restarts
// from the rounded FP64 value, exactly what a re-integration from a
// checkpoint starts from, and f(y_new) is reused only when that copy equals
// the attempt's own (it does unless a double-word split rounds at a tie).
template <class M, class Tab, class S>
__host__ __device__ __forceinline__ void accept_state(double (&y)[M::N], S (&ys)[M::N], S (&k0)[M::N],
                                                      const double (&ynew)[M::N], const S (&ynew_s)[M::N],
                                                      const S (&knew)[M::N], const S (&p)[M::P], double t)
{
    constexpr int N = M::N;
    bool same = true;
#pragma unroll
    for (int i = 0; i < N; i++) {
        if constexpr (std::is_same<S, dword>::value) {
            y[i] = to_d(ynew_s[i]); // the one rounding to FP64 per accepted step
            // from_d(y) returns the same pair exactly when y = hi + lo holds
            // without rounding (false for about 1 in 32 components: lo more
            // than 29 binades below hi carries bits under the FP64 grid) and
            // the float sum hi + lo rounds back to hi (false only at ties)
            if ((y[i] - (double)ynew_s[i].hi) == (double)ynew_s[i].lo &&
                ynew_s[i].hi + ynew_s[i].lo == ynew_s[i].hi) {
                ys[i] = ynew_s[i];
            } else {
                ys[i] = from_d<S>(y[i]);
                same = false;
            }
        } else {
            y[i] = ynew[i];
            ys[i] = ynew_s[i];
        }
    }
    if (Tab::FSAL && same) {
#pragma unroll
        for (int i = 0; i < N; i++)
            k0[i] = knew[i];
    } else {
        M::template rhs<S>(ys, p, from_d<S>(t), k0);
    }
}

// k = f(y) at an FP64 state, in stage precision.
template <class M, class S>
__host__ __device__ __forceinline__ void eval_rhs(const double (&y)[M::N], const S (&p)[M::P], double t,
                                                  S (&k)[M::N])
{
    S ys[M::N];
#pragma unroll
    for (int i = 0; i < M::N; i++)
        ys[i] = from_d<S>(y[i]);
    M::template rhs<S>(ys, p, from_d<S>(t), k);
}

// Checkpoint pool helpers.  Record j of an instance lives in chunk j / CH of
// its chain, slot j % CH.
template <int RS>
__device__ __forceinline__ double *record_ptr(const Pool &pool, int chunk, int slot)
{
    return pool.rec + ((size_t)chunk * pool.chunk_len + slot) * RS;
}

template <int N>
__device__ __forceinline__ void write_record(double *r, double t, double dt, const double (&y)[N])
{
    constexpr int RS = record_doubles(N);
    double v[RS];
    v[0] = t;
    v[1] = dt;
#pragma unroll
    for (int i = 0; i < N; i++)
        v[2 + i] = y[i];
#pragma unroll
    for (int i = 2 + N; i < RS; i++)
        v[i] = 0.0;
#pragma unroll
    for (int i = 0; i < RS; i += 2)
        *reinterpret_cast<double2 *>(r + i) = make_double2(v[i], v[i + 1]);
}

template <int N>
__device__ __forceinline__ void read_record(const double *r, double &t, double (&y)[N])
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
#pragma unroll
    for (int i = 0; i < N; i++)
        y[i] = v[2 + i];
}

// ------------------------------------------------------------ forward sweep

template <class M, class Tab, class S>
__global__ void __launch_bounds__(256) forward_kernel(FwdParams a)
{
    constexpr int N = M::N, P = M::P;
    constexpr int RS = record_doubles(N);
    const int CH = a.pool.chunk_len;

    int b = -1;
    double y[N], t = 0.0, t1 = 0.0, dt = 0.0, t_start = 0.0;
    S ys[N], k0[N], p[P]; // ys: y in stage precision, carried across steps
    int count = 0, rej = 0, fails = 0, status = ST_OK, chunk = -1, slot = 0;
    bool at_top = true;

    // Take the next instance; false when the batch is exhausted.
    auto fetch = [&]() -> bool {
        b = (int)atomicAdd(&a.ctl->fwd_next, 1u);
        if (b >= a.B)
            return false;
        if (a.order)
            b = a.order[b];
#pragma unroll
        for (int i = 0; i < N; i++)
            y[i] = a.y0[(size_t)b * N + i];
#pragma unroll
        for (int k = 0; k < P; k++)
            p[k] = from_d<S>(a.par[(size_t)b * P + k]);
        t = t_start = a.t0[b];
        t1 = a.t1[b];
        dt = a.dt0;
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
        // k_1 = f(y_0): odeint computes it on the first call (FSAL) or on
        // every attempt (non-FSAL, same value for the same y, t).
#pragma unroll
        for (int i = 0; i < N; i++)
            ys[i] = from_d<S>(y[i]);
        M::template rhs<S>(ys, p, from_d<S>(t), k0);
        return true;
    };

    // Reserve the slot of the next stored record; false if the pool ran out.
    auto reserve = [&]() -> bool {
        if (chunk < 0)
            return false;
        if (slot == CH) {
            int c = (int)atomicAdd(&a.ctl->pool_next, 1u);
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
                write_record<N>(record_ptr<RS>(a.pool, chunk, slot), t, dt, y);
                slot++;
            } else {
                status = ST_CKPT_BUDGET;
            }
#pragma unroll
            for (int i = 0; i < N; i++)
                if (!isfinite(y[i]))
                    status = ST_NONFINITE;
        }
        if (a.yT) {
#pragma unroll
            for (int i = 0; i < N; i++)
                a.yT[(size_t)b * N + i] = y[i];
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
            // while (less_with_sign(t, t1, dt))  (runge_kutta.hpp:155); fixed
            // steps: while (less_eq_with_sign(t + dt, t1, dt))  (:54)
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
                write_record<N>(record_ptr<RS>(a.pool, chunk, slot), t, dt, y);
                slot++;
            }
            // end clamp (runge_kutta.hpp:160-163)
            if (!Tab::FIXED && (t + dt) - t1 > kDblEps)
                dt = t1 - t;
            fails = 0;
            at_top = false;
        }
        double ynew[N];
        S ynew_s[N], knew[N];
        const double err = attempt<M, Tab, S>(y, ys, k0, p, t, dt, a.atol, a.rtol, ynew, ynew_s, knew);
        bool ok;
        if (err != err) {
            status = ST_NONFINITE;
            continue;
        }
        if (err > 1.0) {
            dt = decrease_step<Tab, S>(dt, err, a.step_pow, &a.ctl->pow_undecided);
            rej++;
            ok = false;
        } else {
            if constexpr (Tab::FIXED) {
                t = fixed_time(t_start, count + 1, dt); // t_0 + n dt (:61-62)
            } else {
                t += dt;
                dt = increase_step<Tab, S>(dt, err, a.step_pow, &a.ctl->pow_undecided);
            }
            accept_state<M, Tab, S>(y, ys, k0, ynew, ynew_s, knew, p, t);
            ok = true;
        }
        // failed_step_checker: at most max_fail attempts per accepted step
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

// One back_prop_step (backpropagation.hpp:160-229) for step n with state y_n,
// start time tn and h = t_{n+1} - t_n.  lam: in lambda_{n+1}, out lambda_n.
template <class M, class Tab, class S>
__host__ __device__ __forceinline__ void back_step(const double (&y)[M::N], double tn, double h,
                                          const S (&p)[M::P], double (&lam)[M::N],
                                          double (&mu)[M::PG])
{
    constexpr int N = M::N, P = M::PG, NS = Tab::S;
    S K[NS][N];
    S X[NS][N];
    S ys[N];
#pragma unroll
    for (int i = 0; i < N; i++)
        ys[i] = from_d<S>(y[i]);
    const S shh = from_d<S>(h);
    // recompute the stages from y_n (compute_intermediate_states, :24-64)
#pragma unroll
    for (int m = 0; m < NS; m++) {
        form_stage<Tab, N, S>(m, y, ys, K, h, shh, X[m]);
        M::template rhs<S>(X[m], p, from_d<S>(tn + Tab::c(m) * h), K[m]);
    }
    S Kbar[NS][N];
    if constexpr (std::is_same<S, double>::value) {
        // seeds: ybar = lambda, Kbar_m = (b_m h) lambda  (:178-184)
        double ybar[N];
#pragma unroll
        for (int i = 0; i < N; i++) {
            ybar[i] = lam[i];
#pragma unroll
            for (int m = 0; m < NS; m++)
                Kbar[m][i] = (Tab::b(m) * h) * lam[i];
        }
        // stages s..1 (:196-224)
#pragma unroll
        for (int m = NS - 1; m >= 0; m--) {
            S gx[N], gp[P];
            M::template vjp<S>(Kbar[m], X[m], p, S(tn + Tab::c(m) * h), gx, gp);
#pragma unroll
            for (int i = 0; i < N; i++) {
                ybar[i] += gx[i];
#pragma unroll
                for (int k = 0; k < NS - 1; k++)
                    if (k < m)
                        Kbar[k][i] += gx[i] * Tab::a(m, k) * h;
            }
#pragma unroll
            for (int k = 0; k < P; k++)
                mu[k] += gp[k];
        }
#pragma unroll
        for (int i = 0; i < N; i++)
            lam[i] = ybar[i];
    } else {
        // Same recurrence with stage-precision seeds and VJPs; the per-step
        // sums of J^T Kbar are added to the FP64 lambda / mu once per step.
        const S sdt = shh;
        S sl[N];
#pragma unroll
        for (int i = 0; i < N; i++)
            sl[i] = from_d<S>(lam[i]);
#pragma unroll
        for (int m = 0; m < NS; m++) {
            const S bh = S(Tab::b(m)) * sdt;
#pragma unroll
            for (int i = 0; i < N; i++)
                Kbar[m][i] = bh * sl[i];
        }
        S dx[N], dp[P];
#pragma unroll
        for (int m = NS - 1; m >= 0; m--) {
            S gx[N], gp[P];
            M::template vjp<S>(Kbar[m], X[m], p, from_d<S>(tn + Tab::c(m) * h), gx, gp);
#pragma unroll
            for (int i = 0; i < N; i++) {
                dx[i] = m == NS - 1 ? gx[i] : dx[i] + gx[i];
#pragma unroll
                for (int k = 0; k < NS - 1; k++)
                    if (k < m)
                        Kbar[k][i] = madd(gx[i] * S(Tab::a(m, k)), sdt, Kbar[k][i]);
            }
#pragma unroll
            for (int k = 0; k < P; k++)
                dp[k] = m == NS - 1 ? gp[k] : dp[k] + gp[k];
        }
#pragma unroll
        for (int i = 0; i < N; i++)
            lam[i] += to_d(dx[i]);
#pragma unroll
        for (int k = 0; k < P; k++)
            mu[k] += to_d(dp[k]);
    }
}

template <class M, class Tab, class S>
__global__ void __launch_bounds__(256) backward_kernel(AdjParams a)
{
    constexpr int N = M::N, P = M::P;
    constexpr int RS = record_doubles(N);
    const int CH = a.pool.chunk_len;

    int b = -1, q = 0, j = -1, chunk = -1, slot = 0, T = 0, last = -1;
    double lam[N], mu[P], t_next = 0.0;
    S p[P];
    bool alive = true, live = false;

    // Position the walk on record T of instance b and seed cost q.
    auto start_seed = [&]() {
        chunk = last;
        slot = T % a.pool.chunk_len;
        double yTl[N];
        read_record<N>(record_ptr<RS>(a.pool, chunk, slot), t_next, yTl);
        const size_t o = ((size_t)b * a.nout + q);
#pragma unroll
        for (int i = 0; i < N; i++) {
            if (a.cost == 0)
                lam[i] = 2.0 * yTl[i];
            else if (a.cost == 1)
                lam[i] = 1.0;
            else
                lam[i] = a.lambdaT[o * N + i];
        }
#pragma unroll
        for (int k = 0; k < P; k++)
            mu[k] = 0.0;
        note_lambda<N>(a, b, q, T, lam);
        j = T - 1;
    };

    auto fetch = [&]() -> bool {
        for (;;) {
            unsigned w = atomicAdd(&a.ctl->adj_next, 1u);
            if ((int)w >= a.B)
                return false;
            b = a.order ? a.order[w] : (int)w;
            const int st = a.inst_status[b];
            if (st != ST_OK) {
                // no trajectory to differentiate: report the forward status
                for (int qq = 0; qq < a.nout; qq++) {
                    const size_t o = ((size_t)b * a.nout + qq);
                    for (int i = 0; i < N; i++)
                        a.dy0[o * N + i] = __longlong_as_double(0x7ff8000000000000ll);
                    for (int k = 0; k < P; k++)
                        a.dpar[o * P + k] = __longlong_as_double(0x7ff8000000000000ll);
                }
                if (a.status_out)
                    a.status_out[b] = st;
                continue;
            }
#pragma unroll
            for (int k = 0; k < P; k++)
                p[k] = from_d<S>(a.par[(size_t)b * P + k]);
            T = a.inst_T[b];
            last = a.inst_last[b];
            q = 0;
            start_seed();
            return true;
        }
    };

    auto finish_seed = [&]() {
        const size_t o = ((size_t)b * a.nout + q);
        bool finite = true;
#pragma unroll
        for (int i = 0; i < N; i++) {
            a.dy0[o * N + i] = lam[i];
            finite = finite && isfinite(lam[i]);
        }
#pragma unroll
        for (int k = 0; k < P; k++) {
            // mu_direct + accumulated alphabar (backpropagation.hpp:317-321)
            const double d = a.mu_direct ? a.mu_direct[o * P + k] : 0.0;
            a.dpar[o * P + k] = d + mu[k];
            finite = finite && isfinite(mu[k]);
        }
        if (a.status_out && (q == a.nout - 1 || !finite))
            a.status_out[b] = finite ? ST_OK : ST_NONFINITE;
    };

    live = fetch();
    alive = live;
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
        // step back to record j
        if (slot == 0) {
            chunk = a.pool.chunk_prev[chunk];
            slot = CH - 1;
        } else {
            slot--;
        }
        double y[N], tn;
        read_record<N>(record_ptr<RS>(a.pool, chunk, slot), tn, y);
        const double h = t_next - tn;
        back_step<M, Tab, S>(y, tn, h, p, lam, mu);
        note_lambda<N>(a, b, q, j, lam);
        t_next = tn;
        j--;
    }
}

// --------------------------------------------- backward sweep, two levels

// Backward sweep over checkpoints stored every `stride` accepted steps (plus
// the last).  For each segment, last first: re-run the forward controller
// from the segment's checkpoint (t, dt, y) -- the same device code, so the
// same bits -- for the segment's accepted steps into this thread's scratch,
// check that it lands exactly on the next checkpoint's t and y, then run
// back_step through the segment in reverse.  Memory: one record per stride
// steps plus (stride + 1) scratch records per thread, for one extra forward
// evaluation of every step.
template <class M, class Tab, class S>
__global__ void __launch_bounds__(256) backward_kernel_2level(AdjParams a)
{
    constexpr int N = M::N, P = M::P;
    constexpr int RS = record_doubles(N);
    const int CH = a.pool.chunk_len, SK = a.stride;
    double *scr = a.scratch + ((size_t)blockIdx.x * blockDim.x + threadIdx.x) * (SK + 1) * RS;

    int b = -1, q = 0, T = 0, R = 0, k = 0, last = -1, chunk = -1, slot = 0, L = 0, done = 0, jb = 0, fails = 0;
    int first = 0;          // step index of the segment's first record
    double t_start = 0.0;   // t_0 (fixed-step tableaux)
    int phase = 0; // 0: re-integrate segment k, 1: back-step through it
    double lam[N], mu[P], t = 0.0, dt = 0.0, t1 = 0.0, y[N], t_end = 0.0, y_end[N];
    S p[P], ys[N], k0[N];
    bool at_top = true;

    // Record r of the instance: chunk r / CH of its chain.  The walk only
    // moves backwards, one record at a time.
    auto step_back = [&]() {
        if (slot == 0) {
            chunk = a.pool.chunk_prev[chunk];
            slot = CH - 1;
        } else {
            slot--;
        }
    };

    auto fail_instance = [&](int st) {
        for (int qq = 0; qq < a.nout; qq++) {
            const size_t o = ((size_t)b * a.nout + qq);
            for (int i = 0; i < N; i++)
                a.dy0[o * N + i] = __longlong_as_double(0x7ff8000000000000ll);
            for (int kk = 0; kk < P; kk++)
                a.dpar[o * P + kk] = __longlong_as_double(0x7ff8000000000000ll);
        }
        if (a.status_out)
            a.status_out[b] = st;
    };

    // Load the start of segment k (the walk is on record k + 1) and set up
    // its re-integration.
    auto begin_segment = [&]() {
        step_back();
        double rec_t, rec_y[N];
        const double *r = record_ptr<RS>(a.pool, chunk, slot);
        read_record<N>(r, rec_t, rec_y);
        t = rec_t;
        dt = r[1];
        first = k * SK;
        L = (k == R - 2) ? T - first : SK;
#pragma unroll
        for (int i = 0; i < N; i++) {
            y[i] = rec_y[i];
            ys[i] = from_d<S>(y[i]);
            scr[2 + i] = y[i];
        }
        scr[0] = t;
        M::template rhs<S>(ys, p, from_d<S>(t), k0);
        done = 0;
        fails = 0;
        at_top = true;
        phase = 0;
    };

    auto start_seed = [&]() {
        chunk = last;
        slot = (R - 1) % CH;
        double yTl[N];
        read_record<N>(record_ptr<RS>(a.pool, chunk, slot), t_end, yTl);
        const size_t o = ((size_t)b * a.nout + q);
#pragma unroll
        for (int i = 0; i < N; i++) {
            y_end[i] = yTl[i];
            lam[i] = a.cost == 0 ? 2.0 * yTl[i] : a.cost == 1 ? 1.0 : a.lambdaT[o * N + i];
        }
#pragma unroll
        for (int kk = 0; kk < P; kk++)
            mu[kk] = 0.0;
        note_lambda<N>(a, b, q, T, lam);
        k = R - 2;
        if (k >= 0)
            begin_segment();
    };

    auto finish_seed = [&](int st) {
        const size_t o = ((size_t)b * a.nout + q);
        bool finite = st == ST_OK;
#pragma unroll
        for (int i = 0; i < N; i++) {
            a.dy0[o * N + i] = st == ST_OK ? lam[i] : __longlong_as_double(0x7ff8000000000000ll);
            finite = finite && isfinite(lam[i]);
        }
#pragma unroll
        for (int kk = 0; kk < P; kk++) {
            const double d = a.mu_direct ? a.mu_direct[o * P + kk] : 0.0;
            a.dpar[o * P + kk] = st == ST_OK ? d + mu[kk] : __longlong_as_double(0x7ff8000000000000ll);
            finite = finite && isfinite(mu[kk]);
        }
        if (a.status_out && (q == a.nout - 1 || !finite))
            a.status_out[b] = st != ST_OK ? st : (finite ? ST_OK : ST_NONFINITE);
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
                p[kk] = from_d<S>(a.par[(size_t)b * P + kk]);
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
            finish_seed(ST_OK);
            if (q + 1 < a.nout) {
                q++;
                start_seed();
            } else {
                alive = fetch();
            }
            continue;
        }
        if (phase == 0) {
            // one attempt of the forward controller, as forward_kernel does
            if (at_top) {
                if (!Tab::FIXED && (t + dt) - t1 > kDblEps)
                    dt = t1 - t;
                fails = 0;
                at_top = false;
            }
            double ynew[N];
            S ynew_s[N], knew[N];
            const double err = attempt<M, Tab, S>(y, ys, k0, p, t, dt, a.atol, a.rtol, ynew, ynew_s, knew);
            if (err != err || fails >= a.max_fail) {
                fail_instance(ST_RECOMPUTE_MISMATCH);
                alive = fetch();
                continue;
            }
            fails++;
            if (err > 1.0) {
                dt = decrease_step<Tab, S>(dt, err, a.step_pow, &a.ctl->pow_undecided);
                continue;
            }
            if constexpr (Tab::FIXED) {
                t = fixed_time(t_start, first + done + 1, dt);
            } else {
                t += dt;
                dt = increase_step<Tab, S>(dt, err, a.step_pow, &a.ctl->pow_undecided);
            }
            accept_state<M, Tab, S>(y, ys, k0, ynew, ynew_s, knew, p, t);
            at_top = true;
            done++;
            double *r = scr + (size_t)done * RS;
            r[0] = t;
#pragma unroll
            for (int i = 0; i < N; i++)
                r[2 + i] = y[i];
            if (done == L) {
                // the re-integration must land exactly on the next checkpoint
                bool same = t == t_end;
#pragma unroll
                for (int i = 0; i < N; i++)
                    same = same && y[i] == y_end[i];
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
            const double *r = scr + (size_t)jb * RS;
            double yj[N];
#pragma unroll
            for (int i = 0; i < N; i++)
                yj[i] = r[2 + i];
            const double tn = r[0];
            const double h = scr[(size_t)(jb + 1) * RS] - tn;
            back_step<M, Tab, S>(yj, tn, h, p, lam, mu);
            note_lambda<N>(a, b, q, first + jb, lam);
            jb--;
            if (jb < 0) {
                // the segment's start becomes the next segment's end
                t_end = scr[0];
#pragma unroll
                for (int i = 0; i < N; i++)
                    y_end[i] = scr[2 + i];
                k--;
                if (k >= 0)
                    begin_segment();
            }
        }
    }
}

} // namespace va
