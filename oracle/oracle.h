/*
 * CPU oracle for the discrete adjoint of controlled explicit Runge-Kutta
 * integration.  TEST INFRASTRUCTURE ONLY: this code is the checker that the
 * CUDA product path is compared against (tests, smoke check, bench CPU
 * baseline).  Nothing in the product library links or calls it.
 *
 * It restates, in plain C99 and FP64, the reference's algorithm:
 *   - forward loop  : lib/include/detail/runge_kutta.hpp:137-180
 *                     (end clamp, retry loop, failed_step_checker, record of
 *                      every accepted (t_n, y_n))
 *   - controller    : Boost.odeint 1.74.0 controlled_runge_kutta::try_step,
 *                     default_error_checker and default_step_adjuster
 *                     (third-party, not vendored with the reference; restated
 *                      from its published formulas)
 *   - tableaux      : Cash-Karp 5(4) as in lib/include/ButcherTable.hpp:259-308
 *                     (coefficients from Cash & Karp 1990), Dormand-Prince 5(4)
 *                     (Dormand & Prince 1980; absent from the reference's
 *                      ButcherTable, added here from the published tableau),
 *                     Fehlberg 7(8) as in ButcherTable.hpp:191-246 (odeint's
 *                     runge_kutta_fehlberg78; coefficients from Fehlberg 1968);
 *                     fixed-step runge_kutta4 and euler (ButcherTable.hpp:39-125)
 *                     with the fixed-step loop of detail/runge_kutta.hpp:37-72
 *   - adjoint       : lib/include/detail/backpropagation.hpp:24-81 (stage
 *                     recompute), :160-229 (back_prop_step), :256-278
 *                     (back_prop), :280-348 (seed / write-back semantics)
 *   - step size     : h_n = t_{n+1} - t_n, lib/include/StateStorage.hpp:22
 *   - models        : VdP (lib example form examples/VanDerPol/main.cpp:38-43
 *                     and the Lienard form), damped oscillator, generalized
 *                     Lotka-Volterra examples/GeneralizedLotkaVolterra/main.cpp:105-119
 *                     (parameter layout p[N(i+1)+j] = A_ij).
 *
 * Pinning: the adjoint side is checked against the reference's own headers
 * compiled here with a Boost shim and the shipped AADC runtime
 * (oracle/ref/, golden fixtures under tests/golden/).  The forward controller
 * lives in Boost.odeint 1.74.0, which is not available in this container, so
 * forward-sweep parity with real odeint is unpinned (the shim restates the
 * same formulas).
 *
 * Stage times are t_n + c_m h (the reference evaluates every recomputed stage
 * at t_n, detail/backpropagation.hpp:48, which only matters for
 * non-autonomous right-hand sides; all models here are autonomous).
 */
#ifndef VA_ORACLE_H
#define VA_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
    ORC_MODEL_VDP = 0,       /* x0' = x1, x1' = mu (1 - x0^2) x1 - x0           */
    ORC_MODEL_VDP_PETSC = 1, /* x0' = x1, x1' = mu ((1 - x0^2) x1 - x0)         */
    ORC_MODEL_DHO = 2,       /* x' = v, v' = -w^2 x - 2 z w v, p = (w, z)       */
    ORC_MODEL_GLV = 3,       /* x_i' = x_i (r_i + sum_j A_ij x_j), p = (r, A)  */
    ORC_MODEL_DECAY = 4,     /* y_i' = -p_i y_i (analytic test model)          */
    ORC_MODEL_USER = 6       /* the callbacks user_rhs / user_vjp of orc_problem */
};

enum { ORC_TAB_DOPRI5 = 0, ORC_TAB_CK54 = 1, ORC_TAB_RKF78 = 2, ORC_TAB_RK4 = 3, ORC_TAB_EULER = 4 };

enum { ORC_COST_SUMSQ = 0, ORC_COST_SUM = 1 };

enum {
    ORC_OK = 0,
    ORC_MAX_REJECTS = 1, /* failed_step_checker limit exceeded        */
    ORC_MAX_STEPS = 2,   /* checkpoint capacity (max_steps) exceeded  */
    ORC_NONFINITE = 3,
    ORC_BAD_ARGS = 5
};

typedef struct {
    int model;
    int tableau;
    int n;         /* state dimension                         */
    int npar;      /* parameter count                         */
    double atol, rtol;
    double dt0;    /* initial step                            */
    long max_steps;/* accepted-step capacity                  */
    int max_fail;  /* consecutive failed attempts (odeint 500) */
    int pow_mode;  /* step-size factor err^(-1.0/k): 0 = fixed IEEE-only Newton
                      scheme shared with the CUDA library's fast controller
                      (bit-comparable), 1 = the C library's pow (as odeint's
                      std::pow), 2 = the correctly rounded pow (binary128
                      evaluation rounded once; the CUDA library's
                      reference-parity controller gives the same values) */
    /* ORC_MODEL_USER: f = rhs(x, p, t) and (gx, gp) = (J_x^T w, J_p^T w) */
    void (*user_rhs)(const double *x, const double *p, double t, double *f);
    void (*user_vjp)(const double *w, const double *x, const double *p, double t, double *gx, double *gp);
} orc_problem;

/* Trace of the C library's pow in pow_mode 1: calls, calls whose result is
 * not the correctly rounded power (checked against the binary128 value), and
 * the accepted-step index and argument of the first such call (-1, 0: none).
 * orc_set_powtrace(tr) zeroes *tr and traces the calling thread's later
 * forward sweeps into it; NULL stops tracing. */
typedef struct {
    long calls, noncr, first_noncr_step, step;
    double first_noncr_arg;
} orc_powtrace;
void orc_set_powtrace(orc_powtrace *tr);

/* The step-size factor pow(a, -1.0/k) in the given pow_mode (a >= 1e30: 0). */
double orc_step_pow(double a, int k, int pow_mode);

/* Right-hand side and vector-Jacobian product of the built-in models. */
void orc_rhs(const orc_problem *pb, const double *x, const double *p, double t, double *f);
void orc_vjp(const orc_problem *pb, const double *w, const double *x, const double *p, double t,
             double *gx, double *gp);

/* Forward sweep.  times[0..T], states[(T+1)*n] receive every accepted
 * (t_n, y_n); dt_trial[0..T-1] (may be NULL) the trial step at the top of
 * each loop iteration.  cap = capacity in accepted steps. */
int orc_forward(const orc_problem *pb, const double *y0, const double *p, double t0, double t1,
                long cap, double *times, double *states, double *dt_trial, double *yT,
                long *n_acc, long *n_rej);

/* Frozen-step replay of a recorded step sequence (h_n = t_{n+1} - t_n). */
void orc_forward_frozen(const orc_problem *pb, const double *y0, const double *p, long T,
                        const double *times, double *yT);

/* Discrete adjoint.  lambda[nout][n]: in = dG/dy(T), out = dG/dy0.
 * mu[nout][npar]: in = direct partials dG/dp, out = total dG/dp. */
int orc_adjoint(const orc_problem *pb, const double *p, long T, const double *times,
                const double *states, int nout, double *lambda, double *mu);

/* orc_adjoint that also stores lambda_n of every seed, n = 0 .. T, in
 * hist[nout][T+1][n] (the values back_prop's observer sees,
 * detail/backpropagation.hpp:256-278); hist may be NULL. */
int orc_adjoint_history(const orc_problem *pb, const double *p, long T, const double *times,
                        const double *states, int nout, double *lambda, double *mu, double *hist);

/* One gradient (forward + adjoint) for a built-in scalar cost. */
int orc_gradient(const orc_problem *pb, int cost, const double *y0, const double *p, double t0,
                 double t1, double *yT, double *dy0, double *dp, long *n_acc, long *n_rej);

/* Checkpoint bytes of one gradient: stored by the forward sweep (a time
 * and a state per accepted point) and read back by the adjoint sweep. */
typedef struct {
    long long store_bytes, load_bytes;
} orc_traffic;

/* orc_gradient that counts its checkpoint traffic into *traffic. */
int orc_gradient_traffic(const orc_problem *pb, int cost, const double *y0, const double *p, double t0,
                         double t1, long *n_acc, orc_traffic *traffic);

/* B independent gradients over nthreads POSIX threads (static partition). */
int orc_gradient_batch(const orc_problem *pb, int cost, long B, const double *y0, const double *p,
                       const double *t0, const double *t1, int nthreads, double *yT, double *dy0,
                       double *dp, long *n_acc, long *n_rej, int *status);

#ifdef __cplusplus
}
#endif
#endif
