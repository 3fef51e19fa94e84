/*
 * CPU oracle (test infrastructure only) -- see oracle.h for what it restates
 * and where each part comes from in the reference.  Compiled with
 * -ffp-contract=off so that every product and sum is rounded separately, in
 * the operation order of the reference / Boost.odeint expressions.
 */
#include "oracle.h"
#if !(defined(__aarch64__) || (defined(__LDBL_MANT_DIG__) && __LDBL_MANT_DIG__ == 113))
#include <quadmath.h>
#endif

#include <float.h>
#include <stdint.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define SMAX 16  /* largest stage count (Fehlberg 7(8): 13) */
#define NMAX 256 /* largest state dimension */

typedef struct {
    int s;                 /* stages that feed y_{n+1}                        */
    int fsal;              /* derivative at the new point is the next k_1     */
    double a[SMAX][SMAX];  /* strictly lower triangular                       */
    double b[SMAX];        /* higher-order weights                            */
    double c[SMAX];
    double e[SMAX];        /* error weights on k_1..k_s                       */
    double e_new;          /* error weight on f(y_{n+1}) (FSAL stage)        */
    int error_order;       /* odeint error_order_value                        */
    int stepper_order;     /* odeint stepper_order_value                      */
    int fixed;             /* no error estimate: fixed-step loop              */
} tableau;

/* Checkpoint traffic counter of orc_gradient_traffic: the bytes the
 * reference's StateStorage (StateStorage.hpp:4-43) stores in the forward --
 * one time and one state per accepted (t_n, y_n), n = 0 .. T -- and the
 * bytes the adjoint reads back per step (t_n, t_{n+1} for h_n, and y_n). */
static __thread orc_traffic *g_traffic = NULL;

static void count_store(int n)
{
    if (g_traffic)
        g_traffic->store_bytes += (long long)sizeof(double) * (1 + n);
}

/* Cash-Karp 5(4): Cash & Karp (1990), the coefficients the reference reads
 * through odeint's rk54_ck_coefficients_* (ButcherTable.hpp:259-308). */
static void tab_ck54(tableau *T)
{
    memset(T, 0, sizeof(*T));
    T->s = 6;
    T->fsal = 0;
    T->a[1][0] = 1.0 / 5.0;
    T->a[2][0] = 3.0 / 40.0;
    T->a[2][1] = 9.0 / 40.0;
    T->a[3][0] = 3.0 / 10.0;
    T->a[3][1] = -9.0 / 10.0;
    T->a[3][2] = 6.0 / 5.0;
    T->a[4][0] = -11.0 / 54.0;
    T->a[4][1] = 5.0 / 2.0;
    T->a[4][2] = -70.0 / 27.0;
    T->a[4][3] = 35.0 / 27.0;
    T->a[5][0] = 1631.0 / 55296.0;
    T->a[5][1] = 175.0 / 512.0;
    T->a[5][2] = 575.0 / 13824.0;
    T->a[5][3] = 44275.0 / 110592.0;
    T->a[5][4] = 253.0 / 4096.0;
    T->b[0] = 37.0 / 378.0;
    T->b[1] = 0.0;
    T->b[2] = 250.0 / 621.0;
    T->b[3] = 125.0 / 594.0;
    T->b[4] = 0.0;
    T->b[5] = 512.0 / 1771.0;
    T->c[0] = 0.0;
    T->c[1] = 1.0 / 5.0;
    T->c[2] = 3.0 / 10.0;
    T->c[3] = 3.0 / 5.0;
    T->c[4] = 1.0;
    T->c[5] = 7.0 / 8.0;
    /* b - b_hat, each difference of two rounded quotients */
    T->e[0] = 37.0 / 378.0 - 2825.0 / 27648.0;
    T->e[1] = 0.0;
    T->e[2] = 250.0 / 621.0 - 18575.0 / 48384.0;
    T->e[3] = 125.0 / 594.0 - 13525.0 / 55296.0;
    T->e[4] = -277.0 / 14336.0;
    T->e[5] = 512.0 / 1771.0 - 1.0 / 4.0;
    T->e_new = 0.0;
    T->error_order = 4;
    T->stepper_order = 5;
}

/* Dormand-Prince 5(4): Dormand & Prince (1980).  Seven stages, the seventh
 * (b_7 = 0) is f(y_{n+1}) and is reused as the next step's first stage. */
static void tab_dopri5(tableau *T)
{
    memset(T, 0, sizeof(*T));
    T->s = 6;
    T->fsal = 1;
    T->a[1][0] = 1.0 / 5.0;
    T->a[2][0] = 3.0 / 40.0;
    T->a[2][1] = 9.0 / 40.0;
    T->a[3][0] = 44.0 / 45.0;
    T->a[3][1] = -56.0 / 15.0;
    T->a[3][2] = 32.0 / 9.0;
    T->a[4][0] = 19372.0 / 6561.0;
    T->a[4][1] = -25360.0 / 2187.0;
    T->a[4][2] = 64448.0 / 6561.0;
    T->a[4][3] = -212.0 / 729.0;
    T->a[5][0] = 9017.0 / 3168.0;
    T->a[5][1] = -355.0 / 33.0;
    T->a[5][2] = 46732.0 / 5247.0;
    T->a[5][3] = 49.0 / 176.0;
    T->a[5][4] = -5103.0 / 18656.0;
    T->b[0] = 35.0 / 384.0;
    T->b[1] = 0.0;
    T->b[2] = 500.0 / 1113.0;
    T->b[3] = 125.0 / 192.0;
    T->b[4] = -2187.0 / 6784.0;
    T->b[5] = 11.0 / 84.0;
    T->c[0] = 0.0;
    T->c[1] = 1.0 / 5.0;
    T->c[2] = 3.0 / 10.0;
    T->c[3] = 4.0 / 5.0;
    T->c[4] = 8.0 / 9.0;
    T->c[5] = 1.0;
    T->e[0] = 35.0 / 384.0 - 5179.0 / 57600.0;
    T->e[1] = 0.0;
    T->e[2] = 500.0 / 1113.0 - 7571.0 / 16695.0;
    T->e[3] = 125.0 / 192.0 - 393.0 / 640.0;
    T->e[4] = -2187.0 / 6784.0 - -92097.0 / 339200.0;
    T->e[5] = 11.0 / 84.0 - 187.0 / 2100.0;
    T->e_new = -1.0 / 40.0;
    T->error_order = 4;
    T->stepper_order = 5;
}

/* Fehlberg 7(8): E. Fehlberg, "Classical fifth-, sixth-, seventh-, and
 * eighth-order Runge-Kutta formulas with stepsize control", NASA TR R-287
 * (1968).  Thirteen stages; the eighth-order weights propagate (odeint's
 * runge_kutta_fehlberg78, read by the reference's ButcherTable.hpp:191-246),
 * the error weights are b8 - b7, nonzero on k_1, k_11, k_12, k_13. */
static void tab_rkf78(tableau *T)
{
    memset(T, 0, sizeof(*T));
    T->s = 13;
    T->fsal = 0;
    T->a[1][0] = 2.0 / 27.0;
    T->a[2][0] = 1.0 / 36.0;
    T->a[2][1] = 1.0 / 12.0;
    T->a[3][0] = 1.0 / 24.0;
    T->a[3][2] = 1.0 / 8.0;
    T->a[4][0] = 5.0 / 12.0;
    T->a[4][2] = -25.0 / 16.0;
    T->a[4][3] = 25.0 / 16.0;
    T->a[5][0] = 1.0 / 20.0;
    T->a[5][3] = 1.0 / 4.0;
    T->a[5][4] = 1.0 / 5.0;
    T->a[6][0] = -25.0 / 108.0;
    T->a[6][3] = 125.0 / 108.0;
    T->a[6][4] = -65.0 / 27.0;
    T->a[6][5] = 125.0 / 54.0;
    T->a[7][0] = 31.0 / 300.0;
    T->a[7][4] = 61.0 / 225.0;
    T->a[7][5] = -2.0 / 9.0;
    T->a[7][6] = 13.0 / 900.0;
    T->a[8][0] = 2.0;
    T->a[8][3] = -53.0 / 6.0;
    T->a[8][4] = 704.0 / 45.0;
    T->a[8][5] = -107.0 / 9.0;
    T->a[8][6] = 67.0 / 90.0;
    T->a[8][7] = 3.0;
    T->a[9][0] = -91.0 / 108.0;
    T->a[9][3] = 23.0 / 108.0;
    T->a[9][4] = -976.0 / 135.0;
    T->a[9][5] = 311.0 / 54.0;
    T->a[9][6] = -19.0 / 60.0;
    T->a[9][7] = 17.0 / 6.0;
    T->a[9][8] = -1.0 / 12.0;
    T->a[10][0] = 2383.0 / 4100.0;
    T->a[10][3] = -341.0 / 164.0;
    T->a[10][4] = 4496.0 / 1025.0;
    T->a[10][5] = -301.0 / 82.0;
    T->a[10][6] = 2133.0 / 4100.0;
    T->a[10][7] = 45.0 / 82.0;
    T->a[10][8] = 45.0 / 164.0;
    T->a[10][9] = 18.0 / 41.0;
    T->a[11][0] = 3.0 / 205.0;
    T->a[11][5] = -6.0 / 41.0;
    T->a[11][6] = -3.0 / 205.0;
    T->a[11][7] = -3.0 / 41.0;
    T->a[11][8] = 3.0 / 41.0;
    T->a[11][9] = 6.0 / 41.0;
    T->a[12][0] = -1777.0 / 4100.0;
    T->a[12][3] = -341.0 / 164.0;
    T->a[12][4] = 4496.0 / 1025.0;
    T->a[12][5] = -289.0 / 82.0;
    T->a[12][6] = 2193.0 / 4100.0;
    T->a[12][7] = 51.0 / 82.0;
    T->a[12][8] = 33.0 / 164.0;
    T->a[12][9] = 12.0 / 41.0;
    T->a[12][11] = 1.0;
    T->b[5] = 34.0 / 105.0;
    T->b[6] = 9.0 / 35.0;
    T->b[7] = 9.0 / 35.0;
    T->b[8] = 9.0 / 280.0;
    T->b[9] = 9.0 / 280.0;
    T->b[11] = 41.0 / 840.0;
    T->b[12] = 41.0 / 840.0;
    T->c[1] = 2.0 / 27.0;
    T->c[2] = 1.0 / 9.0;
    T->c[3] = 1.0 / 6.0;
    T->c[4] = 5.0 / 12.0;
    T->c[5] = 1.0 / 2.0;
    T->c[6] = 5.0 / 6.0;
    T->c[7] = 1.0 / 6.0;
    T->c[8] = 2.0 / 3.0;
    T->c[9] = 1.0 / 3.0;
    T->c[10] = 1.0;
    T->c[12] = 1.0;
    T->e[0] = -41.0 / 840.0;
    T->e[10] = -41.0 / 840.0;
    T->e[11] = 41.0 / 840.0;
    T->e[12] = 41.0 / 840.0;
    T->e_new = 0.0;
    T->error_order = 7;
    T->stepper_order = 8;
}

/* Fixed-step steppers the reference's ButcherTable accepts
 * (ButcherTable.hpp:39-125): odeint's runge_kutta4 (classic fourth-order
 * tableau) and euler. */
static void tab_rk4(tableau *T)
{
    memset(T, 0, sizeof(*T));
    T->s = 4;
    T->a[1][0] = 1.0 / 2.0;
    T->a[2][1] = 1.0 / 2.0;
    T->a[3][2] = 1.0;
    T->b[0] = 1.0 / 6.0;
    T->b[1] = 1.0 / 3.0;
    T->b[2] = 1.0 / 3.0;
    T->b[3] = 1.0 / 6.0;
    T->c[1] = 1.0 / 2.0;
    T->c[2] = 1.0 / 2.0;
    T->c[3] = 1.0;
    T->stepper_order = 4;
    T->fixed = 1;
}

static void tab_euler(tableau *T)
{
    memset(T, 0, sizeof(*T));
    T->s = 1;
    T->b[0] = 1.0;
    T->stepper_order = 1;
    T->fixed = 1;
}

static int get_tableau(int id, tableau *T)
{
    if (id == ORC_TAB_DOPRI5) {
        tab_dopri5(T);
        return 0;
    }
    if (id == ORC_TAB_CK54) {
        tab_ck54(T);
        return 0;
    }
    if (id == ORC_TAB_RKF78) {
        tab_rkf78(T);
        return 0;
    }
    if (id == ORC_TAB_RK4) {
        tab_rk4(T);
        return 0;
    }
    if (id == ORC_TAB_EULER) {
        tab_euler(T);
        return 0;
    }
    return -1;
}

/* ------------------------------------------------------------------ models */

void orc_rhs(const orc_problem *pb, const double *x, const double *p, double t, double *f)
{
    (void)t;
    int n = pb->n;
    switch (pb->model) {
    case ORC_MODEL_VDP:
        f[0] = x[1];
        f[1] = p[0] * (1.0 - x[0] * x[0]) * x[1] - x[0];
        break;
    case ORC_MODEL_VDP_PETSC: /* examples/VanDerPol/main.cpp:41-42 */
        f[0] = x[1];
        f[1] = p[0] * ((1.0 - x[0] * x[0]) * x[1] - x[0]);
        break;
    case ORC_MODEL_DHO:
        f[0] = x[1];
        f[1] = -p[0] * p[0] * x[0] - 2.0 * p[1] * p[0] * x[1];
        break;
    case ORC_MODEL_GLV: /* examples/GeneralizedLotkaVolterra/main.cpp:109-118 */
        for (int i = 0; i < n; i++) {
            double sum = 0.0;
            for (int j = 0; j < n; j++)
                sum += p[n * (i + 1) + j] * x[j];
            f[i] = x[i] * (p[i] + sum);
        }
        break;
    case ORC_MODEL_DECAY:
        for (int i = 0; i < n; i++)
            f[i] = -p[i] * x[i];
        break;
    case ORC_MODEL_USER:
        pb->user_rhs(x, p, t, f);
        break;
    }
}

/* gx = J_x^T w, gp = J_p^T w (overwritten, not accumulated). */
void orc_vjp(const orc_problem *pb, const double *w, const double *x, const double *p, double t,
             double *gx, double *gp)
{
    (void)t;
    int n = pb->n;
    switch (pb->model) {
    case ORC_MODEL_VDP: {
        double mu = p[0];
        gx[0] = w[1] * (-2.0 * mu * x[0] * x[1] - 1.0);
        gx[1] = w[0] + w[1] * (mu * (1.0 - x[0] * x[0]));
        gp[0] = w[1] * ((1.0 - x[0] * x[0]) * x[1]);
        break;
    }
    case ORC_MODEL_VDP_PETSC: {
        double mu = p[0];
        gx[0] = w[1] * (mu * (-2.0 * x[0] * x[1] - 1.0));
        gx[1] = w[0] + w[1] * (mu * (1.0 - x[0] * x[0]));
        gp[0] = w[1] * ((1.0 - x[0] * x[0]) * x[1] - x[0]);
        break;
    }
    case ORC_MODEL_DHO: {
        double om = p[0], ze = p[1];
        gx[0] = w[1] * (-om * om);
        gx[1] = w[0] + w[1] * (-2.0 * ze * om);
        gp[0] = w[1] * (-2.0 * om * x[0] - 2.0 * ze * x[1]);
        gp[1] = w[1] * (-2.0 * om * x[1]);
        break;
    }
    case ORC_MODEL_GLV: {
        /* f_i = x_i s_i,  s_i = r_i + sum_j A_ij x_j
         * gx_k = w_k s_k + sum_i A_ik w_i x_i ; gr_i = w_i x_i ; gA_ij = w_i x_i x_j */
        for (int k = 0; k < n; k++) {
            double sum = 0.0;
            for (int j = 0; j < n; j++)
                sum += p[n * (k + 1) + j] * x[j];
            gx[k] = w[k] * (p[k] + sum);
        }
        for (int i = 0; i < n; i++) {
            double v = w[i] * x[i];
            gp[i] = v;
            for (int k = 0; k < n; k++) {
                gx[k] += p[n * (i + 1) + k] * v;
                gp[n * (i + 1) + k] = v * x[k];
            }
        }
        break;
    }
    case ORC_MODEL_DECAY:
        for (int i = 0; i < n; i++) {
            gx[i] = -p[i] * w[i];
            gp[i] = -x[i] * w[i];
        }
        break;
    case ORC_MODEL_USER:
        pb->user_vjp(w, x, p, t, gx, gp);
        break;
    }
}

/* ------------------------------------------------------------- controller */

/* odeint detail::less_with_sign for dt > 0: t2 - t1 > epsilon */
static int less_with_sign(double t1, double t2) { return t2 - t1 > DBL_EPSILON; }

/* One odeint error-stepper step from (x, dxdt, t) with step dt.  Writes the
 * new state, the derivative at the new point (FSAL tableaux only) and the
 * error vector.  K[0] must hold dxdt on entry. */
static void rk_error_step(const orc_problem *pb, const tableau *T, const double *x, double t,
                          double dt, const double *p, double K[SMAX][NMAX], double *out,
                          double *dxdt_new, double *xerr, double *xtmp)
{
    int n = pb->n;
    for (int m = 1; m < T->s; m++) {
        for (int i = 0; i < n; i++) {
            double acc = x[i];
            for (int j = 0; j < m; j++)
                acc = acc + (T->a[m][j] * dt) * K[j][i];
            xtmp[i] = acc;
        }
        orc_rhs(pb, xtmp, p, t + T->c[m] * dt, K[m]);
    }
    for (int i = 0; i < n; i++) {
        double acc = x[i];
        for (int j = 0; j < T->s; j++)
            if (T->b[j] != 0.0)
                acc = acc + (T->b[j] * dt) * K[j][i];
        out[i] = acc;
    }
    if (T->fsal)
        orc_rhs(pb, out, p, t + dt, dxdt_new);
    for (int i = 0; i < n; i++) {
        double acc = 0.0;
        int first = 1;
        for (int j = 0; j < T->s; j++) {
            if (T->e[j] == 0.0)
                continue; /* an exact zero term leaves the sum unchanged */
            double term = (T->e[j] * dt) * K[j][i];
            acc = first ? term : acc + term;
            first = 0;
        }
        if (T->fsal)
            acc = acc + (T->e_new * dt) * dxdt_new[i];
        xerr[i] = acc;
    }
}

/* default_error_checker::error with a_x = a_dxdt = 1: max-norm of
 * |err_i| / (atol + rtol (|x_i| + |dt| |dxdt_i|)) at the step start. */
static double error_norm(const orc_problem *pb, const double *x, const double *dxdt,
                         const double *xerr, double dt)
{
    double m = 0.0;
    double adt = fabs(dt);
    for (int i = 0; i < pb->n; i++) {
        double r = fabs(xerr[i]) / (pb->atol + pb->rtol * (1.0 * fabs(x[i]) + adt * fabs(dxdt[i])));
        if (isnan(r))
            return r;
        if (r > m)
            m = r;
    }
    return m;
}

/* pow(a, -1.0/k) correctly rounded: the power evaluated in binary128
 * (113-bit significand; the C library's powl where long double is binary128,
 * as on aarch64 Linux, else GCC's libquadmath powq, both accurate to about an
 * ulp of binary128) and rounded once to double.  The rounding to double can
 * only differ from the correctly rounded result when the exact power lies
 * within ~2^-110 of a midpoint between doubles (probability ~2^-57 per
 * call).  Independent of the CUDA library's double-double evaluation, which
 * it checks. */
static double cr_pow_q(double a, double y)
{
#if defined(__aarch64__) || (defined(__LDBL_MANT_DIG__) && __LDBL_MANT_DIG__ == 113)
    return (double)powl((long double)a, (long double)y);
#else
    return (double)powq((__float128)a, (__float128)y);
#endif
}

/* err^(-1/k).  pow_mode 1: the C library's pow, as odeint calls std::pow.
 * pow_mode 2: the correctly rounded pow (cr_pow_q), what a correctly rounded
 * libm returns; the CUDA library's reference-parity controller computes the
 * same values.  pow_mode 0: a fixed IEEE-only scheme -- Newton's iteration
 * for the inverse k-th root x <- x + x (1 - a x^k) / k from a seed read off
 * the float bit pattern (exponent field scaled by -1/k), four FP32 steps then
 * two FP64 steps -- whose result is the same bits on every IEEE machine, so
 * step sequences can be compared bit for bit with the CUDA library's fast
 * controller, which uses the same scheme.  The modes differ in the last bit
 * of some factors (libm against correctly rounded: ~0.1% of calls with
 * glibc 2.39). */
/* pow trace of the calling thread (orc_set_powtrace): libm pow calls, and
 * those whose result is not the correctly rounded one */
static __thread orc_powtrace *g_pow = NULL;

void orc_set_powtrace(orc_powtrace *tr)
{
    g_pow = tr;
    if (tr) {
        tr->calls = tr->noncr = tr->step = 0;
        tr->first_noncr_step = -1;
        tr->first_noncr_arg = 0.0;
    }
}

static double inv_root(double a, int k, int pow_mode)
{
    if (pow_mode == 1) {
        const double r = pow(a, -1.0 / k);
        if (g_pow) {
            g_pow->calls++;
            if (a < 1e30 && r != cr_pow_q(a, -1.0 / k) && g_pow->noncr++ == 0) {
                g_pow->first_noncr_step = g_pow->step;
                g_pow->first_noncr_arg = a;
            }
        }
        return r;
    }
    if (pow_mode == 2)
        return a < 1e30 ? cr_pow_q(a, -1.0 / k) : 0.0;
    if (!(a < 1e30))
        return 0.0;
    float af = (float)a;
    int32_t bits;
    memcpy(&bits, &af, 4);
    int32_t c = (int32_t)(((int64_t)(k + 1) * 0x3F800000LL) / k);
    int32_t xb = c - bits / k;
    float x;
    memcpy(&x, &xb, 4);
    const float rk = 1.0f / (float)k;
    for (int it = 0; it < 4; it++) {
        float xk = x;
        for (int j = 1; j < k; j++)
            xk = xk * x;
        float r = fmaf(-af, xk, 1.0f);
        x = fmaf(x * r, rk, x);
    }
    double xd = (double)x;
    for (int it = 0; it < 2; it++) {
        double xk = xd;
        for (int j = 1; j < k; j++)
            xk = xk * xd;
        double r = fma(-a, xk, 1.0);
        xd = fma(xd * r, 1.0 / k, xd);
    }
    return xd;
}

double orc_step_pow(double a, int k, int pow_mode) { return inv_root(a, k, pow_mode); }

/* default_step_adjuster::decrease_step / increase_step */
static double decrease_step(double dt, double err, int error_order, int pow_mode)
{
    double f = 9.0 / 10.0 * inv_root(err, error_order - 1, pow_mode);
    double lo = 1.0 / 5.0;
    return dt * (f > lo ? f : lo);
}

static double increase_step(double dt, double err, int stepper_order, int pow_mode)
{
    if (err < 0.5) {
        /* pow(5.0, -p): 5^-5 = 1/3125 and 5^-8 = 1/390625, rounded (a
         * correctly rounded pow returns the same quotients) */
        double floor_ = stepper_order == 5   ? 1.0 / 3125.0
                        : stepper_order == 8 ? 1.0 / 390625.0
                                             : pow(5.0, -(double)stepper_order);
        if (err < floor_)
            err = floor_;
        dt *= 9.0 / 10.0 * inv_root(err, stepper_order, pow_mode);
    }
    return dt;
}

int orc_forward(const orc_problem *pb, const double *y0, const double *p, double t0, double t1,
                long cap, double *times, double *states, double *dt_trial, double *yT,
                long *n_acc, long *n_rej)
{
    tableau T;
    int n = pb->n;
    if (n < 1 || n > NMAX || get_tableau(pb->tableau, &T) != 0)
        return ORC_BAD_ARGS;
    double y[NMAX], dxdt[NMAX], dxdt_new[NMAX], out[NMAX], xerr[NMAX], xtmp[NMAX];
    double K[SMAX][NMAX];
    memcpy(y, y0, sizeof(double) * n);
    double t = t0, dt = pb->dt0;
    long count = 0, rej = 0;
    int status = ORC_OK;
    int first_call = 1;
    int max_fail = pb->max_fail > 0 ? pb->max_fail : 500;

    if (T.fixed) {
        /* runge_kutta for non-controlled steppers (detail/runge_kutta.hpp:
         * 37-72): t_n = t0 + n dt while (t_n + dt) - t1 <= eps (odeint's
         * less_eq_with_sign for dt > 0), every step recorded; do_step is the
         * tableau's stages and y + sum_j (b_j dt) k_j. */
        while ((t + dt) - t1 <= DBL_EPSILON) {
            if (count >= cap || count >= pb->max_steps) {
                status = ORC_MAX_STEPS;
                break;
            }
            times[count] = t;
            memcpy(states + (size_t)count * n, y, sizeof(double) * n);
            count_store(n);
            if (dt_trial)
                dt_trial[count] = dt;
            orc_rhs(pb, y, p, t, K[0]);
            rk_error_step(pb, &T, y, t, dt, p, K, out, dxdt_new, xerr, xtmp);
            memcpy(y, out, sizeof(double) * n);
            count++;
            t = t0 + (double)count * dt;
        }
        if (status == ORC_OK) {
            times[count] = t;
            memcpy(states + (size_t)count * n, y, sizeof(double) * n);
            count_store(n);
            for (int i = 0; i < n; i++)
                if (!isfinite(y[i]))
                    status = ORC_NONFINITE;
        }
        if (yT)
            memcpy(yT, y, sizeof(double) * n);
        if (n_acc)
            *n_acc = count;
        if (n_rej)
            *n_rej = 0;
        return status;
    }

    while (less_with_sign(t, t1)) {
        if (count >= cap) {
            status = ORC_MAX_STEPS;
            break;
        }
        times[count] = t;
        memcpy(states + (size_t)count * n, y, sizeof(double) * n);
        count_store(n);
        if (dt_trial)
            dt_trial[count] = dt;
        if (g_pow)
            g_pow->step = count;
        if (less_with_sign(t1, t + dt))
            dt = t1 - t;
        int fails = 0;
        for (;;) {
            /* try_step: CK54 recomputes dxdt on every attempt; DOPRI5
             * computes it on the first call and then carries it (FSAL). */
            if (!T.fsal || first_call) {
                orc_rhs(pb, y, p, t, dxdt);
                first_call = 0;
            }
            memcpy(K[0], dxdt, sizeof(double) * n);
            rk_error_step(pb, &T, y, t, dt, p, K, out, dxdt_new, xerr, xtmp);
            double err = error_norm(pb, y, dxdt, xerr, dt);
            int ok;
            if (isnan(err)) {
                status = ORC_NONFINITE;
                break;
            }
            if (err > 1.0) {
                dt = decrease_step(dt, err, T.error_order, pb->pow_mode);
                ok = 0;
                rej++;
            } else {
                t += dt;
                dt = increase_step(dt, err, T.stepper_order, pb->pow_mode);
                memcpy(y, out, sizeof(double) * n);
                if (T.fsal)
                    memcpy(dxdt, dxdt_new, sizeof(double) * n);
                ok = 1;
            }
            /* failed_step_checker::operator(): throws once m_steps reaches max */
            if (fails >= max_fail) {
                status = ORC_MAX_REJECTS;
                break;
            }
            fails++;
            if (ok)
                break;
            if (!isfinite(dt) || dt == 0.0) {
                status = ORC_NONFINITE;
                break;
            }
        }
        if (status != ORC_OK)
            break;
        count++;
    }
    if (status == ORC_OK) {
        times[count] = t;
        memcpy(states + (size_t)count * n, y, sizeof(double) * n);
        count_store(n);
        for (int i = 0; i < n; i++)
            if (!isfinite(y[i]))
                status = ORC_NONFINITE;
    }
    if (yT)
        memcpy(yT, y, sizeof(double) * n);
    if (n_acc)
        *n_acc = count;
    if (n_rej)
        *n_rej = rej;
    return status;
}

void orc_forward_frozen(const orc_problem *pb, const double *y0, const double *p, long T,
                        const double *times, double *yT)
{
    tableau tab;
    int n = pb->n;
    get_tableau(pb->tableau, &tab);
    double y[NMAX], xtmp[NMAX], K[SMAX][NMAX];
    memcpy(y, y0, sizeof(double) * n);
    for (long k = 0; k < T; k++) {
        double t = times[k], h = times[k + 1] - times[k];
        orc_rhs(pb, y, p, t, K[0]);
        for (int m = 1; m < tab.s; m++) {
            for (int i = 0; i < n; i++) {
                double acc = y[i];
                for (int j = 0; j < m; j++)
                    acc = acc + (tab.a[m][j] * h) * K[j][i];
                xtmp[i] = acc;
            }
            orc_rhs(pb, xtmp, p, t + tab.c[m] * h, K[m]);
        }
        for (int i = 0; i < n; i++) {
            double acc = y[i];
            for (int j = 0; j < tab.s; j++)
                if (tab.b[j] != 0.0)
                    acc = acc + (tab.b[j] * h) * K[j][i];
            y[i] = acc;
        }
    }
    memcpy(yT, y, sizeof(double) * n);
}

/* ---------------------------------------------------------------- adjoint */

/* back_prop_step (detail/backpropagation.hpp:160-229) for one seed. */
static void back_prop_step(const orc_problem *pb, const tableau *T, const double *p, double tn,
                           double h, const double *u, double *lam, double *alphabar,
                           double *K /* [s][n] */, double *X /* [s][n] */, double *Kbar /* [s][n] */,
                           double *ybar, double *gx, double *gp)
{
    int n = pb->n, s = T->s, np = pb->npar;
    /* compute_intermediate_states (:24-64): X_m = u + sum_{j<m} (h a_mj) K_j */
    for (int m = 0; m < s; m++) {
        for (int i = 0; i < n; i++) {
            double acc = u[i];
            for (int j = 0; j < m; j++)
                acc += h * T->a[m][j] * K[j * n + i];
            X[m * n + i] = acc;
        }
        orc_rhs(pb, X + m * n, p, tn + T->c[m] * h, K + m * n);
    }
    /* step s+1 (:178-184): ybar = lambda, Kbar_m = b_m h lambda */
    for (int i = 0; i < n; i++) {
        ybar[i] = 0.0 + lam[i];
        for (int m = 0; m < s; m++)
            Kbar[m * n + i] = 0.0 + T->b[m] * h * lam[i];
    }
    /* steps s..1 (:196-224) */
    for (int m = s - 1; m >= 0; m--) {
        orc_vjp(pb, Kbar + m * n, X + m * n, p, tn + T->c[m] * h, gx, gp);
        for (int i = 0; i < n; i++) {
            ybar[i] += gx[i];
            for (int k = 0; k < m; k++)
                Kbar[k * n + i] += gx[i] * T->a[m][k] * h;
        }
        for (int k = 0; k < np; k++)
            alphabar[k] += gp[k];
    }
    for (int i = 0; i < n; i++)
        lam[i] = ybar[i];
}

int orc_adjoint(const orc_problem *pb, const double *p, long T, const double *times,
                const double *states, int nout, double *lambda, double *mu)
{
    return orc_adjoint_history(pb, p, T, times, states, nout, lambda, mu, NULL);
}

int orc_adjoint_history(const orc_problem *pb, const double *p, long T, const double *times,
                        const double *states, int nout, double *lambda, double *mu, double *hist)
{
    tableau tab;
    if (get_tableau(pb->tableau, &tab) != 0 || pb->n < 1 || pb->n > NMAX || nout < 1)
        return ORC_BAD_ARGS;
    int n = pb->n, np = pb->npar, s = tab.s;
    double *work = (double *)malloc(sizeof(double) * ((size_t)4 * s * n + 2 * n + 2 * (size_t)np));
    if (!work)
        return ORC_BAD_ARGS;
    double *K = work, *X = K + s * n, *Kbar = X + s * n, *ybar = Kbar + s * n;
    double *gx = ybar + n, *gp = gx + n, *alphabar = gp + np;
    int status = ORC_OK;
    for (int q = 0; q < nout; q++) {
        double *lam = lambda + (size_t)q * n;
        for (int k = 0; k < np; k++)
            alphabar[k] = 0.0;
        /* back_prop (:256-278): n = T-1 .. 0; its observer sees lambda_T,
         * then lambda_n after each step (:268, :274) */
        double *hq = hist ? hist + (size_t)q * (T + 1) * n : NULL;
        if (hq)
            memcpy(hq + (size_t)T * n, lam, sizeof(double) * n);
        for (long k = T - 1; k >= 0; k--) {
            double tn = times[k];
            double h = times[k + 1] - times[k];
            if (g_traffic) /* times[k], times[k + 1], y_k (GetState / GetDt) */
                g_traffic->load_bytes += (long long)sizeof(double) * (2 + n);
            back_prop_step(pb, &tab, p, tn, h, states + (size_t)k * n, lam, alphabar, K, X, Kbar,
                           ybar, gx, gp);
            if (hq)
                memcpy(hq + (size_t)k * n, lam, sizeof(double) * n);
        }
        /* write-back (:317-321): mu += alphabar */
        for (int k = 0; k < np; k++)
            mu[(size_t)q * np + k] += alphabar[k];
        for (int i = 0; i < n; i++)
            if (!isfinite(lam[i]))
                status = ORC_NONFINITE;
    }
    free(work);
    return status;
}

/* --------------------------------------------------------------- gradient */

int orc_gradient(const orc_problem *pb, int cost, const double *y0, const double *p, double t0,
                 double t1, double *yT, double *dy0, double *dp, long *n_acc, long *n_rej)
{
    int n = pb->n;
    long cap = pb->max_steps > 0 ? pb->max_steps : 100000;
    double *times = (double *)malloc(sizeof(double) * (size_t)(cap + 1));
    double *states = (double *)malloc(sizeof(double) * (size_t)(cap + 1) * n);
    if (!times || !states) {
        free(times);
        free(states);
        return ORC_BAD_ARGS;
    }
    double yT_local[NMAX];
    long T = 0;
    int st = orc_forward(pb, y0, p, t0, t1, cap, times, states, NULL, yT_local, &T, n_rej);
    if (yT)
        memcpy(yT, yT_local, sizeof(double) * n);
    if (n_acc)
        *n_acc = T;
    if (st == ORC_OK) {
        for (int i = 0; i < n; i++)
            dy0[i] = cost == ORC_COST_SUMSQ ? 2.0 * yT_local[i] : 1.0;
        for (int k = 0; k < pb->npar; k++)
            dp[k] = 0.0;
        st = orc_adjoint(pb, p, T, times, states, 1, dy0, dp);
    }
    free(times);
    free(states);
    return st;
}

typedef struct {
    const orc_problem *pb;
    int cost;
    long lo, hi;
    long *next;  /* the shared counter of the next unclaimed instance */
    long chunk;  /* instances claimed at a time */
    const double *y0, *p, *t0, *t1;
    double *yT, *dy0, *dp;
    long *n_acc, *n_rej;
    int *status;
} batch_job;

// Instances are handed out in chunks from a shared counter (instance
// lengths vary by an order of magnitude: a static partition left cores idle
// while the thread with the longest instances finished); a chunk is at most
// 32 instances and at most 1/8 of a thread's share, so that small batches
// still spread over every thread.

static void *batch_worker(void *arg)
{
    batch_job *J = (batch_job *)arg;
    int n = J->pb->n, np = J->pb->npar;
    for (;;) {
        const long lo = __atomic_fetch_add(J->next, J->chunk, __ATOMIC_RELAXED);
        if (lo >= J->hi)
            break;
        const long hi = lo + J->chunk < J->hi ? lo + J->chunk : J->hi;
        for (long b = lo; b < hi; b++) {
        long na = 0, nr = 0;
        int st = orc_gradient(J->pb, J->cost, J->y0 + b * n, J->p + b * np, J->t0[b], J->t1[b],
                              J->yT ? J->yT + b * n : NULL, J->dy0 + b * n, J->dp + b * np, &na,
                              &nr);
        if (J->n_acc)
            J->n_acc[b] = na;
        if (J->n_rej)
            J->n_rej[b] = nr;
        if (J->status)
            J->status[b] = st;
        }
    }
    return NULL;
}

int orc_gradient_batch(const orc_problem *pb, int cost, long B, const double *y0, const double *p,
                       const double *t0, const double *t1, int nthreads, double *yT, double *dy0,
                       double *dp, long *n_acc, long *n_rej, int *status)
{
    if (nthreads < 1)
        nthreads = 1;
    if (nthreads > 256)
        nthreads = 256;
    pthread_t th[256];
    int created[256];
    batch_job jobs[256];
    if (B < 1)
        return ORC_OK;
    if (nthreads > B)
        nthreads = (int)B; /* no idle threads to create */
    long chunk = B / (8L * nthreads);
    chunk = chunk < 1 ? 1 : (chunk > 32 ? 32 : chunk);
    long next = 0;
    if (nthreads == 1) { /* on the calling thread */
        batch_job J = {pb, cost, 0, B, &next, chunk, y0, p, t0, t1, yT, dy0, dp, n_acc, n_rej, status};
        batch_worker(&J);
        return ORC_OK;
    }
    for (int k = 0; k < nthreads; k++) {
        batch_job J = {pb, cost, 0, B, &next, chunk, y0, p, t0, t1, yT, dy0, dp, n_acc, n_rej, status};
        jobs[k] = J;
        created[k] = 0;
    }
    for (int k = 0; k < nthreads; k++) {
        if (pthread_create(&th[k], NULL, batch_worker, &jobs[k]) == 0)
            created[k] = 1;
        else
            batch_worker(&jobs[k]);
    }
    for (int k = 0; k < nthreads; k++)
        if (created[k])
            pthread_join(th[k], NULL);
    return ORC_OK;
}

int orc_gradient_traffic(const orc_problem *pb, int cost, const double *y0, const double *p, double t0,
                         double t1, long *n_acc, orc_traffic *traffic)
{
    double yT[NMAX], dy0[NMAX];
    double *dp = (double *)malloc(sizeof(double) * (size_t)(pb->npar > 0 ? pb->npar : 1));
    if (!dp || pb->n < 1 || pb->n > NMAX) {
        free(dp);
        return ORC_BAD_ARGS;
    }
    traffic->store_bytes = traffic->load_bytes = 0;
    g_traffic = traffic;
    long n_rej = 0;
    int st = orc_gradient(pb, cost, y0, p, t0, t1, yT, dy0, dp, n_acc, &n_rej);
    g_traffic = NULL;
    free(dp);
    return st;
}
