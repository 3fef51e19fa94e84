// Reference-backed checker (TEST INFRASTRUCTURE ONLY).  Compiles the
// reference's unchanged lib/include headers (Driver, runge_kutta,
// adjointSolve, ButcherTable, AadData) against the project's Boost stand-in
// (boost_shim/) and links the AADC runtime shipped with the reference, then
// exposes one C entry point that runs the reference's own call sequence --
// as in examples/VanDerPol/main.cpp:89-117 -- for one instance:
//   Driver(N, Nout, Npar); runge_kutta(make_controlled<stepper>(atol, rtol),
//   f, x0, alphas, t0, t1, dt, driver); setCostGradients(driver, lambda, mu);
//   constructDriverButcherTableau(driver, stepper);
//   recordDriverRHSFunction(driver, f); adjointSolve(driver, alphas).
// Built by oracle/ref/Makefile into oracle/_ref/ (git-ignored), only where
// the reference sources are present; it generates the golden fixtures of
// tests/golden/.  The reference's ButcherTable has no Dormand-Prince entry
// (ButcherTable.hpp:365-368); the explicit specialization below adds the
// published 7-stage FSAL tableau without editing the reference.
#include <cstring>
#include <exception>
#include <iostream>
#include <vector>

#include "lib.hpp"

namespace odeint = boost::numeric::odeint;
using State = std::vector<double>;
using Dopri5 = odeint::runge_kutta_dopri5<State>;
using CashKarp = odeint::runge_kutta_cash_karp54<State>;
using Fehlberg78 = odeint::runge_kutta_fehlberg78<State>;
using RK4 = odeint::runge_kutta4<State>;
using Euler = odeint::euler<State>;

template <>
void ButcherTable::initialize<Dopri5>(Dopri5 stepper, odeint::error_stepper_tag)
{
    (void)stepper;
    const odeint::shim_tableau t = Dopri5::tableau();
    const int s = t.s;
    p_a = std::make_unique<std::vector<double>>(s * s, 0.0);
    p_b = std::make_unique<std::vector<double>>(t.b);
    p_c = std::make_unique<std::vector<double>>(t.c);
    for (int i = 0; i < s; i++)
        for (std::size_t j = 0; j < t.a[i].size(); j++)
            (*p_a)[i * s + j] = t.a[i][j];
}

// Right-hand sides with the reference functor signature.
struct VanDerPol { // x1' = mu (1 - x0^2) x1 - x0
    template <typename T> void operator()(const std::vector<T> &x, std::vector<T> &dxdt, const std::vector<T> &p, T t) const
    {
        (void)t;
        dxdt[0] = x[1];
        dxdt[1] = p[0] * (1.0 - x[0] * x[0]) * x[1] - x[0];
    }
};
struct VanDerPolPETSc { // examples/VanDerPol/main.cpp:38-43
    template <typename T> void operator()(const std::vector<T> &x, std::vector<T> &dxdt, const std::vector<T> &mu, const T t) const
    {
        (void)t;
        dxdt[0] = x[1];
        dxdt[1] = mu[0] * ((1.0 - x[0] * x[0]) * x[1] - x[0]);
    }
};
struct DampedOscillator { // p = (omega, zeta)
    template <typename T> void operator()(const std::vector<T> &x, std::vector<T> &dxdt, const std::vector<T> &p, T t) const
    {
        (void)t;
        dxdt[0] = x[1];
        dxdt[1] = -p[0] * p[0] * x[0] - 2.0 * p[1] * p[0] * x[1];
    }
};
struct LotkaVolterra { // examples/GeneralizedLotkaVolterra/main.cpp:105-119
    template <typename T> void operator()(const std::vector<T> &x, std::vector<T> &dxdt, const std::vector<T> &parameters, T t)
    {
        (void)t;
        int N = x.size();
        for (int i = 0; i < (int)x.size(); i++) {
            T sum = 0.0;
            for (int j = 0; j < (int)x.size(); j++) {
                int id = N * (i + 1) + j;
                sum += parameters[id] * x[j];
            }
            dxdt[i] = x[i] * (parameters[i] + sum);
        }
    }
};

// The test suite's device models (tests/cpp/user_models.cuh), wrapped in the
// reference's functor signature: the reference tapes them with AADC like any
// user functor, so they pin the bring-your-own-model path.
#include "../../tests/cpp/user_models.cuh"
template <class Model> struct UserFunctor {
    template <typename T> void operator()(const std::vector<T> &x, std::vector<T> &dxdt, const std::vector<T> &p, T t) const
    {
        Model::template rhs<T>(x.data(), p.data(), t, dxdt.data());
    }
};
using DuffingFunctor = UserFunctor<ForcedDuffing>;
using BrusselatorFunctor = UserFunctor<Brusselator>;

template <class Stepper, class System>
static int run(System sys, int n, int nout, int npar, double atol, double rtol, double dt0, const double *y0,
               const double *p, double t0, double t1, const double *lam_in, const double *mu_in, long cap,
               double *times, double *states, long *T, double *yT, double *lam_out, double *mu_out)
{
    using namespace vectorizedadjoint;
    Driver driver(n, nout, npar);
    State x0(y0, y0 + n), alphas(p, p + npar);
    size_t steps = 0;
    try {
        if constexpr (std::is_same<typename Stepper::stepper_category, odeint::stepper_tag>::value)
            steps = runge_kutta(Stepper(), sys, x0, alphas, t0, t1, dt0, driver); // fixed step dt0
        else
            steps = runge_kutta(odeint::make_controlled<Stepper>(atol, rtol), sys, x0, alphas, t0, t1, dt0, driver);
    } catch (std::exception &e) {
        std::cerr << "runge_kutta: " << e.what() << std::endl;
        return 1;
    }
    *T = (long)steps;
    std::memcpy(yT, x0.data(), sizeof(double) * n);
    const int nrec = driver.GetT();
    for (int k = 0; k < nrec && k <= cap; k++) {
        times[k] = driver.GetTime(k);
        State u(n);
        driver.GetState(u, k);
        std::memcpy(states + (size_t)k * n, u.data(), sizeof(double) * n);
    }
    std::vector<std::vector<double>> lambda(nout, std::vector<double>(n)), mu(nout, std::vector<double>(npar));
    for (int q = 0; q < nout; q++) {
        for (int i = 0; i < n; i++)
            lambda[q][i] = lam_in[(size_t)q * n + i];
        for (int k = 0; k < npar; k++)
            mu[q][k] = mu_in[(size_t)q * npar + k];
    }
    setCostGradients(driver, lambda, mu);
    constructDriverButcherTableau(driver, Stepper());
    recordDriverRHSFunction(driver, sys);
    adjointSolve(driver, alphas);
    for (int q = 0; q < nout; q++) {
        for (int i = 0; i < n; i++)
            lam_out[(size_t)q * n + i] = lambda[q][i];
        for (int k = 0; k < npar; k++)
            mu_out[(size_t)q * npar + k] = mu[q][k];
    }
    return 0;
}

// The reference's SIMD back_prop (detail/backpropagation.hpp:230-254) with
// an observer that records what it is shown: (wbarend, t_n) for n = T .. 0,
// the seeds of up to four costs in the lanes (as adjointSolve packs them).
// hist[q][n][i] = lambda_n of seed q; times[n] = t_n.
template <class Stepper, class System>
static int run_history(System sys, int n, int nout, int npar, double atol, double rtol, double dt0,
                       const double *y0, const double *p, double t0, double t1, const double *lam_in, long cap,
                       double *times, double *hist, long *T)
{
    using namespace vectorizedadjoint;
    const int lanes = (int)(sizeof(mmType) / sizeof(double));
    if (nout < 1 || nout > lanes)
        return 3;
    Driver driver(n, nout, npar);
    State x0(y0, y0 + n), alphas(p, p + npar);
    size_t steps = 0;
    try {
        if constexpr (std::is_same<typename Stepper::stepper_category, odeint::stepper_tag>::value)
            steps = runge_kutta(Stepper(), sys, x0, alphas, t0, t1, dt0, driver);
        else
            steps = runge_kutta(odeint::make_controlled<Stepper>(atol, rtol), sys, x0, alphas, t0, t1, dt0, driver);
    } catch (std::exception &e) {
        std::cerr << "runge_kutta: " << e.what() << std::endl;
        return 1;
    }
    *T = (long)steps;
    if ((long)steps + 1 > cap)
        return 4;
    std::vector<std::vector<double>> lambda(nout, std::vector<double>(n)), mu(nout, std::vector<double>(npar, 0.0));
    setCostGradients(driver, lambda, mu);
    constructDriverButcherTableau(driver, Stepper());
    recordDriverRHSFunction(driver, sys);
    aadc::mmVector<mmType> wbarend(n);
    for (int i = 0; i < n; i++)
        for (int j = 0; j < lanes; j++)
            wbarend[i][j] = j < nout ? lam_in[(size_t)j * n + i] : 0.0;
    long k = (long)steps;
    auto observer = [&](const aadc::mmVector<mmType> &w, double t) {
        if (k < 0)
            return;
        times[k] = t;
        for (int q = 0; q < nout; q++)
            for (int i = 0; i < n; i++)
                hist[((size_t)q * (steps + 1) + k) * n + i] = w[i][q];
        k--;
    };
    detail::back_prop(driver, wbarend, alphas, observer);
    return k == -1 ? 0 : 5;
}

// model: 0 VdP (Lienard), 1 VdP (reference example form), 2 damped
// oscillator, 3 GLV, 10 forced Duffing and 11 Brusselator (the test suite's
// own models); tableau: 0 DOPRI5, 1 Cash-Karp, 2 Fehlberg 7(8) (the
// reference's own ButcherTable branch), 3 fixed-step RK4, 4 fixed-step Euler
// (step dt0).  Returns 0 on success.
extern "C" int ref_solve(int model, int tableau, int n, int nout, int npar, double atol, double rtol, double dt0,
                         const double *y0, const double *p, double t0, double t1, const double *lam_in,
                         const double *mu_in, long cap, double *times, double *states, long *T, double *yT,
                         double *lam_out, double *mu_out)
{
#define VA_ARGS n, nout, npar, atol, rtol, dt0, y0, p, t0, t1, lam_in, mu_in, cap, times, states, T, yT, lam_out, mu_out
#define VA_RUN(SYS)                                                                                \
    (tableau == 0   ? run<Dopri5>(SYS(), VA_ARGS)                                                  \
     : tableau == 1 ? run<CashKarp>(SYS(), VA_ARGS)                                                \
     : tableau == 2 ? run<Fehlberg78>(SYS(), VA_ARGS)                                              \
     : tableau == 3 ? run<RK4>(SYS(), VA_ARGS)                                                     \
                    : run<Euler>(SYS(), VA_ARGS))
    switch (model) {
    case 0:
        return VA_RUN(VanDerPol);
    case 1:
        return VA_RUN(VanDerPolPETSc);
    case 2:
        return VA_RUN(DampedOscillator);
    case 3:
        return VA_RUN(LotkaVolterra);
    case 10:
        return VA_RUN(DuffingFunctor);
    case 11:
        return VA_RUN(BrusselatorFunctor);
    default:
        return 2;
    }
#undef VA_RUN
#undef VA_ARGS
}

// back_prop's observer record of one instance (run_history); same model and
// tableau codes as ref_solve.  hist: [nout][T+1][n], nout <= 4.
extern "C" int ref_history(int model, int tableau, int n, int nout, int npar, double atol, double rtol, double dt0,
                           const double *y0, const double *p, double t0, double t1, const double *lam_in, long cap,
                           double *times, double *hist, long *T)
{
#define VA_ARGS n, nout, npar, atol, rtol, dt0, y0, p, t0, t1, lam_in, cap, times, hist, T
#define VA_RUN(SYS)                                                                                \
    (tableau == 0   ? run_history<Dopri5>(SYS(), VA_ARGS)                                          \
     : tableau == 1 ? run_history<CashKarp>(SYS(), VA_ARGS)                                        \
     : tableau == 2 ? run_history<Fehlberg78>(SYS(), VA_ARGS)                                      \
     : tableau == 3 ? run_history<RK4>(SYS(), VA_ARGS)                                             \
                    : run_history<Euler>(SYS(), VA_ARGS))
    switch (model) {
    case 0:
        return VA_RUN(VanDerPol);
    case 1:
        return VA_RUN(VanDerPolPETSc);
    case 2:
        return VA_RUN(DampedOscillator);
    case 3:
        return VA_RUN(LotkaVolterra);
    case 10:
        return VA_RUN(DuffingFunctor);
    case 11:
        return VA_RUN(BrusselatorFunctor);
    default:
        return 2;
    }
#undef VA_RUN
#undef VA_ARGS
}
