// va_driver.hpp -- the reference's single-instance C++ API on top of the C ABI.
//
// Same names, argument meaning and error behaviour as the reference's
// lib/include headers, so a program written against them switches by
// including this header instead of lib.hpp and linking libva_gb300.so:
//
//   Driver(Nin, Nout, Npar)                        Driver.hpp:39-42
//   runge_kutta(stepper, system, x0, alphas,
//               t0, t1, dt, driver) -> steps       runge_kutta.hpp:47-59
//   setCostGradients(driver, lambda, mu)           Driver.hpp:103-114
//   constructDriverButcherTableau(driver, st)      Driver.hpp:87-93
//   recordDriverRHSFunction(driver, system)        Driver.hpp:95-100
//   adjointSolve(driver, alphas)                   backpropagation.hpp:18-43
//   computeSensitivityMatrix(driver, alphas)       backpropagation.hpp:69-87
//   computeSensitivityMatrixNoSIMD(driver, alphas) backpropagation.hpp:46-66
//
// Differences, by design: the right-hand side is device code -- one of the
// built-in models (VanDerPol, VanDerPolPETSc, DampedOscillator,
// LotkaVolterra, Decay) or a model of your own compiled with
// include/va_model.cuh, passed as a tag struct with
//   static const va_model_kernels *va_kernels();
// returning its VA_DEFINE_MODEL table -- instead of an arbitrary host
// functor, and the steppers are tags carrying the tableau and tolerances.  Step sizes are
// frozen in the adjoint, as in the reference.  runge_kutta throws
// std::runtime_error where odeint throws (failed step checker); adjointSolve
// prints errors and returns, like the reference.
//
// No CUDA header is needed: everything goes through va.h's host entry points.
#ifndef VA_DRIVER_HPP
#define VA_DRIVER_HPP

#include <cstdint>
#include <iostream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "va.h"

namespace vectorizedadjoint_gb300 {

// ---------------------------------------------------------------- steppers
template <class State> struct runge_kutta_dopri5 {
    static constexpr int32_t tableau = VA_TAB_DOPRI5;
};
template <class State> struct runge_kutta_cash_karp54 {
    static constexpr int32_t tableau = VA_TAB_CK54;
};
template <class State> struct runge_kutta_fehlberg78 {
    static constexpr int32_t tableau = VA_TAB_RKF78;
};
// Fixed-step steppers, passed to runge_kutta directly (no make_controlled),
// as odeint's runge_kutta4 / euler are; the tolerances are unused.
template <class State> struct runge_kutta4 {
    static constexpr int32_t tableau = VA_TAB_RK4;
    double atol = 1e-6, rtol = 1e-6;
};
template <class State> struct euler {
    static constexpr int32_t tableau = VA_TAB_EULER;
    double atol = 1e-6, rtol = 1e-6;
};
template <class ErrorStepper> struct controlled_runge_kutta {
    double atol, rtol;
    static constexpr int32_t tableau = ErrorStepper::tableau;
};
// odeint::make_controlled<Stepper>(abs, rel)
template <class ErrorStepper>
controlled_runge_kutta<ErrorStepper> make_controlled(double atol, double rtol)
{
    return controlled_runge_kutta<ErrorStepper>{atol, rtol};
}

// ------------------------------------------------------------------ models
struct VanDerPol { static constexpr int32_t model = VA_MODEL_VDP; };
struct VanDerPolPETSc { static constexpr int32_t model = VA_MODEL_VDP_PETSC; };
struct DampedOscillator { static constexpr int32_t model = VA_MODEL_DHO; };
struct LotkaVolterra { static constexpr int32_t model = VA_MODEL_GLV; };
struct Decay { static constexpr int32_t model = VA_MODEL_DECAY; };

// a model compiled outside the library: System::va_kernels() gives its table
template <class System, class = void> struct is_device_model : std::false_type {};
template <class System>
struct is_device_model<System, std::void_t<decltype(System::va_kernels())>> : std::true_type {};

// ------------------------------------------------------------------ driver
class Driver {
  public:
    Driver(int Nin, int Nout, int Npar) : m_Nin(Nin), m_Nout(Nout), m_Npar(Npar) {}
    ~Driver() { release(); }
    Driver(const Driver &) = delete;
    Driver &operator=(const Driver &) = delete;

    int GetNin() const { return m_Nin; }
    int GetNout() const { return m_Nout; }
    int GetNpar() const { return m_Npar; }
    // accepted-step record of the last forward sweep (StateStorage contents)
    int GetT() const { return m_T + 1; }

    std::vector<std::vector<double>> *p_lambda = nullptr;
    std::vector<std::vector<double>> *p_mu = nullptr;
    int32_t m_model = -1;
    const va_model_kernels *m_user = nullptr;
    int32_t m_tableau = -1;
    double m_atol = 1e-6, m_rtol = 1e-6, m_dt0 = 1e-3;
    int32_t m_T = -1;

    // (Re)creates the handle when the problem or the stepper changed; `user`
    // is the table of a model compiled outside the library (model
    // VA_MODEL_USER), null for the built-in models.
    va_handle *handle(int32_t model, int32_t tableau, double atol, double rtol, double dt0,
                      const va_model_kernels *user = nullptr)
    {
        if (m_h && model == m_model && tableau == m_tableau && atol == m_atol && rtol == m_rtol &&
            dt0 == m_dt0 && user == m_user)
            return m_h;
        release();
        va_problem p{model, m_Nin, m_Npar, 1, m_Nout};
        va_options o;
        va_default_options(&o);
        o.tableau = tableau;
        o.atol = atol;
        o.rtol = rtol;
        o.dt0 = dt0;
        va_status st = user ? va_create_model(&p, &o, user, &m_h) : va_create(&p, &o, &m_h);
        if (st != VA_OK) {
            m_h = nullptr;
            throw std::runtime_error(std::string("va_create failed: ") + va_status_string(st));
        }
        m_model = model;
        m_user = user;
        m_tableau = tableau;
        m_atol = atol;
        m_rtol = rtol;
        m_dt0 = dt0;
        return m_h;
    }
    va_handle *handle() const { return m_h; }

  private:
    void release()
    {
        if (m_h)
            va_destroy(m_h);
        m_h = nullptr;
    }
    int m_Nin, m_Nout, m_Npar;
    va_handle *m_h = nullptr;
};

inline void delete_driver_handle(void *ptr) { delete static_cast<Driver *>(ptr); }

// Forward sweep of one instance; x0 is overwritten with y(t1) and the number
// of accepted steps is returned, as the reference does.
template <class Stepper, class System, class State, class Time>
size_t runge_kutta(Stepper stepper, System system, State &start_state, const State &alphas,
                   Time start_time, const Time end_time, Time dt, Driver &driver)
{
    (void)system;
    va_handle *h;
    if constexpr (is_device_model<System>::value)
        h = driver.handle(VA_MODEL_USER, Stepper::tableau, stepper.atol, stepper.rtol, (double)dt,
                          System::va_kernels());
    else
        h = driver.handle(System::model, Stepper::tableau, stepper.atol, stepper.rtol, (double)dt);
    const double t0 = (double)start_time, t1 = (double)end_time;
    std::vector<double> y0(start_state.begin(), start_state.end()), p(alphas.begin(), alphas.end()),
        yT(y0.size());
    int32_t nacc = 0, nrej = 0, status = 0;
    va_status st = va_forward_host(h, y0.data(), p.data(), &t0, &t1, yT.data(), &nacc, &nrej, &status);
    if (st != VA_OK)
        throw std::runtime_error(std::string("runge_kutta: ") + va_last_error(h));
    if (status != VA_OK)
        throw std::runtime_error(std::string("runge_kutta: ") + va_status_string(status));
    for (size_t i = 0; i < yT.size(); i++)
        start_state[i] = yT[i];
    driver.m_T = nacc;
    return (size_t)nacc;
}

// With observer (runge_kutta.hpp:16-29): observer(state, t) for every
// record (t_n, y_n), n = 0 .. T, in order, as the reference's loop calls it
// (detail/runge_kutta.hpp:94,113); here replayed from the checkpoint record
// after the sweep.
template <class Stepper, class System, class State, class Time, class Observer>
size_t runge_kutta(Stepper stepper, System system, State &start_state, const State &alphas,
                   Time start_time, const Time end_time, Time dt, Driver &driver, Observer observer)
{
    const size_t steps = runge_kutta(stepper, system, start_state, alphas, start_time, end_time, dt, driver);
    va_handle *h = driver.handle();
    const int n = driver.GetNin(), nrec = driver.GetT();
    std::vector<double> t(nrec), y((size_t)nrec * n);
    int32_t got = 0;
    if (va_trajectory(h, 0, nrec, t.data(), nullptr, y.data(), &got) != VA_OK)
        throw std::runtime_error(std::string("runge_kutta: ") + va_last_error(h));
    for (int k = 0; k < nrec; k++) {
        State x(y.begin() + (size_t)k * n, y.begin() + (size_t)(k + 1) * n);
        observer(x, (Time)t[k]);
    }
    return steps;
}

inline void setCostGradients(Driver &driver, std::vector<std::vector<double>> &lambda,
                             std::vector<std::vector<double>> &mu)
{
    driver.p_lambda = &lambda;
    driver.p_mu = &mu;
}

// The tableau travels with the stepper tag passed to runge_kutta; these two
// calls exist so reference programs compile unchanged.
template <class Stepper> void constructDriverButcherTableau(Driver &, Stepper) {}
template <class System> void recordDriverRHSFunction(Driver &, System) {}

// lambda[j] <- dG_j/dy0, mu[j] += dG_j/dalpha (frozen step sizes).
template <class State> void adjointSolve(Driver &driver, const State &parameters)
{
    try {
        if (!(driver.p_lambda && driver.p_mu))
            throw std::runtime_error("Must call setCostGradients() first!");
        va_handle *h = driver.handle();
        if (!h || driver.m_T < 0)
            throw std::runtime_error("Must call runge_kutta() first!");
        const int nin = driver.GetNin(), nout = driver.GetNout(), npar = driver.GetNpar();
        std::vector<double> lam((size_t)nout * nin), mu((size_t)nout * npar), p(parameters.begin(), parameters.end());
        for (int j = 0; j < nout; j++) {
            for (int i = 0; i < nin; i++)
                lam[(size_t)j * nin + i] = (*driver.p_lambda)[j][i];
            for (int k = 0; k < npar; k++)
                mu[(size_t)j * npar + k] = (*driver.p_mu)[j][k];
        }
        std::vector<double> dy0(lam.size()), dp(mu.size());
        int32_t status = 0;
        va_status st = va_backward_host(h, p.data(), lam.data(), mu.data(), dy0.data(), dp.data(), &status);
        if (st != VA_OK)
            throw std::runtime_error(std::string("adjointSolve: ") + va_last_error(h));
        if (status != VA_OK)
            throw std::runtime_error(std::string("adjointSolve: ") + va_status_string(status));
        for (int j = 0; j < nout; j++) {
            for (int i = 0; i < nin; i++)
                (*driver.p_lambda)[j][i] = dy0[(size_t)j * nin + i];
            for (int k = 0; k < npar; k++)
                (*driver.p_mu)[j][k] = dp[(size_t)j * npar + k];
        }
    } catch (std::exception &e) {
        std::cout << e.what() << std::endl;
    }
}

// adjointSolve with the back_prop observer of detail/backpropagation.hpp:
// 230-254 exposed: observer(lambda_n, t_n) with lambda_n = [Nout][Nin] after
// every back step, n = T .. 0 (the reference passes null_observer there).
template <class State, class Observer>
void adjointSolve(Driver &driver, const State &parameters, Observer observer)
{
    va_handle *h = driver.handle();
    const int nin = driver.GetNin(), nout = driver.GetNout(), nrec = driver.GetT();
    if (!h || driver.m_T < 0 || va_set_adjoint_history(h, nrec) != VA_OK) {
        std::cout << "Must call runge_kutta() first!" << std::endl;
        return;
    }
    adjointSolve(driver, parameters);
    std::vector<double> t(nrec), lam((size_t)nout * nrec * nin);
    int32_t got = 0;
    if (va_adjoint_history(h, 0, nrec, t.data(), lam.data(), &got) == VA_OK) {
        std::vector<std::vector<double>> rows(nout, std::vector<double>(nin));
        for (int k = nrec - 1; k >= 0; k--) {
            for (int q = 0; q < nout; q++)
                for (int i = 0; i < nin; i++)
                    rows[q][i] = lam[((size_t)q * nrec + k) * nin + i];
            observer(rows, t[k]);
        }
    } else {
        std::cout << "adjointSolve: " << va_last_error(h) << std::endl;
    }
    va_set_adjoint_history(h, 0);
}

// d x_i(T) / d alpha_k (Nin x Npar), identity seeds (backpropagation.hpp:69-87).
// Needs a Driver created with Nout == Nin.
template <class State> std::vector<std::vector<double>> computeSensitivityMatrix(Driver &driver, const State &parameters)
{
    const int nin = driver.GetNin(), npar = driver.GetNpar();
    std::vector<std::vector<double>> lam(nin, std::vector<double>(nin, 0.0)), mu(nin, std::vector<double>(npar, 0.0));
    for (int i = 0; i < nin; i++)
        lam[i][i] = 1.0;
    auto *pl = driver.p_lambda, *pm = driver.p_mu;
    setCostGradients(driver, lam, mu);
    adjointSolve(driver, parameters);
    driver.p_lambda = pl;
    driver.p_mu = pm;
    return mu;
}

// The reference's one-cost-at-a-time variant (backpropagation.hpp:46-66):
// the same matrix; here every seed row shares one backward sweep either way.
template <class State> std::vector<std::vector<double>> computeSensitivityMatrixNoSIMD(Driver &driver, const State &parameters)
{
    return computeSensitivityMatrix(driver, parameters);
}

} // namespace vectorizedadjoint_gb300

#endif
