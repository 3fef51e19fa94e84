// Stand-in for the parts of Boost (odeint, uBLAS, array) that the
// reference's lib/include headers include.  Boost is not installed in this
// container, so this project-written shim lets the reference's own forward
// loop (lib/include/detail/runge_kutta.hpp) and discrete adjoint
// (lib/include/detail/backpropagation.hpp) compile unchanged.  TEST
// INFRASTRUCTURE ONLY: it builds the reference-backed checker under
// oracle/_ref and is never part of the CUDA library.
//
// The stepper and controller restate Boost.odeint 1.74.0 from its published
// formulas (controlled_runge_kutta::try_step, default_error_checker with
// a_x = a_dxdt = 1, default_step_adjuster, failed_step_checker(500),
// generic_rk / runge_kutta_dopri5 stage sums evaluated left to right as
// odeint's scale_sum operations do).  They are the same formulas the C
// oracle restates, so forward-sweep parity with real odeint stays unpinned;
// what this shim pins is the reference's own adjoint code and the AADC
// vector-Jacobian products it calls.
#ifndef VA_BOOST_SHIM_HPP
#define VA_BOOST_SHIM_HPP

#include <array>
#include <cfloat>
#include <limits>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <typeinfo>
#include <vector>

#define BOOST_THROW_EXCEPTION(e) throw(e)

namespace boost {

template <class T, std::size_t N> using array = std::array<T, N>;
template <class A, class B> struct is_same : std::is_same<A, B> {};

namespace numeric {
namespace ublas {

template <class T> class matrix {
  public:
    matrix() = default;
    matrix(std::size_t r, std::size_t c) : m_r(r), m_c(c), m_v(r * c, T()) {}
    T &operator()(std::size_t i, std::size_t j) { return m_v[i * m_c + j]; }
    const T &operator()(std::size_t i, std::size_t j) const { return m_v[i * m_c + j]; }
    std::size_t size1() const { return m_r; }
    std::size_t size2() const { return m_c; }

  private:
    std::size_t m_r = 0, m_c = 0;
    std::vector<T> m_v;
};

template <class T> using vector = std::vector<T>;

} // namespace ublas

namespace odeint {

// stepper categories (odeint/stepper/stepper_categories.hpp)
struct stepper_tag {};
struct error_stepper_tag {};
struct explicit_error_stepper_tag : error_stepper_tag {};
struct explicit_error_stepper_fsal_tag : error_stepper_tag {};
struct controlled_stepper_tag {};
struct explicit_controlled_stepper_tag : controlled_stepper_tag {};
struct explicit_controlled_stepper_fsal_tag : controlled_stepper_tag {};

enum controlled_step_result { success, fail };

template <class T> struct unwrap_reference { typedef T type; };
template <class T> struct unwrap_reference<std::reference_wrapper<T>> { typedef T type; };
template <class T> struct unit_value_type { typedef T type; };

struct null_observer {
    template <class State, class Time> void operator()(const State &, Time) const {}
};

class step_adjustment_error : public std::runtime_error {
  public:
    explicit step_adjustment_error(const std::string &s) : std::runtime_error(s) {}
};

// failed_step_checker: throws once more than max_steps attempts were made
// without a reset.
class failed_step_checker {
  public:
    explicit failed_step_checker(int max_steps = 500) : m_max_steps(max_steps) {}
    void operator()()
    {
        if (m_steps++ >= m_max_steps) {
            char msg[200];
            std::snprintf(msg, sizeof(msg), "Max number of iterations exceeded (%d). A new step size was not found.",
                          m_max_steps);
            BOOST_THROW_EXCEPTION(step_adjustment_error(msg));
        }
    }
    void reset() { m_steps = 0; }

  private:
    int m_max_steps;
    int m_steps = 0;
};

namespace detail {
template <class T> bool less_with_sign(T t1, T t2, T dt)
{
    if (dt > 0)
        return t2 - t1 > std::numeric_limits<T>::epsilon();
    return t1 - t2 > std::numeric_limits<T>::epsilon();
}
template <class T> bool less_eq_with_sign(T t1, T t2, T dt)
{
    if (dt > 0)
        return t1 - t2 <= std::numeric_limits<T>::epsilon();
    return t2 - t1 <= std::numeric_limits<T>::epsilon();
}
} // namespace detail

// ------------------------------------------------------------ coefficients
// Classic RK4 and Cash-Karp 5(4) (Cash & Karp 1990) as odeint names them.
template <class V> array<V, 1> rk4_coefficients_a1() { return {V(1) / V(2)}; }
template <class V> array<V, 2> rk4_coefficients_a2() { return {V(0), V(1) / V(2)}; }
template <class V> array<V, 3> rk4_coefficients_a3() { return {V(0), V(0), V(1)}; }
template <class V> array<V, 4> rk4_coefficients_b() { return {V(1) / V(6), V(1) / V(3), V(1) / V(3), V(1) / V(6)}; }
template <class V> array<V, 4> rk4_coefficients_c() { return {V(0), V(1) / V(2), V(1) / V(2), V(1)}; }

template <class V> array<V, 1> rk54_ck_coefficients_a1() { return {V(1) / V(5)}; }
template <class V> array<V, 2> rk54_ck_coefficients_a2() { return {V(3) / V(40), V(9) / V(40)}; }
template <class V> array<V, 3> rk54_ck_coefficients_a3() { return {V(3) / V(10), V(-9) / V(10), V(6) / V(5)}; }
template <class V> array<V, 4> rk54_ck_coefficients_a4()
{
    return {V(-11) / V(54), V(5) / V(2), V(-70) / V(27), V(35) / V(27)};
}
template <class V> array<V, 5> rk54_ck_coefficients_a5()
{
    return {V(1631) / V(55296), V(175) / V(512), V(575) / V(13824), V(44275) / V(110592), V(253) / V(4096)};
}
template <class V> array<V, 6> rk54_ck_coefficients_b()
{
    return {V(37) / V(378), V(0), V(250) / V(621), V(125) / V(594), V(0), V(512) / V(1771)};
}
template <class V> array<V, 6> rk54_ck_coefficients_db()
{
    return {V(37) / V(378) - V(2825) / V(27648), V(0), V(250) / V(621) - V(18575) / V(48384),
            V(125) / V(594) - V(13525) / V(55296), V(-277) / V(14336), V(512) / V(1771) - V(1) / V(4)};
}
template <class V> array<V, 6> rk54_ck_coefficients_c()
{
    return {V(0), V(1) / V(5), V(3) / V(10), V(3) / V(5), V(1), V(7) / V(8)};
}

// Fehlberg 7(8) (E. Fehlberg, NASA TR R-287, 1968): the coefficient functions
// odeint's runge_kutta_fehlberg78 provides and the reference's ButcherTable
// reads (ButcherTable.hpp:191-246); b propagates (eighth order), db = b - b_hat.
template <class V> array<V, 1> rk78_coefficients_a1() { return {V(2) / V(27)}; }
template <class V> array<V, 2> rk78_coefficients_a2() { return {V(1) / V(36), V(1) / V(12)}; }
template <class V> array<V, 3> rk78_coefficients_a3() { return {V(1) / V(24), V(0), V(1) / V(8)}; }
template <class V> array<V, 4> rk78_coefficients_a4() { return {V(5) / V(12), V(0), V(-25) / V(16), V(25) / V(16)}; }
template <class V> array<V, 5> rk78_coefficients_a5() { return {V(1) / V(20), V(0), V(0), V(1) / V(4), V(1) / V(5)}; }
template <class V> array<V, 6> rk78_coefficients_a6() { return {V(-25) / V(108), V(0), V(0), V(125) / V(108), V(-65) / V(27), V(125) / V(54)}; }
template <class V> array<V, 7> rk78_coefficients_a7() { return {V(31) / V(300), V(0), V(0), V(0), V(61) / V(225), V(-2) / V(9), V(13) / V(900)}; }
template <class V> array<V, 8> rk78_coefficients_a8() { return {V(2) / V(1), V(0), V(0), V(-53) / V(6), V(704) / V(45), V(-107) / V(9), V(67) / V(90), V(3) / V(1)}; }
template <class V> array<V, 9> rk78_coefficients_a9() { return {V(-91) / V(108), V(0), V(0), V(23) / V(108), V(-976) / V(135), V(311) / V(54), V(-19) / V(60), V(17) / V(6), V(-1) / V(12)}; }
template <class V> array<V, 10> rk78_coefficients_a10() { return {V(2383) / V(4100), V(0), V(0), V(-341) / V(164), V(4496) / V(1025), V(-301) / V(82), V(2133) / V(4100), V(45) / V(82), V(45) / V(164), V(18) / V(41)}; }
template <class V> array<V, 11> rk78_coefficients_a11() { return {V(3) / V(205), V(0), V(0), V(0), V(0), V(-6) / V(41), V(-3) / V(205), V(-3) / V(41), V(3) / V(41), V(6) / V(41), V(0)}; }
template <class V> array<V, 12> rk78_coefficients_a12() { return {V(-1777) / V(4100), V(0), V(0), V(-341) / V(164), V(4496) / V(1025), V(-289) / V(82), V(2193) / V(4100), V(51) / V(82), V(33) / V(164), V(12) / V(41), V(0), V(1) / V(1)}; }
template <class V> array<V, 13> rk78_coefficients_b() { return {V(0), V(0), V(0), V(0), V(0), V(34) / V(105), V(9) / V(35), V(9) / V(35), V(9) / V(280), V(9) / V(280), V(0), V(41) / V(840), V(41) / V(840)}; }
template <class V> array<V, 13> rk78_coefficients_c() { return {V(0), V(2) / V(27), V(1) / V(9), V(1) / V(6), V(5) / V(12), V(1) / V(2), V(5) / V(6), V(1) / V(6), V(2) / V(3), V(1) / V(3), V(1) / V(1), V(0), V(1) / V(1)}; }
template <class V> array<V, 13> rk78_coefficients_db() { return {V(-41) / V(840), V(0), V(0), V(0), V(0), V(0), V(0), V(0), V(0), V(0), V(-41) / V(840), V(41) / V(840), V(41) / V(840)}; }

// ------------------------------------------------------------------ steppers
// Explicit embedded pairs held as dense tables; do_step evaluates every sum
// left to right (x + (a0 dt) k0 + (a1 dt) k1 + ...) as odeint's scale_sum
// operators do, skipping exact-zero weights only where odeint's own code
// omits the term.
struct shim_tableau {
    int s;                    // stages (FSAL pairs: the last one is f(y_new))
    bool fsal;
    std::vector<std::vector<double>> a;
    std::vector<double> b, c, db; // db: b - b_hat
    int stepper_order, error_order;
};

template <class State> struct runge_kutta_cash_karp54 {
    typedef State state_type;
    typedef double value_type;
    typedef explicit_error_stepper_tag stepper_category;
    static shim_tableau tableau()
    {
        shim_tableau t;
        t.s = 6;
        t.fsal = false;
        auto a1 = rk54_ck_coefficients_a1<double>();
        auto a2 = rk54_ck_coefficients_a2<double>();
        auto a3 = rk54_ck_coefficients_a3<double>();
        auto a4 = rk54_ck_coefficients_a4<double>();
        auto a5 = rk54_ck_coefficients_a5<double>();
        t.a = {{}, {a1.begin(), a1.end()}, {a2.begin(), a2.end()}, {a3.begin(), a3.end()},
               {a4.begin(), a4.end()}, {a5.begin(), a5.end()}};
        auto b = rk54_ck_coefficients_b<double>();
        auto db = rk54_ck_coefficients_db<double>();
        auto c = rk54_ck_coefficients_c<double>();
        t.b.assign(b.begin(), b.end());
        t.db.assign(db.begin(), db.end());
        t.c.assign(c.begin(), c.end());
        t.stepper_order = 5;
        t.error_order = 4;
        return t;
    }
};

// Dormand-Prince 5(4) (Dormand & Prince 1980), 7 stages, FSAL.
template <class State> struct runge_kutta_dopri5 {
    typedef State state_type;
    typedef double value_type;
    typedef explicit_error_stepper_fsal_tag stepper_category;
    static shim_tableau tableau()
    {
        shim_tableau t;
        t.s = 7;
        t.fsal = true;
        t.a = {{},
               {1.0 / 5.0},
               {3.0 / 40.0, 9.0 / 40.0},
               {44.0 / 45.0, -56.0 / 15.0, 32.0 / 9.0},
               {19372.0 / 6561.0, -25360.0 / 2187.0, 64448.0 / 6561.0, -212.0 / 729.0},
               {9017.0 / 3168.0, -355.0 / 33.0, 46732.0 / 5247.0, 49.0 / 176.0, -5103.0 / 18656.0},
               {35.0 / 384.0, 0.0, 500.0 / 1113.0, 125.0 / 192.0, -2187.0 / 6784.0, 11.0 / 84.0}};
        t.b = {35.0 / 384.0, 0.0, 500.0 / 1113.0, 125.0 / 192.0, -2187.0 / 6784.0, 11.0 / 84.0, 0.0};
        t.c = {0.0, 1.0 / 5.0, 3.0 / 10.0, 4.0 / 5.0, 8.0 / 9.0, 1.0, 1.0};
        const double c1 = 35.0 / 384.0, c3 = 500.0 / 1113.0, c4 = 125.0 / 192.0, c5 = -2187.0 / 6784.0,
                     c6 = 11.0 / 84.0;
        t.db = {c1 - 5179.0 / 57600.0, 0.0, c3 - 7571.0 / 16695.0, c4 - 393.0 / 640.0, c5 - -92097.0 / 339200.0,
                c6 - 187.0 / 2100.0, -1.0 / 40.0};
        t.stepper_order = 5;
        t.error_order = 4;
        return t;
    }
};

// Fixed-step steppers for the reference's non-controlled loop
// (detail/runge_kutta.hpp:37-72).  euler: out = 1 x + dt f(x) (odeint's
// scale_sum2(1, dt)); runge_kutta4: odeint's generic explicit RK with the
// rk4 coefficients, each stage x + (a_m0 dt) k_0 + ... left to right with
// every coefficient of the row, then x + (b_0 dt) k_0 + ... + (b_3 dt) k_3.
template <class State> struct euler {
    typedef State state_type;
    typedef stepper_tag stepper_category;
    template <class System> void do_step(System system, State &x, double t, double dt)
    {
        State dxdt(x.size());
        system(x, dxdt, t);
        for (std::size_t i = 0; i < x.size(); i++)
            x[i] = 1.0 * x[i] + dt * dxdt[i];
    }
};
template <class State> struct runge_kutta4 {
    typedef State state_type;
    typedef stepper_tag stepper_category;
    template <class System> void do_step(System system, State &x, double t, double dt)
    {
        const std::size_t n = x.size();
        const auto a1 = rk4_coefficients_a1<double>();
        const auto a2 = rk4_coefficients_a2<double>();
        const auto a3 = rk4_coefficients_a3<double>();
        const auto b = rk4_coefficients_b<double>();
        const auto c = rk4_coefficients_c<double>();
        const std::vector<std::vector<double>> a = {{}, {a1.begin(), a1.end()}, {a2.begin(), a2.end()},
                                                    {a3.begin(), a3.end()}};
        std::vector<State> K(4, State(n));
        State xtmp(n);
        system(x, K[0], t);
        for (int m = 1; m < 4; m++) {
            for (std::size_t i = 0; i < n; i++) {
                double acc = 1.0 * x[i];
                for (int j = 0; j < m; j++)
                    acc = acc + (a[m][j] * dt) * K[j][i];
                xtmp[i] = acc;
            }
            system(xtmp, K[m], t + c[m] * dt);
        }
        for (std::size_t i = 0; i < n; i++) {
            double acc = 1.0 * x[i];
            for (int j = 0; j < 4; j++)
                acc = acc + (b[j] * dt) * K[j][i];
            x[i] = acc;
        }
    }
};
template <class State> struct runge_kutta4_classic : runge_kutta4<State> {
};
template <class State> struct runge_kutta_fehlberg78 {
    typedef State state_type;
    typedef double value_type;
    typedef explicit_error_stepper_tag stepper_category;
    static shim_tableau tableau()
    {
        shim_tableau t;
        t.s = 13;
        t.fsal = false;
        auto a1 = rk78_coefficients_a1<double>();
        auto a2 = rk78_coefficients_a2<double>();
        auto a3 = rk78_coefficients_a3<double>();
        auto a4 = rk78_coefficients_a4<double>();
        auto a5 = rk78_coefficients_a5<double>();
        auto a6 = rk78_coefficients_a6<double>();
        auto a7 = rk78_coefficients_a7<double>();
        auto a8 = rk78_coefficients_a8<double>();
        auto a9 = rk78_coefficients_a9<double>();
        auto a10 = rk78_coefficients_a10<double>();
        auto a11 = rk78_coefficients_a11<double>();
        auto a12 = rk78_coefficients_a12<double>();
        t.a = {{},
               {a1.begin(), a1.end()},   {a2.begin(), a2.end()},   {a3.begin(), a3.end()},
               {a4.begin(), a4.end()},   {a5.begin(), a5.end()},   {a6.begin(), a6.end()},
               {a7.begin(), a7.end()},   {a8.begin(), a8.end()},   {a9.begin(), a9.end()},
               {a10.begin(), a10.end()}, {a11.begin(), a11.end()}, {a12.begin(), a12.end()}};
        auto b = rk78_coefficients_b<double>();
        auto db = rk78_coefficients_db<double>();
        auto c = rk78_coefficients_c<double>();
        t.b.assign(b.begin(), b.end());
        t.db.assign(db.begin(), db.end());
        t.c.assign(c.begin(), c.end());
        t.stepper_order = 8;
        t.error_order = 7;
        return t;
    }
};

// controlled_runge_kutta<ErrorStepper> with odeint's default error checker
// and step adjuster.
template <class ErrorStepper> class controlled_runge_kutta {
  public:
    typedef typename ErrorStepper::state_type state_type;
    typedef typename std::conditional<std::is_same<typename ErrorStepper::stepper_category,
                                                   explicit_error_stepper_fsal_tag>::value,
                                      explicit_controlled_stepper_fsal_tag,
                                      explicit_controlled_stepper_tag>::type stepper_category;

    controlled_runge_kutta(double eps_abs = 1e-6, double eps_rel = 1e-6)
        : m_abs(eps_abs), m_rel(eps_rel), m_tab(ErrorStepper::tableau())
    {
    }

    template <class System>
    controlled_step_result try_step(System system, state_type &x, double &t, double &dt)
    {
        const std::size_t n = x.size();
        if (m_first || !m_tab.fsal) {
            // non-FSAL: dxdt = f(x, t) on every attempt; FSAL: on the first call
            m_dxdt.assign(n, 0.0);
            system(x, m_dxdt, t);
            m_first = false;
        }
        std::vector<std::vector<double>> K(m_tab.s, std::vector<double>(n));
        K[0] = m_dxdt;
        state_type xtmp(n), out(n), err(n);
        const int s_eval = m_tab.fsal ? m_tab.s - 1 : m_tab.s;
        for (int m = 1; m < s_eval; m++) {
            for (std::size_t i = 0; i < n; i++) {
                double acc = 1.0 * x[i];
                for (int j = 0; j < m; j++)
                    acc = acc + (m_tab.a[m][j] * dt) * K[j][i];
                xtmp[i] = acc;
            }
            system(xtmp, K[m], t + m_tab.c[m] * dt);
        }
        for (std::size_t i = 0; i < n; i++) {
            double acc = 1.0 * x[i];
            for (int j = 0; j < s_eval; j++)
                if (!(m_tab.fsal && m_tab.b[j] == 0.0)) // dopri5 omits k2
                    acc = acc + (m_tab.b[j] * dt) * K[j][i];
            out[i] = acc;
        }
        std::vector<double> dxdt_new;
        if (m_tab.fsal) {
            dxdt_new.assign(n, 0.0);
            system(out, dxdt_new, t + dt);
        }
        for (std::size_t i = 0; i < n; i++) {
            double acc = 0.0;
            bool first = true;
            for (int j = 0; j < s_eval; j++) {
                if (m_tab.fsal && m_tab.db[j] == 0.0) // dopri5 omits k2
                    continue;
                const double term = (m_tab.db[j] * dt) * K[j][i];
                acc = first ? term : acc + term;
                first = false;
            }
            if (m_tab.fsal)
                acc = acc + (m_tab.db[m_tab.s - 1] * dt) * dxdt_new[i];
            err[i] = acc;
        }
        // default_error_checker::error: max_i |err_i| / (eps_abs + eps_rel (|x_i| + |dt| |dxdt_i|))
        double max_rel = 0.0;
        for (std::size_t i = 0; i < n; i++) {
            const double r =
                std::abs(err[i]) / (m_abs + m_rel * (1.0 * std::abs(x[i]) + std::abs(dt) * std::abs(m_dxdt[i])));
            max_rel = std::max(max_rel, r);
        }
        if (max_rel > 1.0) {
            // default_step_adjuster::decrease_step
            dt *= std::max(9.0 / 10.0 * std::pow(max_rel, -1.0 / (m_tab.error_order - 1)), 1.0 / 5.0);
            return fail;
        }
        t += dt;
        // default_step_adjuster::increase_step
        if (max_rel < 0.5) {
            max_rel = std::max(std::pow(5.0, -(double)m_tab.stepper_order), max_rel);
            dt *= 9.0 / 10.0 * std::pow(max_rel, -1.0 / m_tab.stepper_order);
        }
        x = out;
        if (m_tab.fsal)
            m_dxdt = dxdt_new;
        return success;
    }

  private:
    double m_abs, m_rel;
    shim_tableau m_tab;
    bool m_first = true;
    std::vector<double> m_dxdt;
};

template <class ErrorStepper>
controlled_runge_kutta<ErrorStepper> make_controlled(double abs_error, double rel_error,
                                                     ErrorStepper = ErrorStepper())
{
    return controlled_runge_kutta<ErrorStepper>(abs_error, rel_error);
}

} // namespace odeint
} // namespace numeric
} // namespace boost

#endif
