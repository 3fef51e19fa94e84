// A reference-style program (the call sequence of the reference's
// examples/VanDerPol/main.cpp) against va_driver.hpp.  Usage:
//   driver_example <mu> <x0> <v0> <t1> <tol> [dopri5|rkf78|rk4|euler] [dt] [observe]
// Prints: steps, x(T), then the Nout x Nin lambda and Nout x Npar mu rows
// after adjointSolve with identity seeds, then the sensitivity matrix.
// With "observe": the forward observer's (t, x) records ("obs") and the
// adjoint observer's (t, lambda rows) records ("aobs") as well.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "va_driver.hpp"

using namespace vectorizedadjoint_gb300;
using State = std::vector<double>;

template <class Stepper, class StepperTag>
static int run(Stepper stepper, StepperTag tag, State mu, State x0, double t1, double dt, bool observe)
{
    const int N = 2, Npar = 1;
    Driver driver(N, N, Npar);
    auto vdp = VanDerPol();
    size_t steps = 0;
    if (observe) {
        auto obs = [](const State &x, double t) { std::printf("obs %.17g %.17g %.17g\n", t, x[0], x[1]); };
        steps = runge_kutta(stepper, vdp, x0, mu, 0.0, t1, dt, driver, obs);
    } else {
        steps = runge_kutta(stepper, vdp, x0, mu, 0.0, t1, dt, driver);
    }
    std::printf("steps %zu\nx %.17g %.17g\n", steps, x0[0], x0[1]);
    auto lambda = std::vector<std::vector<double>>(N, std::vector<double>(N, 0.0));
    lambda[0][0] = 1.0;
    lambda[1][1] = 1.0;
    auto muadj = std::vector<std::vector<double>>(N, std::vector<double>(Npar, 0.0));
    setCostGradients(driver, lambda, muadj);
    constructDriverButcherTableau(driver, tag);
    recordDriverRHSFunction(driver, vdp);
    if (observe) {
        auto aobs = [](const std::vector<std::vector<double>> &l, double t) {
            std::printf("aobs %.17g %.17g %.17g %.17g %.17g\n", t, l[0][0], l[0][1], l[1][0], l[1][1]);
        };
        adjointSolve(driver, mu, aobs);
    } else {
        adjointSolve(driver, mu);
    }
    for (int i = 0; i < N; i++)
        std::printf("lambda %.17g %.17g\n", lambda[i][0], lambda[i][1]);
    for (int i = 0; i < N; i++)
        std::printf("mu %.17g\n", muadj[i][0]);
    auto S = computeSensitivityMatrix(driver, mu);
    for (int i = 0; i < N; i++)
        std::printf("sens %.17g\n", S[i][0]);
    auto S1 = computeSensitivityMatrixNoSIMD(driver, mu);
    for (int i = 0; i < N; i++)
        std::printf("sens1 %.17g\n", S1[i][0]);
    return 0;
}

int main(int argc, char **argv)
{
    if (argc < 6) {
        std::fprintf(stderr, "usage: %s mu x0 v0 t1 tol [dopri5|rkf78|rk4|euler] [dt] [observe]\n", argv[0]);
        return 1;
    }
    State mu = {std::atof(argv[1])};
    State x0 = {std::atof(argv[2]), std::atof(argv[3])};
    const double t1 = std::atof(argv[4]), tol = std::atof(argv[5]);
    const char *name = argc > 6 ? argv[6] : "dopri5";
    const double dt = argc > 7 ? std::atof(argv[7]) : 1e-3;
    const bool ob = argc > 8 && !std::strcmp(argv[8], "observe");
    if (!std::strcmp(name, "rkf78")) {
        typedef runge_kutta_fehlberg78<State> stepper_type;
        return run(make_controlled<stepper_type>(tol, tol), stepper_type(), mu, x0, t1, dt, ob);
    }
    if (!std::strcmp(name, "rk4"))
        return run(runge_kutta4<State>(), runge_kutta4<State>(), mu, x0, t1, dt, ob);
    if (!std::strcmp(name, "euler"))
        return run(euler<State>(), euler<State>(), mu, x0, t1, dt, ob);
    typedef runge_kutta_dopri5<State> stepper_type;
    return run(make_controlled<stepper_type>(tol, tol), stepper_type(), mu, x0, t1, dt, ob);
}
