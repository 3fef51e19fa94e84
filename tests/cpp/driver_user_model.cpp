// The reference's call sequence (examples/VanDerPol/main.cpp) with a model of
// the caller's own: the Brusselator of tests/cpp/user_models.cuh, compiled
// into its own library (tests/cpp/user_model_brusselator.cu) and named here by
// a host tag, the way a reference program names its functor.  Usage:
//   driver_user_model <a> <b> <x0> <y0> <t1> <tol>
// Prints steps, the state at t1 and the lambda / mu rows after adjointSolve
// with identity seeds.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "va_driver.hpp"

extern "C" const va_model_kernels *brusselator_kernels(void);

struct Brusselator {
    static const va_model_kernels *va_kernels() { return brusselator_kernels(); }
};

using namespace vectorizedadjoint_gb300;
using State = std::vector<double>;

int main(int argc, char **argv)
{
    if (argc < 7) {
        std::fprintf(stderr, "usage: %s a b x0 y0 t1 tol\n", argv[0]);
        return 1;
    }
    State alphas = {std::atof(argv[1]), std::atof(argv[2])};
    State x0 = {std::atof(argv[3]), std::atof(argv[4])};
    const double t1 = std::atof(argv[5]), tol = std::atof(argv[6]);
    const int N = 2, Npar = 2;
    typedef runge_kutta_dopri5<State> stepper_type;
    Driver driver(N, N, Npar);
    size_t steps = runge_kutta(make_controlled<stepper_type>(tol, tol), Brusselator(), x0, alphas, 0.0, t1, 1e-3,
                               driver);
    std::printf("steps %zu\nx %.17g %.17g\n", steps, x0[0], x0[1]);
    std::vector<std::vector<double>> lambda = {{1.0, 0.0}, {0.0, 1.0}};
    std::vector<std::vector<double>> mu(N, std::vector<double>(Npar, 0.0));
    setCostGradients(driver, lambda, mu);
    constructDriverButcherTableau(driver, stepper_type());
    recordDriverRHSFunction(driver, Brusselator());
    adjointSolve(driver, alphas);
    for (int i = 0; i < N; i++)
        std::printf("lambda %.17g %.17g\n", lambda[i][0], lambda[i][1]);
    for (int i = 0; i < N; i++)
        std::printf("mu %.17g %.17g\n", mu[i][0], mu[i][1]);
    return 0;
}
