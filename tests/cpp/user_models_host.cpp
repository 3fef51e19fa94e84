// Host callbacks of the test models for the oracle (g++ -ffp-contract=off:
// the same operation order as the FP64 device code built with -fmad=false).
#include "user_models.cuh"

extern "C" {
void duffing_rhs(const double *x, const double *p, double t, double *f) { ForcedDuffing::rhs<double>(x, p, t, f); }
void duffing_vjp(const double *w, const double *x, const double *p, double t, double *gx, double *gp)
{
    ForcedDuffing::vjp<double>(w, x, p, t, gx, gp);
}
void brusselator_rhs(const double *x, const double *p, double t, double *f) { Brusselator::rhs<double>(x, p, t, f); }
void brusselator_vjp(const double *w, const double *x, const double *p, double t, double *gx, double *gp)
{
    Brusselator::vjp<double>(w, x, p, t, gx, gp);
}
}
