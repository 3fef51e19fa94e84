// Host build of the library's step-factor power (csrc/va_stepfactor.cuh) for
// tests/test_stepfactor.py, which checks it against an arbitrary-precision
// power.  Compiled with g++ -ffp-contract=off, as the FP64 kernels are built
// without contraction.
#include "../../vectorizedadjoint_gb300/csrc/va_stepfactor.cuh"

extern "C" {
// correctly rounded pow(x, -1.0/k), k in {3, 5, 6, 8}; *undecided counts
// failed rounding tests
double sf_cr_pow(int k, double x, unsigned int *undecided)
{
    switch (k) {
    case 3: return va::cr_step_pow<3>(x, undecided);
    case 5: return va::cr_step_pow<5>(x, undecided);
    case 6: return va::cr_step_pow<6>(x, undecided);
    case 8: return va::cr_step_pow<8>(x, undecided);
    default: return -1.0;
    }
}
// the double-double value before rounding: x^(-1.0/k) ~ ph + pl
void sf_dd(int k, double x, double *ph, double *pl)
{
    switch (k) {
    case 3: va::step_pow_dd<3>(x, *ph, *pl); break;
    case 5: va::step_pow_dd<5>(x, *ph, *pl); break;
    case 6: va::step_pow_dd<6>(x, *ph, *pl); break;
    default: va::step_pow_dd<8>(x, *ph, *pl); break;
    }
}
// the first pass of cr_step_pow: ln x from the float logarithm
void sf_dd_fastln(int k, double x, double *ph, double *pl)
{
    const double lnx = (double)logf((float)x);
    switch (k) {
    case 3: va::step_pow_dd_ln<3>(x, lnx, *ph, *pl); break;
    case 5: va::step_pow_dd_ln<5>(x, lnx, *ph, *pl); break;
    case 6: va::step_pow_dd_ln<6>(x, lnx, *ph, *pl); break;
    default: va::step_pow_dd_ln<8>(x, 0.0, *ph, *pl); break;
    }
}
// the Newton root the fast controller uses
double sf_inv_root(int k, double x)
{
    switch (k) {
    case 3: return va::inv_root<3, 2>(x);
    case 5: return va::inv_root<5, 2>(x);
    case 6: return va::inv_root<6, 2>(x);
    case 8: return va::inv_root<8, 2>(x);
    default: return -1.0;
    }
}
}
