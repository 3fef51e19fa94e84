// Checks va_endtests.h against the FP64 expressions it replaces: for many
// end times t1 (log-uniform over 1.3e-15 .. 1e15, plus round values and the
// smallest fast one, 4 eps) and every
// double within 3000 ulps of each threshold, plus random points in [-3 t1, 3 t1],
// end_loop / end_clamp must equal fl(t1 - t) > eps / fl(x - t1) > eps.
// Prints the number of comparisons and of mismatches; exit code 1 on any.
#include <cmath>
#include <cstdio>
#include <random>

#include "../../vectorizedadjoint_gb300/csrc/va_endtests.h"

using namespace va;

static double from_bits(int64_t b)
{
    double x;
    std::memcpy(&x, &b, 8);
    return x;
}

int main()
{
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> u(0.0, 1.0);
    long checks = 0, bad = 0;
    auto check = [&](const EndTests &e, double x, double t1) {
        if (!std::isfinite(x))
            return;
        const bool l_ref = t1 - x > kEndEps, c_ref = x - t1 > kEndEps;
        if (end_loop(e, x, t1) != l_ref || end_clamp(e, x, t1) != c_ref) {
            if (bad < 10)
                std::printf("mismatch t1=%.17g x=%.17g\n", t1, x);
            bad++;
        }
        checks++;
    };
    double fixed[] = {1.0, 2.0, 10.0, 20.0, 50.0, 0.5, 1e-3, 3.0, 7.0, 1e6, 8.881784197001252e-16,
                      1.1102230246251565e-15, 1e-15, 1e15};
    for (int k = 0; k < 20000; k++) {
        const double t1 = k < 14 ? fixed[k] : std::pow(10.0, -14.9 + 29.9 * u(rng));
        const EndTests e = end_tests(t1);
        if (!e.fast) {
            std::printf("not fast: t1=%.17g\n", t1);
            return 1;
        }
        for (int64_t d = -3000; d <= 3000; d++) {
            check(e, from_bits(e.lo + d), t1);
            check(e, from_bits(e.hi + d), t1);
        }
        for (int r = 0; r < 200; r++) {
            check(e, 3.0 * t1 * u(rng), t1);
            check(e, -3.0 * t1 * u(rng), t1);
        }
        check(e, 0.0, t1);
        check(e, -0.0, t1);
    }
    std::printf("%ld checks, %ld mismatches\n", checks, bad);
    return bad ? 1 : 0;
}
