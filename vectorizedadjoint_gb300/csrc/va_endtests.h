// The two time tests of the controlled loop (lib/include/detail/
// runge_kutta.hpp:155-163, odeint's less_with_sign with dt > 0):
//   loop      while (fl(t1 - t) > eps)
//   end clamp if (fl(fl(t + dt) - t1) > eps) dt = t1 - t
// as comparisons of the doubles' bit patterns against two per-instance
// thresholds, without FP64 arithmetic on the step's critical path (each FP64
// operation of a warp occupies the FP64 pipe for 64 FP32 slots on this part).
//
// For t <= t1 and t1 >= 4 eps (the fast case):
//  - fl(t1 - x) is monotone in x and exact for x >= t1/2 (Sterbenz), so
//    fl(t1 - x) > eps  <=>  x < t1 - eps (real)  <=>  x <= lo, with lo the
//    largest double below the real t1 - eps; for x < t1/2 both sides hold
//    (fl(t1 - x) >= t1/2 > eps: t1 = 2 eps fails here, hence the margin).
//  - likewise fl(x - t1) > eps  <=>  x > hi, with hi the largest double not
//    above the real t1 + eps (x < t1/2: both false; x > 2 t1: both true).
// lo and hi come from one 2Sum each.  As signed 64-bit integers, the bit
// patterns of non-negative doubles order like the doubles and those of
// negative doubles fall below every non-negative one, which is all the
// comparisons against the positive thresholds need.  Instances whose end
// time is below 4 eps or not finite keep the FP64 expressions.  The equivalence is checked exhaustively around both
// thresholds by tests/test_endtests.py (tests/cpp/endtests_check.cpp).
#pragma once

#include <cstdint>
#include <cstring>

#ifndef __CUDACC__
#define VA_HD
#else
#define VA_HD __host__ __device__
#endif

namespace va {

constexpr double kEndEps = 2.220446049250313080847e-16; // std::numeric_limits<double>::epsilon()

VA_HD inline int64_t dbits(double x)
{
#ifdef __CUDA_ARCH__
    return __double_as_longlong(x);
#else
    int64_t i;
    std::memcpy(&i, &x, 8);
    return i;
#endif
}

struct EndTests {
    bool fast;  // the thresholds apply
    int64_t lo; // bits of the largest double x with fl(t1 - x) > eps
    int64_t hi; // bits of the largest double x with fl(x - t1) <= eps
};

// a + b = s + e exactly (Knuth's 2Sum)
VA_HD inline double two_sum_err(double a, double b, double s)
{
    const double bb = s - a;
    return (a - (s - bb)) + (b - bb);
}

VA_HD inline EndTests end_tests(double t1)
{
    EndTests e{};
    e.fast = t1 >= 4.0 * kEndEps && t1 < 1e300;
    if (!e.fast)
        return e;
    const double y = t1 - kEndEps; // t1 - eps = y + ey
    const double ey = two_sum_err(t1, -kEndEps, y);
    e.lo = ey > 0.0 ? dbits(y) : dbits(y) - 1; // y < t1 - eps, else the double below y
    const double z = t1 + kEndEps; // t1 + eps = z + ez
    const double ez = two_sum_err(t1, kEndEps, z);
    e.hi = ez >= 0.0 ? dbits(z) : dbits(z) - 1;
    return e;
}

// while (less_with_sign(t, t1, dt)): fl(t1 - t) > eps
VA_HD inline bool end_loop(const EndTests &e, double t, double t1)
{
    return e.fast ? dbits(t) <= e.lo : t1 - t > kEndEps;
}

// end clamp: fl(x - t1) > eps for x = fl(t + dt)
VA_HD inline bool end_clamp(const EndTests &e, double x, double t1)
{
    return e.fast ? dbits(x) > e.hi : x - t1 > kEndEps;
}

} // namespace va
