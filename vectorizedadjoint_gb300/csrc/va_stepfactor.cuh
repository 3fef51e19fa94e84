// Step-size factors of odeint's default_step_adjuster (Boost 1.74, called
// from controlled_runge_kutta::try_step at lib/include/detail/
// runge_kutta.hpp:103-107):
//   decrease_step: dt *= max(0.9 pow(err, -1.0/(q-1)), 0.2)
//   increase_step: dt *= 0.9 pow(max(err, pow(5.0, -p)), -1.0/p)
// with q the error order and p the stepper order (5(4) pairs: -1.0/3 and
// -1.0/5; Fehlberg 7(8): -1.0/6 and -1.0/8).  Two ways to form the power:
//
//  - inv_root<K>: Newton's iteration for the inverse K-th root (fast; a few
//    ulps from the true power).
//  - cr_step_pow<K>: the correctly rounded value of pow(x, -1.0/K), the
//    exponent being the DOUBLE -1.0/K that odeint passes (for K = 3, 5, 6
//    it is not exactly -1/K).  A correctly rounded pow is the platform-
//    independent meaning of odeint's std::pow; with it the forward sweep
//    takes the reference's accepted steps wherever the host's libm pow
//    returns the correctly rounded value too.
//
// Self-contained (IEEE adds, multiplies and fused multiply-adds, one call
// of log), so the same code compiles for the host and is checked there
// against an arbitrary-precision power (tests/test_stepfactor.py).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#ifndef __CUDACC__
#ifndef VA_HD
#define VA_HD
#endif
#define VA_HD_NOINLINE
#else
#ifndef VA_HD
#define VA_HD __host__ __device__
#endif
#define VA_HD_NOINLINE __host__ __device__ __noinline__
#endif

namespace va {

VA_HD inline int32_t f32_bits(float f)
{
#ifdef __CUDA_ARCH__
    return __float_as_int(f);
#else
    int32_t i;
    std::memcpy(&i, &f, 4);
    return i;
#endif
}
VA_HD inline float f32_from_bits(int32_t i)
{
#ifdef __CUDA_ARCH__
    return __int_as_float(i);
#else
    float f;
    std::memcpy(&f, &i, 4);
    return f;
#endif
}

// a^(-1/K) for the step-size controller, without a double-precision pow
// (FP64 issues at 1/61 of the FP32 rate on this part).  Newton's iteration
// for the inverse K-th root, x <- x + x (1 - a x^K) / K, from a seed built on
// the float bit pattern (log2 read off the exponent field and scaled by
// -1/K, the idea of the classic fast inverse square root): four FP32 steps
// (seed error ~6% -> ~1e-7), two FP64 steps (-> ~1e-14 -> rounding).  Only
// IEEE adds, multiplies and fused multiply-adds, in a fixed order: the
// result has the same bits on any IEEE machine, which the oracle relies on
// for a bit-exact comparison of step sequences.  a >= 1e30 (decrease only)
// returns 0, which the 0.2 limiter turns into the same factor pow would.
template <int K>
VA_HD inline float inv_root_f32(float af)
{
    constexpr int32_t c = (int32_t)(((int64_t)(K + 1) * 0x3F800000LL) / K);
    float x = f32_from_bits(c - f32_bits(af) / K);
    const float rk = 1.0f / (float)K;
#pragma unroll
    for (int it = 0; it < 4; it++) {
        float xk = x;
#pragma unroll
        for (int k = 1; k < K; k++)
            xk = xk * x;
        const float r = fmaf(-af, xk, 1.0f);
        x = fmaf(x * r, rk, x);
    }
    return x;
}

template <int K, int FP64_STEPS = 2>
VA_HD inline double inv_root(double a)
{
    if (!(a < 1e30))
        return 0.0;
    const float x = inv_root_f32<K>((float)a);
    double xd = (double)x;
#pragma unroll
    for (int it = 0; it < FP64_STEPS; it++) {
        double xk = xd;
#pragma unroll
        for (int k = 1; k < K; k++)
            xk = xk * xd;
        const double r = fma(-a, xk, 1.0);
        xd = fma(xd * r, 1.0 / K, xd);
    }
    return xd;
}

// ------------------------------------------------- correctly rounded power
//
// pow(x, y) for y = fl(-1/K), K in {3, 5, 6, 8}.  Write y = -(1 + e)/K with
// e = K fl(1/K) - 1 (exactly -2^-54 for K = 3 and 6, +2^-54 for K = 5, 0 for
// K = 8).  Then x^y = R^(1+e) = R exp(e ln R), R = x^(-1/K).
//
//  1. r0 = inv_root<K>(x), within a few ulps of R.
//  2. rho = 1 - x r0^K, formed with error-free products (double-double,
//     relative error < 2^-101), so that R = r0 (1 - rho)^(-1/K)
//     = r0 (1 + rho/K + (K+1) rho^2/(2K^2) + O(rho^3)), |rho| < 2^-49.
//  3. exp(e ln R) = 1 + u + u^2/2 + O(u^3), u = -(e/K) ln x, |u| < 2^-49
//     for x < 1e30 (ln x from log(), within an ulp: its error moves the
//     result by < 2^-101).
//  4. P = r0 (1 + w), w = c + v + c v with c and v the two corrections,
//     the product r0 w taken exactly (TwoProd): P = ph + pl with
//     |P - x^y| < 2^-98 x^y.
//  5. Ziv's rounding test (Ziv 1991, "Fast evaluation of elementary
//     mathematical functions with correctly rounded last bit"): round the
//     two ends of [P - 2^-95 ph, P + 2^-95 ph]; rounding is monotone, so if
//     both give the same double, that double is the correctly rounded
//     x^y.  Otherwise (probability ~2^-42 per call) the value is too close
//     to a rounding boundary for this precision: the nearer end is returned
//     and *undecided is incremented, so that such a call is never silent.
//
// Domain: 0 < x < 1e30 (the controller's errors: increase_step takes
// err >= 5^-p >= 2.56e-6, decrease_step err > 1; for err >= 1e30 the 0.2
// limiter makes the factor irrelevant and 0 is returned, as inv_root does).
// x = 1 gives exactly 1.

struct DD {
    double hi, lo;
};

VA_HD inline DD dd_two_prod(double a, double b)
{
    const double p = a * b;
    return {p, fma(a, b, -p)};
}
// |a| >= |b| (or a = 0)
VA_HD inline DD dd_fast_two_sum(double a, double b)
{
    const double s = a + b;
    return {s, b - (s - a)};
}
// (a.hi + a.lo) b, |a.lo| <= ulp(a.hi)/2: relative error < 2^-104
VA_HD inline DD dd_mul_d(DD a, double b)
{
    const DD p = dd_two_prod(a.hi, b);
    return dd_fast_two_sum(p.hi, fma(a.lo, b, p.lo));
}
// (a.hi + a.lo)(b.hi + b.lo): relative error < 2^-103
VA_HD inline DD dd_mul(DD a, DD b)
{
    const DD p = dd_two_prod(a.hi, b.hi);
    return dd_fast_two_sum(p.hi, fma(a.hi, b.lo, fma(a.lo, b.hi, p.lo)));
}

// r^K as a double-double
template <int K>
VA_HD inline DD dd_ipow(double r)
{
    static_assert(K == 3 || K == 5 || K == 6 || K == 8, "step-factor roots of odeint's 5(4) and 7(8) pairs");
    const DD r2 = dd_two_prod(r, r);
    if constexpr (K == 3)
        return dd_mul_d(r2, r);
    if constexpr (K == 5)
        return dd_mul_d(dd_mul(r2, r2), r);
    if constexpr (K == 6) {
        const DD r3 = dd_mul_d(r2, r);
        return dd_mul(r3, r3);
    }
    const DD r4 = dd_mul(r2, r2);
    return dd_mul(r4, r4);
}

// e / K with e = K fl(1/K) - 1: the exponent's offset from -1/K
template <int K>
struct StepPowExp {
    static constexpr double e_over_k = (K == 5 ? 0x1p-54 : (K == 8 ? 0.0 : -0x1p-54)) / K;
};

// Steps 1-4 with ln x given: x^y = ph + pl within 2^-98 relative plus
// (e/K) |ln x - lnx| (0 < x < 1e30)
template <int K>
VA_HD inline void step_pow_dd_ln(double x, double lnx, double &ph, double &pl)
{
    const double r0 = inv_root<K, 2>(x);
    // rho = 1 - x r0^K (1 - q.hi is exact: q.hi is within 2^-48 of 1)
    const DD q = dd_mul_d(dd_ipow<K>(r0), x);
    const double rho = (1.0 - q.hi) - q.lo;
    // (1 - rho)^(-1/K) - 1 to second order
    constexpr double c1 = 1.0 / K, c2 = (K + 1.0) / (2.0 * K * K);
    const double c = rho * fma(c2, rho, c1);
    // R^e - 1 = u + u^2/2, u = e ln R = -(e/K) ln x
    double v = 0.0;
    if constexpr (K != 8) {
        const double u = -StepPowExp<K>::e_over_k * lnx;
        v = fma(0.5 * u, u, u);
    }
    const double w = fma(c, v, c + v);
    // P = r0 + r0 w, the product exact
    const DD t = dd_two_prod(r0, w);
    const DD s = dd_fast_two_sum(r0, t.hi);
    ph = s.hi;
    pl = s.lo + t.lo;
}

// Steps 1-4: x^y = ph + pl within 2^-98 relative (0 < x < 1e30)
template <int K>
VA_HD inline void step_pow_dd(double x, double &ph, double &pl)
{
    step_pow_dd_ln<K>(x, K != 8 ? log(x) : 0.0, ph, pl);
}

// Step 5 and the domain ends, in two passes.  The first takes ln x from
// the float logarithm, (double)logf((float)x): within 2^-24 (the rounding
// of x to float) + 1 ulp of |ln x| < 70, i.e. < 2^-16.9 absolute, which
// moves u by < 2^-72.5 relative (|e/K| <= 2^-55.6); its rounding test uses
// the window 2^-70 and decides all but ~2^-17 of the calls.  The others
// take the second pass with the double logarithm and the window 2^-95.
// Both return the correctly rounded value: the same double either way.
template <int K>
VA_HD_NOINLINE double cr_step_pow(double x, unsigned int *undecided)
{
    if (!(x < 1e30))
        return x != x ? x : 0.0;
    double ph, pl;
    if constexpr (K != 8) {
        step_pow_dd_ln<K>(x, (double)logf((float)x), ph, pl);
        const double E1 = 0x1p-70 * ph;
        const double a1 = ph + (pl - E1), b1 = ph + (pl + E1);
        if (a1 == b1)
            return ph + pl;
    }
    step_pow_dd<K>(x, ph, pl);
    // Ziv's rounding test over [P - E, P + E], E = 2^-95 ph
    const double E = 0x1p-95 * ph;
    const double a = ph + (pl - E), b = ph + (pl + E);
    if (a != b && undecided) {
#ifdef __CUDA_ARCH__
        atomicAdd(undecided, 1u);
#else
        ++*undecided;
#endif
    }
    return ph + pl;
}

} // namespace va
