// Right-hand sides and hand-written vector-Jacobian products of the built-in
// models (N states, P parameters read by the RHS, PG parameter gradients).  They take the place of the user functor the reference records
// with AADC (lib/include/AadData.hpp:124-171) and of the JIT reverse code it
// replays in AadData::VectorTimesJacobians (AadData.hpp:291-330): every
// model gives f(x, p, t) and (J_x^T w, J_p^T w) at the same point.
//
// The argument order (x, p, t) keeps the reference functor's
// (x, dxdt, params, t) meaning (examples/VanDerPol/main.cpp:38-43).  S is the
// stage arithmetic type: double for the FP64 path, float for the mixed path,
// dword for the double-word path.  The double-word forms write each sum of
// products through the compensated accumulator (dacc) instead of a
// double-word multiply followed by a double-word add: the same O(u^2)
// accuracy in about half the FP32 operations.  The FP64 forms keep the
// reference's operation order (the FP64 path is compared bit for bit).
// Parameter layouts follow the reference examples.
#pragma once

#include <type_traits>

#include "va_dword.cuh"

namespace va {

template <class S>
constexpr bool is_dw = std::is_same<S, dword>::value;

// exact product by -2 of a double-word
__host__ __device__ __forceinline__ dword dw_m2(dword v) { return dword(-2.0f * v.hi, -2.0f * v.lo); }

// 1 - x^2 in double-word
__host__ __device__ __forceinline__ dword dw_one_minus_sq(dword x)
{
    dacc r{1.0f, 0.0f};
    dacc_fma(r, -x, x);
    return dacc_get(r);
}

// c + a b in double-word
__host__ __device__ __forceinline__ dword dw_fma(dword a, dword b, dword c)
{
    dacc r = dacc_of(c);
    dacc_fma(r, a, b);
    return dacc_get(r);
}

// Van der Pol, Lienard form: x0' = x1, x1' = mu (1 - x0^2) x1 - x0.  p = (mu).
struct ModelVdP {
    static constexpr int N = 2, P = 1, PG = 1;
    template <class S>
    __host__ __device__ __forceinline__ static void rhs(const S *x, const S *p, S t, S *f)
    {
        (void)t;
        f[0] = x[1];
        if constexpr (is_dw<S>)
            f[1] = dw_fma(p[0] * dw_one_minus_sq(x[0]), x[1], -x[0]);
        else
            f[1] = p[0] * (S(1) - x[0] * x[0]) * x[1] - x[0];
    }
    template <class S>
    __host__ __device__ __forceinline__ static void vjp(const S *w, const S *x, const S *p, S t, S *gx, S *gp)
    {
        (void)t;
        const S mu = p[0];
        if constexpr (is_dw<S>) {
            const dword a = dw_one_minus_sq(x[0]);
            gx[0] = w[1] * dw_fma(dw_m2(mu * x[0]), x[1], dword(-1.0f, 0.0f));
            gx[1] = dw_fma(w[1], mu * a, w[0]);
            gp[0] = w[1] * (a * x[1]);
        } else {
            gx[0] = w[1] * (S(-2) * mu * x[0] * x[1] - S(1));
            gx[1] = w[0] + w[1] * (mu * (S(1) - x[0] * x[0]));
            gp[0] = w[1] * ((S(1) - x[0] * x[0]) * x[1]);
        }
    }
};

// Van der Pol as in the reference example (examples/VanDerPol/main.cpp:41-42):
// x0' = x1, x1' = mu ((1 - x0^2) x1 - x0).
struct ModelVdPPetsc {
    static constexpr int N = 2, P = 1, PG = 1;
    template <class S>
    __host__ __device__ __forceinline__ static void rhs(const S *x, const S *p, S t, S *f)
    {
        (void)t;
        f[0] = x[1];
        if constexpr (is_dw<S>)
            f[1] = p[0] * dw_fma(dw_one_minus_sq(x[0]), x[1], -x[0]);
        else
            f[1] = p[0] * ((S(1) - x[0] * x[0]) * x[1] - x[0]);
    }
    template <class S>
    __host__ __device__ __forceinline__ static void vjp(const S *w, const S *x, const S *p, S t, S *gx, S *gp)
    {
        (void)t;
        const S mu = p[0];
        if constexpr (is_dw<S>) {
            const dword a = dw_one_minus_sq(x[0]);
            gx[0] = w[1] * (mu * dw_fma(dw_m2(x[0]), x[1], dword(-1.0f, 0.0f)));
            gx[1] = dw_fma(w[1], mu * a, w[0]);
            gp[0] = w[1] * dw_fma(a, x[1], -x[0]);
        } else {
            gx[0] = w[1] * (mu * (S(-2) * x[0] * x[1] - S(1)));
            gx[1] = w[0] + w[1] * (mu * (S(1) - x[0] * x[0]));
            gp[0] = w[1] * ((S(1) - x[0] * x[0]) * x[1] - x[0]);
        }
    }
};

// Damped harmonic oscillator x'' + 2 zeta omega x' + omega^2 x = 0 as a first
// order system; p = (omega, zeta).  (The reference example
// examples/HarmonicOscillator/main.cpp:11-30 uses fixed k = 1 and a friction
// parameter; this is the (omega, zeta) form of the same family.)
struct ModelDHO {
    static constexpr int N = 2, P = 2, PG = 2;
    template <class S>
    __host__ __device__ __forceinline__ static void rhs(const S *x, const S *p, S t, S *f)
    {
        (void)t;
        f[0] = x[1];
        if constexpr (is_dw<S>) {
            dacc r = dacc_mul(-(p[0] * p[0]), x[0]);
            dacc_fma(r, dw_m2(p[1] * p[0]), x[1]);
            f[1] = dacc_get(r);
        } else {
            f[1] = -p[0] * p[0] * x[0] - S(2) * p[1] * p[0] * x[1];
        }
    }
    template <class S>
    __host__ __device__ __forceinline__ static void vjp(const S *w, const S *x, const S *p, S t, S *gx, S *gp)
    {
        (void)t;
        const S om = p[0], ze = p[1];
        if constexpr (is_dw<S>) {
            gx[0] = w[1] * -(om * om);
            gx[1] = dw_fma(w[1], dw_m2(ze * om), w[0]);
            dacc r = dacc_mul(dw_m2(om), x[0]);
            dacc_fma(r, dw_m2(ze), x[1]);
            gp[0] = w[1] * dacc_get(r);
            gp[1] = w[1] * (dw_m2(om) * x[1]);
        } else {
            gx[0] = w[1] * (-om * om);
            gx[1] = w[0] + w[1] * (S(-2) * ze * om);
            gp[0] = w[1] * (S(-2) * om * x[0] - S(2) * ze * x[1]);
            gp[1] = w[1] * (S(-2) * om * x[1]);
        }
    }
};

// Exponential decay y' = -k y; p = (k).  Its discrete adjoint has a closed
// form for a frozen step sequence, which the tests use.
struct ModelDecay {
    static constexpr int N = 1, P = 1, PG = 1;
    template <class S>
    __host__ __device__ __forceinline__ static void rhs(const S *x, const S *p, S t, S *f)
    {
        (void)t;
        f[0] = -p[0] * x[0];
    }
    template <class S>
    __host__ __device__ __forceinline__ static void vjp(const S *w, const S *x, const S *p, S t, S *gx, S *gp)
    {
        (void)t;
        gx[0] = -p[0] * w[0];
        gp[0] = -x[0] * w[0];
    }
};

} // namespace va
