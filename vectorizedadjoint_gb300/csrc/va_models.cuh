// Right-hand sides and hand-written vector-Jacobian products of the built-in
// models (N states, P parameters read by the RHS, PG parameter gradients).  They take the place of the user functor the reference records
// with AADC (lib/include/AadData.hpp:124-171) and of the JIT reverse code it
// replays in AadData::VectorTimesJacobians (AadData.hpp:291-330): every
// model gives f(x, p, t) and (J_x^T w, J_p^T w) at the same point.
//
// The argument order (x, p, t) keeps the reference functor's
// (x, dxdt, params, t) meaning (examples/VanDerPol/main.cpp:38-43).  S is the
// stage arithmetic type: double for the FP64 path, float for the mixed path.
// Parameter layouts follow the reference examples.
#pragma once

namespace va {

// Van der Pol, Lienard form: x0' = x1, x1' = mu (1 - x0^2) x1 - x0.  p = (mu).
struct ModelVdP {
    static constexpr int N = 2, P = 1, PG = 1;
    template <class S>
    __host__ __device__ __forceinline__ static void rhs(const S *x, const S *p, S t, S *f)
    {
        (void)t;
        f[0] = x[1];
        f[1] = p[0] * (S(1) - x[0] * x[0]) * x[1] - x[0];
    }
    template <class S>
    __host__ __device__ __forceinline__ static void vjp(const S *w, const S *x, const S *p, S t, S *gx, S *gp)
    {
        (void)t;
        const S mu = p[0];
        gx[0] = w[1] * (S(-2) * mu * x[0] * x[1] - S(1));
        gx[1] = w[0] + w[1] * (mu * (S(1) - x[0] * x[0]));
        gp[0] = w[1] * ((S(1) - x[0] * x[0]) * x[1]);
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
        f[1] = p[0] * ((S(1) - x[0] * x[0]) * x[1] - x[0]);
    }
    template <class S>
    __host__ __device__ __forceinline__ static void vjp(const S *w, const S *x, const S *p, S t, S *gx, S *gp)
    {
        (void)t;
        const S mu = p[0];
        gx[0] = w[1] * (mu * (S(-2) * x[0] * x[1] - S(1)));
        gx[1] = w[0] + w[1] * (mu * (S(1) - x[0] * x[0]));
        gp[0] = w[1] * ((S(1) - x[0] * x[0]) * x[1] - x[0]);
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
        f[1] = -p[0] * p[0] * x[0] - S(2) * p[1] * p[0] * x[1];
    }
    template <class S>
    __host__ __device__ __forceinline__ static void vjp(const S *w, const S *x, const S *p, S t, S *gx, S *gp)
    {
        (void)t;
        const S om = p[0], ze = p[1];
        gx[0] = w[1] * (-om * om);
        gx[1] = w[0] + w[1] * (S(-2) * ze * om);
        gp[0] = w[1] * (S(-2) * om * x[0] - S(2) * ze * x[1]);
        gp[1] = w[1] * (S(-2) * om * x[1]);
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
