// Butcher tableaux of the embedded explicit Runge-Kutta pairs, as
// compile-time constants that fold into the unrolled stage loops.
//
// Cash-Karp 5(4) (Cash & Karp 1990) and Fehlberg 7(8) (Fehlberg 1968) are
// pairs the reference reads from odeint in lib/include/ButcherTable.hpp
// (:259-308, :191-246).  Dormand-Prince 5(4)
// (Dormand & Prince 1980) is not in the reference's ButcherTable
// (ButcherTable.hpp:365-368 rejects it); it is added here from the published
// tableau.  Each coefficient is the IEEE quotient of its two integers, and
// each error weight the difference of two such quotients, the same values
// odeint 1.74's rk54_ck_coefficients_* and runge_kutta_dopri5 compute.
#pragma once

namespace va {

struct TabDopri5 {
    static constexpr int S = 6;           // stages feeding y_{n+1}
    static constexpr bool FSAL = true;    // f(y_{n+1}) is the next k_1
    static constexpr int ERROR_ORDER = 4; // odeint error_order_value
    static constexpr int STEPPER_ORDER = 5;
    static constexpr double ERR_FLOOR = 1.0 / 3125.0; // 5^-STEPPER_ORDER (increase_step)
    static constexpr bool FIXED = false;  // controlled (embedded error estimate)
    __host__ __device__ static constexpr double a(int i, int j)
    {
        return i == 1 ? (j == 0 ? 1.0 / 5.0 : 0.0)
             : i == 2 ? (j == 0 ? 3.0 / 40.0 : j == 1 ? 9.0 / 40.0 : 0.0)
             : i == 3 ? (j == 0 ? 44.0 / 45.0 : j == 1 ? -56.0 / 15.0 : j == 2 ? 32.0 / 9.0 : 0.0)
             : i == 4 ? (j == 0 ? 19372.0 / 6561.0 : j == 1 ? -25360.0 / 2187.0
                         : j == 2 ? 64448.0 / 6561.0 : j == 3 ? -212.0 / 729.0 : 0.0)
             : i == 5 ? (j == 0 ? 9017.0 / 3168.0 : j == 1 ? -355.0 / 33.0 : j == 2 ? 46732.0 / 5247.0
                         : j == 3 ? 49.0 / 176.0 : j == 4 ? -5103.0 / 18656.0 : 0.0)
             : 0.0;
    }
    __host__ __device__ static constexpr double b(int j)
    {
        return j == 0 ? 35.0 / 384.0 : j == 2 ? 500.0 / 1113.0 : j == 3 ? 125.0 / 192.0
             : j == 4 ? -2187.0 / 6784.0 : j == 5 ? 11.0 / 84.0 : 0.0;
    }
    __host__ __device__ static constexpr double c(int j)
    {
        return j == 1 ? 1.0 / 5.0 : j == 2 ? 3.0 / 10.0 : j == 3 ? 4.0 / 5.0 : j == 4 ? 8.0 / 9.0
             : j == 5 ? 1.0 : 0.0;
    }
    // b - b_hat on k_1..k_6, and on f(y_{n+1})
    __host__ __device__ static constexpr double e(int j)
    {
        return j == 0 ? 35.0 / 384.0 - 5179.0 / 57600.0
             : j == 2 ? 500.0 / 1113.0 - 7571.0 / 16695.0
             : j == 3 ? 125.0 / 192.0 - 393.0 / 640.0
             : j == 4 ? -2187.0 / 6784.0 - -92097.0 / 339200.0
             : j == 5 ? 11.0 / 84.0 - 187.0 / 2100.0 : 0.0;
    }
    static constexpr double E_NEW = -1.0 / 40.0;
};

struct TabCK54 {
    static constexpr int S = 6;
    static constexpr bool FSAL = false;
    static constexpr int ERROR_ORDER = 4;
    static constexpr int STEPPER_ORDER = 5;
    static constexpr double ERR_FLOOR = 1.0 / 3125.0;
    static constexpr bool FIXED = false;
    __host__ __device__ static constexpr double a(int i, int j)
    {
        return i == 1 ? (j == 0 ? 1.0 / 5.0 : 0.0)
             : i == 2 ? (j == 0 ? 3.0 / 40.0 : j == 1 ? 9.0 / 40.0 : 0.0)
             : i == 3 ? (j == 0 ? 3.0 / 10.0 : j == 1 ? -9.0 / 10.0 : j == 2 ? 6.0 / 5.0 : 0.0)
             : i == 4 ? (j == 0 ? -11.0 / 54.0 : j == 1 ? 5.0 / 2.0 : j == 2 ? -70.0 / 27.0
                         : j == 3 ? 35.0 / 27.0 : 0.0)
             : i == 5 ? (j == 0 ? 1631.0 / 55296.0 : j == 1 ? 175.0 / 512.0 : j == 2 ? 575.0 / 13824.0
                         : j == 3 ? 44275.0 / 110592.0 : j == 4 ? 253.0 / 4096.0 : 0.0)
             : 0.0;
    }
    __host__ __device__ static constexpr double b(int j)
    {
        return j == 0 ? 37.0 / 378.0 : j == 2 ? 250.0 / 621.0 : j == 3 ? 125.0 / 594.0
             : j == 5 ? 512.0 / 1771.0 : 0.0;
    }
    __host__ __device__ static constexpr double c(int j)
    {
        return j == 1 ? 1.0 / 5.0 : j == 2 ? 3.0 / 10.0 : j == 3 ? 3.0 / 5.0 : j == 4 ? 1.0
             : j == 5 ? 7.0 / 8.0 : 0.0;
    }
    __host__ __device__ static constexpr double e(int j)
    {
        return j == 0 ? 37.0 / 378.0 - 2825.0 / 27648.0
             : j == 2 ? 250.0 / 621.0 - 18575.0 / 48384.0
             : j == 3 ? 125.0 / 594.0 - 13525.0 / 55296.0
             : j == 4 ? -277.0 / 14336.0
             : j == 5 ? 512.0 / 1771.0 - 1.0 / 4.0 : 0.0;
    }
    static constexpr double E_NEW = 0.0;
};

// Fehlberg 7(8): E. Fehlberg, "Classical fifth-, sixth-, seventh-, and
// eighth-order Runge-Kutta formulas with stepsize control", NASA TR R-287
// (1968) -- odeint's runge_kutta_fehlberg78, which the reference's
// ButcherTable reads (lib/include/ButcherTable.hpp:191-246).  13 stages, not
// FSAL; the eighth-order weights propagate and the error estimate is
// (b8 - b7) . k, nonzero on k_1, k_11, k_12, k_13.
struct TabRKF78 {
    static constexpr int S = 13;
    static constexpr bool FSAL = false;
    static constexpr int ERROR_ORDER = 7;
    static constexpr int STEPPER_ORDER = 8;
    static constexpr double ERR_FLOOR = 1.0 / 390625.0; // 5^-8
    static constexpr bool FIXED = false;
    __host__ __device__ static constexpr double a(int i, int j)
    {
        return i == 1 ? (j == 0 ? 2.0 / 27.0 : 0.0)
             : i == 2 ? (j == 0 ? 1.0 / 36.0 : j == 1 ? 1.0 / 12.0 : 0.0)
             : i == 3 ? (j == 0 ? 1.0 / 24.0 : j == 2 ? 1.0 / 8.0 : 0.0)
             : i == 4 ? (j == 0 ? 5.0 / 12.0 : j == 2 ? -25.0 / 16.0 : j == 3 ? 25.0 / 16.0 : 0.0)
             : i == 5 ? (j == 0 ? 1.0 / 20.0 : j == 3 ? 1.0 / 4.0 : j == 4 ? 1.0 / 5.0 : 0.0)
             : i == 6 ? (j == 0 ? -25.0 / 108.0 : j == 3 ? 125.0 / 108.0 : j == 4 ? -65.0 / 27.0 : j == 5 ? 125.0 / 54.0 : 0.0)
             : i == 7 ? (j == 0 ? 31.0 / 300.0 : j == 4 ? 61.0 / 225.0 : j == 5 ? -2.0 / 9.0 : j == 6 ? 13.0 / 900.0 : 0.0)
             : i == 8 ? (j == 0 ? 2.0 : j == 3 ? -53.0 / 6.0 : j == 4 ? 704.0 / 45.0 : j == 5 ? -107.0 / 9.0 : j == 6 ? 67.0 / 90.0 : j == 7 ? 3.0 : 0.0)
             : i == 9 ? (j == 0 ? -91.0 / 108.0 : j == 3 ? 23.0 / 108.0 : j == 4 ? -976.0 / 135.0 : j == 5 ? 311.0 / 54.0 : j == 6 ? -19.0 / 60.0 : j == 7 ? 17.0 / 6.0 : j == 8 ? -1.0 / 12.0 : 0.0)
             : i == 10 ? (j == 0 ? 2383.0 / 4100.0 : j == 3 ? -341.0 / 164.0 : j == 4 ? 4496.0 / 1025.0 : j == 5 ? -301.0 / 82.0 : j == 6 ? 2133.0 / 4100.0 : j == 7 ? 45.0 / 82.0 : j == 8 ? 45.0 / 164.0 : j == 9 ? 18.0 / 41.0 : 0.0)
             : i == 11 ? (j == 0 ? 3.0 / 205.0 : j == 5 ? -6.0 / 41.0 : j == 6 ? -3.0 / 205.0 : j == 7 ? -3.0 / 41.0 : j == 8 ? 3.0 / 41.0 : j == 9 ? 6.0 / 41.0 : 0.0)
             : i == 12 ? (j == 0 ? -1777.0 / 4100.0 : j == 3 ? -341.0 / 164.0 : j == 4 ? 4496.0 / 1025.0 : j == 5 ? -289.0 / 82.0 : j == 6 ? 2193.0 / 4100.0 : j == 7 ? 51.0 / 82.0 : j == 8 ? 33.0 / 164.0 : j == 9 ? 12.0 / 41.0 : j == 11 ? 1.0 : 0.0)
             : 0.0;
    }
    __host__ __device__ static constexpr double b(int j)
    {
        return j == 5 ? 34.0 / 105.0 : j == 6 ? 9.0 / 35.0 : j == 7 ? 9.0 / 35.0 : j == 8 ? 9.0 / 280.0 : j == 9 ? 9.0 / 280.0 : j == 11 ? 41.0 / 840.0 : j == 12 ? 41.0 / 840.0 : 0.0;
    }
    __host__ __device__ static constexpr double c(int j)
    {
        return j == 1 ? 2.0 / 27.0 : j == 2 ? 1.0 / 9.0 : j == 3 ? 1.0 / 6.0 : j == 4 ? 5.0 / 12.0 : j == 5 ? 1.0 / 2.0 : j == 6 ? 5.0 / 6.0 : j == 7 ? 1.0 / 6.0 : j == 8 ? 2.0 / 3.0 : j == 9 ? 1.0 / 3.0 : j == 10 ? 1.0 : j == 12 ? 1.0 : 0.0;
    }
    __host__ __device__ static constexpr double e(int j)
    {
        return j == 0 ? -41.0 / 840.0 : j == 10 ? -41.0 / 840.0 : j == 11 ? 41.0 / 840.0 : j == 12 ? 41.0 / 840.0 : 0.0;
    }
    static constexpr double E_NEW = 0.0;
};

// Fixed-step steppers the reference's ButcherTable accepts
// (lib/include/ButcherTable.hpp:39-125): odeint's runge_kutta4 (the classic
// fourth-order tableau) and euler.  No error estimate: the sweeps run the
// reference's non-controlled loop (lib/include/detail/runge_kutta.hpp:37-72),
// t_n = t_0 + n dt while (t_n + dt) - t_1 <= eps, every attempt accepted.
// The error weights are zero and the controller constants unused.
struct TabRK4 {
    static constexpr int S = 4;
    static constexpr bool FSAL = false;
    static constexpr int ERROR_ORDER = 4;
    static constexpr int STEPPER_ORDER = 4;
    static constexpr double ERR_FLOOR = 1.0 / 625.0;
    static constexpr bool FIXED = true;
    __host__ __device__ static constexpr double a(int i, int j)
    {
        return i == 1 ? (j == 0 ? 1.0 / 2.0 : 0.0)
             : i == 2 ? (j == 1 ? 1.0 / 2.0 : 0.0)
             : i == 3 ? (j == 2 ? 1.0 : 0.0)
             : 0.0;
    }
    __host__ __device__ static constexpr double b(int j)
    {
        return j == 0 ? 1.0 / 6.0 : j == 1 ? 1.0 / 3.0 : j == 2 ? 1.0 / 3.0 : j == 3 ? 1.0 / 6.0 : 0.0;
    }
    __host__ __device__ static constexpr double c(int j)
    {
        return j == 1 ? 1.0 / 2.0 : j == 2 ? 1.0 / 2.0 : j == 3 ? 1.0 : 0.0;
    }
    __host__ __device__ static constexpr double e(int) { return 0.0; }
    static constexpr double E_NEW = 0.0;
};

struct TabEuler {
    static constexpr int S = 1;
    static constexpr bool FSAL = false;
    static constexpr int ERROR_ORDER = 1;
    static constexpr int STEPPER_ORDER = 1;
    static constexpr double ERR_FLOOR = 1.0 / 5.0;
    static constexpr bool FIXED = true;
    __host__ __device__ static constexpr double a(int, int) { return 0.0; }
    __host__ __device__ static constexpr double b(int j) { return j == 0 ? 1.0 : 0.0; }
    __host__ __device__ static constexpr double c(int) { return 0.0; }
    __host__ __device__ static constexpr double e(int) { return 0.0; }
    static constexpr double E_NEW = 0.0;
};

// t_0 + n dt of the fixed-step loop, rounded twice as the reference computes
// it (no fused multiply-add, whatever the translation unit contracts)
__host__ __device__ __forceinline__ double fixed_time(double t0, int n, double dt)
{
#ifdef __CUDA_ARCH__
    return __dadd_rn(t0, __dmul_rn((double)n, dt));
#else
    return t0 + (double)n * dt;
#endif
}

} // namespace va
