// Two right-hand sides defined only here, compiled by the tests into their
// own shared libraries (tests/cpp/user_model_*.cu, nvcc) and, for the oracle,
// into host callbacks (tests/cpp/user_models_host.cpp, g++): the
// bring-your-own-model path of include/va_model.cuh.  They are written once,
// with S arithmetic only, so the same expressions run in FP64, float and
// double-word on the GPU and in FP64 on the host.
#pragma once

#ifdef __CUDACC__
#define UM_HD __host__ __device__
#else
#define UM_HD
#endif

// Duffing oscillator under a decaying rational forcing (non-autonomous):
//   x' = v,  v' = -delta v - alpha x - beta x^3 + gamma / (1 + (omega t)^2)
// p = (delta, alpha, beta, gamma, omega).  The forcing needs only IEEE
// division, so host and device evaluate it to the same bits.
struct ForcedDuffing {
    static constexpr int N = 2, P = 5;
    template <class S>
    UM_HD static void rhs(const S *x, const S *p, S t, S *f)
    {
        const S wt = p[4] * t;
        f[0] = x[1];
        f[1] = -p[0] * x[1] - p[1] * x[0] - p[2] * (x[0] * x[0] * x[0]) + p[3] / (S(1) + wt * wt);
    }
    template <class S>
    UM_HD static void vjp(const S *w, const S *x, const S *p, S t, S *gx, S *gp)
    {
        const S wt = p[4] * t, d = S(1) + wt * wt;
        gx[0] = w[1] * (-p[1] - S(3) * p[2] * (x[0] * x[0]));
        gx[1] = w[0] - w[1] * p[0];
        gp[0] = -(w[1] * x[1]);
        gp[1] = -(w[1] * x[0]);
        gp[2] = -(w[1] * (x[0] * x[0] * x[0]));
        gp[3] = w[1] / d;
        gp[4] = -(w[1] * p[3] * (S(2) * wt * t) / (d * d));
    }
};

// Brusselator (autonomous): x' = a + x^2 y - (b + 1) x,  y' = b x - x^2 y;
// p = (a, b).
struct Brusselator {
    static constexpr int N = 2, P = 2;
    template <class S>
    UM_HD static void rhs(const S *x, const S *p, S t, S *f)
    {
        (void)t;
        const S x2y = x[0] * x[0] * x[1];
        f[0] = p[0] + x2y - (p[1] + S(1)) * x[0];
        f[1] = p[1] * x[0] - x2y;
    }
    template <class S>
    UM_HD static void vjp(const S *w, const S *x, const S *p, S t, S *gx, S *gp)
    {
        (void)t;
        const S dw = w[0] - w[1];
        gx[0] = dw * (S(2) * x[0] * x[1]) - w[0] * (p[1] + S(1)) + w[1] * p[1];
        gx[1] = dw * (x[0] * x[0]);
        gp[0] = w[0];
        gp[1] = (w[1] - w[0]) * x[0];
    }
};
