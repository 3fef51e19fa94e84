// Frozen-step replay: the forward map whose exact derivative the discrete
// adjoint computes.  Step sizes are not chosen by a controller but taken
// from a recorded accepted-step sequence, h_n = t_{n+1} - t_n (the step the
// backward sweep uses, StateStorage.hpp:22), and every step is
//   K_0 = f(y_n, t_n),  X_m = y_n + sum_{j<m} (a_mj h_n) K_j,
//   K_m = f(X_m, t_n + c_m h_n),  y_{n+1} = y_n + sum_j (b_j h_n) K_j,
// the arithmetic of the forward sweep's accepted attempts.  Central finite
// differences of this map with respect to y_0 and the parameters check the
// backward sweep's gradients on the GPU (the reference's back_prop_step,
// detail/backpropagation.hpp:83-158, differentiates the same map).
//
// FP64 only.  One thread per lane for the one-thread models (each model's
// own device RHS); for the Lotka-Volterra models one CTA of n threads per
// lane, thread i carrying component i, the stage point shared through
// shared memory.
#pragma once

#include "va_kernels.cuh"

namespace va {

struct ReplayParams {
    int count;            // lanes
    int stride;           // doubles per row of `times`
    int n, np;            // state dimension, per-lane parameters
    const double *times;  // [count][stride]: t_0 .. t_T of each lane
    const int *n_steps;   // [count]: T of each lane
    const double *y0;     // [count][n]
    const double *par;    // [count][np]
    const double *shared; // Lotka-Volterra with a shared matrix: A[n][n] (else null)
    double *yT;           // [count][n]
};

template <class M, class Tab>
__global__ void __launch_bounds__(128) replay_kernel(ReplayParams r)
{
    constexpr int N = M::N, P = M::P;
    const int lane = blockIdx.x * blockDim.x + threadIdx.x;
    if (lane >= r.count)
        return;
    double y[N], p[P];
#pragma unroll
    for (int i = 0; i < N; i++)
        y[i] = r.y0[(size_t)lane * N + i];
#pragma unroll
    for (int k = 0; k < P; k++)
        p[k] = r.par[(size_t)lane * P + k];
    const double *tt = r.times + (size_t)lane * r.stride;
    const int T = min(r.n_steps[lane], r.stride - 1);
    for (int s = 0; s < T; s++) {
        const double t = tt[s], h = tt[s + 1] - t;
        double k0[N], ynew[N], ys[N];
        M::template rhs<double>(y, p, t, k0);
        step_fixed<M, Tab, double>(y, y, k0, p, t, h, ynew, ys);
#pragma unroll
        for (int i = 0; i < N; i++)
            y[i] = ynew[i];
    }
#pragma unroll
    for (int i = 0; i < N; i++)
        r.yT[(size_t)lane * N + i] = y[i];
}

// x_i (r_i + sum_j A_ij x_j) for component i, x in shared memory
__device__ __forceinline__ double glv_component(const double *A, double ri, const double *x, int n, int i)
{
    double sum = 0.0;
    for (int j = 0; j < n; j++)
        sum = sum + A[(size_t)i * n + j] * x[j];
    return x[i] * (ri + sum);
}

// Lotka-Volterra x' = x (r + A x): params [r, A row-major] per lane
// (examples/GeneralizedLotkaVolterra/main.cpp:105-119) or r per lane with a
// shared A.  blockDim.x = n, n doubles of dynamic shared memory.
template <class Tab>
__global__ void __launch_bounds__(256) replay_glv_kernel(ReplayParams r)
{
    constexpr int NS = Tab::S;
    extern __shared__ double xs[];
    const int lane = blockIdx.x, i = threadIdx.x, n = r.n;
    if (lane >= r.count || i >= n)
        return;
    const double *pl = r.par + (size_t)lane * r.np;
    const double *A = r.shared ? r.shared : pl + n;
    const double ri = pl[i];
    double y = r.y0[(size_t)lane * n + i];
    const double *tt = r.times + (size_t)lane * r.stride;
    const int T = min(r.n_steps[lane], r.stride - 1);
    for (int s = 0; s < T; s++) {
        const double t = tt[s], h = tt[s + 1] - t;
        double K[NS];
        xs[i] = y;
        __syncthreads();
        K[0] = glv_component(A, ri, xs, n, i);
        __syncthreads();
#pragma unroll
        for (int m = 1; m < NS; m++) {
            double X = y;
#pragma unroll
            for (int j = 0; j < NS - 1; j++)
                if (j < m)
                    X = X + (Tab::a(m, j) * h) * K[j];
            xs[i] = X;
            __syncthreads();
            K[m] = glv_component(A, ri, xs, n, i);
            __syncthreads();
        }
        double acc = y;
#pragma unroll
        for (int j = 0; j < NS; j++)
            if (Tab::b(j) != 0.0)
                acc = acc + (Tab::b(j) * h) * K[j];
        y = acc;
    }
    r.yT[(size_t)lane * n + i] = y;
}

// the Lotka-Volterra replay kernel of a tableau (va_inst_replay_fp64.cu)
const void *replay_glv(int tableau);

} // namespace va
