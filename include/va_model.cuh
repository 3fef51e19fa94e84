// va_model.cuh -- bring your own right-hand side.
//
// The reference differentiates any templated functor
//   template <class T> void operator()(const std::vector<T> &x,
//       std::vector<T> &dxdt, const std::vector<T> &p, T t)
// by taping it once with AADC (recordDriverRHSFunction, Driver.hpp:95-100 ->
// AadData::Record, AadData.hpp:124-171).  On the GPU a right-hand side has to
// be device code, and the adjoint needs its vector-Jacobian product, so a
// model here is a struct with two templated device functions:
//
//   struct MyModel {
//       static constexpr int N = ..., P = ...;        // states, parameters
//       template <class S> __host__ __device__ static void
//       rhs(const S *x, const S *p, S t, S *f);        // f = dx/dt at (x, p, t)
//       template <class S> __host__ __device__ static void
//       vjp(const S *w, const S *x, const S *p, S t,   // gx = (df/dx)^T w,
//           S *gx, S *gp);                             // gp = (df/dp)^T w (overwritten)
//   };
//
// S is double (the FP64 sweeps) or float (the mixed-precision sweeps); with
// VA_DEFINE_MODEL_DW also va::dword, a pair of floats with +, -, *, / and
// construction from double/int, for the double-word sweeps.  Write the
// bodies with S arithmetic only (S(2) * x[0], not 2.0 * x[0]).
//
// In ONE nvcc translation unit of your own (built with
//   nvcc -gencode arch=compute_103a,code=sm_103a -std=c++17 -O3
//        --expt-relaxed-constexpr -fmad=false -Xcompiler -fPIC -shared
//        -I<this directory> my_model.cu -o libmy_model.so
// -fmad=false keeps every FP64 product and sum rounded on its own, so the
// FP64 sweeps give the same bits as a CPU evaluation of the same
// expressions; without it they contract multiply-adds):
//
//   #include "va_model.cuh"
//   struct MyModel { ... };
//   VA_DEFINE_MODEL(MyModel, my_model_kernels)
//
// VA_DEFINE_MODEL instantiates the library's sweep kernels (forward,
// backward, two-level backward and frozen-step replay, for the Dormand-Prince
// and Cash-Karp 5(4) pairs, Fehlberg 7(8), runge_kutta4 and euler, FP64 and
// float stages) for the model and defines
//   extern "C" const va_model_kernels *my_model_kernels(void);
// Pass its result to va_create_model (va.h) with a va_problem of model
// VA_MODEL_USER, n = N, npar = P; everything else -- va_forward, va_backward,
// va_gradient, two-level checkpointing, multi-cost seeds, trajectories,
// adjoint histories, va_forward_frozen -- works as for the built-in models.
// The C++ facade (va_driver.hpp) takes a host tag struct with
//   static const va_model_kernels *va_kernels() { return my_model_kernels(); }
// wherever the reference takes the functor.
//
// Kernels are launched through a launcher compiled in the same unit, so the
// model's library may link its own copy of the CUDA runtime.
#pragma once

#include <cuda_runtime.h>

#include "va.h"
#include "../vectorizedadjoint_gb300/csrc/va_kernels.cuh"
#include "../vectorizedadjoint_gb300/csrc/va_kernels_dw.cuh"
#include "../vectorizedadjoint_gb300/csrc/va_registry.h"
#include "../vectorizedadjoint_gb300/csrc/va_replay.cuh"

namespace va {
namespace {

cudaError_t model_launch(const void *fn, unsigned grid, unsigned block, void *params, size_t smem, cudaStream_t s)
{
    void *args[] = {params};
    return cudaLaunchKernel(fn, dim3(grid), dim3(block), args, smem, s);
}

cudaError_t model_occupancy(int *blocks, const void *fn, int block, size_t smem)
{
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, fn, block, smem);
}

// the sweeps' model concept: a gradient for every parameter (PG = P)
template <class M>
struct DeviceModel : M {
    static constexpr int PG = M::P;
};

template <class M, int I, class Tab, bool DW>
void model_fill_tableau(KernelSet &k)
{
    k.fwd[I][0] = (const void *)forward_kernel<M, Tab, double>;
    k.bwd[I][0] = (const void *)backward_kernel<M, Tab, double>;
    k.bwd2[I][0] = (const void *)backward_kernel_2level<M, Tab, double>;
    k.fwd[I][1] = (const void *)forward_kernel<M, Tab, float>;
    k.bwd[I][1] = (const void *)backward_kernel<M, Tab, float>;
    k.bwd2[I][1] = (const void *)backward_kernel_2level<M, Tab, float>;
    k.replay[I] = (const void *)replay_kernel<M, Tab>;
    if constexpr (DW) {
        k.fwd[I][2] = (const void *)forward_kernel_dw<M, Tab, true>;
        k.fwd2[I][2] = (const void *)forward_kernel_dw<M, Tab, false>;
        k.bwd[I][2] = (const void *)backward_kernel_dw<M, Tab, true>;
        k.bwd1[I][2] = (const void *)backward_kernel_dw<M, Tab, false>;
        k.bwd2[I][2] = (const void *)backward_kernel_2level_dw<M, Tab>;
        k.rs_stage[I] = stage_record_doubles(M::N, Tab::S);
    }
}

template <class U, bool DW>
ModelKernels make_model_kernels(const char *name)
{
    static_assert(U::N >= 1 && U::P >= 1, "a model needs N >= 1 states and P >= 1 parameters");
    using M = DeviceModel<U>;
    ModelKernels mk{};
    mk.magic = kModelMagic;
    mk.abi = kModelAbi;
    KernelSet &k = mk.set;
    k.N = M::N;
    k.P = M::P;
    k.tpi = 1;
    k.dw_records = true;
    model_fill_tableau<M, 0, TabDopri5, DW>(k);
    model_fill_tableau<M, 1, TabCK54, DW>(k);
    model_fill_tableau<M, 2, TabRKF78, DW>(k);
    model_fill_tableau<M, 3, TabRK4, DW>(k);
    model_fill_tableau<M, 4, TabEuler, DW>(k);
    mk.launch = model_launch;
    mk.occupancy = model_occupancy;
    mk.name = name;
    return mk;
}

} // namespace
} // namespace va

#define VA_DEFINE_MODEL_IMPL_(Model, symbol, dw)                                                  \
    extern "C" __attribute__((visibility("default"))) const va_model_kernels *symbol(void)       \
    {                                                                                             \
        static const va::ModelKernels mk = va::make_model_kernels<Model, dw>(#Model);             \
        return reinterpret_cast<const va_model_kernels *>(&mk);                                   \
    }

// FP64 and float-stage sweeps of Model; `symbol` names the table's accessor.
#define VA_DEFINE_MODEL(Model, symbol) VA_DEFINE_MODEL_IMPL_(Model, symbol, false)
// ... and the double-word sweeps (Model's rhs / vjp must compile for va::dword).
#define VA_DEFINE_MODEL_DW(Model, symbol) VA_DEFINE_MODEL_IMPL_(Model, symbol, true)
