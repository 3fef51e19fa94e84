/*
 * va.h -- C ABI of the GB300 discrete-adjoint library (libva_gb300.so).
 *
 * The reference exposes its solver as a C++ template API
 * (lib/include/runge_kutta.hpp, lib/include/backpropagation.hpp,
 * lib/include/Driver.hpp).  This header is the thin C layer under which the
 * same operations run on one GPU.  Each entry point cites the reference
 * interface it replaces.  Plain pointers and sizes only: no CUDA or C++
 * types, so ctypes, cgo, JNI or any C FFI can bind it.
 *
 * Conventions
 *  - A handle describes one batch of B independent instances of one model
 *    (one ODE, parameters and horizon per instance).  It owns the device
 *    checkpoint pool and scratch; the caller owns every input and output
 *    buffer.
 *  - Unless a name ends in _host, array arguments are DEVICE pointers in
 *    row-major per-instance layout: y0[B][n], params[B][npar], t0[B], t1[B],
 *    seeds lambdaT[B][nout][n], mu_direct[B][nout][npar].
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy default).
 *  - Functions return va_status.  Per-instance outcomes go to status[B].
 *  - A handle is not thread-safe; use one handle per host thread/stream.
 */
#ifndef VA_GB300_H
#define VA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VA_ABI_VERSION 1

#if defined(__GNUC__)
#define VA_API __attribute__((visibility("default")))
#else
#define VA_API
#endif

typedef struct va_handle va_handle;

/* Built-in right-hand sides (the reference records the user functor with
 * AADC, lib/include/AadData.hpp:124-171; here each model ships a
 * hand-written device RHS and vector-Jacobian product). */
typedef enum {
    VA_MODEL_VDP = 0,       /* x0'=x1, x1'=mu(1-x0^2)x1-x0;          n=2, npar=1        */
    VA_MODEL_VDP_PETSC = 1, /* x0'=x1, x1'=mu((1-x0^2)x1-x0)  (examples/VanDerPol/main.cpp:41-42) */
    VA_MODEL_DHO = 2,       /* x'=v, v'=-w^2 x-2 z w v, p=(w,z);     n=2, npar=2        */
    VA_MODEL_GLV = 3,       /* x_i'=x_i(r_i+sum_j A_ij x_j), p=(r, A row-major)
                               per instance (examples/GeneralizedLotkaVolterra/main.cpp:105-119);
                               npar = n + n*n                                            */
    VA_MODEL_DECAY = 4,     /* y'=-k y;                              n=1, npar=1        */
    VA_MODEL_GLV_SHARED = 5, /* GLV with one A shared by the batch; per-instance
                               params = r[n]; shared params = A[n][n]                   */
    VA_MODEL_USER = 6       /* a device model compiled by the caller (include/va_model.cuh,
                               VA_DEFINE_MODEL), passed to va_create_model               */
} va_model;

/* Kernel table of a device model compiled outside the library: the struct
 * that VA_DEFINE_MODEL (include/va_model.cuh) builds in the caller's nvcc
 * translation unit and returns from the function it defines.  Opaque here. */
typedef struct va_model_kernels va_model_kernels;

/* Embedded pairs (ButcherTable.hpp:259-308 for Cash-Karp, :191-246 for
 * Fehlberg 7(8); Dormand-Prince is added from the published tableau) and
 * the fixed-step steppers (ButcherTable.hpp:39-125: runge_kutta4, euler),
 * which run the reference's non-controlled loop
 * (detail/runge_kutta.hpp:37-72) with step dt0: t_n = t0 + n dt0 while
 * t_n + dt0 <= t1 (to within DBL_EPSILON), so the last record can lie short
 * of t1, as in the reference.  Every tableau is compiled for the one-thread
 * models and the per-instance GLV lane groups; VA_MODEL_GLV_SHARED takes the
 * 5(4) pairs and the fixed-step steppers (va_create rejects Fehlberg 7(8),
 * whose 13 stages do not fit the bundle sweeps' shared memory). */
typedef enum {
    VA_TAB_DOPRI5 = 0,
    VA_TAB_CK54 = 1,
    VA_TAB_RKF78 = 2,
    VA_TAB_RK4 = 3,  /* fixed step */
    VA_TAB_EULER = 4 /* fixed step */
} va_tableau;

typedef enum {
    VA_PREC_FP64 = 0, /* all arithmetic FP64: the drop-in path                          */
    VA_PREC_MIXED = 1, /* FP32 stages and VJPs; FP64 t, h, y, error norm, controller and
                          gradient accumulators                                          */
    VA_PREC_MIXED_DW = 2 /* as VA_PREC_MIXED, but stages and VJPs in double-word arithmetic
                            (pairs of FP32, ~48-bit significand) on the FP32 pipe         */
} va_precision;

typedef enum { VA_COST_SEEDS = -1, VA_COST_SUMSQ = 0, VA_COST_SUM = 1 } va_cost;

typedef enum {
    VA_OK = 0,
    VA_MAX_REJECTS = 1,  /* odeint failed_step_checker: > max_rejects attempts on one step */
    VA_MAX_STEPS = 2,    /* more than max_steps accepted steps                             */
    VA_NONFINITE = 3,    /* NaN/Inf in the state, error norm or gradient                   */
    VA_CKPT_BUDGET = 4,  /* checkpoint pool exhausted under the stated budget              */
    VA_BAD_ARGS = 5,
    VA_CUDA_ERROR = 6,
    VA_NOT_READY = 7,    /* backward called before a forward                               */
    VA_RECOMPUTE_MISMATCH = 8, /* two-level re-integration did not land on the checkpoint */
    VA_NOT_RUN = 9
} va_status;

typedef struct {
    int32_t model;  /* va_model                                                   */
    int32_t n;      /* state dimension                                            */
    int32_t npar;   /* per-instance parameter count                               */
    int32_t batch;  /* B                                                          */
    int32_t nout;   /* cost functions (seed rows) per instance, >= 1              */
} va_problem;

typedef struct {
    int32_t tableau;     /* va_tableau                                            */
    int32_t precision;   /* va_precision                                          */
    double atol, rtol;   /* odeint make_controlled(abs, rel)                      */
    double dt0;          /* initial step (runge_kutta(..., dt, ...)); the step of
                            the fixed-step tableaux                               */
    int32_t max_steps;   /* accepted-step cap per instance                        */
    int32_t max_rejects; /* odeint failed_step_checker limit (500)                */
    int64_t ckpt_budget_bytes; /* HBM budget for checkpoints (0 = default 16 GiB) */
    int32_t ckpt_stride; /* 0 or 1: every accepted step is checkpointed (pool
                            exhaustion -> VA_CKPT_BUDGET per instance).  k > 1:
                            two-level checkpointing -- every k-th accepted step is
                            stored and the backward sweep re-integrates each segment
                            from its checkpoint into scratch (bit-identical steps,
                            checked; one extra forward evaluation per step), for
                            every model family: one-thread, lane-group (GLV N=5,10)
                            and shared-matrix bundles.  -1: automatic -- va_forward
                            (and the first va_gradient call on the handle) checks
                            the pool after the sweep (synchronously) and, if it
                            overflowed, reruns: first without stage records, then
                            with a 4x larger stride until the checkpoints fit (up
                            to 1024); later va_gradient calls keep that layout  */
    int32_t block_size;  /* 0 = autotuned / default                               */
    int32_t blocks_per_sm; /* 0 = occupancy limit                                 */
    int32_t chunk_len;   /* records per checkpoint chunk (0 = 64)                 */
    int32_t schedule;    /* 0: longest instances first (forward: by the previous
                            forward's attempt counts, else by t1 - t0; backward:
                            by accepted steps), 1: index order                    */
    int32_t stage_records; /* mixed_dw, every step checkpointed: 1 (default) --
                            each record also holds the step's RK stage values
                            (GLV: also their rates r + A X_m) and the backward
                            sweep reads them instead of recomputing them (one-thread
                            models: 2 + 6N doubles instead of 2 + N); 0 -- [t, dt, y]
                            records and stage recompute, the reference's scheme.
                            With ckpt_stride = -1 a pool overflow first drops the
                            stage values, then thins the checkpoints              */
    int32_t step_pow;    /* FP64 step-size controller (odeint default_step_adjuster,
                            called from detail/runge_kutta.hpp:103-107): 1 (default)
                            -- the factors pow(err, -1.0/(q-1)) and pow(err, -1.0/p)
                            correctly rounded, i.e. what odeint's std::pow gives
                            wherever the host libm rounds correctly, so the sweep
                            takes the reference's accepted steps; 0 -- Newton's
                            inverse root (a few ulps off, ~25% cheaper per attempt).
                            The reduced precisions keep their own controllers     */
    int32_t tensor_products; /* shared-matrix GLV, N = 256, mixed_dw, every step
                            checkpointed with stage records: 0 (default) -- the
                            sweeps' stage products run on the tensor cores
                            (clusters of 8 CTAs carry 64 instances in lockstep;
                            error-free digit split): the backward's A^T v for
                            DOPRI5 and CK54, the forward's A X for DOPRI5, where
                            the GPU can schedule such clusters; -1 -- double-word
                            dot products on the FP32 pipe                      */
    int32_t reserved[2];
} va_options;

/* Fills the reference's defaults: DOPRI5, FP64, atol=rtol=1e-6, dt0=1e-3,
 * max_rejects=500 (odeint failed_step_checker), max_steps=1000000, and the
 * correctly rounded step factor (step_pow = 1). */
VA_API va_status va_default_options(va_options *opt);

/* Replaces Driver(Nin, Nout, Npar) (Driver.hpp:39-42) together with
 * constructDriverButcherTableau (Driver.hpp:87-93) and
 * recordDriverRHSFunction (Driver.hpp:95-100): the model id stands for the
 * recorded RHS, opt->tableau for the tableau. */
VA_API va_status va_create(const va_problem *prob, const va_options *opt, va_handle **out);

/* va_create for a model the caller compiled (prob->model = VA_MODEL_USER):
 * replaces recordDriverRHSFunction (Driver.hpp:95-100, which tapes any
 * templated functor through AadData::Record, AadData.hpp:124-171) for device
 * code.  `model` is what the function defined by VA_DEFINE_MODEL returns;
 * prob->n and prob->npar must equal the model's N and P.  The tableaux and
 * precisions are those the model was instantiated for; the handle keeps the
 * pointer, which must outlive it.  VA_BAD_ARGS for a table built from
 * another version of the sweep templates. */
VA_API va_status va_create_model(const va_problem *prob, const va_options *opt, const va_model_kernels *model,
                                 va_handle **out);

/* Replaces delete_driver_handle (Driver.hpp:81-85). */
VA_API va_status va_destroy(va_handle *h);

/* Forward sweep over all B instances; replaces the controlled overload of
 * runge_kutta (runge_kutta.hpp:47-59 -> detail/runge_kutta.hpp:137-180).
 * Writes y(T) (the reference overwrites x0), the accepted-step count
 * (runge_kutta's return value), the rejected-attempt count and a status per
 * instance; every accepted (t_n, y_n) goes to the handle's checkpoint pool.
 * yT, n_acc, n_rej and status may be NULL. */
VA_API va_status va_forward(va_handle *h, const double *y0, const double *params, const double *t0,
                     const double *t1, double *yT, int32_t *n_acc, int32_t *n_rej,
                     int32_t *status, void *stream);

/* Backward sweep; replaces setCostGradients (Driver.hpp:103-114) plus
 * adjointSolve (backpropagation.hpp:18-43 -> detail/backpropagation.hpp:280-348).
 * lambdaT[B][nout][n] = dG/dy(T), mu_direct[B][nout][npar] = direct dG/dp
 * (NULL = 0).  Outputs dy0[B][nout][n] (the reference's overwritten lambda)
 * and dparams[B][nout][npar] = mu_direct + sum J_p^T Kbar (its accumulated
 * mu).  params must be the ones the forward ran with.  Step sizes are frozen
 * (h_n = t_{n+1} - t_n as in StateStorage.hpp:22). */
VA_API va_status va_backward(va_handle *h, const double *params, const double *lambdaT,
                      const double *mu_direct, double *dy0, double *dparams, int32_t *status,
                      void *stream);

/* Forward + backward for a built-in scalar cost (nout must be 1):
 * VA_COST_SUMSQ g = sum_i y_i(T)^2, VA_COST_SUM g = sum_i y_i(T).  The two
 * sweeps are captured in one CUDA graph on the first call and replayed. */
VA_API va_status va_gradient(va_handle *h, int32_t cost, const double *y0, const double *params,
                      const double *t0, const double *t1, double *yT, double *dy0,
                      double *dparams, int32_t *n_acc, int32_t *status, void *stream);

/* va_gradient with HOST buffers: copies inputs to the device, runs both
 * sweeps and copies the results back, then synchronises `stream`.  Pinned
 * host memory gives the fastest copies.  Any output may be NULL. */
VA_API va_status va_gradient_host(va_handle *h, int32_t cost, const double *y0, const double *params,
                           const double *t0, const double *t1, double *yT, double *dy0,
                           double *dparams, int32_t *n_acc, int32_t *status, void *stream);

/* va_forward with HOST buffers (synchronous; device staging owned by the
 * handle).  The single-instance C++ facade (va_driver.hpp) runs on this. */
VA_API va_status va_forward_host(va_handle *h, const double *y0, const double *params,
                                 const double *t0, const double *t1, double *yT, int32_t *n_acc,
                                 int32_t *n_rej, int32_t *status);

/* va_backward with HOST buffers (synchronous). */
VA_API va_status va_backward_host(va_handle *h, const double *params, const double *lambdaT,
                                  const double *mu_direct, double *dy0, double *dparams,
                                  int32_t *status);

/* Size of the fixed device array va_gradient_noalloc works in. */
#define VA_NOALLOC_SCRATCH_BYTES (64u << 20)

/* va_gradient without any allocation, for callers that may not allocate
 * device memory while they run (e.g. a host whose device memory is owned by
 * another runtime's caching allocator, or a plugin host that forbids
 * allocation in callbacks).  No counterpart in the reference.  No handle:
 * the problem and options are arguments; inputs and outputs are the
 * caller's DEVICE buffers as for va_gradient (nout = 1; yT, n_acc, status
 * may be NULL).  Models whose state fits one thread only: VA_MODEL_VDP,
 * VA_MODEL_VDP_PETSC, VA_MODEL_DHO, VA_MODEL_DECAY.
 * All scratch -- work counters, per-instance metadata and the checkpoint
 * pool -- lives in one file-scope device array of VA_NOALLOC_SCRATCH_BYTES
 * (64 MiB) that every GPU loading the library holds until exit.  A batch
 * whose metadata plus one checkpoint chunk per instance does not fit is
 * rejected with VA_BAD_ARGS before any GPU work; instances that outgrow the
 * pool at run time report VA_CKPT_BUDGET in status.
 * The first call on a device looks up the array's device address (with that
 * device current): make it before any stream capture.  Calls share the
 * array and it keeps the last call's contents; calls whose GPU work overlaps
 * race on it. */
VA_API va_status va_gradient_noalloc(int32_t model, int32_t tableau, int32_t precision,
                                     double atol, double rtol, double dt0, int32_t max_steps,
                                     int32_t max_rejects, int32_t cost, int32_t batch,
                                     const double *y0, const double *params, const double *t0,
                                     const double *t1, double *yT, double *dy0, double *dparams,
                                     int32_t *n_acc, int32_t *status, void *stream);

/* Frozen-step replay of the handle's model and tableau in FP64: for each of
 * `count` lanes, integrates from y0[lane] with params[lane] over the given
 * accepted-step sequence, h_n = t_{n+1} - t_n with t_n =
 * times[lane][n], n = 0..n_steps[lane], no step-size control, and writes
 * y(T) to yT[lane].  This is the map whose exact derivative the backward
 * sweep computes (the reference's back_prop_step,
 * detail/backpropagation.hpp:83-158, differentiates it with step sizes
 * frozen): central differences of it check va_backward on the GPU.  All
 * arrays are DEVICE arrays: times[count][times_stride], n_steps[count],
 * y0[count][n], params[count][npar], yT[count][n].  `shared` (may be NULL):
 * the matrix A of VA_MODEL_GLV_SHARED for this call (NULL: the one of
 * va_set_shared).  Times come from va_trajectory of a forward sweep. */
VA_API va_status va_forward_frozen(va_handle *h, int32_t count, int32_t times_stride, const double *times,
                                   const int32_t *n_steps, const double *y0, const double *params,
                                   const double *shared, double *yT, void *stream);

/* Picks the launch shape by timing candidate runs of both sweeps on the given
 * inputs (device pointers) and keeps it in the handle: for the one-thread
 * and lane-group models the block size and resident blocks per SM of each
 * sweep, for the shared-matrix model the bundle width (instances per CTA:
 * 2 or 4).  Runs forward+backward several times per candidate.  The choice
 * is also kept on disk, one line per problem (GPU, model, sizes, tableau,
 * precision, record layout, batch size's power of two), in the file named
 * by the environment variable VA_AUTOTUNE_CACHE ("" or "off": none), else
 * $XDG_CACHE_HOME/vectorizedadjoint_gb300/autotune.tsv or
 * $HOME/.cache/vectorizedadjoint_gb300/autotune.tsv; a later call for the
 * same problem applies the stored shape without timing anything. */
VA_API va_status va_autotune(va_handle *h, int32_t cost, const double *y0, const double *params,
                      const double *t0, const double *t1, void *stream);

/* Launch configuration in use: block size and grid of each sweep. */
VA_API va_status va_get_launch(const va_handle *h, int32_t *fwd_block, int32_t *fwd_grid,
                        int32_t *bwd_block, int32_t *bwd_grid);

/* Checkpoint pool: bytes reserved, bytes used by the last forward, stride. */
VA_API va_status va_checkpoint_info(const va_handle *h, int64_t *capacity_bytes, int64_t *used_bytes,
                             int32_t *stride);

/* Copies the accepted-step record of one instance from the checkpoint pool
 * to HOST buffers (synchronous): t[k], dt[k] (trial step at the top of step
 * k) and y[k][n] for k = 0..T, the reference's StateStorage contents
 * (StateStorage.hpp:23-42).  *n_records = T + 1; at most `capacity` records
 * are written.  Valid after a forward sweep with stride 1. */
VA_API va_status va_trajectory(va_handle *h, int32_t instance, int32_t capacity, double *t,
                               double *dt, double *y, int32_t *n_records);

/* Adjoint history -- the reference's back_prop observer
 * (detail/backpropagation.hpp:230-254), which sees (lambda_n, t_n) after
 * every back step, n = T .. 0.  capacity > 0: every later backward sweep
 * (va_backward, va_gradient) also stores lambda_n of every seed for record
 * indices n < capacity, in a device buffer the handle owns
 * (batch * nout * capacity * n doubles, NaN where nothing was stored);
 * 0 turns the history off and frees the buffer.  Any checkpoint stride.
 * VA_BAD_ARGS for VA_MODEL_GLV_SHARED. */
VA_API va_status va_set_adjoint_history(va_handle *h, int32_t capacity);

/* Copies one instance's adjoint history to HOST buffers (synchronous):
 * lambda[q][k][i] (row stride `capacity`) = lambda_k of seed q for
 * k < min(capacity, history capacity, T + 1), and, when t is not NULL, the
 * record times t[k] (as va_trajectory; checkpoint stride 1 only).
 * *n_records = T + 1.  VA_NOT_READY before a backward sweep with the
 * history on. */
VA_API va_status va_adjoint_history(va_handle *h, int32_t instance, int32_t capacity, double *t,
                                    double *lambda, int32_t *n_records);

/* The history buffer on the device, layout [batch][nout][capacity][n], and
 * its capacity (NULL, 0 when off). */
VA_API va_status va_adjoint_history_buffer(const va_handle *h, double **buf, int32_t *capacity);

/* Shared parameters of VA_MODEL_GLV_SHARED (n = 64 or 256, npar = n, nout = 1):
 * A[n][n] row-major (DEVICE, read by every later sweep) and dA[n][n] (DEVICE,
 * may be NULL), which each backward sweep overwrites with the gradient of
 * the SUM of the batch's costs with respect to the shared A.  The reference
 * has no shared-parameter batch; per instance this is its GLV parameter
 * layout (examples/GeneralizedLotkaVolterra/main.cpp:105-119) with A common. */
VA_API va_status va_set_shared(va_handle *h, const double *A, double *dA);

/* Step factors of the last forward sweep whose correctly rounded value could
 * not be decided at double-double precision (Ziv's rounding test failed;
 * expected ~2^-42 per factor, so 0 in practice); such a factor is the
 * nearest rounding of a value within 2^-98 of the power.  Synchronous. */
VA_API va_status va_step_pow_undecided(va_handle *h, int64_t *count);

/* Message of the last failing call on this handle ("" if none). */
VA_API const char *va_last_error(const va_handle *h);

/* Name of a va_status value. */
VA_API const char *va_status_string(int32_t status);

#ifdef __cplusplus
}
#endif
#endif
