// Table of compiled sweep kernels per built-in model: one entry per
// (tableau, precision).  Each model's kernels live in their own translation
// units so the library builds in parallel.  A null entry is a combination
// that is not compiled (va_create rejects it).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace va {

// tableaux: 0 Dormand-Prince 5(4), 1 Cash-Karp 5(4), 2 Fehlberg 7(8),
// 3 fixed-step runge_kutta4, 4 fixed-step euler
constexpr int kTableaux = 5;

struct KernelSet {
    int N, P;          // state and parameter counts (0 = runtime n)
    int tpi;           // threads that carry one instance
    const void *fwd[kTableaux][3]; // [tableau][precision] -> __global__ void(FwdParams)
    const void *bwd[kTableaux][3]; // [tableau][precision] -> __global__ void(AdjParams)
    const void *fwd2[kTableaux][3]; // forward writing [t, dt, y] records when fwd writes stage
                                    // records; null: fwd handles every layout
    const void *bwd1[kTableaux][3]; // every-step backward over [t, dt, y] records when bwd reads
                                    // stage records; null: bwd
    const void *bwd2[kTableaux][3]; // two-level backward (checkpoint stride > 1); null if unsupported
    bool dw_records;                // mixed_dw [t, dt, y] records hold double-words (t stays
                                    // FP64); stage records always do
    int rs_stage[kTableaux];        // mixed_dw: doubles per stage record (0: no stage records)
    const void *replay[kTableaux];  // FP64 frozen-step replay, one thread per lane
                                    // (one-thread models); __global__ void(ReplayParams)
};

// whether the sweeps keep stage records: mixed_dw kernels that have them,
// every step checkpointed, and stage storage enabled
inline bool stage_records_on(const KernelSet *ks, int tableau, int precision, int stride, bool enabled)
{
    return enabled && ks && ks->rs_stage[tableau] > 0 && precision == 2 && stride <= 1;
}

// doubles per checkpoint record: the stage record, or [t, dt, y] padded to even
inline int record_doubles_for(const KernelSet *ks, int tableau, int precision, int stride, int n, bool enabled)
{
    return stage_records_on(ks, tableau, precision, stride, enabled) ? ks->rs_stage[tableau] : (2 + n + 1) & ~1;
}

// A device model compiled outside the library (include/va_model.cuh,
// VA_DEFINE_MODEL): its kernel table plus a launcher and an occupancy query
// compiled in the same translation unit, so its kernels are launched through
// the CUDA runtime they were registered with (the model's shared object may
// link its own copy of the runtime).  magic and abi guard against a table
// built from another version of the sweep templates.
constexpr uint32_t kModelMagic = 0x4B4D4156u; // "VAMK"
constexpr uint32_t kModelAbi = 1;
struct ModelKernels {
    uint32_t magic, abi;
    KernelSet set;
    cudaError_t (*launch)(const void *fn, unsigned grid, unsigned block, void *params, size_t smem,
                          cudaStream_t s);
    cudaError_t (*occupancy)(int *blocks, const void *fn, int block, size_t smem);
    const char *name;
};

const KernelSet *kernels_vdp();
const KernelSet *kernels_vdp_petsc();
const KernelSet *kernels_dho();
const KernelSet *kernels_decay();
const KernelSet *kernels_glv(int n); // nullptr when n has no compiled kernels

// Fehlberg 7(8) entries of the one-thread models (their own translation units)
void fill_rkf78_vdp(KernelSet &k);
void fill_rkf78_vdp_petsc(KernelSet &k);
void fill_rkf78_dho(KernelSet &k);
void fill_rkf78_decay(KernelSet &k);

// FP64 frozen-step replay kernels of the one-thread models, every tableau
// (va_inst_replay_fp64.cu)
void fill_replay_vdp(KernelSet &k);
void fill_replay_vdp_petsc(KernelSet &k);
void fill_replay_dho(KernelSet &k);
void fill_replay_decay(KernelSet &k);

// fixed-step runge_kutta4 and euler entries (their own translation units)
void fill_fixed_vdp(KernelSet &k);
void fill_fixed_vdp_petsc(KernelSet &k);
void fill_fixed_dho(KernelSet &k);
void fill_fixed_decay(KernelSet &k);
void fill_fixed_glv5(KernelSet &k);
void fill_fixed_glv10(KernelSet &k);

// Shared-matrix GLV: bundles of kBundleNB instances per CTA of N threads
// (FP64, FP32); the double-word sweeps take bundles of kBundleNBdw, whose
// 128 registers per thread let two CTAs share an SM (GLV-256: 8% faster
// than one CTA of 4; the FP32 sweeps measured 38% slower so).
constexpr int kBundleNB = 4;
constexpr int kBundleNBdw = 2;
struct BundleKernelSet {
    int N;
    int nb[3];                     // instances per CTA, per precision
    const void *fwd[kTableaux][3]; // __global__ void(BundleParams), blockDim = N (mixed_dw: stage records)
    const void *bwd[kTableaux][3];
    const void *fwd1[kTableaux][3]; // mixed_dw sweeps over [t, dt, y] records (stage records off); null: fwd
    const void *bwd1[kTableaux][3];
    int rs_stage[kTableaux];        // mixed_dw: doubles per stage record (0: none)
    size_t smem_fwd[3], smem_bwd[3]; // dynamic shared memory per precision
    const void *prepare;   // prepare_A_kernel: A -> A^T and double-word copies
    const void *reduce;    // reduce_dA_kernel: CTA partials -> dA
    int nsv[kTableaux];    // factor rows per step of the deferred dA (stages that can be non-zero)
    // the other bundle width, one more point for the autotuner (null where not
    // compiled: the 5(4) pairs only): FP64 / FP32 bundles of kBundleNBdw,
    // double-word bundles of kBundleNB
    int nb_alt[3];
    const void *fwd_alt[kTableaux][3], *bwd_alt[kTableaux][3];
    const void *fwd1_alt[kTableaux][3], *bwd1_alt[kTableaux][3];
    size_t smem_fwd_alt[3], smem_bwd_alt[3];
    // two-level backward (checkpoint stride > 1) in bundles of nb[precision];
    // its dynamic shared memory is smem_bwd2[precision]
    const void *bwd2[kTableaux][3];
    size_t smem_bwd2[3];
};
// two-level bundle kernels (va_inst_bundle_2level.cu, va_inst_bundle_2level_fp64.cu)
void fill_bundle_2level64(BundleKernelSet &k);
void fill_bundle_2level256(BundleKernelSet &k);
// alternate-width bundle kernels (va_inst_bundle_alt.cu, va_inst_bundle_alt_fp64.cu)
void fill_bundle_alt64(BundleKernelSet &k);
void fill_bundle_alt256(BundleKernelSet &k);
void fill_bundle_alt_fp64_64(BundleKernelSet &k);
void fill_bundle_alt_fp64_256(BundleKernelSet &k);
const BundleKernelSet *kernels_glv_shared(int n); // n = 64 or 256

} // namespace va
