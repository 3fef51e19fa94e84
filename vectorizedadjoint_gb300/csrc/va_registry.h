// Table of compiled sweep kernels per built-in model: one entry per
// (tableau, precision).  Each model's kernels live in their own translation
// unit so the library builds in parallel.
#pragma once

namespace va {

struct KernelSet {
    int N, P;          // state and parameter counts (0 = runtime n)
    int tpi;           // threads that carry one instance
    const void *fwd[2][3]; // [tableau][precision] -> __global__ void(FwdParams)
    const void *bwd[2][3]; // [tableau][precision] -> __global__ void(AdjParams)
};

const KernelSet *kernels_vdp();
const KernelSet *kernels_vdp_petsc();
const KernelSet *kernels_dho();
const KernelSet *kernels_decay();
const KernelSet *kernels_glv(int n); // nullptr when n has no compiled kernels

} // namespace va
