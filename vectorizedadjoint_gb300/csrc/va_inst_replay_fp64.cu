// FP64 frozen-step replay kernels (va_replay.cuh) of every built-in model and
// tableau.  Built with -fmad=false, like the other FP64 units.
#include "va_models.cuh"
#include "va_registry.h"
#include "va_replay.cuh"

namespace va {

template <class M>
static void fill(KernelSet &k)
{
    k.replay[0] = (const void *)replay_kernel<M, TabDopri5>;
    k.replay[1] = (const void *)replay_kernel<M, TabCK54>;
    k.replay[2] = (const void *)replay_kernel<M, TabRKF78>;
    k.replay[3] = (const void *)replay_kernel<M, TabRK4>;
    k.replay[4] = (const void *)replay_kernel<M, TabEuler>;
}

void fill_replay_vdp(KernelSet &k) { fill<ModelVdP>(k); }
void fill_replay_vdp_petsc(KernelSet &k) { fill<ModelVdPPetsc>(k); }
void fill_replay_dho(KernelSet &k) { fill<ModelDHO>(k); }
void fill_replay_decay(KernelSet &k) { fill<ModelDecay>(k); }

const void *replay_glv(int tableau)
{
    switch (tableau) {
    case 0: return (const void *)replay_glv_kernel<TabDopri5>;
    case 1: return (const void *)replay_glv_kernel<TabCK54>;
    case 2: return (const void *)replay_glv_kernel<TabRKF78>;
    case 3: return (const void *)replay_glv_kernel<TabRK4>;
    case 4: return (const void *)replay_glv_kernel<TabEuler>;
    default: return nullptr;
    }
}

} // namespace va
