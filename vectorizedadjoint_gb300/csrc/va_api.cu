// C ABI of the discrete-adjoint library (include/va.h): handle, checkpoint
// pool, launch configuration, CUDA-graph capture of forward+backward and the
// host-buffer entry point.  Replaces the reference's Driver
// (lib/include/Driver.hpp), runge_kutta (lib/include/runge_kutta.hpp) and
// adjointSolve (lib/include/backpropagation.hpp) for built-in models.
#include <cuda_runtime.h>

#include <sys/stat.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <initializer_list>
#include <string>
#include <vector>

#include "../../include/va.h"
#include "va_bundle.cuh"
#include "va_contract.cuh"
#include "va_bundle_2level.cuh"
#include "va_bundle_tc.cuh"
#include "va_group_2level.cuh"
#include "va_kernels.cuh"
#include "va_order.h"
#include "va_registry.h"
#include "va_replay.cuh"

namespace {

constexpr int64_t kDefaultBudget = 16LL << 30; // 16 GiB of checkpoints
constexpr int kMaxAutoStride = 1024;            // automatic two-level stride cap

struct GraphKey {
    int cost = -2;
    const void *ptrs[10] = {};
    void *stream = nullptr;
    const void *extra = nullptr;
    bool operator==(const GraphKey &o) const
    {
        if (cost != o.cost || stream != o.stream || extra != o.extra)
            return false;
        for (int i = 0; i < 10; i++)
            if (ptrs[i] != o.ptrs[i])
                return false;
        return true;
    }
};

} // namespace

struct va_handle {
    va_problem prob{};
    va_options opt{};
    int device = 0;
    int sm_count = 0;
    const va::KernelSet *ks = nullptr;
    const va::ModelKernels *user = nullptr; // a device model compiled outside the library
    int N = 0, P = 0;
    int RS = 0; // doubles per checkpoint record at the current stride (record_layout)
    bool stages_on = true; // opt.stage_records, cleared by the automatic checkpoint ladder
    size_t pool_bytes = 0;
    int64_t worst_chunks = 0;

    // checkpoint pool and per-instance metadata
    double *pool_rec = nullptr;
    int *chunk_prev = nullptr;
    int n_chunks = 0;
    int chunk_len = 64;
    int *inst_T = nullptr, *inst_last = nullptr, *inst_status = nullptr;
    va::Control *ctl = nullptr;

    // staging buffers of the host entry point
    double *s_y0 = nullptr, *s_par = nullptr, *s_t0 = nullptr, *s_t1 = nullptr;
    double *s_yT = nullptr, *s_dy0 = nullptr, *s_dpar = nullptr;
    int *s_nacc = nullptr, *s_status = nullptr, *s_nrej = nullptr;
    double *s_lam = nullptr, *s_mu = nullptr;

    int fwd_block = 128, fwd_grid = 0, bwd_block = 128, bwd_grid = 0;
    bool forward_done = false;
    bool ladder_settled = false; // ckpt_stride = -1: va_gradient ran the memory ladder once
    std::string err;

    cudaGraphExec_t graph = nullptr;
    GraphKey graph_key;

    // longest-first work order of the two sweeps; inst_work[B] (+ flag) holds
    // the last forward sweep's attempt counts, the next forward's order key
    int *order_fwd = nullptr, *order_bwd = nullptr, *order_work = nullptr, *inst_work = nullptr;

    // two-level checkpointing: stride, end times, re-integration scratch
    int stride = 1;
    double *inst_t1 = nullptr;
    double *inst_t0 = nullptr; // start times (fixed-step two-level backward)
    // adjoint history (va_set_adjoint_history): [batch][nout][hist_cap][N]
    double *hist = nullptr;
    int hist_cap = 0;
    bool hist_done = false; // a backward sweep has been enqueued with the history on
    double *scratch = nullptr;
    size_t scratch_doubles = 0;

    // shared-matrix bundle path (VA_MODEL_GLV_SHARED)
    const va::BundleKernelSet *bks = nullptr;
    const double *shared_A = nullptr;
    double *shared_dA = nullptr;
    double *At = nullptr, *dA_part = nullptr;
    va::dword *Aw = nullptr, *Atw = nullptr;
    bool bundle_alt = false; // the other bundle width (va_autotune's choice)
    // deferred dA on the tensor pipe (N = 256, double-word sweeps with stage
    // records): factor rows, their x pointers, per-instance row offsets,
    // contraction partials and its error flag
    double *fac_v = nullptr;
    const double **fac_xp = nullptr;
    int *k_base = nullptr;
    double *c_part = nullptr;
    unsigned *c_err = nullptr;
    int64_t fac_rows = 0;
    // tensor-core cluster backward (va_bundle_tc.cuh): digit planes of A^T
    // and their exponents (null: the bundle backward)
    uint8_t *bt_adig = nullptr;
    int *bt_aexp = nullptr;
    double *bt_rpk = nullptr; // r as packed double-words
    uint8_t *bt_adig_f = nullptr; // the forward's digit planes of A (null: the bundle forward)
    int *bt_aexp_f = nullptr;
    unsigned *bt_ferr = nullptr;

    bool buffers_ready = false; // ensure_buffers / ensure_staging completed
    bool staging_ready = false;
};

namespace {

va_status fail(va_handle *h, va_status st, const char *fmt, const char *detail = "")
{
    if (h) {
        char buf[512];
        std::snprintf(buf, sizeof(buf), fmt, detail);
        h->err = buf;
    }
    return st;
}

va_status cuda_fail(va_handle *h, cudaError_t e, const char *where)
{
    if (h) {
        h->err = std::string(where) + ": " + cudaGetErrorString(e);
    }
    return VA_CUDA_ERROR;
}

#define VA_CUDA(h, call)                                                                           \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return cuda_fail((h), e_, #call);                                                      \
    } while (0)

const va::KernelSet *kernel_set(const va_problem &p)
{
    switch (p.model) {
    case VA_MODEL_VDP:
        return va::kernels_vdp();
    case VA_MODEL_VDP_PETSC:
        return va::kernels_vdp_petsc();
    case VA_MODEL_DHO:
        return va::kernels_dho();
    case VA_MODEL_DECAY:
        return va::kernels_decay();
    case VA_MODEL_GLV:
        return va::kernels_glv(p.n);
    default:
        return nullptr;
    }
}

// Resident blocks per SM of a sweep kernel: a model compiled outside the
// library answers through its own runtime (its kernels are registered there).
int occupancy_of(const va_handle *h, const void *fn, int block)
{
    int occ = 0;
    const cudaError_t e = h->user ? h->user->occupancy(&occ, fn, block, 0)
                                  : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, block, 0);
    return e == cudaSuccess ? occ : 0;
}

int grid_for(va_handle *h, const void *fn, int block, int instances)
{
    int occ = occupancy_of(h, fn, block);
    if (occ < 1)
        occ = 1;
    int bps = h->opt.blocks_per_sm > 0 ? std::min(h->opt.blocks_per_sm, occ) : occ;
    long need = ((long)instances * h->ks->tpi + block - 1) / block;
    long g = (long)h->sm_count * bps;
    return (int)std::max(1L, std::min(g, need));
}

// Record size and chunk count of the checkpoint pool at the current stride:
// the double-word sweeps store stage records when every step is kept and
// [t, dt, y] records otherwise, so the same bytes hold more chunks at a
// stride > 1.
bool stages_now(const va_handle *h)
{
    if (h->bks)
        return h->stages_on && h->stride <= 1 && h->opt.precision == VA_PREC_MIXED_DW &&
               h->bks->rs_stage[h->opt.tableau] > 0;
    return va::stage_records_on(h->ks, h->opt.tableau, h->opt.precision, h->stride, h->stages_on);
}

// Whether the handle's shared-matrix gradient can be contracted on the
// tensor pipe (va_contract.cu): N = 256, double-word sweeps, stage records
// (the backward points at the stage points X_m they hold).
bool deferred_possible(const va_handle *h)
{
    return h->bks && h->N == va::kContractN && h->opt.precision == VA_PREC_MIXED_DW &&
           h->bks->rs_stage[h->opt.tableau] > 0 && h->opt.stage_records != 0;
}
bool deferred_now(const va_handle *h) { return deferred_possible(h) && stages_now(h) && h->fac_v && h->shared_dA; }
// the tensor-core cluster backward (with the deferred dA)
bool tc_backward_now(const va_handle *h)
{
    return deferred_now(h) && h->bt_adig && h->opt.tensor_products == 0 && va::bundle_tc_available(h->opt.tableau);
}
// the tensor-core cluster forward (stage records, every step checkpointed)
bool tc_forward_now(const va_handle *h)
{
    return deferred_possible(h) && stages_now(h) && h->bt_adig_f && h->opt.tensor_products == 0 &&
           va::bundle_tc_forward_available(h->opt.tableau);
}

// whether the other bundle width is compiled for the handle's tableau and precision
bool bundle_alt_available(const va_handle *h)
{
    const int t = h->opt.tableau, p = h->opt.precision;
    return h->bks && h->bks->fwd_alt[t][p] && h->bks->bwd_alt[t][p];
}
bool use_alt(const va_handle *h) { return h->bundle_alt && bundle_alt_available(h); }
int bundle_nb(const va_handle *h)
{
    const int p = h->opt.precision;
    return use_alt(h) ? h->bks->nb_alt[p] : h->bks->nb[p];
}
size_t bundle_smem_fwd(const va_handle *h)
{
    const int p = h->opt.precision;
    return use_alt(h) ? h->bks->smem_fwd_alt[p] : h->bks->smem_fwd[p];
}
size_t bundle_smem_bwd(const va_handle *h)
{
    const int p = h->opt.precision;
    return use_alt(h) ? h->bks->smem_bwd_alt[p] : h->bks->smem_bwd[p];
}

// the bundle sweep for the current record layout and width
const void *bundle_fwd(const va_handle *h)
{
    const int t = h->opt.tableau, p = h->opt.precision;
    const auto &f = use_alt(h) ? h->bks->fwd_alt : h->bks->fwd;
    const auto &f1 = use_alt(h) ? h->bks->fwd1_alt : h->bks->fwd1;
    return !stages_now(h) && f1[t][p] ? f1[t][p] : f[t][p];
}
const void *bundle_bwd(const va_handle *h)
{
    const int t = h->opt.tableau, p = h->opt.precision;
    const auto &b = use_alt(h) ? h->bks->bwd_alt : h->bks->bwd;
    const auto &b1 = use_alt(h) ? h->bks->bwd1_alt : h->bks->bwd1;
    return !stages_now(h) && b1[t][p] ? b1[t][p] : b[t][p];
}

void record_layout(va_handle *h)
{
    h->RS = h->bks ? (stages_now(h) ? h->bks->rs_stage[h->opt.tableau] : va::record_doubles(h->N))
                   : va::record_doubles_for(h->ks, h->opt.tableau, h->opt.precision, h->stride, h->N, h->stages_on);
    if (!h->pool_bytes)
        return;
    const int64_t chunk_bytes = (int64_t)h->RS * sizeof(double) * h->chunk_len;
    int64_t nch = std::min<int64_t>(h->worst_chunks, (int64_t)h->pool_bytes / chunk_bytes);
    nch = std::max<int64_t>(nch, 1);
    h->n_chunks = (int)std::min<int64_t>(nch, 0x7fffffff);
}

// doubles per record of the two-level re-integration scratch (the
// double-word kernels keep stage records there)
int scratch_record_doubles(const va_handle *h)
{
    return va::record_doubles_for(h->ks, h->opt.tableau, h->opt.precision, 1, h->N, true);
}

// Frees each buffer of a failed all-or-nothing allocation and clears its
// pointer, so that the next call allocates again instead of running on a
// half-built handle.
void release(std::initializer_list<void **> ptrs)
{
    for (void **p : ptrs) {
        if (*p)
            cudaFree(*p);
        *p = nullptr;
    }
    (void)cudaGetLastError(); // the failed allocation's error is reported, not left for the next launch check
}

va_status alloc_buffers(va_handle *h)
{
    const int B = h->prob.batch;
    // the pool is sized for the largest record layout of the handle; the
    // chunk links for the smallest (most chunks)
    const int rs_small = va::record_doubles(h->N);
    const int rs_big = h->bks ? (stages_now(h) ? h->bks->rs_stage[h->opt.tableau] : rs_small)
                              : va::record_doubles_for(h->ks, h->opt.tableau, h->opt.precision, 1, h->N, h->stages_on);
    int64_t budget = h->opt.ckpt_budget_bytes > 0 ? h->opt.ckpt_budget_bytes : kDefaultBudget;
    const int64_t per_inst_chunks = ((int64_t)h->opt.max_steps + 1 + h->chunk_len - 1) / h->chunk_len;
    h->worst_chunks = per_inst_chunks * B;
    const int64_t big_chunk = (int64_t)rs_big * sizeof(double) * h->chunk_len;
    const int64_t small_chunk = (int64_t)rs_small * sizeof(double) * h->chunk_len;
    // with the deferred dA, every stored step also needs nsv factor rows (a v
    // row and an x pointer): the budget is shared in proportion
    const int64_t rec_bytes = (int64_t)rs_big * sizeof(double);
    const int64_t fac_per_rec = deferred_possible(h)
                                    ? (int64_t)h->bks->nsv[h->opt.tableau] * (h->N * (int64_t)sizeof(double) + 8)
                                    : 0;
    const int64_t pool_budget = fac_per_rec ? (int64_t)((double)budget * rec_bytes / (rec_bytes + fac_per_rec)) : budget;
    int64_t bytes = std::min<int64_t>(pool_budget, h->worst_chunks * big_chunk);
    bytes = std::max<int64_t>(bytes, big_chunk);
    h->pool_bytes = (size_t)bytes;
    int64_t links = std::min<int64_t>(h->worst_chunks, bytes / small_chunk);
    links = std::max<int64_t>(std::min<int64_t>(links, 0x7fffffff), 1);
    record_layout(h);
    VA_CUDA(h, cudaMalloc(&h->pool_rec, h->pool_bytes));
    VA_CUDA(h, cudaMalloc(&h->chunk_prev, (size_t)links * sizeof(int)));
    VA_CUDA(h, cudaMalloc(&h->inst_T, (size_t)B * sizeof(int)));
    VA_CUDA(h, cudaMalloc(&h->inst_last, (size_t)B * sizeof(int)));
    VA_CUDA(h, cudaMalloc(&h->inst_status, (size_t)B * sizeof(int)));
    VA_CUDA(h, cudaMalloc(&h->ctl, sizeof(va::Control)));
    VA_CUDA(h, cudaMemset(h->ctl, 0, sizeof(va::Control)));
    VA_CUDA(h, cudaMalloc(&h->inst_t1, (size_t)B * sizeof(double)));
    VA_CUDA(h, cudaMalloc(&h->inst_t0, (size_t)B * sizeof(double)));
    if (!h->bks && h->opt.schedule == 0) {
        VA_CUDA(h, cudaMalloc(&h->order_fwd, (size_t)B * sizeof(int)));
        VA_CUDA(h, cudaMalloc(&h->order_bwd, (size_t)B * sizeof(int)));
        VA_CUDA(h, cudaMalloc(&h->order_work, va::order_work_ints() * sizeof(int)));
        VA_CUDA(h, cudaMemset(h->order_work, 0, va::order_work_ints() * sizeof(int)));
        // attempts per instance of the last forward sweep, then its valid flag
        VA_CUDA(h, cudaMalloc(&h->inst_work, ((size_t)B + 1) * sizeof(int)));
        VA_CUDA(h, cudaMemset(h->inst_work + B, 0, sizeof(int)));
    }
    if (h->bks) {
        const size_t NN = (size_t)h->N * h->N;
        const int nb = std::min({h->bks->nb[0], h->bks->nb[1], h->bks->nb[2], h->bks->nb_alt[0], h->bks->nb_alt[1],
                                 h->bks->nb_alt[2]}); // the most CTAs
        const size_t grid = ((size_t)B + nb - 1) / nb;
        VA_CUDA(h, cudaMalloc(&h->At, NN * sizeof(double)));
        VA_CUDA(h, cudaMalloc(&h->Aw, NN * sizeof(va::dword)));
        VA_CUDA(h, cudaMalloc(&h->Atw, NN * sizeof(va::dword)));
        VA_CUDA(h, cudaMalloc(&h->dA_part, grid * NN * sizeof(double)));
        if (fac_per_rec) {
            // one row set per record the pool can hold
            const int64_t recs = (int64_t)(h->pool_bytes / (size_t)big_chunk) * h->chunk_len;
            h->fac_rows = recs * h->bks->nsv[h->opt.tableau];
            VA_CUDA(h, cudaMalloc(&h->fac_v, (size_t)h->fac_rows * h->N * sizeof(double)));
            VA_CUDA(h, cudaMalloc(&h->fac_xp, (size_t)h->fac_rows * sizeof(double *)));
            VA_CUDA(h, cudaMalloc(&h->k_base, ((size_t)B + 1) * sizeof(int)));
            VA_CUDA(h, cudaMalloc(&h->c_part, (size_t)va::contract_splits(h->sm_count) * NN * sizeof(double)));
            VA_CUDA(h, cudaMalloc(&h->c_err, sizeof(unsigned)));
            VA_CUDA(h, va::contract_prepare());
            if (h->opt.tensor_products == 0 && va::bundle_tc_available(h->opt.tableau)) {
                VA_CUDA(h, cudaMalloc(&h->bt_adig, va::kBtADigitBytes));
                VA_CUDA(h, cudaMalloc(&h->bt_aexp, va::kBtAExpInts * sizeof(int)));
                VA_CUDA(h, cudaMalloc(&h->bt_rpk, (size_t)B * h->N * sizeof(double)));
                if (va::bundle_tc_forward_available(h->opt.tableau)) {
                    VA_CUDA(h, cudaMalloc(&h->bt_adig_f, va::kBtADigitBytes));
                    VA_CUDA(h, cudaMalloc(&h->bt_aexp_f, va::kBtAExpInts * sizeof(int)));
                    VA_CUDA(h, cudaMalloc(&h->bt_ferr, sizeof(unsigned)));
                }
            }
        }
        for (int t = 0; t < va::kTableaux; t++)
            for (int p = 0; p < 3; p++) {
                const void *fns[8] = {h->bks->fwd[t][p],     h->bks->fwd1[t][p],     h->bks->bwd[t][p],
                                      h->bks->bwd1[t][p],    h->bks->fwd_alt[t][p],  h->bks->fwd1_alt[t][p],
                                      h->bks->bwd_alt[t][p], h->bks->bwd1_alt[t][p]};
                const size_t sm[8] = {h->bks->smem_fwd[p],     h->bks->smem_fwd[p],     h->bks->smem_bwd[p],
                                      h->bks->smem_bwd[p],     h->bks->smem_fwd_alt[p], h->bks->smem_fwd_alt[p],
                                      h->bks->smem_bwd_alt[p], h->bks->smem_bwd_alt[p]};
                for (int f = 0; f < 8; f++)
                    if (fns[f])
                        VA_CUDA(h, cudaFuncSetAttribute(fns[f], cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                        (int)sm[f]));
                if (h->bks->bwd2[t][p])
                    VA_CUDA(h, cudaFuncSetAttribute(h->bks->bwd2[t][p], cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                    (int)h->bks->smem_bwd2[p]));
            }
    }
    return VA_OK;
}

va_status ensure_buffers(va_handle *h)
{
    if (h->buffers_ready)
        return VA_OK;
    const va_status st = alloc_buffers(h);
    if (st != VA_OK) {
        release({(void **)&h->pool_rec, (void **)&h->chunk_prev, (void **)&h->inst_T, (void **)&h->inst_last,
                 (void **)&h->inst_status, (void **)&h->ctl, (void **)&h->inst_t1, (void **)&h->inst_t0,
                 (void **)&h->order_fwd, (void **)&h->order_bwd, (void **)&h->order_work, (void **)&h->inst_work,
                 (void **)&h->At, (void **)&h->Aw, (void **)&h->Atw, (void **)&h->dA_part, (void **)&h->fac_v,
                 (void **)&h->fac_xp, (void **)&h->k_base, (void **)&h->c_part, (void **)&h->c_err,
                 (void **)&h->bt_adig, (void **)&h->bt_aexp, (void **)&h->bt_rpk, (void **)&h->bt_adig_f,
                 (void **)&h->bt_aexp_f, (void **)&h->bt_ferr});
        h->pool_bytes = 0;
        h->fac_rows = 0;
        return st;
    }
    h->buffers_ready = true;
    return VA_OK;
}

va::BundleParams bundle_params(va_handle *h)
{
    va::BundleParams bp{};
    bp.A = h->shared_A;
    bp.At = h->At;
    bp.Aw = h->Aw;
    bp.Atw = h->Atw;
    bp.dA_part = h->dA_part;
    bp.nb = bundle_nb(h);
    return bp;
}

int bundle_grid(va_handle *h)
{
    const int nb = bundle_nb(h);
    return (h->prob.batch + nb - 1) / nb;
}

// Two-level backward launch.  One-thread models: 64-thread blocks, at most 4
// per SM, so the re-integration scratch stays (stride + 1) records x 256
// threads per SM.  Lane groups: 256-thread blocks (8 warps of 32 / G groups),
// at most 2 per SM, (stride + 1) records of the group's state per group.
constexpr int kTwoLevelBlock = 64, kTwoLevelBlocksPerSm = 4;
constexpr int kTwoLevelGroupBlock = 256, kTwoLevelGroupBlocksPerSm = 2;

int two_level_block(const va_handle *h) { return h->ks->tpi > 1 ? kTwoLevelGroupBlock : kTwoLevelBlock; }

// instances one block of the two-level backward carries at once
int two_level_per_block(const va_handle *h)
{
    const int g = h->ks->tpi;
    return g > 1 ? kTwoLevelGroupBlock / 32 * (32 / g) : kTwoLevelBlock;
}

int two_level_grid(va_handle *h)
{
    const long per = two_level_per_block(h);
    const long need = ((long)h->prob.batch + per - 1) / per;
    const long bps = h->ks->tpi > 1 ? kTwoLevelGroupBlocksPerSm : kTwoLevelBlocksPerSm;
    return (int)std::max(1L, std::min(need, (long)h->sm_count * bps));
}

// doubles of re-integration scratch the two-level backward needs
size_t two_level_scratch_doubles(va_handle *h)
{
    if (h->bks) // (stride + 1) [t, -, y] records per instance
        return (size_t)h->prob.batch * va::bundle_scratch_doubles(h->N, h->stride);
    const size_t carriers = (size_t)two_level_grid(h) * two_level_per_block(h);
    if (h->ks->tpi > 1)
        return carriers * (size_t)va::group_scratch_doubles(h->N, h->stride);
    return carriers * (h->stride + 1) * scratch_record_doubles(h);
}

// Scratch for the current stride; never called during stream capture.
va_status ensure_scratch(va_handle *h)
{
    if (h->stride <= 1)
        return VA_OK;
    const size_t need = two_level_scratch_doubles(h);
    if (need <= h->scratch_doubles)
        return VA_OK;
    if (h->scratch)
        cudaFree(h->scratch);
    h->scratch = nullptr;
    h->scratch_doubles = 0;
    VA_CUDA(h, cudaMalloc(&h->scratch, need * sizeof(double)));
    h->scratch_doubles = need;
    return VA_OK;
}

va_status alloc_staging(va_handle *h)
{
    const size_t B = h->prob.batch, N = h->N, P = h->P, Q = h->prob.nout;
    VA_CUDA(h, cudaMalloc(&h->s_y0, B * N * sizeof(double)));
    VA_CUDA(h, cudaMalloc(&h->s_par, B * P * sizeof(double)));
    VA_CUDA(h, cudaMalloc(&h->s_t0, B * sizeof(double)));
    VA_CUDA(h, cudaMalloc(&h->s_t1, B * sizeof(double)));
    VA_CUDA(h, cudaMalloc(&h->s_yT, B * N * sizeof(double)));
    VA_CUDA(h, cudaMalloc(&h->s_dy0, B * Q * N * sizeof(double)));
    VA_CUDA(h, cudaMalloc(&h->s_dpar, B * Q * P * sizeof(double)));
    VA_CUDA(h, cudaMalloc(&h->s_nacc, B * sizeof(int)));
    VA_CUDA(h, cudaMalloc(&h->s_status, B * sizeof(int)));
    VA_CUDA(h, cudaMalloc(&h->s_nrej, B * sizeof(int)));
    VA_CUDA(h, cudaMalloc(&h->s_lam, B * Q * N * sizeof(double)));
    VA_CUDA(h, cudaMalloc(&h->s_mu, B * Q * P * sizeof(double)));
    return VA_OK;
}

va_status ensure_staging(va_handle *h)
{
    if (h->staging_ready)
        return VA_OK;
    const va_status st = alloc_staging(h);
    if (st != VA_OK) {
        release({(void **)&h->s_y0, (void **)&h->s_par, (void **)&h->s_t0, (void **)&h->s_t1, (void **)&h->s_yT,
                 (void **)&h->s_dy0, (void **)&h->s_dpar, (void **)&h->s_nacc, (void **)&h->s_status,
                 (void **)&h->s_nrej, (void **)&h->s_lam, (void **)&h->s_mu});
        return st;
    }
    h->staging_ready = true;
    return VA_OK;
}

va::Pool pool_of(va_handle *h)
{
    va::Pool p;
    p.rec = h->pool_rec;
    p.chunk_prev = h->chunk_prev;
    p.n_chunks = h->n_chunks;
    p.chunk_len = h->chunk_len;
    return p;
}

// Launches a sweep kernel of the handle's model with one parameter block;
// kernels of a model compiled outside the library go through its launcher.
cudaError_t launch(const va_handle *h, const void *fn, int grid, int block, void *params, cudaStream_t s,
                   size_t smem = 0)
{
    if (h->user)
        return h->user->launch(fn, (unsigned)grid, (unsigned)block, params, smem, s);
    void *args[] = {params};
    return cudaLaunchKernel(fn, dim3(grid), dim3(block), args, smem, s);
}

va_status enqueue_forward(va_handle *h, const double *y0, const double *params, const double *t0,
                          const double *t1, double *yT, int32_t *n_acc, int32_t *n_rej,
                          int32_t *status, cudaStream_t s)
{
    va::FwdParams a{};
    a.B = h->prob.batch;
    a.y0 = y0;
    a.par = params;
    a.t0 = t0;
    a.t1 = t1;
    a.atol = h->opt.atol;
    a.rtol = h->opt.rtol;
    a.dt0 = h->opt.dt0;
    a.max_steps = h->opt.max_steps;
    a.max_fail = h->opt.max_rejects;
    a.step_pow = h->opt.step_pow;
    a.yT = yT;
    a.n_acc_out = n_acc;
    a.n_rej_out = n_rej;
    a.status_out = status;
    a.inst_T = h->inst_T;
    a.inst_last = h->inst_last;
    a.inst_status = h->inst_status;
    a.inst_t1 = h->inst_t1;
    a.inst_t0 = h->inst_t0;
    a.stride = h->stride;
    a.pool = pool_of(h);
    a.ctl = h->ctl;
    if (h->bks) {
        if (!h->shared_A)
            return fail(h, VA_BAD_ARGS, "shared-matrix model: call va_set_shared first%s");
        const int NN = h->N * h->N;
        void *pargs[] = {(void *)&h->shared_A, (void *)&h->At, (void *)&h->Aw, (void *)&h->Atw};
        VA_CUDA(h, cudaMemsetAsync(h->ctl, 0, sizeof(va::Control), s));
        VA_CUDA(h, cudaLaunchKernel(h->bks->prepare, dim3((NN + 255) / 256), dim3(256), pargs, 0, s));
        va::BundleParams bp = bundle_params(h);
        bp.f = a;
        if (tc_forward_now(h)) {
            // clusters of 8 CTAs, 64 instances each, stage products on the tensor cores
            VA_CUDA(h, cudaMemsetAsync(h->bt_ferr, 0, sizeof(unsigned), s));
            VA_CUDA(h, va::enqueue_bundle_tc_forward(bp, h->shared_A, h->bt_adig_f, h->bt_aexp_f, h->bt_rpk, h->bt_ferr,
                                                     h->opt.tableau, s));
            // CTAs of the cluster sweep (instances past its tiles: the tail)
            h->fwd_grid = va::bundle_tc_tiles(a.B) * va::kBtCluster;
            h->fwd_block = va::kBtThreads;
            return VA_OK;
        }
        void *args[] = {&bp};
        VA_CUDA(h, cudaLaunchKernel(bundle_fwd(h), dim3(bundle_grid(h)), dim3(h->N), args, bundle_smem_fwd(h), s));
        h->fwd_grid = bundle_grid(h);
        h->fwd_block = h->N;
        return VA_OK;
    }
    const void *fn = h->ks->fwd[h->opt.tableau][h->opt.precision];
    if (!stages_now(h) && h->ks->fwd2[h->opt.tableau][h->opt.precision])
        fn = h->ks->fwd2[h->opt.tableau][h->opt.precision];
    if (h->fwd_grid <= 0)
        h->fwd_grid = grid_for(h, fn, h->fwd_block, a.B);
    if (h->order_fwd) {
        const int *valid = h->inst_work + a.B;
        va::OrderArgs o{a.B, nullptr, t0, t1, h->inst_work, valid, h->order_work, h->order_fwd};
        VA_CUDA(h, va::enqueue_order(o, s));
        a.order = h->order_fwd;
        a.inst_work = h->inst_work;
        a.work_valid = h->inst_work + a.B;
    }
    VA_CUDA(h, cudaMemsetAsync(h->ctl, 0, sizeof(va::Control), s));
    VA_CUDA(h, launch(h, fn, h->fwd_grid, h->fwd_block, &a, s));
    return VA_OK;
}

va_status enqueue_backward(va_handle *h, const double *params, const double *lambdaT,
                           const double *mu_direct, int cost, double *dy0, double *dparams,
                           int32_t *status, cudaStream_t s)
{
    va::AdjParams a{};
    a.B = h->prob.batch;
    a.nout = h->prob.nout;
    a.par = params;
    a.lambdaT = lambdaT;
    a.mu_direct = mu_direct;
    a.cost = cost;
    a.dy0 = dy0;
    a.dpar = dparams;
    a.status_out = status;
    a.order = nullptr;
    a.inst_T = h->inst_T;
    a.inst_last = h->inst_last;
    a.inst_status = h->inst_status;
    a.pool = pool_of(h);
    a.ctl = h->ctl;
    if (h->order_bwd) {
        // one-thread models reuse the forward's order (measured: VdP batch
        // +3%); the lane groups sort by their own step counts (GLV-10: the
        // reused order made the backward 11% slower)
        const int *reuse = h->ks->tpi == 1 ? h->order_fwd : nullptr;
        va::OrderArgs o{a.B, h->inst_T, nullptr, nullptr, nullptr, nullptr, h->order_work, h->order_bwd, reuse};
        VA_CUDA(h, va::enqueue_order(o, s));
        a.order = h->order_bwd;
    }
    if (h->bks && h->stride > 1) {
        // two-level: segments re-run from the strided checkpoints, in bundles
        // of the precision's default width
        if (h->scratch_doubles < two_level_scratch_doubles(h))
            return fail(h, VA_BAD_ARGS, "two-level scratch not sized for the stride%s");
        const int p = h->opt.precision;
        va::BundleParams bp = bundle_params(h);
        bp.nb = h->bks->nb[p];
        a.stride = h->stride;
        a.inst_t1 = h->inst_t1;
        a.inst_t0 = h->inst_t0;
        a.scratch = h->scratch;
        a.atol = h->opt.atol;
        a.rtol = h->opt.rtol;
        a.dt0 = h->opt.dt0;
        a.max_fail = h->opt.max_rejects;
        a.step_pow = h->opt.step_pow;
        bp.g = a;
        void *args[] = {&bp};
        int grid = (h->prob.batch + bp.nb - 1) / bp.nb;
        VA_CUDA(h, cudaLaunchKernel(h->bks->bwd2[h->opt.tableau][p], dim3(grid), dim3(h->N), args,
                                    h->bks->smem_bwd2[p], s));
        if (h->shared_dA) {
            const int NN = h->N * h->N;
            int dw = p == VA_PREC_MIXED_DW;
            void *rargs[] = {(void *)&h->dA_part, (void *)&grid, (void *)&dw, (void *)&h->shared_dA};
            VA_CUDA(h, cudaLaunchKernel(h->bks->reduce, dim3((NN + 255) / 256), dim3(256), rargs, 0, s));
        }
        h->bwd_grid = grid;
        h->bwd_block = h->N;
        return VA_OK;
    }
    if (h->bks) {
        va::BundleParams bp = bundle_params(h);
        bp.g = a;
        void *args[] = {&bp};
        const int p = h->opt.precision;
        const int grid = bundle_grid(h);
        const bool defer = deferred_now(h);
        if (defer) {
            VA_CUDA(h, va::enqueue_factor_offsets(h->inst_T, h->inst_status, a.B, h->bks->nsv[h->opt.tableau],
                                                  h->k_base, s));
            bp.fac_v = h->fac_v;
            bp.fac_xp = h->fac_xp;
            bp.k_base = h->k_base;
        }
        const bool tcb = tc_backward_now(h);
        if (defer)
            VA_CUDA(h, cudaMemsetAsync(h->c_err, 0, sizeof(unsigned), s));
        if (tcb) {
            // clusters of 8 CTAs, 64 instances each, stage products on the tensor cores
            VA_CUDA(h, va::enqueue_bundle_tc_backward(bp, h->shared_A, h->bt_adig, h->bt_aexp, h->bt_rpk, h->c_err,
                                                      h->opt.tableau, s));
            h->bwd_grid = va::bundle_tc_tiles(a.B) * va::kBtCluster;
            h->bwd_block = va::kBtThreads;
        } else {
            VA_CUDA(h, cudaLaunchKernel(bundle_bwd(h), dim3(grid), dim3(h->N), args, bundle_smem_bwd(h), s));
            h->bwd_grid = grid;
            h->bwd_block = h->N;
        }
        if (defer) {
            va::ContractParams cp{};
            cp.v = h->fac_v;
            cp.xp = h->fac_xp;
            cp.k_total = h->k_base + a.B;
            cp.partials = h->c_part;
            cp.splits = va::contract_splits(h->sm_count);
            cp.error = h->c_err;
            VA_CUDA(h, va::enqueue_contract(cp, h->shared_dA, s));
        } else if (h->shared_dA) {
            const int NN = h->N * h->N;
            int dw = p == VA_PREC_MIXED_DW;
            void *rargs[] = {(void *)&h->dA_part, (void *)&grid, (void *)&dw, (void *)&h->shared_dA};
            VA_CUDA(h, cudaLaunchKernel(h->bks->reduce, dim3((NN + 255) / 256), dim3(256), rargs, 0, s));
        }
        return VA_OK;
    }
    a.hist = h->hist;
    a.hist_cap = h->hist_cap;
    if (h->hist)
        h->hist_done = true;
    if (h->stride > 1) {
        if (h->scratch_doubles < two_level_scratch_doubles(h))
            return fail(h, VA_BAD_ARGS, "two-level scratch not sized for the stride%s");
        a.stride = h->stride;
        a.inst_t1 = h->inst_t1;
        a.inst_t0 = h->inst_t0;
        a.scratch = h->scratch;
        a.atol = h->opt.atol;
        a.rtol = h->opt.rtol;
        a.dt0 = h->opt.dt0;
        a.max_fail = h->opt.max_rejects;
        a.step_pow = h->opt.step_pow;
        VA_CUDA(h, cudaMemsetAsync(&h->ctl->adj_next, 0, sizeof(unsigned int), s));
        VA_CUDA(h, launch(h, h->ks->bwd2[h->opt.tableau][h->opt.precision], two_level_grid(h), two_level_block(h),
                          &a, s));
        return VA_OK;
    }
    const void *fn = h->ks->bwd[h->opt.tableau][h->opt.precision];
    if (!stages_now(h) && h->ks->bwd1[h->opt.tableau][h->opt.precision])
        fn = h->ks->bwd1[h->opt.tableau][h->opt.precision];
    if (h->bwd_grid <= 0)
        h->bwd_grid = grid_for(h, fn, h->bwd_block, a.B);
    VA_CUDA(h, cudaMemsetAsync(&h->ctl->adj_next, 0, sizeof(unsigned int), s));
    VA_CUDA(h, launch(h, fn, h->bwd_grid, h->bwd_block, &a, s));
    return VA_OK;
}

// CUDA events of one autotune sweep, destroyed on every return path
struct AutotuneEvents {
    cudaEvent_t e[3] = {nullptr, nullptr, nullptr};
    ~AutotuneEvents()
    {
        for (cudaEvent_t x : e)
            if (x)
                cudaEventDestroy(x);
    }
};

// A tuned launch shape: block size and resident blocks per SM of each sweep
// (one-thread and lane-group models) and the bundle width (shared matrix).
struct TunedShape {
    int fb = 0, fbps = 0, bb = 0, bbps = 0, alt = 0;
};

// grid of a sweep launched with `block` threads and at most `bps` resident
// blocks per SM (never more CTAs than the batch needs)
int grid_of(va_handle *h, const void *fn, int block, int bps)
{
    const int occ = std::max(1, occupancy_of(h, fn, block));
    const long need = ((long)h->prob.batch * h->ks->tpi + block - 1) / block;
    return (int)std::max(1L, std::min((long)h->sm_count * std::min(bps, occ), need));
}

void apply_shape(va_handle *h, const TunedShape &t)
{
    if (h->bks) {
        h->bundle_alt = t.alt != 0 && bundle_alt_available(h);
        return;
    }
    const void *ffn = h->ks->fwd[h->opt.tableau][h->opt.precision];
    const void *bfn = h->ks->bwd[h->opt.tableau][h->opt.precision];
    h->fwd_block = t.fb;
    h->fwd_grid = grid_of(h, ffn, t.fb, t.fbps);
    h->bwd_block = t.bb;
    h->bwd_grid = grid_of(h, bfn, t.bb, t.bbps);
}

// Forward and backward once untimed, then the best of two timed runs.
va_status time_sweeps(va_handle *h, int32_t cost, const double *y0, const double *params, const double *t0,
                      const double *t1, cudaStream_t s, AutotuneEvents &ev, float &tf, float &tb)
{
    cudaEvent_t e0 = ev.e[0], e1 = ev.e[1], e2 = ev.e[2];
    tf = tb = 1e30f;
    for (int rep = 0; rep < 3; rep++) {
        VA_CUDA(h, cudaEventRecord(e0, s));
        va_status st = enqueue_forward(h, y0, params, t0, t1, h->s_yT, nullptr, nullptr, h->s_status, s);
        if (st != VA_OK)
            return st;
        VA_CUDA(h, cudaEventRecord(e1, s));
        st = enqueue_backward(h, params, nullptr, nullptr, cost, h->s_dy0, h->s_dpar, h->s_status, s);
        if (st != VA_OK)
            return st;
        VA_CUDA(h, cudaEventRecord(e2, s));
        VA_CUDA(h, cudaEventSynchronize(e2));
        float a = 0, b = 0;
        VA_CUDA(h, cudaEventElapsedTime(&a, e0, e1));
        VA_CUDA(h, cudaEventElapsedTime(&b, e1, e2));
        if (rep > 0) {
            tf = std::min(tf, a);
            tb = std::min(tb, b);
        }
    }
    return VA_OK;
}

// Times the candidates and leaves the best shape in `best`.  One-thread and
// lane-group models: every (block size, resident blocks per SM) of each
// sweep; shared-matrix bundles: both compiled bundle widths.
va_status autotune_sweep(va_handle *h, int32_t cost, const double *y0, const double *params,
                         const double *t0, const double *t1, cudaStream_t s, AutotuneEvents &ev, TunedShape &best)
{
    for (cudaEvent_t &x : ev.e)
        VA_CUDA(h, cudaEventCreate(&x));
    if (h->bks) {
        float best_t = 1e30f;
        for (int alt = 0; alt <= (bundle_alt_available(h) ? 1 : 0); alt++) {
            h->bundle_alt = alt != 0;
            float tf, tb;
            const va_status st = time_sweeps(h, cost, y0, params, t0, t1, s, ev, tf, tb);
            if (st != VA_OK)
                return st;
            if (tf + tb < best_t) {
                best_t = tf + tb;
                best.alt = alt;
            }
        }
        return VA_OK;
    }
    const void *ffn = h->ks->fwd[h->opt.tableau][h->opt.precision];
    const void *bfn = h->ks->bwd[h->opt.tableau][h->opt.precision];
    float best_f = 1e30f, best_b = 1e30f;
    const int blocks[] = {64, 128, 256};
    for (int blk : blocks) {
        const int occf = occupancy_of(h, ffn, blk), occb = occupancy_of(h, bfn, blk);
        // every resident-block count: the best differs between the sweeps and
        // between workloads (stage-record traffic favours fewer warps in the
        // backward, issue rate more in the forward)
        const int maxocc = std::max(1, std::max(occf, occb));
        for (int bps = 1; bps <= maxocc; bps++) {
            TunedShape cand{blk, bps, blk, bps, 0};
            apply_shape(h, cand);
            float tf, tb;
            const va_status st = time_sweeps(h, cost, y0, params, t0, t1, s, ev, tf, tb);
            if (st != VA_OK)
                return st;
            if (tf < best_f) {
                best_f = tf;
                best.fb = blk;
                best.fbps = bps;
            }
            if (tb < best_b) {
                best_b = tb;
                best.bb = blk;
                best.bbps = bps;
            }
        }
    }
    return VA_OK;
}

// ------------------------------------------------------ autotune cache
//
// One line per tuned problem, "key<TAB>fb fbps bb bbps alt", in the file
// named by $VA_AUTOTUNE_CACHE ("" or "off": no cache), else
// $XDG_CACHE_HOME/vectorizedadjoint_gb300/autotune.tsv or
// $HOME/.cache/vectorizedadjoint_gb300/autotune.tsv.  The key: GPU name and
// SM count, model (and a model compiled outside the library's name), n,
// npar, nout, tableau, precision, stage records, checkpoint stride, step
// factor and the batch size's power of two.  The last matching line wins.

std::string cache_path()
{
    const char *e = std::getenv("VA_AUTOTUNE_CACHE");
    if (e)
        return (!*e || !std::strcmp(e, "off")) ? std::string() : std::string(e);
    const char *x = std::getenv("XDG_CACHE_HOME"), *home = std::getenv("HOME");
    std::string dir = (x && *x) ? std::string(x) : ((home && *home) ? std::string(home) + "/.cache" : std::string());
    return dir.empty() ? std::string() : dir + "/vectorizedadjoint_gb300/autotune.tsv";
}

std::string cache_key(const va_handle *h)
{
    cudaDeviceProp prop{};
    if (cudaGetDeviceProperties(&prop, h->device) != cudaSuccess)
        return std::string();
    int lb = 0;
    while ((1L << (lb + 1)) <= (long)h->prob.batch)
        lb++;
    char buf[512];
    std::snprintf(buf, sizeof(buf), "%s|%d|%d%s%s|%d|%d|%d|%d|%d|%d|%d|%d|%d", prop.name, h->sm_count,
                  h->prob.model, h->user ? ":" : "", h->user && h->user->name ? h->user->name : "", h->prob.n,
                  h->prob.npar, h->prob.nout, h->opt.tableau, h->opt.precision, (int)h->stages_on, h->stride,
                  h->opt.step_pow, lb);
    for (char *c = buf; *c; c++)
        if (*c == '\t' || *c == '\n')
            *c = ' ';
    return buf;
}

bool cache_lookup(const std::string &key, TunedShape &t)
{
    const std::string path = cache_path();
    if (path.empty() || key.empty())
        return false;
    FILE *f = std::fopen(path.c_str(), "r");
    if (!f)
        return false;
    char line[1024];
    bool found = false;
    while (std::fgets(line, sizeof(line), f)) {
        char *tab = std::strchr(line, '\t');
        if (!tab)
            continue;
        *tab = 0;
        TunedShape v;
        if (key == line && std::sscanf(tab + 1, "%d %d %d %d %d", &v.fb, &v.fbps, &v.bb, &v.bbps, &v.alt) == 5) {
            t = v;
            found = true;
        }
    }
    std::fclose(f);
    return found;
}

void cache_store(const std::string &key, const TunedShape &t)
{
    const std::string path = cache_path();
    if (path.empty() || key.empty())
        return;
    // create the directories of the path (an existing one is fine)
    for (size_t k = path.find('/', 1); k != std::string::npos; k = path.find('/', k + 1))
        mkdir(path.substr(0, k).c_str(), 0755);
    FILE *f = std::fopen(path.c_str(), "a");
    if (!f)
        return;
    std::fprintf(f, "%s\t%d %d %d %d %d\n", key.c_str(), t.fb, t.fbps, t.bb, t.bbps, t.alt);
    std::fclose(f);
}

void drop_graph(va_handle *h)
{
    if (h->graph) {
        cudaGraphExecDestroy(h->graph);
        h->graph = nullptr;
    }
    h->graph_key = GraphKey{};
}

} // namespace

extern "C" {

const char *va_status_string(int32_t s)
{
    switch (s) {
    case VA_OK:
        return "VA_OK";
    case VA_MAX_REJECTS:
        return "VA_MAX_REJECTS";
    case VA_MAX_STEPS:
        return "VA_MAX_STEPS";
    case VA_NONFINITE:
        return "VA_NONFINITE";
    case VA_CKPT_BUDGET:
        return "VA_CKPT_BUDGET";
    case VA_BAD_ARGS:
        return "VA_BAD_ARGS";
    case VA_CUDA_ERROR:
        return "VA_CUDA_ERROR";
    case VA_NOT_READY:
        return "VA_NOT_READY";
    case VA_RECOMPUTE_MISMATCH:
        return "VA_RECOMPUTE_MISMATCH";
    case VA_NOT_RUN:
        return "VA_NOT_RUN";
    default:
        return "VA_UNKNOWN";
    }
}

const char *va_last_error(const va_handle *h) { return h ? h->err.c_str() : "null handle"; }

va_status va_step_pow_undecided(va_handle *h, int64_t *count)
{
    if (!h || !count)
        return fail(h, VA_BAD_ARGS, "va_step_pow_undecided: null argument%s");
    *count = 0;
    if (!h->ctl)
        return VA_OK; // no sweep has run
    unsigned int c = 0;
    VA_CUDA(h, cudaMemcpy(&c, &h->ctl->pow_undecided, sizeof(c), cudaMemcpyDeviceToHost));
    *count = c;
    return VA_OK;
}

va_status va_default_options(va_options *o)
{
    if (!o)
        return VA_BAD_ARGS;
    std::memset(o, 0, sizeof(*o));
    o->tableau = VA_TAB_DOPRI5;
    o->precision = VA_PREC_FP64;
    o->atol = 1e-6;
    o->rtol = 1e-6;
    o->dt0 = 1e-3;
    o->max_steps = 1000000;
    o->max_rejects = 500;
    o->ckpt_budget_bytes = 0;
    o->ckpt_stride = 0;
    o->block_size = 0;
    o->blocks_per_sm = 0;
    o->chunk_len = 0;
    o->stage_records = 1;
    o->step_pow = 1;
    return VA_OK;
}

} // extern "C"

namespace {

// va_create / va_create_model: `user` is null for the built-in models
va_status create_handle(const va_problem *prob, const va_options *opt, const va::ModelKernels *user,
                        va_handle **out)
{
    if (!prob || !out)
        return VA_BAD_ARGS;
    *out = nullptr;
    va_options o;
    if (opt)
        o = *opt;
    else
        va_default_options(&o);
    if (prob->batch < 1 || prob->nout < 1 || prob->n < 1)
        return VA_BAD_ARGS;
    if (o.tableau < 0 || o.tableau >= va::kTableaux)
        return VA_BAD_ARGS;
    if (o.precision != VA_PREC_FP64 && o.precision != VA_PREC_MIXED && o.precision != VA_PREC_MIXED_DW)
        return VA_BAD_ARGS;
    if (!(o.atol >= 0.0) || !(o.rtol >= 0.0) || !(o.atol + o.rtol > 0.0) || !(o.dt0 > 0.0))
        return VA_BAD_ARGS;
    if (o.max_steps < 1 || o.max_rejects < 1)
        return VA_BAD_ARGS;
    const va::KernelSet *ks = nullptr;
    const va::BundleKernelSet *bks = nullptr;
    int N = 0, P = 0;
    if (user) {
        if (prob->model != VA_MODEL_USER || user->magic != va::kModelMagic || user->abi != va::kModelAbi ||
            !user->launch || !user->occupancy)
            return VA_BAD_ARGS;
        ks = &user->set;
        if (!ks->fwd[o.tableau][o.precision])
            return VA_BAD_ARGS;
        N = ks->N;
        P = ks->P;
    } else if (prob->model == VA_MODEL_GLV_SHARED) {
        bks = va::kernels_glv_shared(prob->n);
        // a (tableau, precision) pair without compiled kernels is rejected
        if (!bks || prob->nout != 1 || !bks->fwd[o.tableau][o.precision])
            return VA_BAD_ARGS;
        N = P = prob->n;
    } else {
        ks = kernel_set(*prob);
        if (!ks || !ks->fwd[o.tableau][o.precision])
            return VA_BAD_ARGS;
        N = ks->N > 0 ? ks->N : prob->n;
        P = ks->P > 0 ? ks->P : prob->npar;
    }
    if (prob->n != N || prob->npar != P)
        return VA_BAD_ARGS;
    // checkpoint stride: -1 automatic, 0/1 every step, k > 1 every k-th step
    // (two-level checkpointing: every model family whose two-level backward
    // is compiled for the tableau and precision)
    if (o.ckpt_stride < -1 ||
        (o.ckpt_stride > 1 && !(ks && ks->bwd2[o.tableau][o.precision]) && !(bks && bks->bwd2[o.tableau][o.precision])))
        return VA_BAD_ARGS;
    va_handle *h = new va_handle();
    h->stride = o.ckpt_stride > 1 ? o.ckpt_stride : 1;
    h->stages_on = o.stage_records != 0;
    h->prob = *prob;
    h->opt = o;
    h->ks = ks;
    h->user = user;
    h->bks = bks;
    h->N = N;
    h->P = P;
    h->chunk_len = o.chunk_len > 0 ? o.chunk_len : 64;
    record_layout(h);
    if (o.block_size > 0) {
        h->fwd_block = h->bwd_block = o.block_size;
    }
    cudaError_t e = cudaGetDevice(&h->device);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, h->device);
    if (e != cudaSuccess) {
        delete h;
        return VA_CUDA_ERROR;
    }
    *out = h;
    return VA_OK;
}

} // namespace

extern "C" {

va_status va_create(const va_problem *prob, const va_options *opt, va_handle **out)
{
    return create_handle(prob, opt, nullptr, out);
}

va_status va_create_model(const va_problem *prob, const va_options *opt, const va_model_kernels *model,
                          va_handle **out)
{
    if (!model) {
        if (out)
            *out = nullptr;
        return VA_BAD_ARGS;
    }
    return create_handle(prob, opt, reinterpret_cast<const va::ModelKernels *>(model), out);
}

va_status va_forward_frozen(va_handle *h, int32_t count, int32_t times_stride, const double *times,
                            const int32_t *n_steps, const double *y0, const double *params,
                            const double *shared, double *yT, void *stream)
{
    if (!h)
        return VA_BAD_ARGS;
    if (count < 1 || times_stride < 2 || !times || !n_steps || !y0 || !params || !yT)
        return fail(h, VA_BAD_ARGS, "va_forward_frozen: bad count, stride or null pointer%s");
    va::ReplayParams r{};
    r.count = count;
    r.stride = times_stride;
    r.n = h->N;
    r.np = h->P;
    r.times = times;
    r.n_steps = n_steps;
    r.y0 = y0;
    r.par = params;
    r.yT = yT;
    cudaStream_t s = (cudaStream_t)stream;
    const int tab = h->opt.tableau;
    if (h->ks && h->ks->tpi == 1) {
        const void *fn = h->ks->replay[tab];
        if (!fn)
            return fail(h, VA_BAD_ARGS, "va_forward_frozen: no replay kernel for this model and tableau%s");
        VA_CUDA(h, launch(h, fn, (count + 127) / 128, 128, &r, s));
        return VA_OK;
    }
    // Lotka-Volterra (per-instance matrix, or the shared one): a CTA per lane
    if (h->bks) {
        r.shared = shared ? shared : h->shared_A;
        if (!r.shared)
            return fail(h, VA_BAD_ARGS, "va_forward_frozen: shared-matrix model without a matrix%s");
    }
    const void *fn = va::replay_glv(tab);
    if (!fn || h->N > 1024)
        return fail(h, VA_BAD_ARGS, "va_forward_frozen: no replay kernel for this model and tableau%s");
    void *args[] = {&r};
    VA_CUDA(h, cudaLaunchKernel(fn, dim3(count), dim3(h->N), args, sizeof(double) * h->N, s));
    return VA_OK;
}

va_status va_destroy(va_handle *h)
{
    if (!h)
        return VA_BAD_ARGS;
    drop_graph(h);
    void *ptrs[] = {h->pool_rec, h->chunk_prev, h->inst_T,  h->inst_last, h->inst_status,
                    h->ctl,      h->s_y0,       h->s_par,   h->s_t0,      h->s_t1,
                    h->s_yT,     h->s_dy0,      h->s_dpar,  h->s_nacc,    h->s_status,
                    h->s_nrej,   h->s_lam,      h->s_mu,    h->At,        h->Aw,
                    h->Atw,      h->dA_part,    h->inst_t1, h->scratch, h->order_fwd,
                    h->order_bwd, h->order_work, h->inst_work, h->inst_t0, h->hist, h->fac_v,
                    h->fac_xp,    h->k_base,    h->c_part,  h->c_err,     h->bt_adig, h->bt_aexp, h->bt_rpk, h->bt_adig_f, h->bt_aexp_f, h->bt_ferr};
    for (void *p : ptrs)
        if (p)
            cudaFree(p);
    delete h;
    return VA_OK;
}

va_status va_forward(va_handle *h, const double *y0, const double *params, const double *t0,
                     const double *t1, double *yT, int32_t *n_acc, int32_t *n_rej, int32_t *status,
                     void *stream)
{
    if (!h)
        return VA_BAD_ARGS;
    if (!y0 || !params || !t0 || !t1)
        return fail(h, VA_BAD_ARGS, "va_forward: null input pointer%s");
    va_status st = ensure_buffers(h);
    if (st != VA_OK)
        return st;
    for (;;) {
        st = enqueue_forward(h, y0, params, t0, t1, yT, n_acc, n_rej, status, (cudaStream_t)stream);
        if (st != VA_OK || h->opt.ckpt_stride != -1)
            break;
        // automatic stride: if the pool ran out, store 4x fewer steps and rerun
        va::Control c{};
        VA_CUDA(h, cudaMemcpyAsync(&c, h->ctl, sizeof(c), cudaMemcpyDeviceToHost, (cudaStream_t)stream));
        VA_CUDA(h, cudaStreamSynchronize((cudaStream_t)stream));
        if (!c.pool_fail || h->stride >= kMaxAutoStride)
            break;
        // the ladder: drop the stage values first, then thin the checkpoints
        // (where a two-level backward exists)
        if (stages_now(h))
            h->stages_on = false;
        else if ((h->ks && h->ks->bwd2[h->opt.tableau][h->opt.precision]) ||
                 (h->bks && h->bks->bwd2[h->opt.tableau][h->opt.precision]))
            h->stride *= 4;
        else
            break;
        record_layout(h);
        drop_graph(h);
    }
    if (st == VA_OK)
        st = ensure_scratch(h);
    if (st == VA_OK)
        h->forward_done = true;
    return st;
}

va_status va_backward(va_handle *h, const double *params, const double *lambdaT,
                      const double *mu_direct, double *dy0, double *dparams, int32_t *status,
                      void *stream)
{
    if (!h)
        return VA_BAD_ARGS;
    if (!h->forward_done)
        return fail(h, VA_NOT_READY, "va_backward: no forward sweep has run on this handle%s");
    if (!params || !lambdaT || !dy0 || !dparams)
        return fail(h, VA_BAD_ARGS, "va_backward: null pointer%s");
    va_status st = ensure_scratch(h);
    if (st != VA_OK)
        return st;
    return enqueue_backward(h, params, lambdaT, mu_direct, VA_COST_SEEDS, dy0, dparams, status,
                            (cudaStream_t)stream);
}

va_status va_gradient(va_handle *h, int32_t cost, const double *y0, const double *params,
                      const double *t0, const double *t1, double *yT, double *dy0, double *dparams,
                      int32_t *n_acc, int32_t *status, void *stream)
{
    if (!h)
        return VA_BAD_ARGS;
    if (cost != VA_COST_SUMSQ && cost != VA_COST_SUM)
        return fail(h, VA_BAD_ARGS, "va_gradient: cost must be VA_COST_SUMSQ or VA_COST_SUM%s");
    if (h->prob.nout != 1)
        return fail(h, VA_BAD_ARGS, "va_gradient: built-in costs need nout == 1%s");
    if (!y0 || !params || !t0 || !t1 || !dy0 || !dparams)
        return fail(h, VA_BAD_ARGS, "va_gradient: null pointer%s");
    va_status st = ensure_buffers(h);
    if (st == VA_OK)
        st = ensure_scratch(h);
    if (st != VA_OK)
        return st;
    cudaStream_t s = (cudaStream_t)stream;
    if (h->opt.ckpt_stride == -1 && !h->ladder_settled) {
        // automatic checkpointing: the first call runs the forward with its
        // memory ladder (synchronous checks of the pool between reruns), then
        // the backward; later calls capture the layout it settled on
        st = va_forward(h, y0, params, t0, t1, yT, n_acc, nullptr, status, stream);
        if (st != VA_OK)
            return st;
        h->ladder_settled = true;
        return enqueue_backward(h, params, nullptr, nullptr, cost, dy0, dparams, status, s);
    }
    GraphKey key;
    key.cost = cost;
    const void *ptrs[10] = {y0, params, t0, t1, yT, dy0, dparams, n_acc, status, h->shared_A};
    std::memcpy(key.ptrs, ptrs, sizeof(ptrs));
    key.stream = stream;
    key.extra = h->shared_dA;
    // The legacy default stream cannot be captured: launch directly there.
    if (s == nullptr) {
        st = enqueue_forward(h, y0, params, t0, t1, yT, n_acc, nullptr, status, s);
        if (st != VA_OK)
            return st;
        h->forward_done = true;
        return enqueue_backward(h, params, nullptr, nullptr, cost, dy0, dparams, status, s);
    }
    if (!h->graph || !(h->graph_key == key)) {
        drop_graph(h);
        // size the persistent grids before capture (occupancy queries)
        if (h->ks && h->fwd_grid <= 0)
            h->fwd_grid = grid_for(h, h->ks->fwd[h->opt.tableau][h->opt.precision], h->fwd_block,
                                   h->prob.batch);
        if (h->ks && h->bwd_grid <= 0)
            h->bwd_grid = grid_for(h, h->ks->bwd[h->opt.tableau][h->opt.precision], h->bwd_block,
                                   h->prob.batch);
        VA_CUDA(h, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        va_status s1 = enqueue_forward(h, y0, params, t0, t1, yT, n_acc, nullptr, status, s);
        va_status s2 = s1 == VA_OK
                           ? enqueue_backward(h, params, nullptr, nullptr, cost, dy0, dparams, status, s)
                           : s1;
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(s, &g);
        if (s2 != VA_OK) {
            if (g)
                cudaGraphDestroy(g);
            return s2;
        }
        if (e != cudaSuccess)
            return cuda_fail(h, e, "cudaStreamEndCapture");
        e = cudaGraphInstantiate(&h->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            h->graph = nullptr;
            return cuda_fail(h, e, "cudaGraphInstantiate");
        }
        h->graph_key = key;
    }
    VA_CUDA(h, cudaGraphLaunch(h->graph, s));
    h->forward_done = true;
    return VA_OK;
}

va_status va_gradient_host(va_handle *h, int32_t cost, const double *y0, const double *params,
                           const double *t0, const double *t1, double *yT, double *dy0,
                           double *dparams, int32_t *n_acc, int32_t *status, void *stream)
{
    if (!h)
        return VA_BAD_ARGS;
    if (!y0 || !params || !t0 || !t1)
        return fail(h, VA_BAD_ARGS, "va_gradient_host: null input pointer%s");
    va_status st = ensure_staging(h);
    if (st != VA_OK)
        return st;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t B = h->prob.batch, N = h->N, P = h->P;
    VA_CUDA(h, cudaMemcpyAsync(h->s_y0, y0, B * N * sizeof(double), cudaMemcpyHostToDevice, s));
    VA_CUDA(h, cudaMemcpyAsync(h->s_par, params, B * P * sizeof(double), cudaMemcpyHostToDevice, s));
    VA_CUDA(h, cudaMemcpyAsync(h->s_t0, t0, B * sizeof(double), cudaMemcpyHostToDevice, s));
    VA_CUDA(h, cudaMemcpyAsync(h->s_t1, t1, B * sizeof(double), cudaMemcpyHostToDevice, s));
    st = va_gradient(h, cost, h->s_y0, h->s_par, h->s_t0, h->s_t1, h->s_yT, h->s_dy0, h->s_dpar,
                     h->s_nacc, h->s_status, stream);
    if (st != VA_OK)
        return st;
    if (yT)
        VA_CUDA(h, cudaMemcpyAsync(yT, h->s_yT, B * N * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (dy0)
        VA_CUDA(h, cudaMemcpyAsync(dy0, h->s_dy0, B * N * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (dparams)
        VA_CUDA(h, cudaMemcpyAsync(dparams, h->s_dpar, B * P * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (n_acc)
        VA_CUDA(h, cudaMemcpyAsync(n_acc, h->s_nacc, B * sizeof(int), cudaMemcpyDeviceToHost, s));
    if (status)
        VA_CUDA(h, cudaMemcpyAsync(status, h->s_status, B * sizeof(int), cudaMemcpyDeviceToHost, s));
    VA_CUDA(h, cudaStreamSynchronize(s));
    return VA_OK;
}

va_status va_forward_host(va_handle *h, const double *y0, const double *params, const double *t0,
                          const double *t1, double *yT, int32_t *n_acc, int32_t *n_rej, int32_t *status)
{
    if (!h)
        return VA_BAD_ARGS;
    if (!y0 || !params || !t0 || !t1)
        return fail(h, VA_BAD_ARGS, "va_forward_host: null input pointer%s");
    va_status st = ensure_staging(h);
    if (st != VA_OK)
        return st;
    const size_t B = h->prob.batch, N = h->N, P = h->P;
    VA_CUDA(h, cudaMemcpy(h->s_y0, y0, B * N * sizeof(double), cudaMemcpyHostToDevice));
    VA_CUDA(h, cudaMemcpy(h->s_par, params, B * P * sizeof(double), cudaMemcpyHostToDevice));
    VA_CUDA(h, cudaMemcpy(h->s_t0, t0, B * sizeof(double), cudaMemcpyHostToDevice));
    VA_CUDA(h, cudaMemcpy(h->s_t1, t1, B * sizeof(double), cudaMemcpyHostToDevice));
    st = va_forward(h, h->s_y0, h->s_par, h->s_t0, h->s_t1, h->s_yT, h->s_nacc, h->s_nrej, h->s_status,
                    nullptr);
    if (st != VA_OK)
        return st;
    VA_CUDA(h, cudaDeviceSynchronize());
    if (yT)
        VA_CUDA(h, cudaMemcpy(yT, h->s_yT, B * N * sizeof(double), cudaMemcpyDeviceToHost));
    if (n_acc)
        VA_CUDA(h, cudaMemcpy(n_acc, h->s_nacc, B * sizeof(int), cudaMemcpyDeviceToHost));
    if (n_rej)
        VA_CUDA(h, cudaMemcpy(n_rej, h->s_nrej, B * sizeof(int), cudaMemcpyDeviceToHost));
    if (status)
        VA_CUDA(h, cudaMemcpy(status, h->s_status, B * sizeof(int), cudaMemcpyDeviceToHost));
    return VA_OK;
}

va_status va_backward_host(va_handle *h, const double *params, const double *lambdaT,
                           const double *mu_direct, double *dy0, double *dparams, int32_t *status)
{
    if (!h)
        return VA_BAD_ARGS;
    if (!params || !lambdaT)
        return fail(h, VA_BAD_ARGS, "va_backward_host: null input pointer%s");
    va_status st = ensure_staging(h);
    if (st != VA_OK)
        return st;
    const size_t B = h->prob.batch, N = h->N, P = h->P, Q = h->prob.nout;
    VA_CUDA(h, cudaMemcpy(h->s_par, params, B * P * sizeof(double), cudaMemcpyHostToDevice));
    VA_CUDA(h, cudaMemcpy(h->s_lam, lambdaT, B * Q * N * sizeof(double), cudaMemcpyHostToDevice));
    if (mu_direct)
        VA_CUDA(h, cudaMemcpy(h->s_mu, mu_direct, B * Q * P * sizeof(double), cudaMemcpyHostToDevice));
    st = va_backward(h, h->s_par, h->s_lam, mu_direct ? h->s_mu : nullptr, h->s_dy0, h->s_dpar,
                     h->s_status, nullptr);
    if (st != VA_OK)
        return st;
    VA_CUDA(h, cudaDeviceSynchronize());
    if (dy0)
        VA_CUDA(h, cudaMemcpy(dy0, h->s_dy0, B * Q * N * sizeof(double), cudaMemcpyDeviceToHost));
    if (dparams)
        VA_CUDA(h, cudaMemcpy(dparams, h->s_dpar, B * Q * P * sizeof(double), cudaMemcpyDeviceToHost));
    if (status)
        VA_CUDA(h, cudaMemcpy(status, h->s_status, B * sizeof(int), cudaMemcpyDeviceToHost));
    return VA_OK;
}

va_status va_get_launch(const va_handle *h, int32_t *fwd_block, int32_t *fwd_grid,
                        int32_t *bwd_block, int32_t *bwd_grid)
{
    if (!h)
        return VA_BAD_ARGS;
    if (fwd_block)
        *fwd_block = h->fwd_block;
    if (fwd_grid)
        *fwd_grid = h->fwd_grid;
    if (bwd_block)
        *bwd_block = h->bwd_block;
    if (bwd_grid)
        *bwd_grid = h->bwd_grid;
    return VA_OK;
}

va_status va_checkpoint_info(const va_handle *h, int64_t *capacity_bytes, int64_t *used_bytes,
                             int32_t *stride)
{
    if (!h)
        return VA_BAD_ARGS;
    const int64_t chunk_bytes = (int64_t)h->RS * sizeof(double) * h->chunk_len;
    if (capacity_bytes)
        *capacity_bytes = (int64_t)h->n_chunks * chunk_bytes;
    if (used_bytes) {
        *used_bytes = 0;
        if (h->ctl) {
            va::Control c{};
            if (cudaMemcpy(&c, h->ctl, sizeof(c), cudaMemcpyDeviceToHost) == cudaSuccess)
                *used_bytes = (int64_t)std::min<unsigned>(c.pool_next, (unsigned)h->n_chunks) * chunk_bytes;
        }
    }
    if (stride)
        *stride = h->stride;
    return VA_OK;
}

va_status va_trajectory(va_handle *h, int32_t instance, int32_t capacity, double *t, double *dt,
                        double *y, int32_t *n_records)
{
    if (!h || instance < 0 || instance >= h->prob.batch || capacity < 0)
        return VA_BAD_ARGS;
    if (h->stride > 1)
        return fail(h, VA_BAD_ARGS, "va_trajectory: checkpoint stride > 1 keeps only every k-th step%s");
    if (!h->forward_done || !h->inst_T)
        return fail(h, VA_NOT_READY, "va_trajectory: no forward sweep has run%s");
    VA_CUDA(h, cudaDeviceSynchronize());
    int T = 0, last = -1, st = 0;
    VA_CUDA(h, cudaMemcpy(&T, h->inst_T + instance, sizeof(int), cudaMemcpyDeviceToHost));
    VA_CUDA(h, cudaMemcpy(&last, h->inst_last + instance, sizeof(int), cudaMemcpyDeviceToHost));
    VA_CUDA(h, cudaMemcpy(&st, h->inst_status + instance, sizeof(int), cudaMemcpyDeviceToHost));
    if (n_records)
        *n_records = T + 1;
    if (st != VA_OK || last < 0)
        return fail(h, (va_status)st, "va_trajectory: instance has no complete record%s");
    const int CH = h->chunk_len, RS = h->RS, N = h->N;
    // mixed_dw stage records, and the one-thread kernels' [t, dt, y] records,
    // hold double-words (float pairs {hi, lo} in 8 bytes) after the FP64 time
    // (bundle stage records: t and dt FP64, the state as double-words)
    const bool dw = h->ks && h->opt.precision == VA_PREC_MIXED_DW && (h->ks->dw_records || stages_now(h));
    const bool ydw = dw || (h->bks && stages_now(h));
    auto unpack = [](double v) {
        const va::dword d = va::dw_unpack(v);
        return (double)d.hi + (double)d.lo;
    };
    std::vector<double> buf((size_t)CH * RS);
    int chunk = last;
    int first_in_chunk = (T / CH) * CH; // record index at slot 0 of the last chunk
    while (chunk >= 0 && first_in_chunk >= 0) {
        const int cnt = std::min(CH, T + 1 - first_in_chunk);
        VA_CUDA(h, cudaMemcpy(buf.data(), h->pool_rec + (size_t)chunk * CH * RS,
                              (size_t)cnt * RS * sizeof(double), cudaMemcpyDeviceToHost));
        for (int k = 0; k < cnt; k++) {
            const int j = first_in_chunk + k;
            if (j >= capacity)
                continue;
            if (t)
                t[j] = buf[(size_t)k * RS];
            if (dt)
                dt[j] = dw ? unpack(buf[(size_t)k * RS + 1]) : buf[(size_t)k * RS + 1];
            if (y)
                for (int i = 0; i < N; i++) {
                    const double v = buf[(size_t)k * RS + 2 + i];
                    y[(size_t)j * N + i] = ydw ? unpack(v) : v;
                }
        }
        int prev = -1;
        VA_CUDA(h, cudaMemcpy(&prev, h->chunk_prev + chunk, sizeof(int), cudaMemcpyDeviceToHost));
        chunk = prev;
        first_in_chunk -= CH;
    }
    return VA_OK;
}

va_status va_set_adjoint_history(va_handle *h, int32_t capacity)
{
    if (!h || capacity < 0)
        return VA_BAD_ARGS;
    if (capacity > 0 && h->bks)
        return fail(h, VA_BAD_ARGS, "va_set_adjoint_history: not available for the shared-matrix model%s");
    drop_graph(h); // captured sweeps hold the old buffer
    if (h->hist) {
        VA_CUDA(h, cudaDeviceSynchronize());
        VA_CUDA(h, cudaFree(h->hist));
        h->hist = nullptr;
    }
    h->hist_cap = 0;
    h->hist_done = false;
    if (capacity == 0)
        return VA_OK;
    const size_t n = (size_t)h->prob.batch * h->prob.nout * capacity * h->N;
    VA_CUDA(h, cudaMalloc(&h->hist, n * sizeof(double)));
    // all-ones bytes: a NaN in every slot no sweep writes
    VA_CUDA(h, cudaMemset(h->hist, 0xff, n * sizeof(double)));
    h->hist_cap = capacity;
    return VA_OK;
}

va_status va_adjoint_history(va_handle *h, int32_t instance, int32_t capacity, double *t, double *lambda,
                             int32_t *n_records)
{
    if (!h || instance < 0 || instance >= h->prob.batch || capacity < 0)
        return VA_BAD_ARGS;
    if (!h->hist)
        return fail(h, VA_NOT_READY, "va_adjoint_history: call va_set_adjoint_history first%s");
    if (!h->hist_done)
        return fail(h, VA_NOT_READY, "va_adjoint_history: no backward sweep has run with the history on%s");
    int32_t nrec = 0;
    if (t) { // the record times, as va_trajectory reads them (stride 1)
        const va_status st = va_trajectory(h, instance, capacity, t, nullptr, nullptr, &nrec);
        if (st != VA_OK)
            return st;
    } else {
        VA_CUDA(h, cudaDeviceSynchronize());
        int T = 0;
        VA_CUDA(h, cudaMemcpy(&T, h->inst_T + instance, sizeof(int), cudaMemcpyDeviceToHost));
        nrec = T + 1;
    }
    if (n_records)
        *n_records = nrec;
    const int N = h->N, Q = h->prob.nout;
    const int k = std::min(std::min(capacity, h->hist_cap), nrec);
    if (lambda && k > 0) {
        for (int q = 0; q < Q; q++)
            VA_CUDA(h, cudaMemcpy(lambda + (size_t)q * capacity * N,
                                  h->hist + (((size_t)instance * Q + q) * h->hist_cap) * N,
                                  (size_t)k * N * sizeof(double), cudaMemcpyDeviceToHost));
    }
    return VA_OK;
}

va_status va_adjoint_history_buffer(const va_handle *h, double **buf, int32_t *capacity)
{
    if (!h)
        return VA_BAD_ARGS;
    if (buf)
        *buf = h->hist;
    if (capacity)
        *capacity = h->hist_cap;
    return VA_OK;
}

va_status va_set_shared(va_handle *h, const double *A, double *dA)
{
    if (!h)
        return VA_BAD_ARGS;
    if (!h->bks)
        return fail(h, VA_BAD_ARGS, "va_set_shared: the model has no shared parameters%s");
    if (!A)
        return fail(h, VA_BAD_ARGS, "va_set_shared: A is null%s");
    h->shared_A = A;
    h->shared_dA = dA;
    return VA_OK;
}

va_status va_autotune(va_handle *h, int32_t cost, const double *y0, const double *params,
                      const double *t0, const double *t1, void *stream)
{
    if (!h)
        return VA_BAD_ARGS;
    va_status st = ensure_buffers(h);
    if (st != VA_OK)
        return st;
    st = ensure_staging(h);
    if (st == VA_OK)
        st = ensure_scratch(h);
    if (st != VA_OK)
        return st;
    const std::string key = cache_key(h);
    TunedShape t;
    if (cache_lookup(key, t) && (h->bks || (t.fb > 0 && t.bb > 0 && t.fbps > 0 && t.bbps > 0))) {
        apply_shape(h, t);
        drop_graph(h);
        return VA_OK;
    }
    cudaStream_t s = (cudaStream_t)stream;
    // the launch shape before tuning, restored if a candidate run fails
    const int prev[4] = {h->fwd_block, h->fwd_grid, h->bwd_block, h->bwd_grid};
    const bool prev_alt = h->bundle_alt;
    AutotuneEvents ev;
    st = autotune_sweep(h, cost, y0, params, t0, t1, s, ev, t);
    if (st != VA_OK) {
        h->fwd_block = prev[0];
        h->fwd_grid = prev[1];
        h->bwd_block = prev[2];
        h->bwd_grid = prev[3];
        h->bundle_alt = prev_alt;
        drop_graph(h);
        return st;
    }
    apply_shape(h, t);
    cache_store(key, t);
    drop_graph(h);
    h->forward_done = true;
    return VA_OK;
}

} // extern "C"
