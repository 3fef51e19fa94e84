// va_gradient_noalloc: forward + backward sweeps that allocate nothing.
//
// Who needs it: callers that may not allocate device memory once they are
// running -- for example a host application whose device memory is carved
// out up front and owned by another runtime's caching allocator (any
// cudaMalloc outside it fails or fragments that pool), or a plugin whose host
// forbids allocation inside its callbacks.  The regular entry points keep
// their scratch (checkpoint pool, per-instance metadata, work counters) in a
// handle that cudaMallocs it; this one takes all of it from a fixed array
// compiled into the library instead.
//
// The array is a file-scope __device__ array of VA_NOALLOC_SCRATCH_BYTES
// (64 MiB): every GPU that loads the library holds it until the process
// exits.  Host code cannot use the array's name as a device address (it is a
// host-side stand-in), so the device address is looked up with
// cudaGetSymbolAddress once per device, with that device current, on the
// first call made on that device; make that first call before any stream
// capture.  All calls share the array and it keeps the previous call's
// contents: each call clears the work counters it needs zeroed and writes
// everything else before reading it.  Calls whose GPU work overlaps (two
// streams, or two host threads) race on the array and corrupt each other.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/va.h"
#include "va_kernels.cuh"
#include "va_registry.h"

namespace {

constexpr size_t kScratchBytes = VA_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;
constexpr int kChunkLen = 64;
constexpr size_t kStageChunks = 4; // chunks per instance below which stage records are dropped

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

} // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

static unsigned char *g_scratch_addr[kMaxDevices];
static std::mutex g_scratch_mutex;

// Device address of the scratch array on the current device (looked up once).
static va_status scratch_address(unsigned char **out)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess)
        return VA_CUDA_ERROR;
    if (dev < 0 || dev >= kMaxDevices)
        return VA_BAD_ARGS;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p)
            return VA_CUDA_ERROR;
        g_scratch_addr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_scratch_addr[dev];
    return VA_OK;
}

extern "C" va_status va_gradient_noalloc(int32_t model, int32_t tableau, int32_t precision, double atol,
                                         double rtol, double dt0, int32_t max_steps, int32_t max_rejects,
                                         int32_t cost, int32_t batch, const double *y0,
                                         const double *params, const double *t0, const double *t1,
                                         double *yT, double *dy0, double *dparams, int32_t *n_acc,
                                         int32_t *status, void *stream)
{
    const va::KernelSet *ks = nullptr;
    switch (model) {
    case VA_MODEL_VDP:
        ks = va::kernels_vdp();
        break;
    case VA_MODEL_VDP_PETSC:
        ks = va::kernels_vdp_petsc();
        break;
    case VA_MODEL_DHO:
        ks = va::kernels_dho();
        break;
    case VA_MODEL_DECAY:
        ks = va::kernels_decay();
        break;
    default:
        return VA_BAD_ARGS;
    }
    if (tableau < 0 || tableau >= va::kTableaux)
        return VA_BAD_ARGS;
    if (precision != VA_PREC_FP64 && precision != VA_PREC_MIXED && precision != VA_PREC_MIXED_DW)
        return VA_BAD_ARGS;
    if (!ks->fwd[tableau][precision])
        return VA_BAD_ARGS;
    if (cost != VA_COST_SUMSQ && cost != VA_COST_SUM)
        return VA_BAD_ARGS;
    if (!(atol >= 0.0) || !(rtol >= 0.0) || !(atol + rtol > 0.0) || !(dt0 > 0.0) || max_steps < 1 ||
        max_rejects < 1 || batch < 1)
        return VA_BAD_ARGS;
    if (!y0 || !params || !t0 || !t1 || !dy0 || !dparams)
        return VA_BAD_ARGS;

    // Carve the array: control block | inst_T | inst_last | inst_status |
    // chunk_prev | checkpoint chunks.  Every instance needs at least one
    // chunk; a batch whose metadata and first chunks do not fit is rejected.
    const size_t B = (size_t)batch;
    const size_t off_T = 256, off_last = off_T + align256(B * 4), off_st = off_last + align256(B * 4);
    const size_t off_prev = off_st + align256(B * 4);
    if (off_prev >= kScratchBytes)
        return VA_BAD_ARGS;
    const size_t room = kScratchBytes - off_prev;
    auto chunks_for = [&](size_t rec_doubles) {
        const size_t chunk_bytes = rec_doubles * sizeof(double) * kChunkLen;
        size_t n = room / (chunk_bytes + sizeof(int));
        while (n > 0 && align256(n * sizeof(int)) + n * chunk_bytes > room)
            n--;
        return n;
    };
    // Every step is checkpointed.  The double-word sweeps keep stage records
    // (the step's stage values too) while the array holds kStageChunks
    // chunks per instance; below that they switch to [t, dt, y] records and
    // recompute the stages in the backward sweep (the kernels va_create uses
    // with stage_records = 0), which fits ~4x more steps.
    const void *ffn = ks->fwd[tableau][precision];
    const void *bfn = ks->bwd[tableau][precision];
    size_t n_chunks = chunks_for((size_t)va::record_doubles_for(ks, tableau, precision, 1, ks->N, true));
    if (n_chunks < kStageChunks * B && ks->fwd2[tableau][precision] && ks->bwd1[tableau][precision]) {
        n_chunks = chunks_for((size_t)va::record_doubles_for(ks, tableau, precision, 1, ks->N, false));
        ffn = ks->fwd2[tableau][precision];
        bfn = ks->bwd1[tableau][precision];
    }
    if (n_chunks < B || n_chunks > 0x7fffffff)
        return VA_BAD_ARGS;
    const size_t off_pool = off_prev + align256(n_chunks * sizeof(int));

    unsigned char *base = nullptr;
    va_status st = scratch_address(&base);
    if (st != VA_OK)
        return st;
    va::Control *ctl = reinterpret_cast<va::Control *>(base);
    int *inst_T = reinterpret_cast<int *>(base + off_T);
    int *inst_last = reinterpret_cast<int *>(base + off_last);
    int *inst_status = reinterpret_cast<int *>(base + off_st);
    va::Pool pool;
    pool.rec = reinterpret_cast<double *>(base + off_pool);
    pool.chunk_prev = reinterpret_cast<int *>(base + off_prev);
    pool.n_chunks = (int)n_chunks;
    pool.chunk_len = kChunkLen;

    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return VA_CUDA_ERROR;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int block = 128;
    auto grid = [&](const void *fn) {
        int occ = 1;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, block, 0) != cudaSuccess || occ < 1)
            occ = 1;
        const size_t need = (B + block - 1) / block;
        const size_t g = (size_t)sms * occ;
        return (int)(g < need ? g : need);
    };

    // the work counters start at zero on every call; nothing else is read
    // before this call writes it
    if (cudaMemsetAsync(ctl, 0, sizeof(va::Control), s) != cudaSuccess)
        return VA_CUDA_ERROR;

    va::FwdParams fa{};
    fa.B = batch;
    fa.y0 = y0;
    fa.par = params;
    fa.t0 = t0;
    fa.t1 = t1;
    fa.atol = atol;
    fa.rtol = rtol;
    fa.dt0 = dt0;
    fa.max_steps = max_steps;
    fa.max_fail = max_rejects;
    fa.step_pow = 1; // the correctly rounded step factor, as va_default_options
    fa.yT = yT;
    fa.n_acc_out = n_acc;
    fa.n_rej_out = nullptr;
    fa.status_out = status;
    fa.inst_T = inst_T;
    fa.inst_last = inst_last;
    fa.inst_status = inst_status;
    fa.stride = 1; // every accepted step is checkpointed
    fa.pool = pool;
    fa.ctl = ctl;
    void *fargs[] = {&fa};
    if (cudaLaunchKernel(ffn, dim3(grid(ffn)), dim3(block), fargs, 0, s) != cudaSuccess)
        return VA_CUDA_ERROR;

    va::AdjParams ba{};
    ba.B = batch;
    ba.nout = 1;
    ba.par = params;
    ba.lambdaT = nullptr;
    ba.mu_direct = nullptr;
    ba.cost = cost;
    ba.dy0 = dy0;
    ba.dpar = dparams;
    ba.status_out = status;
    ba.order = nullptr;
    ba.inst_T = inst_T;
    ba.inst_last = inst_last;
    ba.inst_status = inst_status;
    ba.pool = pool;
    ba.ctl = ctl;
    void *bargs[] = {&ba};
    if (cudaLaunchKernel(bfn, dim3(grid(bfn)), dim3(block), bargs, 0, s) != cudaSuccess)
        return VA_CUDA_ERROR;
    return VA_OK;
}
