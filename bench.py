"""Benchmark: adjoint gradients/s on one GB300 (forward sweep + backward sweep
per instance), batched vs plain, at a stated error against FP64.

Default workload: the Van der Pol batch (262,144 instances, mu = 10^U[-1,1],
x0 ~ U[-2,2]^2, t in [0,20], DOPRI5, atol = rtol = 1e-6), the configuration
the batched-vs-plain target is quoted on; seeded synthetic inputs.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--config vdpb|dho|glv10|glv256|vdp1]
                  [--precision mixed_dw|mixed|fp64] [--impl ours|reference]

One JSON line on rank 0.  `value` = gradients/s of va_gradient with inputs
resident in HBM (CUDA events around each step, L2 flushed between steps);
`e2e` = the same through va_gradient_host (host buffers, copies inside the
timed region); `roofline` = the dominant sweep kernel's FLOP rate against
the peak of the pipe it runs on, measured in the same run (roofline_of);
`cpu_baseline` = the CPU port of the reference algorithm (oracle/) on the
host cores, on a bounded sample.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# Algorithmic FLOPs (FMA = 2) per attempted forward step and per accepted
# backward step: s_f C_f + 2N(nnz_a + nnz_b + nnz_e) + 6N + 30 and
# s_f C_f + 2N nnz_a + s_f C_v + 2N (nnz_a + nnz_b) + N s_f.
TAB_NNZ = {"dopri5": dict(s=6, a=15, b=5, e=6), "ck54": dict(s=6, a=15, b=4, e=5)}


def model_cost(model, n):
    if model in ("vdp", "vdp_petsc"):
        return 5, 13
    if model == "dho":
        return 6, 12
    if model in ("glv", "glv_shared"):
        return 2 * n * n + 2 * n, 4 * n * n + 4 * n
    return 2, 4


def flops(model, tableau, n, attempts, accepted):
    t = TAB_NNZ[tableau]
    cf, cv = model_cost(model, n)
    fwd = t["s"] * cf + 2 * n * (t["a"] + t["b"] + t["e"]) + 6 * n + 30
    adj = t["s"] * cf + 2 * n * t["a"] + t["s"] * cv + 2 * n * (t["a"] + t["b"]) + n * t["s"]
    return fwd * attempts, adj * accepted


# FP32 FLOPs the double-word sweeps execute per forward attempt and per
# backward step (FADD + FMUL + 2 FFMA, thread level), counted by ncu
# (smsp__sass_thread_inst_executed_op_f{add,mul,fma}_pred_on) on the
# double-word sweep kernels at the named workload's acceptance ratio, per
# instance, stage records on.
# Double-word arithmetic is FADD-heavy (2Sum chains), so its FLOP ceiling
# sits near half the FFMA peak.
DW_FP32_FLOPS = {
    ("vdp", "dopri5"): (1611.2, 1682.2),
    ("dho", "ck54"): (1414.5, 1566.0),
    ("glv", "dopri5"): (16898.1, 25416.7),
    # shared-matrix backward: the A^T v products only; dA is contracted
    # afterwards on the tensor pipe (a kernel of its own)
    ("glv_shared", "dopri5"): (6353397.4, 6316765.2),
}

# Models whose backward phase is more than one kernel: the shared-matrix
# backward sweep is followed by the dA contraction (ncu launch list, cluster
# sweeps: forward 46%, backward sweep 40%, contraction 13.5%), so the forward
# sweep is the single dominant kernel whatever the phase times say.
DOMINANT = {"glv_shared": "forward"}


class Clocks:
    """Samples SM clocks and clock-event (throttle) reasons DURING the timed
    region: read-only NVML queries (libnvidia-ml through ctypes) from a
    background thread every 2 ms, kept only between __enter__ and __exit__;
    nvidia-smi at 200 ms where NVML cannot be loaded.  Nothing is set."""

    NAMES = {0x8: "hw_slowdown", 0x40: "hw_thermal_slowdown", 0x20: "sw_thermal_slowdown", 0x4: "sw_power_cap"}
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.p = None
        self.samples = []  # (sm_mhz, max_mhz, reason bits)
        self.nvml = None

    def _nvml_open(self):
        import ctypes
        try:
            lib = ctypes.CDLL("libnvidia-ml.so.1")
        except OSError:
            return False
        if lib.nvmlInit_v2() != 0:
            return False
        h = ctypes.c_void_p()
        if lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(self.index), ctypes.byref(h)) != 0:
            return False
        reasons = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            getattr(lib, "nvmlDeviceGetCurrentClocksThrottleReasons", None)
        if reasons is None:
            return False
        self.nvml = (lib, h, reasons)
        return True

    def _nvml_sample(self):
        import ctypes
        lib, h, reasons = self.nvml
        clk, mx, bits = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_ulonglong()
        if (lib.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(clk)) == 0 and  # NVML_CLOCK_SM
                lib.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx)) == 0 and reasons(h, ctypes.byref(bits)) == 0):
            return clk.value, mx.value, bits.value
        return None

    def _poll(self):
        while not self.stop.is_set():
            v = self._nvml_sample()
            if v is not None:
                self.samples.append(v)
            time.sleep(0.002)

    def __enter__(self):
        import threading
        if self._nvml_open():
            self.stop = threading.Event()
            v = self._nvml_sample()  # the first sample before the timed work starts
            if v is not None:
                self.samples.append(v)
            self.thread = threading.Thread(target=self._poll, daemon=True)
            self.thread.start()
            return self
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.nvml:
            self.stop.set()
            self.thread.join(timeout=5)
            self.nvml[0].nvmlShutdown()
            return
        if self.p:
            time.sleep(0.3)
            self.p.terminate()
            try:
                out = self.p.communicate(timeout=5)[0]
            except subprocess.TimeoutExpired:
                self.p.kill()
                out = ""
            for l in out.splitlines():
                f = [x.strip() for x in l.split(",")]
                try:
                    bits = sum(bit for bit, v in zip((0x8, 0x40, 0x20, 0x4), f[4:8]) if v.lower() == "active")
                    self.samples.append((float(f[1]), float(f[2]), bits))
                except (ValueError, IndexError):
                    continue

    def summary(self):
        sm = [x[0] for x in self.samples]
        mx = self.samples[-1][1] if self.samples else None
        reasons = sorted({nm for x in self.samples for bit, nm in self.NAMES.items() if x[2] & bit})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(sm), "source": "nvml" if self.nvml else "nvidia-smi"}


def cpu_baseline(cfg_name, w, seconds=10.0, threads=None):
    """The oracle's multi-threaded batch gradient on a bounded sample, with the
    C library's pow in the step-size controller, as the reference calls it."""
    from oracle import oracle_py as O
    c = w["cfg"]
    threads = threads or os.cpu_count() or 1
    B = c["batch"]
    params = w["params"]
    if w["shared"] is not None:
        # per instance the reference's GLV layout: r, then the (common) A
        A = np.asarray(w["shared"]).ravel()
        pb = O.problem("glv", c["tableau"], c["n"], c["n"] + c["n"] ** 2, c["tol"], c["tol"], pow_mode=1)
        params = lambda k: np.concatenate([w["params"][:k], np.broadcast_to(A, (k, A.size))], axis=1)
    else:
        pb = O.problem(c["model"], c["tableau"], c["n"], c["npar"], c["tol"], c["tol"], pow_mode=1)
        params = (lambda k, P=params: P[:k])
    pilot = min(B, (64 if c["n"] <= 16 else 1) * threads)
    t0 = time.perf_counter()
    O.gradient_batch(pb, c["cost"], w["y0"][:pilot], params(pilot), w["t0"][:pilot], w["t1"][:pilot],
                     nthreads=threads)
    dt = time.perf_counter() - t0
    m = int(min(B, max(pilot, pilot * seconds / max(dt, 1e-6))))
    # a whole batch that takes far less than the sample time (one instance,
    # e.g.) is repeated, so that call overheads do not dominate the figure
    reps = 1 if m < B else int(max(1, min(1000, 0.25 * seconds / max(dt * m / pilot, 1e-6))))
    t0 = time.perf_counter()
    for _ in range(reps):
        O.gradient_batch(pb, c["cost"], w["y0"][:m], params(m), w["t0"][:m], w["t1"][:m], nthreads=threads)
    dt = time.perf_counter() - t0
    what = f"first {m} of {B} instances" if m < B else f"all {B} instances" + (f" x {reps} calls" if reps > 1 else "")
    used = min(threads, m)  # one thread per instance at most
    return {"value": reps * m / dt, "unit": "gradients/s", "cores": used, "kind": "port",
            "sample": f"{what} of {cfg_name}, {dt:.1f} s on {used} threads"}


def run_reference(args, rank, world):
    """--impl reference: the reference algorithm's CPU implementation on the host
    cores.  The reference's own build needs AADC (x86-only binary) and Boost; on
    this host the oracle port of the same algorithm stands in for it."""
    from vectorizedadjoint_gb300 import workloads as W
    if rank != 0:
        return
    w = W.make(args.config)
    c = w["cfg"]
    for _ in range(args.warmup):
        cpu_baseline(args.config, w, seconds=1.0)
    vals = []
    for _ in range(args.steps):
        vals.append(cpu_baseline(args.config, w, seconds=max(1.0, 60.0 / max(args.steps, 1))))
    v = float(np.mean([x["value"] for x in vals]))
    cb = dict(vals[-1])
    cb["value"] = v
    print(json.dumps({
        "impl": "reference", "metric": "adjoint gradients/s", "value": v, "unit": "gradients/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        # one step = one pass over the whole batch, at the bounded sample's rate
        "ms_per_step": 1e3 * c["batch"] / v,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded PCG64)",
        "config": {"workload": f"{args.config}: {c['model']} B={c['batch']} {c['tableau']} tol={c['tol']}",
                   "batch": c["batch"], "cost": c["cost"]},
        "cpu_baseline": cb, "e2e": {"value": v, "unit": "gradients/s", "h2d_bytes_per_step": 0,
                                    "d2h_bytes_per_step": 0}}), flush=True)


def max_over_ranks(ms, world, dist, torch, device="cpu"):
    """The job's step time: the slowest rank's (ranks run independent replicas)."""
    if world <= 1:
        return ms
    tt = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def replica_throughput(batch_per_rank, ms, world):
    """Whole-job gradients/s: every rank differentiates its own contiguous
    share of the instances (weak scaling: the share is fixed as ranks grow)."""
    return world * batch_per_rank / (ms * 1e-3)


def fp32_peak_tflops(torch):
    """FP32 (non-tensor) peak of this GPU measured as cuBLAS SGEMM throughput
    with TF32 off (best of 5)."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        return gemm_tflops(torch, torch.float32, 8192)
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


def fp64_peak_tflops(torch):
    """FP64 peak of this GPU measured as cuBLAS DGEMM throughput (best of 5)."""
    return gemm_tflops(torch, torch.float64, 4096)


def gemm_tflops(torch, dtype, n):
    a = torch.randn(n, n, dtype=dtype, device="cuda")
    b = torch.randn(n, n, dtype=dtype, device="cuda")
    for _ in range(2):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e9
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return 2 * n ** 3 / (best * 1e-3) / 1e12


# DRAM bytes (read + write) per launch of the dominant double-word kernel of
# each workload at its full size, one ncu capture each of the timed launch
# (dram__bytes_read.sum, dram__bytes_write.sum): the forwards write the stage
# records (128 B per accepted step for the two-state models, 24.6 KB for the
# shared-matrix GLV), the backwards read them back.
DW_TRAFFIC = {("vdpb", "forward"): 121.0e6 + 5557.4e6, ("vdpb", "backward"): 5655.6e6 + 20.8e6,
              ("dho", "forward"): 9.2e6 + 1586.3e6, ("glv10", "backward"): 745.5e6 + 4.3e6,
              ("vdp1", "forward"): 0.05e6, ("glv256", "forward"): 12.6e6 + 1179.1e6,
              # the tensor-core cluster sweeps of GLV-256 (1,024 instances: the
              # 960 of the 15 cluster tiles; the other 64 run in the tail sweep)
              ("glv256", "tc_forward"): 9.4e6 + 1105.0e6, ("glv256", "tc_backward"): 1161.9e6 + 550.5e6}


def measured_bf16_peak():
    """Dense bf16 TFLOP/s from MEASURED_PEAKS.json (the sustained figure: the
    kernels run inside a multi-millisecond step), else the recipe's fallback."""
    try:
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["bf16_tflops_sustained"]), "MEASURED_PEAKS.json bf16_tflops_sustained"
    except (OSError, KeyError, ValueError):
        return 1700.0, "fallback (no MEASURED_PEAKS.json): sustained bf16 ~1.7 PFLOP/s"


def pipe_rates():
    """This GPU's arithmetic pipe rates from the library's probes
    (va_probe_rate): FP64 FMA, FP32 FMA and FP64 tensor-core MMA, TFLOP/s;
    INT8 dp4a, tera-operations/s (8 per instruction and lane)."""
    import ctypes

    from vectorizedadjoint_gb300 import _lib
    L = _lib.load()
    out = {}
    for kind, name, iters in [(0, "fp64_fma", 4096), (1, "fp32_fma", 65536), (2, "fp64_mma_m8n8k4", 2048),
                              (3, "fp64_mma_m16n8k16", 512), (4, "int8_dp4a_tops", 65536)]:
        tf, ms = ctypes.c_double(), ctypes.c_double()
        st = L.va_probe_rate(kind, iters, ctypes.byref(tf), ctypes.byref(ms))
        out[name] = tf.value if st == 0 else None
    for n, ctas in ((16, 1), (16, 2), (32, 1), (32, 2), (64, 1), (64, 2), (128, 1), (128, 2), (256, 1)):
        tf, ms = ctypes.c_double(), ctypes.c_double()
        st = L.va_probe_mma_bf16(n, 1, ctas, 8192, ctypes.byref(tf), ctypes.byref(ms))
        out[f"bf16_tcgen05_m128n{n}k16_{ctas}cta"] = tf.value if st == 0 else None
    return out


def cluster_mma_flops(attempts_per_instance, forward, n_tiles):
    """bf16 tensor FLOPs the cluster sweeps of the shared-matrix GLV execute
    (csrc/va_bundle_tc.cuh): per tile of 64 instances, per product, 8 CTAs x
    108 MMAs of M 128, N 64, K 16.  Forward: f(y_0), then 6 products (5
    stages and f(y_new)) per attempt of the tile's longest instance; backward:
    6 per accepted step of the tile's longest instance.  The first n_tiles
    tiles (instances past them run in the double-word bundles beside)."""
    per_product = 8 * 108 * 2 * 128 * 64 * 16
    a = np.asarray(attempts_per_instance, dtype=np.int64)[:64 * n_tiles]
    tiles = [int(a[i:i + 64].max()) for i in range(0, len(a), 64)]
    return per_product * sum((1 + 6 * m) if forward else 6 * m for m in tiles)


def glv_shared_launches(launch, B):
    """Kernels per shared-matrix gradient: prepare A, forward, factor offsets,
    backward, dA contraction and partial sum; each tensor-core cluster sweep
    adds the digit planes of A and the packed r, and its tail sweep when the
    clusters leave instances over."""
    n = 6
    for blk, grid in (("fwd_block", "fwd_grid"), ("bwd_block", "bwd_grid")):
        if launch[blk] == 512:
            n += 2 + (launch[grid] // 8 * 64 < B)
    return n


def roofline_of(args, c, torch, fms, bms, fl_f, fl_b, attempts, accepted, launch=None, per_inst=None):
    """Roofline of the dominant sweep kernel.  fp64: algorithmic FP64 FLOPs
    against cuBLAS DGEMM.  mixed_dw: the FP32 FLOPs the double-word
    arithmetic executes (ncu-counted per attempt / per step, scaled by this
    run's attempts and steps) against cuBLAS SGEMM, or, for the shared-matrix
    cluster sweeps on the tensor cores, their executed bf16 MMA FLOPs against
    the measured bf16 peak; mixed: the algorithmic count, executed in FP32,
    against SGEMM.  Every mode also reports the FP64-equivalent rate
    (algorithmic FP64 FLOPs / time) against DGEMM."""
    fwd_dom = DOMINANT.get(c["model"], "forward" if fms >= bms else "backward") == "forward"
    kernel, ms = ("forward", fms) if fwd_dom else ("backward", bms)
    alg = fl_f if fwd_dom else fl_b
    peak64 = fp64_peak_tflops(torch)
    equiv = alg / (ms * 1e-3) / 1e12
    out = {"kernel": kernel, "unit": "TFLOP/s", "launch_ms": ms, "forward_ms": fms, "backward_ms": bms,
           "traffic": DW_TRAFFIC.get((args.config, kernel)) if args.precision == "mixed_dw" else None,
           "fp64_equivalent": {"achieved": equiv, "dgemm_peak": peak64, "ratio": equiv / peak64}}
    cluster = (launch or {}).get("fwd_block" if fwd_dom else "bwd_block") == 512 and c["model"] == "glv_shared"
    if args.precision == "mixed_dw" and cluster and per_inst is not None:
        n_tiles = launch["fwd_grid" if fwd_dom else "bwd_grid"] // 8
        fl = cluster_mma_flops(per_inst[0] if fwd_dom else per_inst[1], fwd_dom, n_tiles)
        peak, src = measured_bf16_peak()
        out.update(kernel=kernel + " (tensor-core cluster sweep)", bound="tensor", achieved=fl / (ms * 1e-3) / 1e12,
                   peak=peak, peak_source=src, flops_per_launch=fl,
                   traffic=DW_TRAFFIC.get((args.config, "tc_" + kernel)),
                   flop_count="bf16 MMA FLOPs executed (8 CTAs x 108 MMAs of 128x64x16 per product and tile; "
                              "per tile the longest instance's attempts; instances past the cluster tiles run "
                              "beside them in double-word bundles and are not counted)")
        out["frac"] = out["achieved"] / out["peak"]
        return out
    dgemm = "cuBLAS DGEMM 4096^3 measured in this run (FP64 is absent from the measured-peaks file)"
    sgemm = "cuBLAS SGEMM 8192^3, TF32 off, measured in this run (FP32 is absent from the measured-peaks file)"
    per = DW_FP32_FLOPS.get((c["model"], c["tableau"]), (None, None))[0 if fwd_dom else 1]
    if args.precision == "fp64":
        out.update(bound="fp64", achieved=equiv, peak=peak64, peak_source=dgemm, flops_per_launch=alg,
                   flop_count="algorithmic FP64 FLOPs (FMA = 2) of stages, VJPs and error norm")
    elif args.precision == "mixed" or per is not None:
        fl = alg if args.precision == "mixed" else per * (attempts if fwd_dom else accepted)
        peak32 = fp32_peak_tflops(torch)
        out.update(bound="fp32", achieved=fl / (ms * 1e-3) / 1e12, peak=peak32, peak_source=sgemm,
                   flops_per_launch=fl,
                   flop_count=("algorithmic FLOPs executed in FP32" if args.precision == "mixed" else
                               f"{per} FP32 FLOPs per {'attempt' if fwd_dom else 'step'} of the double-word "
                               "arithmetic (ncu instruction counts, FFMA = 2)"))
    else:
        out.update(bound="fp64-equivalent", achieved=equiv, peak=peak64, peak_source=dgemm,
                   flops_per_launch=alg,
                   flop_count="algorithmic FP64 FLOPs done in double-word arithmetic (its FP32 count is "
                              "not measured for this kernel)")
    out["frac"] = out["achieved"] / out["peak"]
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--config", default="vdpb")
    ap.add_argument("--precision", default="mixed_dw", choices=["mixed_dw", "mixed", "fp64"])
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--quick", action="store_true",
                    help="only the timed steps of one mode (no autotune sweep, other modes, plain, e2e or CPU "
                         "legs): the small case used for ncu captures")
    ap.add_argument("--tune", action="store_true",
                    help="with --quick: pick the launch shape by the autotune sweep first, as the full run does")
    ap.add_argument("--batch", type=int, default=0, help="override the workload's batch size")
    ap.add_argument("--budget-gb", type=float, default=0.0, help="checkpoint pool budget (GiB)")
    ap.add_argument("--step-pow", type=int, default=1, choices=[0, 1],
                    help="FP64 controller: 1 correctly rounded step factor (default), 0 Newton root")
    ap.add_argument("--probe", action="store_true",
                    help="print this GPU's FP64 / FP32 / FP64-MMA pipe rates as one JSON line and exit")
    args = ap.parse_args()

    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # one process per GPU: relaunch this command under torch.distributed.run
        import socket
        with socket.socket() as sk:
            sk.bind(("127.0.0.1", 0))
            port = sk.getsockname()[1]
        cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
               "--master-addr", "127.0.0.1", f"--master-port={port}", os.path.abspath(__file__)] + sys.argv[1:]
        return subprocess.call(cmd)
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    if world != args.gpus and rank == 0:
        sys.stderr.write(f"bench.py: --gpus {args.gpus} but WORLD_SIZE={world}; using {world} ranks\n")
    if args.impl == "reference":
        return run_reference(args, rank, world)

    import torch
    import torch.distributed as dist

    torch.cuda.set_device(local)
    if args.probe:
        if rank == 0:
            print(json.dumps({"pipe_rates_tflops": pipe_rates(), "gpu": torch.cuda.get_device_name(local)}))
        return
    if world > 1:
        dist.init_process_group("nccl")
    # a non-default stream, so va_gradient captures both sweeps in one CUDA graph
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        _bench(args, rank, world, local, torch, dist)
    if world > 1:
        dist.destroy_process_group()


def _bench(args, rank, world, local, torch, dist):
    from vectorizedadjoint_gb300 import Solver
    from vectorizedadjoint_gb300 import workloads as W

    # rank r solves its contiguous share of a job of world x batch instances
    w = W.make_shard(args.config, rank, world, batch=args.batch or None) if world > 1 else \
        W.make(args.config, batch=args.batch or None)
    c = w["cfg"]
    B = c["batch"]
    if args.budget_gb > 0:
        c["budget"] = int(args.budget_gb * (1 << 30))
    dev = lambda a: torch.tensor(a, dtype=torch.float64, device="cuda")
    y0, par, t0, t1 = dev(w["y0"]), dev(w["params"]), dev(w["t0"]), dev(w["t1"])
    shared = dev(w["shared"]) if w["shared"] is not None else None

    def make_solver(batch, precision, budget=c.get("budget", 0), step_pow=args.step_pow):
        sv = Solver(c["model"], c["n"], c["npar"], batch, tableau=c["tableau"], precision=precision,
                    atol=c["tol"], rtol=c["tol"], ckpt_budget_bytes=budget, step_pow=step_pow)
        if shared is not None:
            sv.set_shared(shared, torch.empty_like(shared))
        return sv

    def exchange_dA(sv):
        """The shared matrix's gradient is the sum over every rank's instances:
        gathered and added in rank order (deterministic for a world size)."""
        if world > 1 and shared is not None:
            dA = sv._shared[1]
            bufs = [torch.empty_like(dA) for _ in range(world)]
            dist.all_gather(bufs, dA)
            acc = bufs[0].clone()
            for b in bufs[1:]:
                acc += b
            dA.copy_(acc)

    s = make_solver(B, args.precision)
    if not args.quick or args.tune:
        s.autotune(c["cost"], y0, par, t0, t1)
    out = s.gradient(c["cost"], y0, par, t0, t1)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # > 129 MB L2
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        s.gradient(c["cost"], y0, par, t0, t1, out=out)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    times = []
    with Clocks(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            # the NVTX range lets a profiler select the timed launches
            # (ncu --nvtx --nvtx-include "timed_step/")
            torch.cuda.nvtx.range_push("timed_step")
            e0.record(stream)
            s.gradient(c["cost"], y0, par, t0, t1, out=out)
            exchange_dA(s)
            e1.record(stream)
            torch.cuda.nvtx.range_pop()
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    ms = max_over_ranks(float(np.mean(times)), world, dist, torch, device="cuda")
    status = out["status"].cpu().numpy()
    n_acc = out["n_acc"].cpu().numpy().astype(np.int64)
    value = replica_throughput(B, ms, world)
    if args.quick:
        if rank == 0:
            print(json.dumps({"metric": "adjoint gradients/s", "value": value, "unit": "gradients/s",
                              "ms_per_step": ms, "quick": True, "precision": args.precision,
                              "step_pow": args.step_pow,
                              "config": {"workload": args.config, "batch": B, "launch": s.launch()},
                              "status_ok": int((status == 0).sum()), "clocks": clk.summary()}), flush=True)
        s.close()
        return

    # per-kernel timing (forward / backward launched separately) for the roofline
    lam = None
    fw_ms, bw_ms = [], []
    for _ in range(3):
        flush.zero_()
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(stream)
        f = s.forward(y0, par, t0, t1)
        e1.record(stream)
        if lam is None:
            torch.cuda.synchronize()
            if c["cost"] == "sumsq":
                lam = (2.0 * f["yT"]).reshape(B, 1, c["n"]).contiguous()
            else:
                lam = torch.ones(B, 1, c["n"], dtype=torch.float64, device="cuda")
            e1.record(stream)
        bwo = s.backward(par, lam)
        e2.record(stream)
        e2.synchronize()
        fw_ms.append(e0.elapsed_time(e1))
        bw_ms.append(e1.elapsed_time(e2))
    n_rej = f["n_rej"].cpu().numpy().astype(np.int64)
    attempts, accepted = int((n_acc + n_rej).sum()), int(n_acc.sum())
    fl_f, fl_b = flops(c["model"], c["tableau"], c["n"], attempts, accepted)
    fms, bms = float(np.median(fw_ms)), float(np.median(bw_ms))
    roofline = roofline_of(args, c, torch, fms, bms, fl_f, fl_b, attempts, accepted, launch=s.launch(),
                           per_inst=(n_acc + n_rej, n_acc))

    # the other precision modes on the same batch: throughput and gradient error vs FP64
    def run_mode(precision, step_pow=args.step_pow):
        sm = make_solver(B, precision, step_pow=step_pow)
        sm.autotune(c["cost"], y0, par, t0, t1)
        o = sm.gradient(c["cost"], y0, par, t0, t1)
        tt = []
        for _ in range(3):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            sm.gradient(c["cost"], y0, par, t0, t1, out=o)
            e1.record(stream)
            e1.synchronize()
            tt.append(e0.elapsed_time(e1))
        sm.close()
        return B / (float(np.median(tt)) * 1e-3), o

    def grad_err(o, o64):
        """Per instance max|g - g64| / max(max|g64|, 1e-8 max|y0|): the floor keeps
        damped instances whose gradient decays to ~1e-100 on a meaningful scale."""
        g = torch.cat([o["dy0"], o["dp"]], 1)
        g64 = torch.cat([o64["dy0"], o64["dp"]], 1)
        scale = torch.maximum(g64.abs().amax(1), 1e-8 * y0.abs().amax(1)).clamp_min(1e-300)
        rel = ((g - g64).abs().amax(1) / scale).cpu().numpy()
        ok = (o["status"].cpu().numpy() == 0) & (o64["status"].cpu().numpy() == 0)
        same = float((o["n_acc"] == o64["n_acc"]).float().mean().item())
        return {"median": float(np.median(rel[ok])), "p99": float(np.quantile(rel[ok], 0.99)),
                "max": float(rel[ok].max()), "same_step_count": same,
                "vs": "FP64 path of this library (oracle-checked in tests)"}

    modes = {}
    if args.precision == "fp64":
        fp64_value, o64 = value, out
    else:
        fp64_value, o64 = run_mode("fp64")
    modes["fp64"] = {"gradients_per_s": fp64_value}
    modes[args.precision] = {"gradients_per_s": value, "grad_err_vs_fp64": grad_err(out, o64)}
    for other in ("mixed_dw", "mixed"):
        if other not in modes:
            v, o = run_mode(other)
            modes[other] = {"gradients_per_s": v, "grad_err_vs_fp64": grad_err(o, o64)}
    # FP64 with the other step-factor power (Newton root <-> correctly rounded)
    v, o = run_mode("fp64", step_pow=1 - args.step_pow)
    modes["fp64_step_pow%d" % (1 - args.step_pow)] = {"gradients_per_s": v, "grad_err_vs_fp64": grad_err(o, o64)}
    err = modes[args.precision].get("grad_err_vs_fp64")

    # plain drop-in: the FP64 path called once per instance through the host entry point
    M = 64 if c["n"] <= 16 else 8
    s1 = make_solver(1, "fp64", budget=0)
    s1.gradient_host(c["cost"], w["y0"][:1], w["params"][:1], w["t0"][:1], w["t1"][:1])
    tp = time.perf_counter()
    for b in range(M):
        s1.gradient_host(c["cost"], w["y0"][b:b + 1], w["params"][b:b + 1], w["t0"][b:b + 1], w["t1"][b:b + 1])
    plain = M / (time.perf_counter() - tp)
    s1.close()

    # e2e: host buffers (pinned) through va_gradient_host, copies inside the timed region
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
    hy0, hpar, ht0, ht1 = pin(w["y0"]), pin(w["params"]), pin(w["t0"]), pin(w["t1"])
    hout = dict(yT=torch.empty(B, c["n"], dtype=torch.float64).pin_memory(),
                dy0=torch.empty(B, c["n"], dtype=torch.float64).pin_memory(),
                dp=torch.empty(B, c["npar"], dtype=torch.float64).pin_memory(),
                n_acc=torch.empty(B, dtype=torch.int32).pin_memory(),
                status=torch.empty(B, dtype=torch.int32).pin_memory())
    s.gradient_host(c["cost"], hy0, hpar, ht0, ht1, out=hout)
    te = []
    for _ in range(max(3, args.steps // 2)):
        flush.zero_()
        torch.cuda.synchronize()
        tq = time.perf_counter()
        s.gradient_host(c["cost"], hy0, hpar, ht0, ht1, out=hout)
        te.append(time.perf_counter() - tq)
    e2e = B / float(np.mean(te))
    h2d = B * (c["n"] + c["npar"] + 2) * 8
    d2h = B * (2 * c["n"] + c["npar"]) * 8 + 2 * B * 4

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(args.config, w)

    if rank == 0:
        line = {
            "metric": "adjoint gradients/s", "value": value, "unit": "gradients/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": {"mixed_dw": "f32x2 (double-word) stages / f64 controller+accumulators",
                      "mixed": "f32 stages / f64 controller+accumulators", "fp64": "f64"}[args.precision],
            "data": "synthetic (seeded PCG64)",
            "config": {"workload": f"{args.config}: {c['model']} B={B} {c['tableau']} tol={c['tol']}",
                       "batch": B, "global_batch": B * world,
                       "parallelism": f"{world} rank(s), contiguous instance shards" + (
                           ", shared dA summed across ranks in rank order" if shared is not None and world > 1
                           else ""),
                       "precision": args.precision, "cost": c["cost"],
                       "l2": "flushed between timed steps (256 MB write)",
                       "launch": s.launch(), "status_ok": int((status == 0).sum())},
            "e2e": {"value": e2e, "unit": "gradients/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            # per gradient: forward order (3) + forward + backward order (3) +
            # backward; shared-matrix bundles: prepare + forward + factor offsets +
            # backward + dA contraction + partial sum, and each tensor-core
            # cluster sweep its digit planes of A and packed r
            "gpu_launches": (glv_shared_launches(s.launch(), B) if c["model"] == "glv_shared" else 8) * args.steps,
            "roofline": roofline,
            "fp64_batched": fp64_value,
            "modes": modes,
            "plain_fp64_per_instance": plain,
            "batched_vs_plain": value / plain,
            "grad_err_vs_fp64": err,
            "steps_per_instance": {"mean_accepted": float(n_acc.mean()), "max_accepted": int(n_acc.max()),
                                   "mean_rejected": float(n_rej.mean())},
            "clocks": clk.summary(),
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    s.close()


if __name__ == "__main__":
    sys.exit(main() or 0)
