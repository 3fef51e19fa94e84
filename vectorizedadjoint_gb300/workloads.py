"""Seeded synthetic workloads (inputs only) for the five benchmark
configurations of the discrete adjoint.

All draws use numpy.random.Generator(PCG64(seed)) in the listed order, FP64,
t0 = 0 and dt0 = 1e-3 (the initial step of the reference examples,
examples/GeneralizedLotkaVolterra/main.cpp:165, examples/VanDerPol/main.cpp:71).
`batch` may be reduced for parity tests: the first k instances of a reduced
draw are NOT the first k of the full one, so tests always regenerate with the
size they use.

  vdp1    Van der Pol, 1 instance, mu~U[0.5,2], x0~U[-2,2]^2, T=10, DOPRI5, tol 1e-8
  dho     damped oscillator, B=65,536, omega~U[0.5,5], zeta~U[0,0.5], x0~U[-1,1]^2,
          T~U[5,50], Cash-Karp, tol 1e-8
  vdpb    Van der Pol, B=262,144, mu=10^U[-1,1], x0~U[-2,2]^2, T=20, DOPRI5, tol 1e-6
  glv10   GLV N=10, B=16,384, r~U[.5,1.5]^N, A diag -1 / off-diag N(0,0.1^2) row-major,
          x0~U[.1,1]^N, T=20, DOPRI5, tol 1e-7
  glv256  GLV N=256, one shared A (diag -1, off-diag N(0,(0.5/sqrt N)^2)), B=1,024 with
          r~U[.5,1.5]^N, x0~U[.1,1]^N, T=10, DOPRI5, tol 1e-7, 8 GB checkpoint budget
Costs: sum of squared terminal state (vdp1, dho, vdpb); sum of terminal state (glv*).
"""
import numpy as np

CONFIGS = {
    "vdp1": dict(model="vdp", n=2, npar=1, batch=1, tableau="dopri5", tol=1e-8, cost="sumsq", seed=1),
    "dho": dict(model="dho", n=2, npar=2, batch=65536, tableau="ck54", tol=1e-8, cost="sumsq", seed=2),
    "vdpb": dict(model="vdp", n=2, npar=1, batch=262144, tableau="dopri5", tol=1e-6, cost="sumsq", seed=3),
    "glv10": dict(model="glv", n=10, npar=110, batch=16384, tableau="dopri5", tol=1e-7, cost="sum", seed=4),
    "glv256": dict(model="glv_shared", n=256, npar=256, batch=1024, tableau="dopri5", tol=1e-7, cost="sum",
                   seed=5, budget=8 << 30),
}


def make(name, batch=None):
    """Returns dict(cfg, y0[B,n], params[B,npar], t0[B], t1[B], shared (glv256 A or None))."""
    cfg = dict(CONFIGS[name])
    B = batch or cfg["batch"]
    cfg["batch"] = B
    rng = np.random.Generator(np.random.PCG64(cfg["seed"]))
    shared = None
    if name == "vdp1" or name == "vdpb":
        if name == "vdp1":
            mu = rng.uniform(0.5, 2.0, B)
        else:
            mu = 10.0 ** rng.uniform(-1.0, 1.0, B)
        x0 = rng.uniform(-2.0, 2.0, (B, 2))
        params = mu[:, None]
        T = np.full(B, 10.0 if name == "vdp1" else 20.0)
    elif name == "dho":
        om = rng.uniform(0.5, 5.0, B)
        ze = rng.uniform(0.0, 0.5, B)
        x0 = rng.uniform(-1.0, 1.0, (B, 2))
        T = rng.uniform(5.0, 50.0, B)
        params = np.stack([om, ze], axis=1)
    elif name == "glv10":
        N = 10
        r = rng.uniform(0.5, 1.5, (B, N))
        A = rng.normal(0.0, 0.1, (B, N, N))
        A[:, np.arange(N), np.arange(N)] = -1.0
        x0 = rng.uniform(0.1, 1.0, (B, N))
        params = np.concatenate([r, A.reshape(B, N * N)], axis=1)
        T = np.full(B, 20.0)
    elif name == "glv256":
        N = 256
        A = rng.normal(0.0, 0.5 / np.sqrt(N), (N, N))
        A[np.arange(N), np.arange(N)] = -1.0
        r = rng.uniform(0.5, 1.5, (B, N))
        x0 = rng.uniform(0.1, 1.0, (B, N))
        params = r
        shared = A
        T = np.full(B, 10.0)
    else:
        raise KeyError(name)
    return dict(cfg=cfg, y0=np.ascontiguousarray(x0), params=np.ascontiguousarray(params),
                t0=np.zeros(B), t1=np.ascontiguousarray(T), shared=shared)


def make_shard(name, rank, world, batch=None):
    """Rank `rank`'s contiguous share of a job of `world` x batch instances:
    the job's workload is drawn once with the global batch (the same draws on
    every rank) and each rank keeps its own range, so ranks solve different
    instances and the shared matrix, where there is one, is common."""
    from .shard import shard_range
    per = batch or CONFIGS[name]["batch"]
    w = make(name, batch=per * world)
    lo, hi = shard_range(per * world, rank, world)
    out = dict(w)
    for k in ("y0", "params", "t0", "t1"):
        out[k] = np.ascontiguousarray(w[k][lo:hi])
    out["cfg"] = dict(w["cfg"], batch=hi - lo, global_batch=per * world, shard=(lo, hi))
    return out
