"""Builds libva_gb300.so in-tree: every CUDA translation unit is compiled for
sm_103a (nvcc -gencode arch=compute_103a,code=sm_103a), in parallel, then
linked into one shared library that exports the C ABI of include/va.h."""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libva_gb300.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
NVCC = os.environ.get("NVCC", "nvcc")
FLAGS = ["-O3", "-lineinfo", "-std=c++17", ARCH, "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
         "--expt-relaxed-constexpr", "-I", os.path.join(HERE, "..", "include")]


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps.append(os.path.join(HERE, "..", "include", "va.h"))
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    procs = []
    objs = []
    for src in sources():
        obj = os.path.join(OUT_DIR, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if _stale(obj, src):
            # FP64 sweeps: no FMA contraction, so they round like the oracle
            extra = ["-fmad=false"] if src.endswith("_fp64.cu") else []
            cmd = [NVCC, *FLAGS, *extra, "-c", src, "-o", obj]
            if verbose:
                print(" ".join(cmd))
            procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for src, p in procs:
        out = p.communicate()[0].decode()
        if p.returncode != 0:
            failed.append((src, out))
        elif verbose and out.strip():
            print(out)
    if failed:
        for src, out in failed:
            sys.stderr.write(f"nvcc failed on {src}:\n{out}\n")
        raise RuntimeError("CUDA build failed")
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [NVCC, ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
