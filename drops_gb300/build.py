"""Builds libtracefem.so (the CUDA path) for sm_103a with nvcc.

Each translation unit is compiled in parallel, then linked into
drops_gb300/_lib/libtracefem.so.  mesh_levelset.cu is compiled with
-fmad=false so that vertex coordinates and level-set values round exactly like
the reference's host arithmetic; refine.cu's host code (the distance tests of
the refinement marks) with -ffp-contract=off for the same reason.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libtracefem.so")
UNITS = ["common.cu", "mesh_levelset.cu", "dofs.cu", "assemble.cu", "krylov.cu", "krylov_res.cu", "ch.cu", "capi.cu", "noalloc.cu", "batch.cu", "mlp.cu", "learned.cu", "gmres2.cu", "tune.cu", "quaqua.cu", "order.cu", "refine.cu", "refine_par.cu"]
NO_FMA = {"mesh_levelset.cu", "learned.cu", "refine.cu", "refine_par.cu"}
# host arithmetic that must round like the reference's (no fused multiply-add)
HOST_NO_CONTRACT = {"refine.cu", "refine_par.cu"}
# kernel bodies written as __host__ __device__ lambdas
EXTENDED_LAMBDA = {"refine_par.cu"}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags(unit, extra=()):
    f = [nvcc(), "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "--expt-relaxed-constexpr", "-I", os.path.join(HERE, "..", "include")]
    if unit in NO_FMA:
        f.append("-fmad=false")
    if unit in HOST_NO_CONTRACT:
        f += ["-Xcompiler", "-ffp-contract=off"]
    if unit in EXTENDED_LAMBDA:
        f.append("--extended-lambda")
    return f + list(extra)


def _stale(obj, deps):
    return not os.path.exists(obj) or any(os.path.getmtime(d) > os.path.getmtime(obj) for d in deps)


def build(force=False, verbose=False, extra=()):
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(SRC, h) for h in sorted(os.listdir(SRC)) if h.endswith(".cuh")]
    headers.append(os.path.join(HERE, "..", "include", "tracefem.h"))
    jobs = []
    for u in UNITS:
        src = os.path.join(SRC, u)
        obj = os.path.join(OUT, u.replace(".cu", ".o"))
        if force or _stale(obj, [src, *headers]):
            jobs.append(_flags(u, extra) + ["-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        results = list(ex.map(lambda cmd: subprocess.run(cmd, capture_output=True, text=True), jobs))
    for cmd, r in zip(jobs, results):
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {cmd[-3]}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
    objs = [os.path.join(OUT, u.replace(".cu", ".o")) for u in UNITS]
    if force or jobs or not os.path.exists(LIB):
        r = subprocess.run([nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
