"""Benchmark of the TraceFEM path (DROPS) on GB300.

Workload (one "step"): the P2 surface-Poisson problem on the sphere |x| = 1 in
[-5/3, 5/3]^3 split into 96^3 Kuhn cubes (5,308,416 tets), P2 level set by
nodal interpolation, f = 13 xyz at ext(x):
    IdxDescCL::DistributeDOFs (P2IF) -> setupFESystem {M, A, C_n, F}
    -> LinComb M + A + h C_n -> Jacobi-PCG to relative residual 1e-10
(FP32 PCG sweeps inside FP64 iterative refinement).  The level set is the
input; everything downstream of it is recomputed every step.

value: cut tets per second through the whole step, inputs resident in HBM.
e2e:   the same through the C ABI from pinned host buffers: level-set upload
       (H2D), the step, solution download (D2H) inside the timed region.
L2 is flushed (2x L2 bytes written) before every timed step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload poisson|batch]

--workload batch: 256 independent P1 ellipsoid problems of uneven size (n^3
cubes, n ~ U{16..64}) through the same calls, solved by one persistent
batched PCG launch (CUDA graph, autotuned lanes per row).

--impl reference times the reference algorithm on the host cores: the C
restatement in oracle/ (the DROPS sources do not exist on the GPU host), same
workload, FP64 Jacobi-PCG as in the reference, all host threads.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_CUBES = 96
HALF = 5.0 / 3.0
SPHERE = [0.0, 0.0, 0.0, 1.0]
RHS = [0.0, 0.0, 0.0, 1.0, 13.0]
TOL = 1e-10
METRIC = "cut tets/s through DistributeDOFs + setupFESystem + Jacobi-PCG to rel. residual 1e-10 (P2 TraceFEM)"
CONFIG = {
    "workload": "surface Poisson, P2 TraceFEM, sphere r=1 in [-5/3,5/3]^3, 96^3 Kuhn cubes (5,308,416 tets), "
                "P2 level set, f=13xyz(ext x), A=M+A_LB+h*C_n, Jacobi-PCG rel 1e-10, FP32 inner / FP64 refinement",
    "mesh": "96^3 x 6 tets", "fe": "P2IF", "solver": "PCG+Jacobi, mixed FP32/FP64 IR", "tol": TOL,
    "l2": "flushed before every timed step (2x L2 size written)", "parallelism": "replicas",
}


# ---------------------------------------------------------------------------
def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=ws)
        return rank, ws, dist
    return 0, 1, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def all_max(dist, v):
    if dist is None:
        return v
    import torch

    t = torch.tensor([float(v)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def all_sum(dist, v):
    if dist is None:
        return v
    import torch

    t = torch.tensor([float(v)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


class Clocks:
    """nvidia-smi samples (200 ms) while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.file, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.3)
            self.proc.terminate()
            try:
                self.proc.wait(5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        self.file.flush()
        rows = []
        with open(self.file.name) as f:
            for line in f:
                p = [x.strip() for x in line.split(",")]
                if len(p) >= 9:
                    rows.append(p)
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ---------------------------------------------------------------------------
def pcg_bytes(m, nnz, iters, fp32):
    """Algorithmic bytes of the persistent PCG per iteration: matrix values and
    column indices once, row pointers once, and per row 12 vector words: the
    FP64 kernel reads z, p, x, r, q, diag and writes p, q, x, r, z (+1 for the
    gathered p); the single-barrier FP32 kernel reads and writes the 4-word
    state {r, w, s, 1/d}, p and the correction dx."""
    vb = 4 if fp32 else 8
    return iters * ((vb + 4) * nnz + 4 * (m + 1) + 12 * vb * m)


def spmv_cold(ctx, tf, m, nnz, kernel=None):
    """Standalone SpMV (y_Ax) on the system matrix, L2 flushed before each of 20 launches; the library
    queues (flush, event, kernel, event) back to back, so the events bracket the kernel alone.  Beside it, the
    streaming floor: a plain coalesced read of the same byte count, timed the same way.  kernel: the
    tf_spmv_options kernel (FP64 FMAs by default; the pair kernel's time includes its split pass of x)."""
    ctx.spmv_options(tf.SPMV_KERNEL_FP64 if kernel is None else kernel)
    t = float(np.median(ctx.spmv_timed(tf.MAT_SYS, tf.VEC_X, tf.VEC_T0, reps=20, cold=1)))
    b = 12 * nnz + 4 * (m + 1) + 16 * m
    floor = float(np.median(ctx.stream_read_timed(b, reps=20, cold=1)))
    # the same with an L2 left clean (flushed by reading), so DRAM serves only this kernel's traffic
    tc = float(np.median(ctx.spmv_timed(tf.MAT_SYS, tf.VEC_X, tf.VEC_T0, reps=20, cold=2)))
    fc = float(np.median(ctx.stream_read_timed(b, reps=20, cold=2)))
    return {"ms": round(t, 4), "bytes": b, "achieved_gbs": round(b / (t / 1e3) / 1e9, 1),
            "stream_read_same_bytes_ms": round(floor, 4), "frac_of_stream_read": round(floor / t, 4),
            "clean_l2": {"ms": round(tc, 4), "achieved_gbs": round(b / (tc / 1e3) / 1e9, 1),
                         "stream_read_same_bytes_ms": round(fc, 4), "frac_of_stream_read": round(fc / tc, 4)},
            "bytes_model": "12*nnz + 4*(m+1) + 16*m (FP64 values + int32 columns, row pointers, x read, y written)",
            "timing": "median of 20 launches, CUDA events on the library stream; L2 flushed before each by writing "
                      "2x its size (dirty lines left, whose write-back shares DRAM with the reads); clean_l2: "
                      "flushed by reading 2x its size"}


def run_ours(args, rank, ws, dist):
    import drops_gb300 as tf

    N = args.size
    H = 2 * HALF / N

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    ctx = tf.TraceFEM(dev)
    ctx.brick_cube(N, HALF)
    ctx.levelset_analytic(tf.LS_SPHERE, SPHERE, p2=True)
    nv, ne, nt = ctx.mesh_info()
    lv_dev, le_dev = ctx.levelset_download()
    pin_v, pin_e = tf.PinnedArray(nv), tf.PinnedArray(ne)
    pin_v.array[:] = lv_dev
    pin_e.array[:] = le_dev

    forms = [tf.FORM_M, tf.FORM_A, tf.FORM_CN]
    state = {}

    def step(precision=tf.PREC_MIXED):
        na, m = ctx.distribute_dofs(tf.P2IF)
        nnz = ctx.setup_fe_system(forms, tf.RHS_SPHERE_XYZ, RHS)
        ctx.lincomb(forms, [1.0, 1.0, H])
        ctx.vec_fill(tf.VEC_X, m, 0.0)
        st, it, res = ctx.pcg_jacobi(tf.MAT_SYS, tf.VEC_RHS, tf.VEC_X, tol=TOL, precision=precision)
        if st != tf.OK or res > TOL:
            raise RuntimeError(f"solve failed: status {st}, residual {res}")
        state.update(na=na, m=m, nnz=nnz, it=it, res=res)
        return na

    for _ in range(max(args.warmup, 3)):
        step()
    barrier(dist)

    # ---- device-resident timed region --------------------------------------
    ctx.timing(True)
    ctx.timing_reset()
    launches0 = ctx.launch_count()
    step_ms, cut = [], 0
    with Clocks(dev) as clk:
        for _ in range(args.steps):
            ctx.flush_l2()
            barrier(dist)
            ctx.marker(0)
            cut += step()
            ctx.marker(1)
            step_ms.append(ctx.elapsed_ms(0, 1))
    launches = ctx.launch_count() - launches0  # L2 flushes are memsets, not counted
    ktimes = {name: ctx.timing_get(k) for k, name in enumerate(tf.KERNEL_NAMES)}
    ctx.timing(False)
    clocks = clk.summary()
    total_ms = all_max(dist, sum(step_ms))
    total_cut = all_sum(dist, cut)
    value = total_cut / (total_ms / 1e3)

    # ---- end to end through the C ABI from pinned host buffers -------------
    pin_x = tf.PinnedArray(state["m"])
    e2e_ms, e2e_cut = [], 0
    for _ in range(args.steps):
        ctx.flush_l2()
        barrier(dist)
        ctx.marker(2)
        ctx.levelset_upload(pin_v.array, pin_e.array)
        e2e_cut += step()
        if pin_x.array.size != state["m"]:
            pin_x.free()
            pin_x = tf.PinnedArray(state["m"])
        ctx.vec_download(tf.VEC_X, out=pin_x.array)
        ctx.marker(3)
        e2e_ms.append(ctx.elapsed_ms(2, 3))
    e2e_total = all_max(dist, sum(e2e_ms))
    e2e_value = all_sum(dist, e2e_cut) / (e2e_total / 1e3)

    # ---- solve time on the same system: FP64 with the reference's recurrences (two grid barriers per
    # iteration), FP64 on the single-barrier resident kernel, mixed precision (the benchmark's solver) -----
    solve = {}
    for prec, k64, name in ((tf.PREC_FP64, tf.PCG_FP64_CLASSIC, "fp64"), (tf.PREC_FP64, tf.PCG_FP64_CG1, "fp64_cg1"),
                            (tf.PREC_MIXED, tf.PCG_FP64_CLASSIC, "mixed")):
        ctx.pcg_options(k64)
        ts = []
        for rep in range(3):
            ctx.vec_fill(tf.VEC_X, state["m"], 0.0)
            ctx.flush_l2()
            ctx.marker(4)
            st, it, res = ctx.pcg_jacobi(tf.MAT_SYS, tf.VEC_RHS, tf.VEC_X, tol=TOL, precision=prec)
            ctx.marker(5)
            ts.append(ctx.elapsed_ms(4, 5))
        solve[name] = {"ms": round(statistics.median(ts), 4), "iters": it, "resid": res,
                       "us_per_iter": round(1e3 * statistics.median(ts) / max(it, 1), 3)}
    ctx.pcg_options(tf.PCG_FP64_CLASSIC)
    solve["note"] = ("median of 3 solves from x = 0, L2 flushed before each; fp64: PCGSolverCL's recurrences "
                     "(two grid barriers per iteration); fp64_cg1: the single-barrier form of the mixed solver in "
                     "FP64; mixed: FP32 iterations in FP64 refinement (the benchmark's solver)")
    solve["mixed_vs_fp64"] = round(solve["fp64"]["ms"] / solve["mixed"]["ms"], 3)
    solve["mixed_vs_fp64_cg1"] = round(solve["fp64_cg1"]["ms"] / solve["mixed"]["ms"], 3)

    # ---- P2 forms: pair-arithmetic kernel (the default) against the FP64 kernel -------------
    asm = {}
    for kern, name in ((tf.ASM_KERNEL_PAIR, "pair"), (tf.ASM_KERNEL_FP64, "fp64")):
        ctx.assemble_options(kern)
        ts = []
        for rep in range(3):
            ctx.flush_l2()
            ctx.timing(True)
            ctx.timing_reset()
            ctx.setup_fe_system(forms, tf.RHS_SPHERE_XYZ, RHS)
            ts.append(ctx.timing_get(tf.K_ASSEMBLE)[0])
            ctx.timing(False)
        asm[name] = round(statistics.median(ts), 4)
    ctx.assemble_options(tf.ASM_KERNEL_PAIR)
    ctx.setup_fe_system(forms, tf.RHS_SPHERE_XYZ, RHS)
    ctx.lincomb(forms, [1.0, 1.0, H])
    asm["pair_vs_fp64"] = round(asm["fp64"] / asm["pair"], 3)
    asm["note"] = ("element-form kernel time (ms, median of 3, L2 flushed): M, A, C_n and the load vector; pair: "
                   "per-point work and element sums in FP32-pair arithmetic (tf_assemble_options default), fp64: "
                   "FP64 throughout")

    # ---- standalone FP64 SpMV (y_Ax) on the system matrix, cold L2 ---------
    spmv = spmv_cold(ctx, tf, state["m"], state["nnz"])
    # the same kernel on the P2 systems of twice and four times the resolution
    # (4x and 16x the bytes), where the launch and the ramp of HBM weigh less
    spmv_big, spmv_pair = {}, {}
    if args.size == N_CUBES and not args.no_large_spmv:
        for f in (2, 4):
            big = tf.TraceFEM(dev)
            nb = f * N_CUBES
            big.brick_cube(nb, HALF)
            big.levelset_analytic(tf.LS_SPHERE, SPHERE, p2=True)
            _, mb = big.distribute_dofs(tf.P2IF)
            nnzb = big.setup_fe_system(forms, tf.RHS_NONE, [])
            big.lincomb(forms, [1.0, 1.0, 2 * HALF / nb])
            big.vec_fill(tf.VEC_X, mb, 1.0)
            spmv_big[f] = spmv_cold(big, tf, mb, nnzb)
            spmv_big[f]["system"] = f"P2 sphere {nb}^3 cubes: m={mb}, nnz={nnzb}"
            spmv_pair[f] = spmv_cold(big, tf, mb, nnzb, tf.SPMV_KERNEL_PAIR)
            spmv_pair[f]["system"] = spmv_big[f]["system"]
            spmv_pair[f]["kernel"] = ("FP32-pair products (tf_spmv_options TF_SPMV_KERNEL_PAIR), split pass of x "
                                      "included; same algorithmic bytes")
            big.close()

    # ---- roofline of the dominant kernel ------------------------------------
    dom = max(ktimes, key=lambda k: ktimes[k][0])
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    for sp in (spmv, *spmv_big.values(), *spmv_pair.values()):
        if sp:
            sp["frac"] = round(sp["achieved_gbs"] / hbm_peak, 4)
            sp["clean_l2"]["frac"] = round(sp["clean_l2"]["achieved_gbs"] / hbm_peak, 4)
    ms_d, n_d = ktimes[dom]
    na, m, nnz = state["na"], state["m"], state["nnz"]
    if dom == "pcg":
        per_launch = pcg_bytes(m, nnz, state["it"], fp32=True)
        note = "FP32 inner iterations of one single-barrier PCG solve: (4+4)*nnz + 4*(m+1) + 48*m bytes per iteration"
    elif dom == "assemble":
        per_launch = na * (10 * 8 + 3 * 55 * 8 + 10 * 8)
        note = "per cut tet: 10 level-set values read, 3 packed 10x10 element matrices + load vector written"
    else:
        per_launch = 0
        note = "no byte model for this kernel"
    achieved = per_launch / ((ms_d / max(n_d, 1)) / 1e3) / 1e9 if ms_d > 0 else 0.0
    # DRAM bytes of one launch from an ncu capture of this workload (96^3):
    # dram__bytes_read.sum + dram__bytes_write.sum of k_pcg_cg1 / k_assemble<10>
    traffic = {"pcg": 69.94e6, "assemble": None}.get(dom) if N == N_CUBES else None
    roofline = {"kernel": dom, "bound": "hbm", "achieved": round(achieved, 1), "peak": hbm_peak, "unit": "GB/s",
                "frac": round(achieved / hbm_peak, 4), "traffic": traffic, "peak_source": peak_src,
                "bytes_model": note, "launch_ms": round(ms_d / max(n_d, 1), 4),
                "bytes_per_launch": per_launch,
                "traffic_note": "DRAM bytes per launch of the resident mixed PCG (ncu, "
                                "profiles/k_pcg_res_p2_sphere96.md): the algorithmic bytes of the iterations are "
                                "served from shared memory and L2 after a one-time load"}

    # ---- products of the step, for the parity check against the oracle (untimed) -----------
    products = {"xs": {}}
    for prec, name in ((tf.PREC_MIXED, "mixed"), (tf.PREC_FP64, "fp64")):
        ctx.vec_fill(tf.VEC_X, state["m"], 0.0)
        ctx.pcg_jacobi(tf.MAT_SYS, tf.VEC_RHS, tf.VEC_X, tol=TOL, precision=prec)
        products["xs"][name] = ctx.vec_download(tf.VEC_X)
    _, _, products["act"], products["l2g"] = ctx.dofs()
    products["mats"] = [ctx.matrix(f) for f in forms]
    products["rhs"] = ctx.vec_download(tf.VEC_RHS)

    out = {
        "metric": METRIC, "value": round(value, 1), "unit": "cut_tets/s", "n_gpus": ws, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": round(total_ms / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32", "data": "synthetic (analytic level set)",
        "config": CONFIG, "_products": products,
        "e2e": {"value": round(e2e_value, 1), "unit": "cut_tets/s", "h2d_bytes_per_step": 8 * (nv + ne),
                "d2h_bytes_per_step": 8 * state["m"], "ms_per_step": round(e2e_total / args.steps, 3)},
        "gpu_launches": int(launches),
        "roofline": roofline,
        "clocks": clocks,
        "problem": {"tets": nt, "cut_tets": na, "dofs": m, "nnz": nnz, "pcg_iters_inner": state["it"]},
        "solve_ms": solve,
        "assemble_ms": asm,
        "spmv_fp64_cold": spmv,
        "spmv_fp64_cold_2x": spmv_big.get(2),
        "spmv_fp64_cold_4x": spmv_big.get(4),
        "spmv_pair_cold_2x": spmv_pair.get(2),
        "spmv_pair_cold_4x": spmv_pair.get(4),
        "kernel_ms": {k: round(v[0] / args.steps, 4) for k, v in ktimes.items() if v[1]},
    }
    ctx.close()
    pin_v.free()
    pin_e.free()
    pin_x.free()
    return out


# ---------------------------------------------------------------------------
BATCH_COUNT, BATCH_NMIN, BATCH_NMAX = 256, 16, 64
BATCH_METRIC = "cut tets/s through DistributeDOFs + setupFESystem + batched Jacobi-PCG to rel. residual 1e-10 " \
               "(256 independent P1 ellipsoid problems, one persistent solve launch)"
BATCH_CONFIG = {
    "workload": "256 independent surface Poisson problems, P1 TraceFEM, ellipsoids (semi-axes U[0.6,1.4], "
                "Haar rotations, centres in the 0.1-ball, seed 1000+i) on [-5/3,5/3]^3 with n^3 Kuhn cubes, "
                "n ~ U{16..64}; A_i = M + A_LB + h_i C_n, f = 13xyz(x/|x|); batched Jacobi-PCG rel 1e-10, "
                "FP32 inner / FP64 reliable updates, CUDA-graph launch, autotuned lanes per row",
    "instances": BATCH_COUNT, "fe": "P1IF", "tol": TOL,
    "l2": "flushed before every timed step (2x L2 size written)", "parallelism": "replicas",
}


def batch_spec(args):
    from drops_gb300.workloads import ellipsoid_batch

    return ellipsoid_batch(args.batch_count, args.batch_nmin, args.batch_nmax, seed=1000)


def run_batch(args, rank, ws, dist):
    import drops_gb300 as tf

    W = batch_spec(args)
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    ctx = tf.TraceFEM(dev)
    ctx.brick_batch(W["n"], W["orig"], W["axes"])
    ctx.levelset_analytic_batch(tf.LS_ELLIPSOID, W["par"], p2=False)
    nv, ne, nt = ctx.mesh_info()
    # the level sets are P1 (LinearLSInit): the host holds the vertex values, the edge values are their means,
    # formed on the device by the upload (bit for bit as the analytic P1 evaluation)
    lv_dev, le_dev = ctx.levelset_download()
    pin_v = tf.PinnedArray(nv)
    pin_v.array[:] = lv_dev
    forms = [tf.FORM_M, tf.FORM_A, tf.FORM_CN]
    coef = np.stack([np.ones(len(W["h"])), np.ones(len(W["h"])), W["h"]], axis=1)
    state = {}

    def step(precision=tf.PREC_MIXED):
        na, m = ctx.distribute_dofs(tf.P1IF)
        nnz = ctx.setup_fe_system(forms, tf.RHS_SPHERE_XYZ, RHS)
        ctx.batch_lincomb(forms, coef)
        ctx.vec_fill(tf.VEC_X, m, 0.0)
        st, its, res = ctx.batch_pcg_jacobi(tf.MAT_SYS, tf.VEC_RHS, tf.VEC_X, tol=TOL, precision=precision)
        if st != tf.OK or np.any(res > TOL):
            raise RuntimeError(f"batched solve failed: status {st}, worst residual {res.max()}")
        state.update(na=na, m=m, nnz=nnz, its=its.copy())
        return na

    for _ in range(max(args.warmup, 3)):
        step()
    lanes, threads = ctx.batch_tune(tf.MAT_SYS, tf.VEC_RHS, tf.PREC_MIXED)
    barrier(dist)
    ctx.timing(True)
    ctx.timing_reset()
    launches0 = ctx.launch_count()
    step_ms, cut = [], 0
    with Clocks(dev) as clk:
        for _ in range(args.steps):
            ctx.flush_l2()
            barrier(dist)
            ctx.marker(0)
            cut += step()
            ctx.marker(1)
            step_ms.append(ctx.elapsed_ms(0, 1))
    launches = ctx.launch_count() - launches0
    ktimes = {name: ctx.timing_get(k) for k, name in enumerate(tf.KERNEL_NAMES)}
    ctx.timing(False)
    clocks = clk.summary()
    total_ms = all_max(dist, sum(step_ms))
    value = all_sum(dist, cut) / (total_ms / 1e3)

    pin_x = tf.PinnedArray(state["m"])
    e2e_ms, e2e_cut = [], 0
    for _ in range(args.steps):
        ctx.flush_l2()
        barrier(dist)
        ctx.marker(2)
        ctx.levelset_upload(pin_v.array)
        e2e_cut += step()
        ctx.vec_download(tf.VEC_X, out=pin_x.array)
        ctx.marker(3)
        e2e_ms.append(ctx.elapsed_ms(2, 3))
    e2e_total = all_max(dist, sum(e2e_ms))
    e2e_value = all_sum(dist, e2e_cut) / (e2e_total / 1e3)
    lv_chk, le_chk = ctx.levelset_download()
    assert np.array_equal(lv_chk, lv_dev) and np.array_equal(le_chk, le_dev), "P1 edge values differ after upload"

    # solve only: FP64 vs mixed, graph replay vs direct launch
    solve = {}
    for prec, name, graph in ((tf.PREC_FP64, "fp64", True), (tf.PREC_MIXED, "mixed", True),
                              (tf.PREC_MIXED, "mixed_no_graph", False)):
        ctx.batch_config(lanes, threads, use_graph=graph)
        ts = []
        for rep in range(3):
            ctx.vec_fill(tf.VEC_X, state["m"], 0.0)
            ctx.flush_l2()
            ctx.marker(4)
            st, its, res = ctx.batch_pcg_jacobi(tf.MAT_SYS, tf.VEC_RHS, tf.VEC_X, tol=TOL, precision=prec)
            ctx.marker(5)
            ts.append(ctx.elapsed_ms(4, 5))
        solve[name] = {"ms": round(min(ts[1:]), 4), "iters_max": int(its.max()), "iters_sum": int(its.sum()),
                       "resid_max": float(res.max())}
    tets, cutr, rows, nnzr = ctx.batch_info()
    sizes = {"tets": int(nt), "cut_tets": int(state["na"]), "dofs": int(state["m"]), "nnz": int(state["nnz"]),
             "rows_min": int(np.diff(rows).min()), "rows_max": int(np.diff(rows).max())}

    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    dom = max(ktimes, key=lambda k: ktimes[k][0])
    ms_d, n_d = ktimes[dom]
    na, m, nnz = state["na"], state["m"], state["nnz"]
    if dom == "assemble":
        per_launch = na * (4 * 8 + 3 * 10 * 8 + 4 * 8)
        note = "per cut tet: 4 level-set values read, 3 packed 4x4 element matrices + load vector written"
    elif dom == "batch":
        per_launch = sum(((4 + 4) * (nnzr[i + 1] - nnzr[i]) + 4 * (rows[i + 1] - rows[i] + 1) +
                          48 * (rows[i + 1] - rows[i])) * int(state["its"][i]) for i in range(len(state["its"])))
        note = "FP32 inner PCG iterations of every instance: (4+4)*nnz_i + 4*(m_i+1) + 48*m_i bytes per iteration"
    else:
        per_launch = 0
        note = "no byte model for this kernel"
    achieved = per_launch / ((ms_d / max(n_d, 1)) / 1e3) / 1e9 if ms_d > 0 else 0.0
    roofline = {"kernel": dom, "bound": "hbm", "achieved": round(achieved, 1), "peak": hbm_peak, "unit": "GB/s",
                "frac": round(achieved / hbm_peak, 4), "traffic": None,
                "peak_source": "measured" if "hbm_gbs" in peaks else "fallback", "bytes_model": note,
                "launch_ms": round(ms_d / max(n_d, 1), 4)}
    out = {
        "metric": BATCH_METRIC, "value": round(value, 1), "unit": "cut_tets/s", "n_gpus": ws, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": round(total_ms / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32", "data": "synthetic (analytic level sets)",
        "config": BATCH_CONFIG,
        "e2e": {"value": round(e2e_value, 1), "unit": "cut_tets/s", "h2d_bytes_per_step": 8 * nv,
                "d2h_bytes_per_step": 8 * state["m"], "ms_per_step": round(e2e_total / args.steps, 3),
                "note": "per step: the P1 level sets' vertex values up (edge values formed on the device), the "
                        "solutions down, from pinned host buffers"},
        "gpu_launches": int(launches), "roofline": roofline, "clocks": clocks, "problem": sizes,
        "autotuned": {"lanes_per_row": lanes, "threads": threads}, "solve_ms": solve,
        "kernel_ms": {k: round(v[0] / args.steps, 4) for k, v in ktimes.items() if v[1]},
    }
    ctx.close()
    pin_v.free()
    pin_x.free()
    return out


def batch_cpu_sample(args, threads, budget_s=20.0):
    """Oracle (C restatement of the reference) on the batch instances, in order, until budget_s has passed."""
    from oracle import pyoracle as O

    O.set_threads(threads)
    W = batch_spec(args)
    opts = O.make_opts(False, [O.FORM_M, O.FORM_A, O.FORM_CN], O.RHS_SPHERE_XYZ, RHS)
    tot_t, tot_cut, done = 0.0, 0, 0
    for i in range(len(W["h"])):
        n = tuple(int(k) for k in W["n"][i])
        mesh = O.brick(n, orig=W["orig"][i], e=W["axes"][i])
        lv, le = O.levelset(mesh, O.LS_ELLIPSOID, W["par"][i], False)
        t0 = time.perf_counter()
        st, na, m, dv, de, act = O.distribute_dofs(mesh, lv, le, False)
        st, rp, ci, vals, rhs = O.assemble(mesh, lv, le, act, dv, None, m, opts)
        S = vals[O.FORM_M] + vals[O.FORM_A] + W["h"][i] * vals[O.FORM_CN]
        O.pcg_jacobi(rp, ci, S, rhs, tol=TOL)
        tot_t += time.perf_counter() - t0
        tot_cut += na
        done += 1
        if tot_t > budget_s:
            break
    return tot_cut / tot_t, f"first {done} of {len(W['h'])} instances, in order ({tot_t:.1f} s, FP64 PCG)"


# ---------------------------------------------------------------------------
CH_N, CH_HALF, CH_DT, CH_EPS, CH_STEPS = 128, 1.6, 1e-3, 0.02, 200
CH_METRIC = "Cahn-Hilliard GMRES(50) solve time to rel. residual 1e-10 per time step, mixed precision + learned " \
            "warm start vs plain FP64 (P1 TraceFEM, torus)"
CH_CONFIG = {
    "workload": "surface Cahn-Hilliard on the torus R=1, r=0.4 in [-1.6,1.6]^3 with 128^3 Kuhn cubes (12,582,912 "
                "tets), P1, 2x2 block system, BDF1 dt=1e-3, mobility 1, eps=0.02, c0=0.5+U(+-0.01) (seed 2024), "
                "GMRES(50) with nodal block-Jacobi to rel 1e-10; learned warm start trained online on the first steps "
                "(train_steps: 100 for 300 steps or more, a third of the steps below)",
    "fe": "P1IF", "tol": TOL, "restart": 50, "parallelism": "replicas",
}


def run_ch(args, rank, ws, dist):
    import drops_gb300 as tf

    n = args.ch_n
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    ctx = tf.TraceFEM(dev)
    ctx.brick_cube(n, CH_HALF)
    ctx.levelset_analytic(tf.LS_TORUS, [1.0, 0.4, 2], False)
    na, nd = ctx.distribute_dofs(tf.P1IF)
    nnz = ctx.setup_fe_system([tf.FORM_M, tf.FORM_A, tf.FORM_CN])
    h = 2 * CH_HALF / n
    rng = np.random.default_rng(2024)
    x0 = np.concatenate([0.5 + rng.uniform(-0.01, 0.01, nd), np.zeros(nd)])
    pin0, pinx = tf.PinnedArray(2 * nd), tf.PinnedArray(2 * nd)
    pin0.array[:] = x0
    steps = args.ch_steps
    # learned: 0 previous state (the reference's warm start), 2 linear extrapolation, 3 minimal-residual
    # projection onto the last 6 states, 1 that projection with the MLP's correction in its basis
    variants = [("fp64_mgs_plain", tf.PREC_FP64, tf.ORTH_MGS, 0), ("fp64_cgs2_plain", tf.PREC_FP64, tf.ORTH_CGS2, 0),
                ("mixed_plain", tf.PREC_MIXED, tf.ORTH_MGS, 0), ("mixed_extrapolated", tf.PREC_MIXED, tf.ORTH_MGS, 2),
                ("mixed_projected", tf.PREC_MIXED, tf.ORTH_MGS, 3), ("mixed_learned", tf.PREC_MIXED, tf.ORTH_MGS, 1)]
    if args.ch_quick:
        variants = [variants[0], variants[5]]
    if args.ch_variants:
        keep = args.ch_variants.split(",")
        variants = [v for v in variants if v[0] in keep]
    train = min(100, max(args.ch_steps // 3, 4))
    runs = {}
    launches0 = ctx.launch_count()
    with Clocks(dev) as clk:
        for name, prec, orth, learned in variants:
            ctx.gmres_options(orth)
            ctx.mlp_init(1234)
            ctx.flush_l2()
            barrier(dist)
            ctx.marker(0)
            ctx.vec_upload(tf.VEC_X, pin0.array)
            st, its, res, used = ctx.ch_steps_learned(steps, CH_DT, 1.0, CH_EPS, 0.0, 1.0, h, restart=50, tol=TOL,
                                                      max_iter=100000, precision=prec, learned=learned,
                                                      train_steps=train, epochs=2, minibatch_tiles=16, lr=1e-3)
            ctx.vec_download(tf.VEC_X, out=pinx.array)
            ctx.marker(1)
            ms = all_max(dist, ctx.elapsed_ms(0, 1))
            if st != tf.OK or np.any(res > TOL):
                raise RuntimeError(f"{name}: status {st}, worst residual {res.max()}")
            runs[name] = {"ms": round(ms, 2), "ms_per_step": round(ms / steps, 3), "gmres_iters": int(its.sum()),
                          "iters_per_step": round(float(its.mean()), 1), "learned_steps": int(used.sum()),
                          "final_chi_mean": float(pinx.array[:nd].mean())}
    ctx.gmres_options(tf.ORTH_MGS)
    launches = ctx.launch_count() - launches0
    clocks = clk.summary()
    base = runs.get("fp64_mgs_plain", next(iter(runs.values())))
    best = runs.get("mixed_learned", next(iter(runs.values())))
    value = steps / (best["ms"] / 1e3)
    ratios = {f"{k}_vs_fp64_mgs_plain": round(base["ms"] / v["ms"], 3) for k, v in runs.items() if k != "fp64_mgs_plain"}
    if "fp64_cgs2_plain" in runs:
        ratios["mixed_learned_vs_fp64_cgs2_plain"] = round(runs["fp64_cgs2_plain"]["ms"] / best["ms"], 3)
    out = {
        "metric": CH_METRIC, "value": round(value, 2), "unit": "time_steps/s", "n_gpus": ws, "steps": steps,
        "warmup": 0, "ms_per_step": best["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64+f32+bf16", "data": "synthetic (analytic level set, seeded noise)",
        "config": dict(CH_CONFIG, steps=steps, n=n, train_steps=train),
        "speedup_vs_plain_fp64": round(base["ms"] / best["ms"], 3), "ratios": ratios,
        "e2e": {"value": round(value, 2), "unit": "time_steps/s", "h2d_bytes_per_step": round(16 * nd / steps, 1),
                "d2h_bytes_per_step": round(16 * nd / steps, 1),
                "note": "each run uploads the initial state and downloads the final state (pinned host buffers)"},
        "gpu_launches": int(launches), "clocks": clocks,
        "problem": {"cut_tets": na, "dofs_per_field": nd, "block_rows": 2 * nd, "nnz_per_block": nnz},
        "runs": runs,
    }
    ctx.close()
    pin0.free()
    pinx.free()
    return out


def ch_cpu_sample(args, threads, budget_s=20.0):
    """Oracle GMRES(50) with block Jacobi on the same CH steps (FP64, previous-state guess) until budget_s."""
    from oracle import pyoracle as O

    O.set_threads(threads)
    n = args.ch_n
    mesh = O.brick(n, a=CH_HALF)
    lv, le = O.levelset(mesh, O.LS_TORUS, [1.0, 0.4, 2], False)
    st, na, m, dv, de, act = O.distribute_dofs(mesh, lv, le, False)
    opts = O.make_opts(False, [O.FORM_M, O.FORM_A, O.FORM_CN])
    st, rp, ci, vals, rhs = O.assemble(mesh, lv, le, act, dv, None, m, opts)
    h = 2 * CH_HALF / n
    alpha = 1.0 / CH_DT
    brp, bci, bv = O.ch_block(rp, ci, vals[O.FORM_M], vals[O.FORM_A], vals[O.FORM_CN], alpha, 1.0, h,
                              CH_EPS * CH_EPS, 0.0)
    rng = np.random.default_rng(2024)
    x = np.concatenate([0.5 + rng.uniform(-0.01, 0.01, m), np.zeros(m)])
    t_tot, k = 0.0, 0
    while t_tot < budget_s and k < args.ch_steps:
        chi = x[:m]
        Mchi = O.spmv(rp, ci, vals[O.FORM_M], chi)
        fp = 2 * chi * (1 - chi) * (1 - 2 * chi)
        b = np.concatenate([alpha * Mchi, -O.spmv(rp, ci, vals[O.FORM_M], fp)])
        t0 = time.perf_counter()
        st, x, it, res = O.gmres_jacobi(brp, bci, bv, b, x0=x, restart=50, tol=TOL, max_iter=100000, block=True)
        t_tot += time.perf_counter() - t0
        k += 1
    return k / t_tot, f"first {k} of {args.ch_steps} time steps, GMRES(50) solves only ({t_tot:.1f} s)"


# ---------------------------------------------------------------------------
CPU_THREADING = ("OpenMP on all host threads where the reference threads or the work is per tet: the distance test of "
                 "every tet, the element matrices (accumulated serially in tet order), the pattern's row sorts and "
                 "PCG's SpMV; serial as in the reference: first-touch DOF numbering, PCG's dots and vector updates")


def cpu_workload(threads, N=N_CUBES):
    """The same step with the oracle (C restatement of the reference) on the host.  step(keep) returns
    (cut tets, seconds, PCG iterations, seconds per phase, the step's products if keep)."""
    from oracle import pyoracle as O

    O.set_threads(threads)
    H = 2 * HALF / N
    mesh = O.brick(N, a=HALF)
    lv, le = O.levelset(mesh, O.LS_SPHERE, SPHERE, True)
    opts = O.make_opts(True, [O.FORM_M, O.FORM_A, O.FORM_CN], O.RHS_SPHERE_XYZ, RHS)

    def step(keep=False):
        t0 = time.perf_counter()
        st, na, m, dv, de, act = O.distribute_dofs(mesh, lv, le, True)
        t1 = time.perf_counter()
        st, rp, ci, vals, rhs = O.assemble(mesh, lv, le, act, dv, de, m, opts)
        t2 = time.perf_counter()
        S = vals[O.FORM_M] + vals[O.FORM_A] + H * vals[O.FORM_CN]
        st, x, it, res = O.pcg_jacobi(rp, ci, S, rhs, tol=TOL)
        t3 = time.perf_counter()
        phases = {"dofs_s": round(t1 - t0, 3), "assemble_s": round(t2 - t1, 3), "solve_s": round(t3 - t2, 3)}
        prod = None
        if keep:
            from tests.helpers import loc2glo

            prod = {"act": np.nonzero(act)[0], "l2g": loc2glo(mesh, act, dv, de, True), "rowptr": rp, "colind": ci,
                    "vals": [vals[O.FORM_M], vals[O.FORM_A], vals[O.FORM_CN]], "rhs": rhs, "S": S, "x": x}
        return na, t3 - t0, it, phases, prod

    return step


def parity_report(gpu, ref):
    """The GPU step's products against the oracle's FP64 ones on the same inputs (outside any timed region):
    pattern and numbering bit for bit, matrix entries per entry against their row's scale (tolerance 1e-12,
    tests/helpers.py), the worst plain per-entry relative error (entries above 1e-12 max|b|), and each GPU
    solution's error against the oracle's FP64 PCG solution with the oracle's FP64 residual of it."""
    from oracle import pyoracle as O
    from tests.helpers import entry_rel_err, mat_close, sha

    same = (sha(gpu["act"].astype(np.int64)) == sha(ref["act"].astype(np.int64))
            and sha(gpu["l2g"].astype(np.int64)) == sha(ref["l2g"].astype(np.int64))
            and all(sha(rp.astype(np.int64)) == sha(ref["rowptr"].astype(np.int64))
                    and sha(ci.astype(np.int64)) == sha(ref["colind"].astype(np.int64)) for rp, ci, _ in gpu["mats"]))
    row_err = max(mat_close(v, rv, ref["rowptr"])[1] for (_, _, v), rv in zip(gpu["mats"], ref["vals"]))
    ent_err = max(entry_rel_err(v, rv) for (_, _, v), rv in zip(gpu["mats"], ref["vals"]))
    nb = np.linalg.norm(ref["rhs"])
    sol = {}
    for name, x in gpu["xs"].items():
        sol[name] = {"rel_err": float(np.linalg.norm(x - ref["x"]) / np.linalg.norm(ref["x"])),
                     "oracle_fp64_resid": float(np.linalg.norm(ref["rhs"] - O.spmv(ref["rowptr"], ref["colind"],
                                                                                    ref["S"], x)) / nb)}
    return {"against": "oracle (C restatement of the reference, FP64; pinned to the reference's outputs)",
            "pattern_numbering_sha_equal": bool(same), "max_row_scaled_entry_err": row_err,
            "max_rel_entry_err": ent_err, "rhs_err": mat_close(gpu["rhs"], ref["rhs"])[1],
            "entry_tolerance": "|a_ij - b_ij| <= 1e-12 * max(max_k |b_ik|, 1e-4 max|b|); rhs: 1e-12 max|b|", "solution": sol}


def run_reference(args, rank, ws, dist):
    if rank != 0:
        return None
    threads = os.cpu_count() or 1
    if args.workload == "batch":
        vals = [batch_cpu_sample(args, threads, budget_s=10.0) for _ in range(max(args.steps, 1))]
        value = statistics.median(v[0] for v in vals)
        return {
            "impl": "reference", "metric": BATCH_METRIC, "value": round(value, 1), "unit": "cut_tets/s",
            "n_gpus": ws, "steps": args.steps, "warmup": 0, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (analytic level sets)", "config": BATCH_CONFIG,
            "cpu_baseline": {"value": round(value, 1), "unit": "cut_tets/s", "cores": threads, "kind": "port",
                             "sample": vals[0][1] + "; C restatement of the reference in oracle/"},
            "e2e": {"value": round(value, 1), "unit": "cut_tets/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
    step = cpu_workload(threads, args.size)
    for _ in range(args.warmup):
        step()
    tot_t, tot_cut = 0.0, 0
    for _ in range(args.steps):
        na, dt, it, phases, _ = step()
        tot_t += dt
        tot_cut += na
    value = tot_cut / tot_t
    return {
        "impl": "reference", "metric": METRIC, "value": round(value, 1), "unit": "cut_tets/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * tot_t / args.steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (analytic level set)", "config": CONFIG,
        "cpu_baseline": {"value": round(value, 1), "unit": "cut_tets/s", "cores": threads, "kind": "port",
                         "sample": "the full workload per step (FP64 Jacobi-PCG as in the reference); "
                                   "C restatement of the reference in oracle/: " + CPU_THREADING,
                         "phases_last_step": phases},
        "e2e": {"value": round(value, 1), "unit": "cut_tets/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def run_quaqua(args):
    """Isoparametric P2 forms with the QuaQua mapper (tf_setup_quaqua_p2) on the headline mesh and surface:
    device time per setup (recovered gradient, per-point Newton base points, mapped quadrature, scatter),
    median of 3 after one warm-up; the discrete area (sum of M) against 4 pi as a size-independent check."""
    import drops_gb300 as tf

    ctx = tf.TraceFEM(0)
    ctx.brick_cube(N_CUBES, HALF)
    ctx.levelset_analytic(tf.LS_SPHERE, SPHERE, p2=True)
    na, m = ctx.distribute_dofs(tf.P2IF)
    newton = ctx.setup_quaqua_p2(13.0, 1e-13, 100)
    ts = []
    for _ in range(3):
        ctx.flush_l2()
        ctx.marker(6)
        newton = ctx.setup_quaqua_p2(13.0, 1e-13, 100)
        ctx.marker(7)
        ts.append(ctx.elapsed_ms(6, 7))
    rp, ci, mv = ctx.matrix(tf.FORM_M)
    ctx.close()
    ms = statistics.median(ts)
    return {"ms": round(ms, 4), "cut_tets": na, "dofs": m, "nnz": len(ci), "cut_tets_per_s": round(na / (ms / 1e3), 1),
            "newton_iters_max": newton, "area": float(mv.sum()), "area_err_vs_4pi": float(mv.sum() - 4 * np.pi),
            "note": "tf_setup_quaqua_p2 on the 96^3 P2 sphere (f = 13xyz at the base points, Newton tol 1e-13), "
                    "device time from the call to the assembled M, A and load vector, median of 3, L2 flushed"}


REFINE_N, REFINE_WIDTH, REFINE_LEVELS = 32, 0.05, 2


def run_refine(args):
    """Narrow-band refinement of a 32^3 brick of the same box towards the same sphere (width 0.05, levels 0..2,
    AdapTriangCL::MakeInitialTriang with DistMarkingStrategyCL) and the P2 TraceFEM path on its last
    triangulation level.  The refinement runs on the device (wall clock of tf_mesh_refine_band, median of 3,
    including reading back the level-0 mesh); the path (level set, DistributeDOFs, setupFESystem of M, A, C_n
    and the load vector, LinComb, mixed PCG to 1e-10) is device time between stream markers, median of 3 after
    one warm-up."""
    import drops_gb300 as tf

    ctx = tf.TraceFEM(0)
    tr = []
    for _ in range(3):
        ctx.brick_cube(REFINE_N, HALF)
        t0 = time.perf_counter()
        last, steps = ctx.mesh_refine_band(tf.LS_SPHERE, SPHERE, REFINE_WIDTH, 0, REFINE_LEVELS)
        tr.append((time.perf_counter() - t0) * 1e3)
    nv, ne, nt = ctx.mesh_info()
    h = 2 * HALF / REFINE_N
    ts, its = [], []
    for rep in range(4):
        ctx.flush_l2()
        ctx.marker(6)
        ctx.levelset_analytic(tf.LS_SPHERE, SPHERE, p2=True)
        na, m = ctx.distribute_dofs(tf.P2IF)
        ctx.setup_fe_system([tf.FORM_M, tf.FORM_A, tf.FORM_CN], tf.RHS_SPHERE_XYZ, list(SPHERE) + [13.0])
        ctx.lincomb([tf.FORM_M, tf.FORM_A, tf.FORM_CN], [1.0, 1.0, h])
        ctx.vec_fill(tf.VEC_X, m, 0.0)
        st, it, res = ctx.pcg_jacobi(tf.MAT_SYS, tf.VEC_RHS, tf.VEC_X, tol=1e-10, precision=tf.PREC_MIXED)
        ctx.marker(7)
        if rep:
            ts.append(ctx.elapsed_ms(6, 7))
            its.append(it)
        assert st == tf.OK and res <= 1e-10
    ctx.close()
    ms = statistics.median(ts)
    return {"refine_ms": round(statistics.median(tr), 1), "refine_first_ms": round(tr[0], 1), "levels": last,
            "steps": steps, "tets": nt, "vertices": nv,
            "cut_tets": na, "dofs": m, "path_ms": round(ms, 3), "cut_tets_per_s": round(na / (ms / 1e3), 1),
            "pcg_iters": int(statistics.median(its)),
            "note": f"{REFINE_N}^3 Kuhn cubes on [-5/3,5/3]^3 refined towards the unit sphere (width "
                    f"{REFINE_WIDTH}, levels 0..{REFINE_LEVELS}); refine_ms: tf_mesh_refine_band on the device (wall "
                    "clock, median of 3 calls in one context; the first call, refine_first_ms, also fills the "
                    "context's memory pool), path_ms: the P2 path with mixed PCG on the device, L2 flushed before each path"}


def refine_cpu_sample():
    """The sequential form of the same refinement (tf_refine_band: the reference's steps on one core, no
    device), on the same brick, median of 3 wall clocks in ms."""
    import drops_gb300 as tf
    from oracle import pyoracle as O

    om = O.brick(REFINE_N, a=HALF)
    ts = []
    for _ in range(3):
        t0 = time.perf_counter()
        r = tf.refine_band(om.coords, om.tet_v, tf.LS_SPHERE, SPHERE, REFINE_WIDTH, 0, REFINE_LEVELS)
        ts.append((time.perf_counter() - t0) * 1e3)
    return statistics.median(ts), len(r["tet_level"])


def quaqua_cpu_sample(threads, sample=4000):
    """The oracle's QuaQua element forms on the first `sample` cut tets of the same problem (one thread: the
    reference accumulates them serially), as cut tets/s."""
    from oracle import pyoracle as O

    mesh = O.brick(N_CUBES, a=HALF)
    lv, le = O.levelset(mesh, O.LS_SPHERE, SPHERE, True)
    st, na, m, dv, de, act = O.distribute_dofs(mesh, lv, le, True)
    tets = np.nonzero(act)[0][:sample]
    t0 = time.perf_counter()
    grad = O.grad_recovery(mesh, lv, le)
    t1 = time.perf_counter()
    O.quaqua_elements(mesh, lv, le, tets, grad=grad)
    t2 = time.perf_counter()
    per_tet = (t2 - t1) / len(tets)
    total = (t1 - t0) + per_tet * na
    return na / total, (f"the oracle on one core: recovered gradient of all {na} cut tets ({t1 - t0:.2f} s) and the "
                        f"mapped forms of the first {len(tets)} ({t2 - t1:.2f} s), extrapolated per tet")


def extra_workloads(args, rank, ws, dist):
    """The batch of 256 ellipsoids and the Cahn-Hilliard loop on the 128^3 torus, run after the headline
    workload with short step counts and reported inside its line (their own lines: --workload batch|ch)."""
    a = argparse.Namespace(**vars(args))
    a.steps, a.warmup = 5, 3
    b = run_batch(a, rank, ws, dist)
    batch = {k: b[k] for k in ("metric", "value", "unit", "ms_per_step", "e2e", "solve_ms", "autotuned", "problem",
                               "roofline", "clocks", "gpu_launches")}
    batch["steps"], batch["warmup"], batch["config"] = a.steps, a.warmup, b["config"]
    c = argparse.Namespace(**vars(args))
    c.ch_steps, c.ch_quick, c.ch_variants = args.extra_ch_steps, False, ""
    r = run_ch(c, rank, ws, dist)
    ch = {k: r[k] for k in ("metric", "value", "unit", "ms_per_step", "speedup_vs_plain_fp64", "ratios", "runs",
                            "problem", "clocks", "gpu_launches", "config")}
    ch["steps"] = c.ch_steps
    return batch, ch


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-large-spmv", action="store_true", help="skip the SpMV timings on the 192^3 and 384^3 systems")
    ap.add_argument("--size", type=int, default=N_CUBES, help="cubes per direction (96 = the benchmark workload; "
                    "smaller sizes are for profiling captures)")
    ap.add_argument("--workload", default="poisson", choices=["poisson", "batch", "ch"],
                    help="poisson: the P2 96^3 sphere problem (headline); batch: 256 independent P1 ellipsoids; "
                         "ch: Cahn-Hilliard steps on the torus, plain FP64 vs mixed + learned warm start")
    ap.add_argument("--ch-n", type=int, default=CH_N)
    ap.add_argument("--ch-steps", type=int, default=CH_STEPS)
    ap.add_argument("--ch-quick", action="store_true", help="only the plain FP64 and the mixed + learned runs")
    ap.add_argument("--ch-variants", default="", help="comma-separated subset of the Cahn-Hilliard variants")
    ap.add_argument("--no-extra", action="store_true",
                    help="poisson only: skip the batch and Cahn-Hilliard runs reported inside the headline line")
    ap.add_argument("--extra-ch-steps", type=int, default=30,
                    help="time steps of the Cahn-Hilliard run inside the headline line")
    ap.add_argument("--batch-count", type=int, default=BATCH_COUNT)
    ap.add_argument("--batch-nmin", type=int, default=BATCH_NMIN)
    ap.add_argument("--batch-nmax", type=int, default=BATCH_NMAX)
    args = ap.parse_args()
    rank, ws, dist = dist_init()
    if args.impl == "reference":
        out = run_reference(args, rank, ws, dist)
        if rank == 0:
            print(json.dumps(out))
        return
    from drops_gb300 import build

    if rank == 0:
        build.build()
    barrier(dist)
    if args.workload == "ch":
        out = run_ch(args, rank, ws, dist)
        if rank == 0:
            if ws == 1 and not args.no_cpu_baseline:
                v, sample = ch_cpu_sample(args, os.cpu_count() or 1)
                out["cpu_baseline"] = {"value": round(v, 3), "unit": "time_steps/s", "cores": os.cpu_count() or 1,
                                       "kind": "port", "sample": sample}
            print(json.dumps(out))
        if dist is not None:
            dist.destroy_process_group()
        return
    if args.workload == "batch":
        out = run_batch(args, rank, ws, dist)
        if (args.batch_count, args.batch_nmin, args.batch_nmax) != (BATCH_COUNT, BATCH_NMIN, BATCH_NMAX):
            out["config"] = dict(out["config"], workload=f"PROFILING SIZE {args.batch_count} instances, "
                                 f"n in [{args.batch_nmin},{args.batch_nmax}] (not the benchmark workload)")
        if rank == 0:
            if ws == 1 and not args.no_cpu_baseline:
                v, sample = batch_cpu_sample(args, os.cpu_count() or 1)
                out["cpu_baseline"] = {"value": round(v, 1), "unit": "cut_tets/s", "cores": os.cpu_count() or 1,
                                       "kind": "port", "sample": sample}
            print(json.dumps(out))
        if dist is not None:
            dist.destroy_process_group()
        return
    out = run_ours(args, rank, ws, dist)
    if args.size != N_CUBES:
        out["config"] = dict(out["config"], workload=f"PROFILING SIZE {args.size}^3 (not the benchmark workload)")
    if rank == 0 and ws == 1 and args.size == N_CUBES and not args.no_extra:
        out["batch"], out["ch"] = extra_workloads(args, rank, ws, dist)
        out["quaqua"] = run_quaqua(args)
        out["refine"] = run_refine(args)
    if rank == 0:
        products = out.pop("_products")
        if ws == 1 and not args.no_cpu_baseline:
            threads = os.cpu_count() or 1
            step = cpu_workload(threads, args.size)
            na, dt, it, phases, ref = step(keep=True)
            out["cpu_baseline"] = {"value": round(na / dt, 1), "unit": "cut_tets/s", "cores": threads, "kind": "port",
                                   "sample": f"one full step of the same workload ({dt:.1f} s, FP64 PCG {it} "
                                             f"iterations); {CPU_THREADING}",
                                   "phases": phases}
            out["parity"] = parity_report(products, ref)
            if "quaqua" in out:
                v, sample = quaqua_cpu_sample(threads)
                out["quaqua"]["cpu_baseline"] = {"value": round(v, 1), "unit": "cut_tets/s", "cores": 1,
                                                 "kind": "port", "sample": sample}
            if "refine" in out:
                ms, ntets = refine_cpu_sample()
                out["refine"]["cpu_baseline"] = {
                    "value": round(ms, 1), "unit": "ms", "cores": 1, "kind": "port",
                    "sample": f"the same refinement ({ntets} tets) by tf_refine_band, the library's sequential form "
                              "of the reference's steps (pinned to its refined meshes), one core, median of 3"}
        print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
