"""Single-barrier Jacobi-PCG with each block's share of the system resident in shared memory
(krylov_res.cu): the mixed-precision solver (default where it fits) and its FP64 form
(tf_pcg_options(TF_PCG_FP64_CG1)), against the reference's PCG solutions, the oracle's FP64 residual,
the non-resident single-barrier kernel and the classic FP64 kernel."""
import os

import numpy as np
import pytest

import drops_gb300 as tf
from oracle import pyoracle as O
from tests.helpers import sol_close
from tests.test_gpu_parity import SYSTEMS, setup_case

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctxs():
    from drops_gb300 import build

    build.build()
    res = tf.TraceFEM()
    res.autotune(False)  # the resident kernel itself, not the tuner's pick
    os.environ["TF_PCG_RESIDENT"] = "0"
    try:
        plain = tf.TraceFEM()
    finally:
        del os.environ["TF_PCG_RESIDENT"]
    yield res, plain
    res.close()
    plain.close()


def _system(ctx, n, fe, kind=tf.LS_SPHERE, par=(0, 0, 0, 1.0)):
    a = 5.0 / 3.0
    ctx.brick_cube(n, a)
    ctx.levelset_analytic(kind, list(par), fe == tf.P2IF)
    _, nd = ctx.distribute_dofs(fe)
    ctx.setup_fe_system([tf.FORM_M, tf.FORM_A, tf.FORM_CN], tf.RHS_SPHERE_XYZ, [0, 0, 0, 1.0, 13.0])
    ctx.lincomb([tf.FORM_M, tf.FORM_A, tf.FORM_CN], [1.0, 1.0, 2 * a / n])
    return nd


def _fp64_resid(ctx, x, vec_b=tf.VEC_RHS):
    rp, ci, S = ctx.matrix(tf.MAT_SYS)
    b = ctx.vec_download(vec_b)
    return np.linalg.norm(b - O.spmv(rp, ci, S, x)) / np.linalg.norm(b)


def _solve(ctx, nd, precision, fp64_kernel=tf.PCG_FP64_CLASSIC, **kw):
    ctx.pcg_options(fp64_kernel)
    try:
        ctx.vec_fill(tf.VEC_X, nd, 0.0)
        st, it, res = ctx.pcg_jacobi(tf.MAT_SYS, tf.VEC_RHS, tf.VEC_X, precision=precision, **kw)
    finally:
        ctx.pcg_options(tf.PCG_FP64_CLASSIC)
    return st, it, res, ctx.vec_download(tf.VEC_X)


@pytest.mark.parametrize("name,kind,par", [s for s in SYSTEMS if s[0] != "torus_p2_n10.npz"])
def test_fp64_cg1_matches_reference(ctxs, golden, name, kind, par):
    """FP64 single-barrier PCG on the reference's systems: the reference's solution within 1e-9 and
    its iteration count within 2% (the same Krylov method, different rounding of the recurrences)."""
    ctx = ctxs[0]
    g = golden(name)
    om, p2, na, nd = setup_case(ctx, g, kind, par)
    ctx.setup_fe_system([tf.FORM_M, tf.FORM_A, tf.FORM_CN], tf.RHS_SPHERE_XYZ, [0, 0, 0, 1.0, 13.0])
    ctx.lincomb([tf.FORM_M, tf.FORM_A, tf.FORM_CN], [1.0, 1.0, 2 * float(g["a"]) / int(g["n"])])
    st, it, res, x = _solve(ctx, nd, tf.PREC_FP64, tf.PCG_FP64_CG1, tol=1e-10)
    rit = int(g["iters"])
    assert st == tf.OK and res <= 1e-10
    assert abs(it - rit) <= max(2, rit // 50), (it, rit)
    assert _fp64_resid(ctx, x) <= 1.01e-10
    ok, err = sol_close(x, g["x"])
    assert ok, err


@pytest.mark.parametrize("n,fe", [(16, tf.P1IF), (24, tf.P2IF), (48, tf.P2IF), (96, tf.P2IF)])
def test_resident_against_plain_and_fp64(ctxs, n, fe):
    """Mixed: resident against the non-resident single-barrier kernel; FP64: single-barrier resident against
    the classic two-barrier kernel.  Every solution meets the FP64 residual; iteration counts agree as the
    rounding allows (the FP32 count moves by up to ~15% with the summation order)."""
    res_ctx, plain_ctx = ctxs
    out = {}
    for key, ctx, prec, k64 in (("mixed_res", res_ctx, tf.PREC_MIXED, 0), ("mixed_plain", plain_ctx, tf.PREC_MIXED, 0),
                                ("fp64_cg1", res_ctx, tf.PREC_FP64, tf.PCG_FP64_CG1),
                                ("fp64_classic", res_ctx, tf.PREC_FP64, tf.PCG_FP64_CLASSIC)):
        nd = _system(ctx, n, fe)
        st, it, r, x = _solve(ctx, nd, prec, k64, tol=1e-10)
        assert st == tf.OK and r <= 1e-10, (key, st, r)
        assert _fp64_resid(ctx, x) <= 1.01e-10, key
        out[key] = (it, x)
    print({k: v[0] for k, v in out.items()})
    it = {k: v[0] for k, v in out.items()}
    assert abs(it["mixed_res"] - it["mixed_plain"]) <= max(10, (15 * it["mixed_plain"]) // 100), it
    assert abs(it["fp64_cg1"] - it["fp64_classic"]) <= max(2, it["fp64_classic"] // 50), it
    ref = out["fp64_classic"][1]
    for k in ("mixed_res", "mixed_plain", "fp64_cg1"):
        ok, err = sol_close(out[k][1], ref)
        assert ok, (k, err)


@pytest.mark.parametrize("prec,k64", [(tf.PREC_MIXED, 0), (tf.PREC_FP64, tf.PCG_FP64_CG1)])
def test_resident_edge_cases_and_determinism(ctxs, prec, k64):
    ctx = ctxs[0]
    nd = _system(ctx, 24, tf.P2IF)
    st, it, res, x1 = _solve(ctx, nd, prec, k64, tol=1e-10)
    assert st == tf.OK
    st2, it2, res2, x2 = _solve(ctx, nd, prec, k64, tol=1e-10)
    assert it2 == it and res2 == res and np.array_equal(x1, x2)  # deterministic
    ctx.pcg_options(k64)
    try:
        # converged start: zero iterations
        st, it, res = ctx.pcg_jacobi(tf.MAT_SYS, tf.VEC_RHS, tf.VEC_X, tol=1e-10, precision=prec)
        assert st == tf.OK and it == 0 and res <= 1e-10
        # zero right-hand side with rel=True: |b| = 0 counts as 1, x = 0 is the answer
        b = ctx.vec_download(tf.VEC_RHS)
        ctx.vec_fill(tf.VEC_B, nd, 0.0)
        ctx.vec_fill(tf.VEC_X, nd, 0.0)
        st, it, res = ctx.pcg_jacobi(tf.MAT_SYS, tf.VEC_B, tf.VEC_X, tol=1e-10, precision=prec)
        assert st == tf.OK and it == 0 and res == 0.0
        # cut off by max_iter: not converged, the count is max_iter, the residual is the true one
        ctx.vec_upload(tf.VEC_B, b)
        ctx.vec_fill(tf.VEC_X, nd, 0.0)
        st, it, res = ctx.pcg_jacobi(tf.MAT_SYS, tf.VEC_B, tf.VEC_X, tol=1e-10, max_iter=7, precision=prec)
        assert st == tf.ERR_NOT_CONVERGED and it == 7 and res > 1e-10
        x = ctx.vec_download(tf.VEC_X)
        assert abs(_fp64_resid(ctx, x, tf.VEC_B) - res) <= 1e-6 * res
        # non-zero start, absolute tolerance
        rng = np.random.default_rng(4)
        ctx.vec_upload(tf.VEC_X, rng.standard_normal(nd))
        st, it, res = ctx.pcg_jacobi(tf.MAT_SYS, tf.VEC_B, tf.VEC_X, tol=1e-9, rel=False, precision=prec)
        assert st == tf.OK and res <= 1e-9
        x = ctx.vec_download(tf.VEC_X)
        rp, ci, S = ctx.matrix(tf.MAT_SYS)
        assert np.linalg.norm(b - O.spmv(rp, ci, S, x)) <= 1.01e-9
    finally:
        ctx.pcg_options(tf.PCG_FP64_CLASSIC)


def test_too_large_for_shared_memory_falls_back(ctxs):
    """P2 on 144^3 cubes (~327k rows): a block's run does not fit the shared memory, so the mixed solve
    runs the non-resident kernel and the FP64 single-barrier request the classic kernel; both converge."""
    ctx = ctxs[0]
    nd = _system(ctx, 144, tf.P2IF)
    for prec, k64 in ((tf.PREC_MIXED, 0), (tf.PREC_FP64, tf.PCG_FP64_CG1)):
        st, it, res, x = _solve(ctx, nd, prec, k64, tol=1e-10)
        assert st == tf.OK and res <= 1e-10
        assert _fp64_resid(ctx, x) <= 1.01e-10


def test_autotune_picks_the_fastest_measured_shape():
    """tf_autotune: the first SpMV and mixed PCG on a matrix structure time the candidate launch shapes on
    that matrix; the kept choice is the fastest measured, the caller's vectors are untouched by the timing
    runs (a non-zero initial guess is honoured), and a rebuilt identical pattern keeps the choice."""
    from drops_gb300 import build

    build.build()
    with tf.TraceFEM() as ctx:
        nd = _system(ctx, 48, tf.P2IF)
        rng = np.random.default_rng(8)
        x0 = rng.standard_normal(nd)
        ctx.vec_upload(tf.VEC_X, x0)
        ctx.spmv(tf.MAT_SYS, tf.VEC_X, tf.VEC_T0)
        rp, ci, S = ctx.matrix(tf.MAT_SYS)
        y = ctx.vec_download(tf.VEC_T0)
        ref = O.spmv(rp, ci, S, x0)
        assert np.abs(y - ref).max() <= 1e-12 * np.abs(ref).max()
        ctx.vec_upload(tf.VEC_X, x0)
        st, it, res = ctx.pcg_jacobi(tf.MAT_SYS, tf.VEC_RHS, tf.VEC_X, tol=1e-10, precision=tf.PREC_MIXED)
        assert st == tf.OK and res <= 1e-10
        assert _fp64_resid(ctx, ctx.vec_download(tf.VEC_X)) <= 1.01e-10
        thr, bps, kind, spmv_us, pcg_us = ctx.autotune_info(tf.MAT_SYS)
        print("spmv", thr, bps, spmv_us, "pcg kind", kind, pcg_us)
        cand = [(512, 1), (512, 2), (256, 2), (256, 4)]
        assert (thr, bps) == cand[int(np.argmin(spmv_us))] and all(t > 0 for t in spmv_us)
        assert kind == int(np.argmin(pcg_us)) and all(t > 0 for t in pcg_us)
        # the same structure again (a rebuilt pattern): the choice is kept
        _system(ctx, 48, tf.P2IF)
        ctx.vec_fill(tf.VEC_X, nd, 0.0)
        st, it2, res = ctx.pcg_jacobi(tf.MAT_SYS, tf.VEC_RHS, tf.VEC_X, tol=1e-10, precision=tf.PREC_MIXED)
        assert st == tf.OK and ctx.autotune_info(tf.MAT_SYS)[2] == kind


def test_locality_order_across_numberings():
    """The solvers' SELL windows follow the Morton order of the DOFs' nodes (order.cu).  One context
    switches between P2 and P1 numberings (a P1 numbering leaves the edge DOF array unset) and solves each
    system in mixed and FP64 precision; the solutions match those of a context without the order."""
    from drops_gb300 import build

    build.build()
    os.environ["TF_LOCALITY_ORDER"] = "0"
    try:
        plain = tf.TraceFEM()
    finally:
        del os.environ["TF_LOCALITY_ORDER"]
    with tf.TraceFEM() as ctx:
        for n, fe in ((24, tf.P2IF), (16, tf.P1IF), (16, tf.P2IF), (22, tf.P1IF)):
            for prec in (tf.PREC_MIXED, tf.PREC_FP64):
                out = []
                for c in (ctx, plain):
                    nd = _system(c, n, fe)
                    st, it, res, x = _solve(c, nd, prec, tol=1e-10)
                    assert st == tf.OK and res <= 1e-10
                    assert _fp64_resid(c, x) <= 1.01e-10
                    out.append(x)
                ok, err = sol_close(out[0], out[1])
                assert ok, (n, fe, prec, err)
    plain.close()
