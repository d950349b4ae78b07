"""Mixed-precision Jacobi-PCG: the single-barrier kernel (Chronopoulos-Gear recurrences, FP32 inner
iterations, FP64 refinement) against the two-barrier kernel and the oracle's FP64 residual."""
import os

import numpy as np
import pytest

import drops_gb300 as tf
from oracle import pyoracle as O
from tests.helpers import sol_close

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctxs():
    from drops_gb300 import build

    build.build()
    one = tf.TraceFEM()
    os.environ["TF_PCG_TWO_BARRIER"] = "1"
    try:
        two = tf.TraceFEM()
    finally:
        del os.environ["TF_PCG_TWO_BARRIER"]
    yield one, two
    one.close()
    two.close()


def _system(ctx, n, fe, kind=tf.LS_SPHERE, par=(0, 0, 0, 1.0)):
    a = 5.0 / 3.0
    ctx.brick_cube(n, a)
    ctx.levelset_analytic(kind, list(par), fe == tf.P2IF)
    _, nd = ctx.distribute_dofs(fe)
    ctx.setup_fe_system([tf.FORM_M, tf.FORM_A, tf.FORM_CN], tf.RHS_SPHERE_XYZ, [0, 0, 0, 1.0, 13.0])
    ctx.lincomb([tf.FORM_M, tf.FORM_A, tf.FORM_CN], [1.0, 1.0, 2 * a / n])
    return nd


def _fp64_resid(ctx, x):
    rp, ci, S = ctx.matrix(tf.MAT_SYS)
    b = ctx.vec_download(tf.VEC_RHS)
    return np.linalg.norm(b - O.spmv(rp, ci, S, x)) / np.linalg.norm(b)


@pytest.mark.parametrize("n,fe", [(16, tf.P1IF), (24, tf.P2IF), (48, tf.P2IF)])
def test_single_barrier_matches_two_barrier(ctxs, n, fe):
    out = []
    for ctx in ctxs:
        nd = _system(ctx, n, fe)
        ctx.vec_fill(tf.VEC_X, nd, 0.0)
        st, it, res = ctx.pcg_jacobi(tf.MAT_SYS, tf.VEC_RHS, tf.VEC_X, tol=1e-10, precision=tf.PREC_MIXED)
        assert st == tf.OK and res <= 1e-10
        x = ctx.vec_download(tf.VEC_X)
        # convergence is decided on the FP64 residual: check it independently
        assert _fp64_resid(ctx, x) <= 1.01e-10
        out.append((it, x))
    (it1, x1), (it2, x2) = out
    print("iterations single-barrier", it1, "two-barrier", it2)
    # the same Krylov method in exact arithmetic; FP32 rounding moves the count (an FP32 emulation of either
    # form needs ~17% more iterations than FP64 PCG on the 48^3 P2 system)
    assert abs(it1 - it2) <= max(10, (15 * it2) // 100), (it1, it2)
    ok, err = sol_close(x1, x2)
    assert ok, err


def test_single_barrier_edge_cases(ctxs):
    ctx = ctxs[0]
    nd = _system(ctx, 16, tf.P1IF)
    # converged start: zero iterations
    ctx.vec_fill(tf.VEC_X, nd, 0.0)
    st, it, res = ctx.pcg_jacobi(tf.MAT_SYS, tf.VEC_RHS, tf.VEC_X, tol=1e-10, precision=tf.PREC_MIXED)
    assert st == tf.OK
    st, it, res = ctx.pcg_jacobi(tf.MAT_SYS, tf.VEC_RHS, tf.VEC_X, tol=1e-10, precision=tf.PREC_MIXED)
    assert st == tf.OK and it == 0 and res <= 1e-10
    # zero right-hand side with rel=True: |b| = 0 counts as 1, x = 0 is the answer
    b = ctx.vec_download(tf.VEC_RHS)
    ctx.vec_fill(tf.VEC_B, nd, 0.0)
    ctx.vec_fill(tf.VEC_X, nd, 0.0)
    st, it, res = ctx.pcg_jacobi(tf.MAT_SYS, tf.VEC_B, tf.VEC_X, tol=1e-10, precision=tf.PREC_MIXED)
    assert st == tf.OK and it == 0 and res == 0.0
    # cut off by max_iter: not converged, the count is max_iter, the iterate is the folded one
    ctx.vec_upload(tf.VEC_B, b)
    ctx.vec_fill(tf.VEC_X, nd, 0.0)
    st, it, res = ctx.pcg_jacobi(tf.MAT_SYS, tf.VEC_B, tf.VEC_X, tol=1e-10, max_iter=7, precision=tf.PREC_MIXED)
    assert st == tf.ERR_NOT_CONVERGED and it == 7 and res > 1e-10
    x = ctx.vec_download(tf.VEC_X)
    assert abs(_fp64_resid(ctx, x) - res) <= 1e-6 * res
    # non-zero start, absolute tolerance
    rng = np.random.default_rng(4)
    ctx.vec_upload(tf.VEC_X, rng.standard_normal(nd))
    st, it, res = ctx.pcg_jacobi(tf.MAT_SYS, tf.VEC_B, tf.VEC_X, tol=1e-9, rel=False, precision=tf.PREC_MIXED)
    assert st == tf.OK and res <= 1e-9
    x = ctx.vec_download(tf.VEC_X)
    rp, ci, S = ctx.matrix(tf.MAT_SYS)
    assert np.linalg.norm(b - O.spmv(rp, ci, S, x)) <= 1.01e-9


def test_single_barrier_large_runs(ctxs):
    """P2 system on 144^3 cubes (~327k rows, ~10k slices): the blocks' slice runs exceed one planned chunk of
    64 slices, so blocks that walk several chunks and keep p and dx in global memory meet blocks that plan
    once and keep them in shared memory; the solution must match FP64 PCG."""
    ctx = ctxs[0]
    nd = _system(ctx, 144, tf.P2IF)
    assert nd > 64 * 32 * 152
    ctx.vec_fill(tf.VEC_X, nd, 0.0)
    st, it, res = ctx.pcg_jacobi(tf.MAT_SYS, tf.VEC_RHS, tf.VEC_X, tol=1e-10, precision=tf.PREC_MIXED)
    assert st == tf.OK and res <= 1e-10
    x = ctx.vec_download(tf.VEC_X)
    assert _fp64_resid(ctx, x) <= 1.01e-10
    ctx.vec_fill(tf.VEC_X, nd, 0.0)
    st, it64, res = ctx.pcg_jacobi(tf.MAT_SYS, tf.VEC_RHS, tf.VEC_X, tol=1e-10, precision=tf.PREC_FP64)
    assert st == tf.OK
    print("iterations mixed", it, "fp64", it64)
    ok, err = sol_close(x, ctx.vec_download(tf.VEC_X))
    assert ok, err
