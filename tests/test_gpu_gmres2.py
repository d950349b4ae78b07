"""CGS2 GMRES (FP64 and FP32 Arnoldi cycles inside FP64 refinement) against the reference's GMRES solutions."""
import numpy as np
import pytest

import drops_gb300 as tf
from oracle import pyoracle as O
from tests.helpers import mat_close
from tests.test_gpu_parity import SYSTEMS, setup_case

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from drops_gb300 import build

    build.build()
    c = tf.TraceFEM()
    yield c
    c.close()


def resid(rp, ci, v, x, b):
    return np.linalg.norm(b - O.spmv(rp, ci, v, x)) / np.linalg.norm(b)


@pytest.mark.parametrize("precision,orth", [(tf.PREC_MIXED, tf.ORTH_MGS), (tf.PREC_FP64, tf.ORTH_CGS2)])
def test_ch_block_gmres2(ctx, golden, precision, orth):
    """CGS2 GMRES (FP32 cycles in FP64 refinement, or FP64) on the Cahn-Hilliard block system against the
    reference's own GMRES(50) solve of the same system (ch_torus_p1_n16.npz): FP64 residual 1e-10 on the
    reference's block matrix, solution within 1e-5 of the reference's (the block system's conditioning
    turns a 1e-10 residual into ~1e-7 differences between two solvers), deterministic."""
    t, g = golden("torus_p1_n16.npz"), golden("ch_torus_p1_n16.npz")
    om, p2, na, nd = setup_case(ctx, t, O.LS_TORUS, [1.0, 0.4, 2])
    ctx.setup_fe_system([tf.FORM_M, tf.FORM_A, tf.FORM_CN])
    dt, eps, rho, beta = float(g["dt"]), float(g["eps"]), float(g["rho"]), float(g["beta_s"])
    alpha = 1.0 / dt
    ctx.ch_block(alpha, 1.0, rho, eps * eps, beta)
    brp, bci, bv = g["B_rowptr"], g["B_colind"], g["B"]
    chi = g["chi0"]
    Mchi = O.spmv(t["rowptr"], t["colind"], t["M"], chi)
    fp = 2 * chi * (1 - chi) * (1 - 2 * chi)
    rhs = np.concatenate([alpha * Mchi, beta * Mchi - O.spmv(t["rowptr"], t["colind"], t["M"], fp)])
    rx, rit = g["block_x"], int(g["block_iters"])
    ctx.gmres_options(orth)
    try:
        ctx.vec_upload(tf.VEC_B, rhs)
        for rep in range(2):
            ctx.vec_fill(tf.VEC_X, 2 * nd, 0.0)
            st, it, res = ctx.gmres_jacobi(tf.MAT_BLOCK, tf.VEC_B, tf.VEC_X, restart=50, tol=1e-10, max_iter=20000,
                                           precision=precision)
            x = ctx.vec_download(tf.VEC_X)
            if rep == 0:
                x0, it0 = x, it
        assert np.array_equal(x, x0) and it == it0  # deterministic
    finally:
        ctx.gmres_options(tf.ORTH_MGS)
    assert st == tf.OK and res <= 1e-10
    r = resid(brp, bci, bv, x, rhs)
    print(f"iterations {it} (reference MGS {rit}), FP64 residual {r:.3e}, |x-x_ref|/|x_ref| "
          f"{np.linalg.norm(x - rx) / np.linalg.norm(rx):.3e}")
    assert r <= 1.01e-10
    assert it <= 1.5 * rit + 60
    assert np.linalg.norm(x - rx) <= 1e-5 * np.linalg.norm(rx)


@pytest.mark.parametrize("name,kind,par", [SYSTEMS[0], SYSTEMS[1]])
def test_point_jacobi_gmres2_mixed(ctx, golden, name, kind, par):
    g = golden(name)
    om, p2, na, nd = setup_case(ctx, g, kind, par)
    ctx.setup_fe_system([tf.FORM_M, tf.FORM_A, tf.FORM_CN], tf.RHS_SPHERE_XYZ, [0, 0, 0, 1.0, 13.0])
    h = 2 * float(g["a"]) / int(g["n"])
    ctx.lincomb([tf.FORM_M, tf.FORM_A, tf.FORM_CN], [1.0, 1.0, h])
    rp, ci, S = ctx.matrix(tf.MAT_SYS)
    ok, err = mat_close(S, g["S"], rp)
    assert ok, err
    ctx.vec_fill(tf.VEC_X, nd, 0.0)
    st, it, res = ctx.gmres_jacobi(tf.MAT_SYS, tf.VEC_RHS, tf.VEC_X, restart=30, tol=1e-10, max_iter=20000,
                                   precision=tf.PREC_MIXED)
    x = ctx.vec_download(tf.VEC_X)
    assert st == tf.OK and resid(g["rowptr"], g["colind"], g["S"], x, g["rhs"]) <= 1.01e-10
    assert np.linalg.norm(x - g["x"]) <= 1e-6 * np.linalg.norm(g["x"])
    # left preconditioning is the MGS solver's only
    with pytest.raises(tf.TraceFEMError):
        ctx.gmres_jacobi(tf.MAT_SYS, tf.VEC_RHS, tf.VEC_X, restart=30, tol=1e-10, method=1, precision=tf.PREC_MIXED)


def test_ch_steps_mixed_matches_fp64(ctx):
    ctx.brick_cube(16, 1.6)
    ctx.levelset_analytic(tf.LS_TORUS, [1.0, 0.4, 2], False)
    na, nd = ctx.distribute_dofs(tf.P1IF)
    ctx.setup_fe_system([tf.FORM_M, tf.FORM_A, tf.FORM_CN])
    h = 3.2 / 16
    rng = np.random.default_rng(4)
    x0 = np.concatenate([0.5 + rng.uniform(-0.01, 0.01, nd), np.zeros(nd)])
    out = {}
    for prec in (tf.PREC_FP64, tf.PREC_MIXED):
        ctx.vec_upload(tf.VEC_X, x0)
        st, its, res, used = ctx.ch_steps_learned(6, 1e-3, 1.0, 0.02, 0.0, 1.0, h, precision=prec, learned=False)
        assert st == tf.OK and np.all(res <= 1e-10)
        out[prec] = (ctx.vec_download(tf.VEC_X), its)
    xa, xb = out[tf.PREC_FP64][0], out[tf.PREC_MIXED][0]
    print("FP64 iterations", out[tf.PREC_FP64][1].tolist(), "mixed", out[tf.PREC_MIXED][1].tolist())
    # both runs solve every step to relative residual 1e-10; the block system's
    # conditioning turns that into ~1e-7 relative differences between two
    # solvers' states (a single solve already differs by ~1e-7, see above)
    assert np.linalg.norm(xa - xb) <= 1e-6 * np.linalg.norm(xa)
