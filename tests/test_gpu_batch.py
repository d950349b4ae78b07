"""Batches of independent ellipsoid problems (one persistent launch) against the oracle, instance by instance."""
import numpy as np
import pytest

import drops_gb300 as tf
from drops_gb300.workloads import ellipsoid_batch
from oracle import pyoracle as O
from tests.helpers import mat_close, sol_close

pytestmark = pytest.mark.gpu

RHS = [0, 0, 0, 1.0, 13.0]
FORMS = [tf.FORM_M, tf.FORM_A, tf.FORM_CN]


@pytest.fixture(scope="module")
def ctx():
    from drops_gb300 import build

    build.build()
    c = tf.TraceFEM()
    yield c
    c.close()


def setup_batch(ctx, W):
    ctx.brick_batch(W["n"], W["orig"], W["axes"])
    ctx.levelset_analytic_batch(tf.LS_ELLIPSOID, W["par"], p2=False)
    na, nd = ctx.distribute_dofs(tf.P1IF)
    ctx.setup_fe_system(FORMS, tf.RHS_SPHERE_XYZ, RHS)
    coef = np.stack([np.ones(len(W["h"])), np.ones(len(W["h"])), W["h"]], axis=1)
    ctx.batch_lincomb(FORMS, coef)
    return na, nd


def oracle_instance(W, i):
    n = tuple(int(k) for k in W["n"][i])
    om = O.brick(n, orig=W["orig"][i], e=W["axes"][i])
    lv, le = O.levelset(om, O.LS_ELLIPSOID, W["par"][i], False)
    st, na, nd, dv, de, act = O.distribute_dofs(om, lv, le, False)
    assert st == O.OK
    opts = O.make_opts(False, FORMS, O.RHS_SPHERE_XYZ, RHS)
    st, rp, ci, vals, rhs = O.assemble(om, lv, le, act, dv, None, nd, opts)
    assert st == O.OK
    S = vals[0] + vals[1] + W["h"][i] * vals[2]
    return dict(mesh=om, na=na, nd=nd, dv=dv, rp=rp, ci=ci, vals=vals, rhs=rhs, S=S)


@pytest.fixture(scope="module")
def batch(ctx):
    W = ellipsoid_batch(7, nmin=6, nmax=14, seed=4242)
    na, nd = setup_batch(ctx, W)
    return W, [oracle_instance(W, i) for i in range(7)]


def test_batch_numbering_and_matrices_bitexact(ctx, batch):
    W, ref = batch
    tets, cut, rows, nnz = ctx.batch_info()
    dv, _, act, _ = ctx.dofs()
    mats = {f: ctx.matrix(f) for f in FORMS}
    rp, ci, _ = mats[tf.FORM_M]
    S = ctx.matrix(tf.MAT_SYS)[2]
    rhs = ctx.vec_download(tf.VEC_RHS)
    v0 = 0
    for i, R in enumerate(ref):
        nv = R["mesh"].nv
        assert cut[i + 1] - cut[i] == R["na"] and rows[i + 1] - rows[i] == R["nd"]
        r0, r1 = rows[i], rows[i + 1]
        odv = np.where(R["dv"] >= 0, R["dv"] + r0, -1)
        assert np.array_equal(dv[v0:v0 + nv], odv)
        v0 += nv
        z0, z1 = rp[r0], rp[r1]
        assert z0 == nnz[i] and z1 == nnz[i + 1]
        assert np.array_equal(rp[r0:r1 + 1] - z0, R["rp"])
        assert np.array_equal(ci[z0:z1] - r0, R["ci"])
        for f in FORMS:
            ok, err = mat_close(mats[f][2][z0:z1], R["vals"][f], R["rp"])
            assert ok, (i, f, err)
        ok, err = mat_close(S[z0:z1], R["S"], R["rp"])
        assert ok, (i, err)
        ok, err = mat_close(rhs[r0:r1], R["rhs"])
        assert ok, (i, err)


@pytest.mark.parametrize("precision", [tf.PREC_FP64, tf.PREC_MIXED])
@pytest.mark.parametrize("lanes,threads", [(0, 0), (2, 128), (8, 512), (16, 1024)])
def test_batch_pcg_parity(ctx, batch, precision, lanes, threads):
    W, ref = batch
    _, _, rows, _ = ctx.batch_info(nnz=False)
    ctx.batch_config(lanes, threads, use_graph=True)
    ctx.vec_upload(tf.VEC_X, np.zeros(int(rows[-1])))
    st, its, res = ctx.batch_pcg_jacobi(tf.MAT_SYS, tf.VEC_RHS, tf.VEC_X, tol=1e-10, precision=precision)
    assert st == tf.OK and np.all(res <= 1e-10)
    x = ctx.vec_download(tf.VEC_X)
    for i, R in enumerate(ref):
        xi = x[rows[i]:rows[i + 1]]
        ost, ox, oit, ores = O.pcg_jacobi(R["rp"], R["ci"], R["S"], R["rhs"], tol=1e-10)
        assert ost == O.OK
        if precision == tf.PREC_FP64:
            assert abs(int(its[i]) - oit) <= 1, (i, its[i], oit)
        r = R["rhs"] - O.spmv(R["rp"], R["ci"], R["S"], xi)
        assert np.linalg.norm(r) / np.linalg.norm(R["rhs"]) <= 1.01e-10, i
        ok, err = sol_close(xi, ox)
        assert ok, (i, err)


def test_batch_graph_replay_and_direct_launch_agree(ctx, batch):
    W, ref = batch
    _, _, rows, _ = ctx.batch_info(nnz=False)
    m = int(rows[-1])
    outs = []
    for use_graph in (True, True, False):
        ctx.batch_config(4, 256, use_graph=use_graph)
        ctx.vec_upload(tf.VEC_X, np.zeros(m))
        st, its, res = ctx.batch_pcg_jacobi(tf.MAT_SYS, tf.VEC_RHS, tf.VEC_X, tol=1e-10, precision=tf.PREC_MIXED)
        assert st == tf.OK
        outs.append((ctx.vec_download(tf.VEC_X), its.copy(), res.copy()))
    for o in outs[1:]:
        assert np.array_equal(o[0], outs[0][0]) and np.array_equal(o[1], outs[0][1])


def test_batch_autotuner_and_limits(ctx, batch):
    W, ref = batch
    _, _, rows, _ = ctx.batch_info(nnz=False)
    ctx.batch_config(0, 0, use_graph=True)
    lanes, threads = ctx.batch_tune(tf.MAT_SYS, tf.VEC_RHS, tf.PREC_MIXED)
    assert lanes in (2, 4, 8, 16) and threads in (128, 256, 512, 1024)
    # a too small iteration budget is reported per instance
    ctx.vec_upload(tf.VEC_X, np.zeros(int(rows[-1])))
    st, its, res = ctx.batch_pcg_jacobi(tf.MAT_SYS, tf.VEC_RHS, tf.VEC_X, tol=1e-10, max_iter=3, check=False)
    assert st == tf.ERR_NOT_CONVERGED and np.all(its == 3) and np.all(res > 1e-10)
    with pytest.raises(tf.TraceFEMError):
        ctx.batch_config(3, 256)
