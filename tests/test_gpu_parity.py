"""CUDA path (through the C ABI) against the oracle and the reference's golden fixtures."""
import numpy as np
import pytest

import drops_gb300 as tf
from oracle import pyoracle as O
from tests.helpers import loc2glo, mat_close, sol_close

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from drops_gb300 import build

    build.build()
    c = tf.TraceFEM()
    yield c
    c.close()


def brick(ctx, n, a=None, orig=None, e=None):
    if isinstance(n, int):
        n = (n, n, n)
    if orig is None:
        orig = np.array([-a, -a, -a])
        e = np.diag([2.0 * a] * 3)
    ctx.brick(orig, e[0], e[1], e[2], *n)
    return O.brick(n, orig=orig, e=e)


@pytest.mark.parametrize("n,a", [((3, 4, 5), 1.3), ((16, 16, 16), 5.0 / 3.0), ((7, 1, 2), 0.9)])
def test_brick_mesh_bitexact(ctx, n, a):
    om = brick(ctx, n, a)
    coords, tv, te, ev = ctx.mesh_download()
    assert np.array_equal(coords, om.coords)
    assert np.array_equal(tv, om.tet_v) and np.array_equal(te, om.tet_e) and np.array_equal(ev, om.edge_v)


@pytest.mark.parametrize("kind,par", [
    (O.LS_SPHERE, [0, 0, 0, 1.0]), (O.LS_SPHERE, [0.1, -0.2, 0.05, 0.8]), (O.LS_TORUS, [1.0, 0.4, 2]),
    (O.LS_PLANE, [0.3, 0.5, -0.2, 0.1]),
    (O.LS_ELLIPSOID, [0.05, -0.03, 0.02, 1.2, 0.8, 0.7] + list(np.linalg.qr(np.arange(9.0).reshape(3, 3) + np.eye(3))[0].ravel())),
])
@pytest.mark.parametrize("p2", [False, True])
def test_levelset_bitexact(ctx, kind, par, p2):
    om = brick(ctx, 12, 1.6)
    ctx.levelset_analytic(kind, par, p2)
    lv, le = ctx.levelset_download()
    olv, ole = O.levelset(om, kind, par, p2)
    assert np.array_equal(lv, olv) and np.array_equal(le, ole)


SYSTEMS = [
    ("c1_sphere_p1_n16.npz", O.LS_SPHERE, [0, 0, 0, 1.0]),
    ("sphere_p2_n8.npz", O.LS_SPHERE, [0, 0, 0, 1.0]),
    ("torus_p1_n16.npz", O.LS_TORUS, [1.0, 0.4, 2]),
    ("torus_p2_n10.npz", O.LS_TORUS, [1.0, 0.4, 2]),
]


def setup_case(ctx, g, kind, par, upload=False):
    n, a = int(g["n"]), float(g["a"])
    om = brick(ctx, n, a)
    if upload:
        ctx.levelset_upload(g["ls_vert"], g["ls_edge"])
    else:
        ctx.levelset_analytic(kind, par, bool(g["ls_p2"]))
    p2 = bool(g["p2"])
    na, nd = ctx.distribute_dofs(tf.P2IF if p2 else tf.P1IF)
    return om, p2, na, nd


@pytest.mark.parametrize("name,kind,par", SYSTEMS)
@pytest.mark.parametrize("upload", [False, True])
def test_dofs_bitexact(ctx, golden, name, kind, par, upload):
    g = golden(name)
    om, p2, na, nd = setup_case(ctx, g, kind, par, upload)
    assert na == int(g["n_active"]) and nd == int(g["n_dofs"])
    dv, de, act, l2g = ctx.dofs()
    assert np.array_equal(act, g["active_tets"])
    assert np.array_equal(l2g, g["loc2glo"])
    # the per-entity maps agree with the oracle's
    lv, le = O.levelset(om, kind, par, bool(g["ls_p2"]))
    st, ona, ond, odv, ode, oact = O.distribute_dofs(om, lv, le, p2)
    assert np.array_equal(dv, odv)
    if p2:
        assert np.array_equal(de, ode)


@pytest.mark.parametrize("name,kind,par", SYSTEMS)
def test_assembly_parity(ctx, golden, name, kind, par):
    g = golden(name)
    om, p2, na, nd = setup_case(ctx, g, kind, par)
    nnz = ctx.setup_fe_system([tf.FORM_M, tf.FORM_A, tf.FORM_CN], tf.RHS_SPHERE_XYZ, [0, 0, 0, 1.0, 13.0])
    assert nnz == len(g["colind"])
    for f, key in ((tf.FORM_M, "M"), (tf.FORM_A, "A"), (tf.FORM_CN, "C")):
        rp, ci, v = ctx.matrix(f)
        assert np.array_equal(rp, g["rowptr"]) and np.array_equal(ci, g["colind"])
        ok, err = mat_close(v, g[key])
        assert ok, (key, err)
    ok, err = mat_close(ctx.vec_download(tf.VEC_RHS), g["rhs"])
    assert ok, err


@pytest.mark.parametrize("name,kind,par", [SYSTEMS[0], SYSTEMS[1], SYSTEMS[2]])
@pytest.mark.parametrize("precision", [tf.PREC_FP64, tf.PREC_MIXED])
def test_pcg_parity(ctx, golden, name, kind, par, precision):
    g = golden(name)
    om, p2, na, nd = setup_case(ctx, g, kind, par)
    ctx.setup_fe_system([tf.FORM_M, tf.FORM_A, tf.FORM_CN], tf.RHS_SPHERE_XYZ, [0, 0, 0, 1.0, 13.0])
    h = 2 * float(g["a"]) / int(g["n"])
    ctx.lincomb([tf.FORM_M, tf.FORM_A, tf.FORM_CN], [1.0, 1.0, h])
    rp, ci, S = ctx.matrix(tf.MAT_SYS)
    ok, err = mat_close(S, g["S"])
    assert ok, err
    ctx.vec_upload(tf.VEC_X, np.zeros(nd))
    st, it, res = ctx.pcg_jacobi(tf.MAT_SYS, tf.VEC_RHS, tf.VEC_X, tol=1e-10, precision=precision)
    assert st == tf.OK and res <= 1e-10
    x = ctx.vec_download(tf.VEC_X)
    if precision == tf.PREC_FP64:
        assert abs(it - int(g["iters"])) <= 1, (it, int(g["iters"]))
    # the FP64 residual of the returned solution, by the oracle
    r = g["rhs"] - O.spmv(g["rowptr"], g["colind"], g["S"], x)
    assert np.linalg.norm(r) / np.linalg.norm(g["rhs"]) <= 1.01e-10
    ok, err = sol_close(x, g["x"])
    assert ok, err


def test_pcg_user_matrix(ctx, golden):
    """PCGSolverCL<JACPcCL>::Solve on a host MatrixCL (size_t CSR) uploaded as is."""
    g = golden("c1_sphere_p1_n16.npz")
    ctx.matrix_upload(g["rowptr"], g["colind"], g["S"])
    ctx.vec_upload(tf.VEC_B, g["rhs"])
    ctx.vec_upload(tf.VEC_X, np.zeros(len(g["rhs"])))
    st, it, res = ctx.pcg_jacobi(tf.MAT_USER, tf.VEC_B, tf.VEC_X, tol=1e-10)
    assert st == tf.OK and abs(it - int(g["iters"])) <= 1
    ok, err = sol_close(ctx.vec_download(tf.VEC_X), g["x"])
    assert ok, err


def test_explicit_mesh_equals_brick(ctx, golden):
    g = golden("sphere_p2_n8.npz")
    om = O.brick(int(g["n"]), a=float(g["a"]))
    ctx.mesh_upload(om.coords, om.tet_v, om.tet_e, om.edge_v)
    ctx.levelset_upload(g["ls_vert"], g["ls_edge"])
    na, nd = ctx.distribute_dofs(tf.P2IF)
    assert na == int(g["n_active"]) and nd == int(g["n_dofs"])
    ctx.setup_fe_system([tf.FORM_M, tf.FORM_A, tf.FORM_CN], tf.RHS_SPHERE_XYZ, [0, 0, 0, 1.0, 13.0])
    for f, key in ((tf.FORM_M, "M"), (tf.FORM_A, "A"), (tf.FORM_CN, "C")):
        rp, ci, v = ctx.matrix(f)
        assert np.array_equal(ci, g["colind"])
        ok, err = mat_close(v, g[key])
        assert ok, (key, err)


def test_zero_node_is_an_error(ctx):
    """distance() throws for an exact zero at a node of a cut tet (geom/subtriangulation.tpp:43-44)."""
    om = brick(ctx, (10, 1, 1), orig=np.zeros(3), e=np.eye(3))
    ctx.levelset_analytic(tf.LS_PLANE, [1, 0, 0, 0.4], True)
    with pytest.raises(tf.TraceFEMError) as ei:
        ctx.distribute_dofs(tf.P1IF)
    assert ei.value.status == tf.ERR_ZERO_NODE
    # the context stays usable
    ctx.levelset_analytic(tf.LS_PLANE, [1, 0, 0, 0.41], True)
    na, nd = ctx.distribute_dofs(tf.P1IF)
    assert nd == 8


def test_assembly_and_pcg_deterministic(ctx):
    brick(ctx, 24, 5.0 / 3.0)
    ctx.levelset_analytic(tf.LS_SPHERE, [0, 0, 0, 1.0], True)
    ctx.distribute_dofs(tf.P2IF)
    outs = []
    for _ in range(2):
        ctx.setup_fe_system([tf.FORM_M, tf.FORM_A, tf.FORM_CN], tf.RHS_SPHERE_XYZ, [0, 0, 0, 1.0, 13.0])
        ctx.lincomb([tf.FORM_M, tf.FORM_A, tf.FORM_CN], [1.0, 1.0, 0.1])
        ctx.vec_upload(tf.VEC_X, np.zeros(ctx.m))
        st, it, res = ctx.pcg_jacobi(tf.MAT_SYS, tf.VEC_RHS, tf.VEC_X, tol=1e-10)
        outs.append((ctx.matrix(tf.MAT_SYS)[2].copy(), ctx.vec_download(tf.VEC_X).copy(), it))
    assert np.array_equal(outs[0][0], outs[1][0])
    assert np.array_equal(outs[0][1], outs[1][1]) and outs[0][2] == outs[1][2]


def test_p2_against_oracle_mid_size(ctx):
    """n = 32 P2 sphere (P2 level set): GPU vs oracle, pattern bit-exact, values 1e-12."""
    n, a = 32, 5.0 / 3.0
    om = brick(ctx, n, a)
    ctx.levelset_analytic(tf.LS_SPHERE, [0, 0, 0, 1.0], True)
    na, nd = ctx.distribute_dofs(tf.P2IF)
    lv, le = O.levelset(om, O.LS_SPHERE, [0, 0, 0, 1.0], True)
    st, ona, ond, odv, ode, oact = O.distribute_dofs(om, lv, le, True)
    assert (na, nd) == (ona, ond)
    ctx.setup_fe_system([tf.FORM_M, tf.FORM_A, tf.FORM_CN], tf.RHS_SPHERE_XYZ, [0, 0, 0, 1.0, 13.0])
    opts = O.make_opts(True, [O.FORM_M, O.FORM_A, O.FORM_CN], O.RHS_SPHERE_XYZ, [0, 0, 0, 1.0, 13.0])
    st, rp, ci, vals, rhs = O.assemble(om, lv, le, oact, odv, ode, ond, opts)
    for f in (tf.FORM_M, tf.FORM_A, tf.FORM_CN):
        grp, gci, gv = ctx.matrix(f)
        assert np.array_equal(grp, rp) and np.array_equal(gci, ci)
        ok, err = mat_close(gv, vals[f])
        assert ok, err
    ok, err = mat_close(ctx.vec_download(tf.VEC_RHS), rhs)
    assert ok, err
