"""The TraceFEM path on narrow-band refined meshes (tf_mesh_refine_band), through the C ABI, against the
reference's own refinement, numbering, forms and PCG solve on the last triangulation level."""
import hashlib

import numpy as np
import pytest

import drops_gb300 as tf
from tests.helpers import mat_close, sol_close

pytestmark = pytest.mark.gpu

CASES = [
    ("refine_sphere_p1_n4.npz", tf.LS_SPHERE, [0.0, 0.0, 0.0, 1.0]),
    ("refine_torus_p2_n3.npz", tf.LS_TORUS, [1.0, 0.4, 2]),
]


@pytest.fixture(scope="module")
def ctx():
    from drops_gb300 import build

    build.build()
    c = tf.TraceFEM()
    yield c
    c.close()


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def setup(ctx, g, kind, par):
    n, a = int(g["n"]), float(g["a"])
    ctx.brick_cube(n, a)
    last, steps = ctx.mesh_refine_band(kind, par, float(g["width"]), int(g["clevel"]), int(g["flevel"]))
    assert last == int(g["flevel"]) and steps >= 1
    coords, tv, te, ev = ctx.mesh_download()
    assert sha(coords[tv]) == str(g["tet_xyz_sha"])
    ctx.levelset_analytic(kind, par, bool(g["ls_p2"]))
    return ctx.distribute_dofs(tf.P2IF if bool(g["p2"]) else tf.P1IF)


@pytest.mark.parametrize("name,kind,par", CASES)
def test_refined_dofs_and_forms(ctx, golden, name, kind, par):
    g = golden(name)
    na, nd = setup(ctx, g, kind, par)
    assert na == int(g["n_active"]) and nd == int(g["n_dofs"])
    dv, de, act, l2g = ctx.dofs()
    assert np.array_equal(act, g["active_tets"])
    assert np.array_equal(l2g, g["loc2glo"])
    nnz = ctx.setup_fe_system([tf.FORM_M, tf.FORM_A, tf.FORM_CN], tf.RHS_SPHERE_XYZ, [0, 0, 0, 1.0, 13.0])
    assert nnz == len(g["colind"])
    for f, key in ((tf.FORM_M, "M"), (tf.FORM_A, "A"), (tf.FORM_CN, "C")):
        rp, ci, v = ctx.matrix(f)
        assert np.array_equal(rp, g["rowptr"]) and np.array_equal(ci, g["colind"])
        ok, err = mat_close(v, g[key], rp)
        assert ok, (key, err)
    ok, err = mat_close(ctx.vec_download(tf.VEC_RHS), g["rhs"])
    assert ok, err


@pytest.mark.parametrize("precision", [tf.PREC_FP64, tf.PREC_MIXED])
def test_refined_pcg(ctx, golden, precision):
    """PCGSolverCL<JACPcCL> on M + A + h C_n of the refined sphere mesh (h the coarse mesh width, as the
    reference driver's)."""
    g = golden("refine_sphere_p1_n4.npz")
    na, nd = setup(ctx, g, tf.LS_SPHERE, [0.0, 0.0, 0.0, 1.0])
    ctx.setup_fe_system([tf.FORM_M, tf.FORM_A, tf.FORM_CN], tf.RHS_SPHERE_XYZ, [0, 0, 0, 1.0, 13.0])
    h = 2 * float(g["a"]) / int(g["n"])
    ctx.lincomb([tf.FORM_M, tf.FORM_A, tf.FORM_CN], [1.0, 1.0, h])
    rp, ci, S = ctx.matrix(tf.MAT_SYS)
    ok, err = mat_close(S, g["S"], rp)
    assert ok, err
    ctx.vec_upload(tf.VEC_X, np.zeros(nd))
    st, it, res = ctx.pcg_jacobi(tf.MAT_SYS, tf.VEC_RHS, tf.VEC_X, tol=1e-10, precision=precision)
    assert st == tf.OK and res <= 1e-10
    if precision == tf.PREC_FP64:
        assert abs(it - int(g["iters"])) <= 1, (it, int(g["iters"]))
    ok, err = sol_close(ctx.vec_download(tf.VEC_X), g["x"])
    assert ok, err


def _rows():
    import os

    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "refine_meshes.npz"))
    return [(str(g["shape"][i]), int(g["n"][i]), float(g["a"][i]), float(g["width"][i]), int(g["clevel"][i]),
             int(g["flevel"][i]), i) for i in range(len(g["n"]))]


@pytest.mark.parametrize("shape,n,a,width,cl,fl,i", _rows())
def test_device_refinement_matches_reference(ctx, golden, shape, n, a, width, cl, fl, i):
    """The device engine's mesh (up to four levels, 330k tets) against the reference's: every tet's vertices'
    coordinates in tet order and local vertex order."""
    g = golden("refine_meshes.npz")
    kind, par = (tf.LS_SPHERE, [0.0, 0.0, 0.0, 1.0]) if shape == "sphere" else (tf.LS_TORUS, [1.0, 0.4, 2])
    ctx.brick_cube(n, a)
    last, steps = ctx.mesh_refine_band(kind, par, width, cl, fl)
    assert last == fl
    coords, tv, te, ev = ctx.mesh_download()
    assert sha(coords[tv]) == str(g["tet_xyz_sha"][i])
    # every edge of every tet is the uploaded edge between its two vertices
    pairs = np.sort(np.stack([tv[:, [0, 0, 1, 0, 1, 2]], tv[:, [1, 2, 2, 3, 3, 3]]], -1), -1)
    assert np.array_equal(np.sort(ev[te], -1), pairs)


@pytest.mark.parametrize("case", [
    ("upload", tf.LS_SPHERE, [0.0, 0.0, 0.0, 1.0], 0.1, 0, 2),
    ("brick", tf.LS_PLANE, [0.3, 0.5, -0.2, 0.1], 0.05, 0, 2),
    ("brick", tf.LS_SPHERE, [0.1, -0.2, 0.05, 0.8], 0.0, 1, 1),
    ("brick", tf.LS_TORUS, [1.0, 0.4, 2], 0.02, 0, 3),
])
def test_device_refinement_equals_sequential_form(ctx, case):
    """The device engine against the sequential form (pinned to the reference above) on other inputs: an
    uploaded mesh, a plane, uniform refinement (coarse = fine level), a thin band at three levels.  Both number
    vertices and edges by first touch in the triangulation's order, so all four arrays agree exactly."""
    from oracle import pyoracle as O

    how, kind, par, width, cl, fl = case
    n, a = 5, 1.55
    om = O.brick(n, a=a)
    if how == "upload":
        ctx.mesh_upload(om.coords, om.tet_v, om.tet_e, om.edge_v)
    else:
        ctx.brick_cube(n, a)
    last, steps = ctx.mesh_refine_band(kind, par, width, cl, fl)
    coords, tv, te, ev = ctx.mesh_download()
    r = tf.refine_band(om.coords, om.tet_v, kind, par, width, cl, fl)
    assert last == r["last_level"] and steps == r["steps"]
    assert np.array_equal(coords[tv], r["coords"][r["tet_v"]])
    for got, key in ((coords, "coords"), (tv, "tet_v"), (te, "tet_e"), (ev, "edge_v")):
        assert np.array_equal(got, r[key]), key


def test_refine_rejects_bad_input_on_device(ctx):
    ctx.brick_cube(3, 1.0)
    with pytest.raises(tf.TraceFEMError):
        ctx.mesh_refine_band(tf.LS_SPHERE, [0.0, 0.0, 0.0, 1.0], 0.1, 2, 1)
    with pytest.raises(tf.TraceFEMError):
        ctx.mesh_refine_band(tf.LS_ELLIPSOID, [0.0] * 15, 0.1, 0, 1)
    # the context keeps its mesh after a refused call
    assert ctx.mesh_info()[2] == 6 * 27


def test_repeated_refinement_from_the_pool(ctx, golden):
    """The refinement's buffers come from a memory pool of the context that keeps freed memory, uncleared, for
    the next call: after a torus band has left its data in the pool, the sphere refinement twice gives the
    reference's mesh both times, with the same vertex and edge numbering."""
    g = golden("refine_meshes.npz")
    i = int(np.argmax(g["n"] * (g["shape"] == "sphere")))
    n, a, width, cl, fl = int(g["n"][i]), float(g["a"][i]), float(g["width"][i]), int(g["clevel"][i]), int(g["flevel"][i])
    c = tf.TraceFEM()
    try:
        c.brick_cube(6, 1.55)
        c.mesh_refine_band(tf.LS_TORUS, [1.0, 0.4, 2], 0.02, 0, 3)
        out = []
        for _ in range(2):
            c.brick_cube(n, a)
            assert c.mesh_refine_band(tf.LS_SPHERE, [0.0, 0.0, 0.0, 1.0], width, cl, fl)[0] == fl
            out.append(c.mesh_download())
        assert sha(out[0][0][out[0][1]]) == str(g["tet_xyz_sha"][i])
        for x, y in zip(out[0], out[1]):
            assert np.array_equal(x, y)
    finally:
        c.close()


def test_refine_then_brick_again(ctx, golden):
    """A refined mesh is replaced by the next mesh call like any uploaded mesh."""
    g = golden("refine_sphere_p1_n4.npz")
    setup(ctx, g, tf.LS_SPHERE, [0.0, 0.0, 0.0, 1.0])
    ctx.brick_cube(4, 1.0)
    nv, ne, nt = ctx.mesh_info()
    assert nt == 6 * 4 ** 3 and nv == 5 ** 3


def ch_setup(ctx, g):
    """The brick refined towards the torus, P1 level set, P1IF numbering, M, A, C_n."""
    ctx.brick_cube(int(g["n"]), float(g["a"]))
    ctx.mesh_refine_band(tf.LS_TORUS, [1.0, 0.4, 2], float(g["width"]), int(g["clevel"]), int(g["flevel"]))
    coords, tv, te, ev = ctx.mesh_download()
    assert sha(coords[tv]) == str(g["tet_xyz_sha"])
    ctx.levelset_analytic(tf.LS_TORUS, [1.0, 0.4, 2], False)
    na, nd = ctx.distribute_dofs(tf.P1IF)
    assert nd == int(g["n_dofs"])
    ctx.setup_fe_system([tf.FORM_M, tf.FORM_A, tf.FORM_CN])
    return nd


def test_refined_ch_block_solve(ctx, golden):
    """One implicit Cahn-Hilliard step on the refined torus mesh: the block matrix of surfphasesep.cpp:431-434
    and GMRES(50) with nodal block Jacobi from a zero guess, against the reference's (iterations within 2,
    solution within 1e-9)."""
    g = golden("ch_torus_refined_n6.npz")
    nd = ch_setup(ctx, g)
    dt, eps, rho, beta, xi = (float(g[k]) for k in ("dt", "eps", "rho", "beta_s", "xi"))
    ctx.ch_block(1.0 / dt, 1.0, rho, eps * eps, beta)
    rp, ci, M = ctx.matrix(tf.FORM_M)
    chi = g["chi0"]
    from oracle import pyoracle as O

    Mc = O.spmv(rp, ci, M, chi)
    Mf = O.spmv(rp, ci, M, xi * 2 * chi * (1 - chi) * (1 - 2 * chi))
    ctx.vec_upload(tf.VEC_B, np.concatenate([Mc / dt, beta * Mc - Mf]))
    ctx.vec_fill(tf.VEC_X, 2 * nd, 0.0)
    st, it, res = ctx.gmres_jacobi(tf.MAT_BLOCK, tf.VEC_B, tf.VEC_X, restart=50, tol=1e-10, max_iter=20000)
    assert st == tf.OK and res <= 1e-10, (st, it, res)
    assert abs(it - int(g["block_iters"])) <= 2, (it, int(g["block_iters"]))
    ok, err = sol_close(ctx.vec_download(tf.VEC_X), g["block_x"])
    assert ok, err


def test_refined_ch_steps(ctx, golden):
    """Three warm-started BDF1 steps on the refined torus mesh (the surface driver's pipeline: refinement,
    interface numbering, forms, block GMRES) against the reference: iterations within 2 per step, state
    within 1e-9 after each step."""
    g = golden("ch_torus_refined_n6.npz")
    nd = ch_setup(ctx, g)
    dt, eps, rho, beta, xi = (float(g[k]) for k in ("dt", "eps", "rho", "beta_s", "xi"))
    ctx.vec_upload(tf.VEC_X, np.concatenate([g["chi0"], np.zeros(nd)]))
    for k in range(len(g["steps_iters"])):
        st, its, res = ctx.ch_steps(1, dt, 1.0, eps, beta, xi, rho, restart=50, tol=1e-10)
        assert st == tf.OK and np.all(res <= 1e-10)
        assert abs(int(its[0]) - int(g["steps_iters"][k])) <= 2, (k, its, g["steps_iters"])
        ok, err = sol_close(ctx.vec_download(tf.VEC_X), g["steps_X"][k])
        assert ok, (k, err)
