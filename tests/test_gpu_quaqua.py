"""Isoparametric P2 TraceFEM on the GPU (tf_setup_quaqua_p2: recovered gradient, QuaQua base points by
Newton, the mapped quadrature and the element forms) against the reference's own accumulation and, at
larger sizes, against the oracle; then a solve of (M + A) u = f on the forms."""
import numpy as np
import pytest
import scipy.sparse as sp

import drops_gb300 as tf
from oracle import pyoracle as O
from tests.helpers import mat_close, sparse_close
from tests.test_oracle_golden import quaqua_system

pytestmark = pytest.mark.gpu

# The base points come out of Newton stopped at |F| < 1e-13; the GPU and the oracle round the iterates
# differently, so the points agree to about that, and the gradient transformation amplifies the difference
# by 1 / (nl . n) where the linear facet is tilted against the surface: 1e-11 row-scaled for the forms at
# sizes past the reference fixture (where the agreement is 1e-12).
QQ_RTOL = 1e-11


@pytest.fixture(scope="module")
def ctx():
    from drops_gb300 import build

    build.build()
    c = tf.TraceFEM()
    yield c
    c.close()


def _setup(ctx, n, kind, par, a=5.0 / 3.0):
    ctx.brick_cube(n, a)
    ctx.levelset_analytic(kind, list(par), True)
    _, nd = ctx.distribute_dofs(tf.P2IF)
    newton = ctx.setup_quaqua_p2(13.0, 1e-13, 100)
    out = []
    for f in (tf.FORM_M, tf.FORM_A):
        rp, ci, v = ctx.matrix(f)
        out.append(sp.csr_matrix((v, ci, rp), shape=(nd, nd)))
    return nd, out[0], out[1], ctx.vec_download(tf.VEC_RHS), newton


def test_quaqua_matches_reference(ctx, golden):
    g = golden("quaqua_sphere_p2_n8.npz")
    m = int(g["n_dofs"])
    nd, M, A, rhs, newton = _setup(ctx, int(g["n"]), tf.LS_SPHERE, (0, 0, 0, 1.0), float(g["a"]))
    assert nd == m and 1 <= newton <= 100
    Mg = sp.csr_matrix((g["M"], g["M_colind"], g["M_rowptr"]), shape=(m, m))
    Ag = sp.csr_matrix((g["A"], g["A_colind"], g["A_rowptr"]), shape=(m, m))
    for X, G in ((M, Mg), (A, Ag)):
        ok, err = sparse_close(X, G)
        assert ok, err
    ok, err = mat_close(rhs, g["rhs"])
    assert ok, err


@pytest.mark.parametrize("n,kind,par", [(32, tf.LS_SPHERE, (0, 0, 0, 1.0)), (24, tf.LS_TORUS, (1.0, 0.4, 2)),
                                        (20, tf.LS_SPHERE, (0.1, -0.2, 0.05, 0.8))])
def test_quaqua_matches_oracle(ctx, n, kind, par):
    nd, M, A, rhs, newton = _setup(ctx, n, kind, par)
    mesh = O.brick(n, a=5.0 / 3.0)
    lv, le = O.levelset(mesh, kind, list(par), True)
    g = {"n_dofs": nd}
    Mo, Ao, ro, npts, onewton = quaqua_system(g, mesh, lv, le, O.grad_recovery(mesh, lv, le))
    for X, G in ((M, Mo), (A, Ao)):
        ok, err = sparse_close(X, G, rtol=QQ_RTOL)
        print(n, kind, err)
        assert ok, err
    ok, err = mat_close(rhs, ro, rtol=QQ_RTOL)
    assert ok, err


def test_quaqua_high_order_on_the_sphere(ctx):
    """Size-independent properties of the isoparametric forms on the unit sphere, taken with
    u = xyz at the DOF positions projected onto the sphere (a spherical harmonic of degree 3, eigenvalue
    12, and f = 13xyz): the discrete area (sum of M), the Rayleigh quotient u'Au / u'Mu - 12 and
    u'b / (13 u'Mu) - 1 all converge at about h^4, so each falls by more than 8 per halving of h."""
    errs = []
    for n in (8, 16, 32):
        nd, M, A, rhs, _ = _setup(ctx, n, tf.LS_SPHERE, (0, 0, 0, 1.0))
        om = O.brick(n, a=5.0 / 3.0)
        lv, le = O.levelset(om, O.LS_SPHERE, [0, 0, 0, 1.0], True)
        st, na, m, dv, de, act = O.distribute_dofs(om, lv, le, True)
        assert m == nd
        pos = np.zeros((m, 3))
        iv, ie = dv >= 0, de >= 0
        pos[dv[iv]] = om.coords[iv]
        pos[de[ie]] = 0.5 * (om.coords[om.edge_v[ie, 0]] + om.coords[om.edge_v[ie, 1]])
        p = pos / np.linalg.norm(pos, axis=1)[:, None]
        u = p[:, 0] * p[:, 1] * p[:, 2]
        um = u @ (M @ u)
        errs.append((abs(M.sum() - 4 * np.pi), abs(u @ (A @ u) / um - 12), abs(u @ rhs / (13 * um) - 1)))
    print(errs)
    e = np.array(errs)
    assert (e[0] < [2e-2, 0.2, 1e-2]).all()
    assert (e[0] / e[1] > 8).all() and (e[1] / e[2] > 8).all(), e
