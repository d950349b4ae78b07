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


@pytest.mark.parametrize("dist", [0.0, -0.0, 0.02, 0.3, -0.1])
@pytest.mark.parametrize("p2", [False, True])
def test_dofs_narrow_band_dist(ctx, dist, p2):
    """DistributeDOFs(level, mg, ls, dist): a tet is active iff distance() <= dist, distance() being min |phi|
    over its 10 values when they share one sign and 0 otherwise (geom/subtriangulation.tpp:38-46).  Bands
    of positive width take uncut tets near the sphere; a negative dist takes none."""
    om = brick(ctx, 12, 5.0 / 3.0)
    ctx.levelset_analytic(tf.LS_SPHERE, [0.03, -0.02, 0.01, 1.0], p2)
    lv, le = O.levelset(om, O.LS_SPHERE, [0.03, -0.02, 0.01, 1.0], p2)
    na, nd = ctx.distribute_dofs(tf.P2IF if p2 else tf.P1IF, dist=dist)
    st, ona, ond, odv, ode, oact = O.distribute_dofs(om, lv, le, p2, dist=dist)
    assert st == 0 and (na, nd) == (ona, ond)
    dv, de, act, l2g = ctx.dofs()
    assert np.array_equal(act[:na], np.flatnonzero(oact))
    assert np.array_equal(dv, odv)
    if p2:
        assert np.array_equal(de, ode)
    if dist < 0:
        assert na == 0
    elif dist > 0.1:
        st0, na0, *_ = O.distribute_dofs(om, lv, le, p2, dist=0.0)
        assert na > na0


@pytest.mark.parametrize("name,kind,par", [s for s in SYSTEMS if "p1" in s[0]])
def test_wind_convection_parity(ctx, golden, name, kind, par):
    """N_P1P1 (surfactant/ifacetransp.h:1590-1600) against the reference's matrix for its vecP2IF wind:
    the one form that is not symmetric (scatter by row-local and column-local index)."""
    g = golden(name)
    om, p2, na, nd = setup_case(ctx, g, kind, par)
    with pytest.raises(tf.TraceFEMError):  # no wind on this mesh yet
        ctx.setup_fe_system([tf.FORM_N])
    ctx.wind_upload(g["wind_vert"], g["wind_edge"])
    nnz = ctx.setup_fe_system([tf.FORM_M, tf.FORM_N])
    assert nnz == len(g["colind"])
    rp, ci, v = ctx.matrix(tf.FORM_N)
    assert np.array_equal(rp, g["rowptr"]) and np.array_equal(ci, g["colind"])
    ok, err = mat_close(v, g["N"], rp)
    assert ok, err
    # alpha M + N, the convective block of surfphasesep.cpp:432
    ctx.lincomb([tf.FORM_M, tf.FORM_N], [1000.0, 1.0])
    rp, ci, s_ = ctx.matrix(tf.MAT_SYS)
    ok, err = mat_close(s_, 1000.0 * g["M"] + g["N"], rp)
    assert ok, err
    # a new mesh drops the wind
    brick(ctx, int(g["n"]), float(g["a"]))
    ctx.levelset_analytic(kind, par, False)
    ctx.distribute_dofs(tf.P1IF)
    with pytest.raises(tf.TraceFEMError):
        ctx.setup_fe_system([tf.FORM_N])


def test_vecdesc_write_read(ctx, golden, tmp_path):
    """tf_vec_write writes exactly the bytes of the reference's VecDescCL::Write(binary); tf_vec_read reads
    them back and rejects a count that differs from the expected one, as VecDescBaseCL::Read throws."""
    import os

    g = golden("c1_sphere_p1_n16.npz")
    ref = open(os.path.join(os.path.dirname(__file__), "golden", "c1_sphere_p1_n16_x.vec"), "rb").read()
    ctx.vec_upload(tf.VEC_X, g["x"])
    out = tmp_path / "x.vec"
    ctx.vec_write(tf.VEC_X, str(out))
    assert out.read_bytes() == ref
    ctx.vec_read(tf.VEC_T1, str(out), n_expected=len(g["x"]))
    assert np.array_equal(ctx.vec_download(tf.VEC_T1), g["x"])
    with pytest.raises(tf.TraceFEMError):
        ctx.vec_read(tf.VEC_T1, str(out), n_expected=len(g["x"]) + 1)
    short = tmp_path / "short.vec"
    short.write_bytes(ref[:100])
    with pytest.raises(tf.TraceFEMError):
        ctx.vec_read(tf.VEC_T1, str(short))
    with pytest.raises(tf.TraceFEMError):
        ctx.vec_read(tf.VEC_T1, str(tmp_path / "missing.vec"))


@pytest.mark.parametrize("name,kind,par", [s for s in SYSTEMS if "p1" in s[0]])
def test_laplace_m_degenerate_parity(ctx, golden, name, kind, par):
    """LaplaceM_P1P1 with the degenerate mobility chi (1 - chi) cut off at 0 (surfactant/ifacetransp.h:
    1533-1544, 1176-1190) against the reference's matrix; chi per interface DOF in TF_VEC_CHI."""
    g = golden(name)
    setup_case(ctx, g, kind, par)
    ctx.vec_upload(tf.VEC_CHI, g["chi"])
    ctx.setup_fe_system([tf.FORM_LAPM])
    rp, ci, v = ctx.matrix(tf.FORM_LAPM)
    assert np.array_equal(ci, g["colind"])
    ok, err = mat_close(v, g["LapM"], rp)
    assert ok, err


def test_ch_block_mobility_and_wind(ctx, golden):
    """[[alpha M + N, mob A_deg + rho C], [eps2 A_one + beta M + eps2 rho C, -M]] (surfphasesep.cpp:431-434):
    the degenerate-mobility matrix only in the upper-right block, A_one below."""
    g = golden("torus_p1_n16.npz")
    om, p2, na, nd = setup_case(ctx, g, tf.LS_TORUS, [1.0, 0.4, 2])
    ctx.vec_upload(tf.VEC_CHI, g["chi"])
    ctx.wind_upload(g["wind_vert"], g["wind_edge"])
    ctx.setup_fe_system([tf.FORM_M, tf.FORM_A, tf.FORM_CN, tf.FORM_LAPM, tf.FORM_N])
    alpha, rho, eps, beta = 1000.0, 0.2, 0.02, 0.3
    ctx.ch_block(alpha, 0.7, rho, eps * eps, beta, tf.CH_DEGENERATE_MOBILITY | tf.CH_WIND)
    brp, bci, bv = O.ch_block(g["rowptr"], g["colind"], g["M"], g["A"], g["C"], alpha, 0.7, rho, eps * eps, beta,
                              Amob=g["LapM"], N=g["N"])
    rp, ci, v = ctx.matrix(tf.MAT_BLOCK)
    assert np.array_equal(rp, brp) and np.array_equal(ci, bci)
    ok, err = mat_close(v, bv, rp)
    assert ok, err


def test_ch_steps_degenerate_mobility_and_wind(ctx, golden):
    """tf_ch_options(TF_CH_DEGENERATE_MOBILITY | TF_CH_WIND): three BDF1 steps on the torus against the
    reference (LaplaceM_P1P1 reassembled every step from the evolving chi, wind block alpha M + N,
    surfphasesep.cpp:414-434): iterations within 2 per step, state within 1e-9."""
    t, g = golden("torus_p1_n16.npz"), golden("ch_torus_p1_n16.npz")
    om, p2, na, nd = setup_case(ctx, t, O.LS_TORUS, [1.0, 0.4, 2])
    ctx.wind_upload(t["wind_vert"], t["wind_edge"])
    ctx.setup_fe_system([tf.FORM_M, tf.FORM_A, tf.FORM_CN])
    dt, eps, rho, beta, xi = float(g["dt"]), float(g["eps"]), float(g["rho"]), float(g["beta_s"]), float(g["xi"])
    try:
        ctx.ch_options(tf.CH_DEGENERATE_MOBILITY | tf.CH_WIND)
        ctx.vec_upload(tf.VEC_X, np.concatenate([g["dm_chi0"], np.zeros(nd)]))
        for k in range(len(g["dm_steps_iters"])):
            st, its, res = ctx.ch_steps(1, dt, 1.0, eps, beta, xi, rho, restart=50, tol=1e-10)
            assert st == tf.OK and np.all(res <= 1e-10)
            if k == 0:
                rp, ci, B = ctx.matrix(tf.MAT_BLOCK)
                assert np.array_equal(rp, g["B_rowptr"]) and np.array_equal(ci, g["B_colind"])
                ok, err = mat_close(B, g["dm_B0"], rp)
                assert ok, err
            assert abs(int(its[0]) - int(g["dm_steps_iters"][k])) <= 2, (k, its, g["dm_steps_iters"])
            ok, err = sol_close(ctx.vec_download(tf.VEC_X), g["dm_steps_X"][k])
            assert ok, (k, err)
    finally:
        ctx.ch_options(0)


def test_wind_convection_is_p1_only(ctx, golden):
    g = golden("sphere_p2_n8.npz")
    setup_case(ctx, g, tf.LS_SPHERE, [0, 0, 0, 1.0])
    nv, ne, nt = ctx.mesh_info()
    ctx.wind_upload(np.zeros((nv, 3)), np.zeros((ne, 3)))
    with pytest.raises(tf.TraceFEMError):
        ctx.setup_fe_system([tf.FORM_N])


@pytest.mark.parametrize("asm", [tf.ASM_KERNEL_PAIR, tf.ASM_KERNEL_FP64])
@pytest.mark.parametrize("name,kind,par", SYSTEMS)
def test_assembly_parity(ctx, golden, name, kind, par, asm):
    """Forms and load vector against the reference's own assembly, with the P2 forms in pair arithmetic
    (the default) and in FP64 (the P1 forms are FP64 either way)."""
    g = golden(name)
    om, p2, na, nd = setup_case(ctx, g, kind, par)
    ctx.assemble_options(asm)
    try:
        nnz = ctx.setup_fe_system([tf.FORM_M, tf.FORM_A, tf.FORM_CN], tf.RHS_SPHERE_XYZ, [0, 0, 0, 1.0, 13.0])
    finally:
        ctx.assemble_options(tf.ASM_KERNEL_PAIR)
    assert nnz == len(g["colind"])
    for f, key in ((tf.FORM_M, "M"), (tf.FORM_A, "A"), (tf.FORM_CN, "C")):
        rp, ci, v = ctx.matrix(f)
        assert np.array_equal(rp, g["rowptr"]) and np.array_equal(ci, g["colind"])
        ok, err = mat_close(v, g[key], rp)
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
    ok, err = mat_close(S, g["S"], rp)
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
        ok, err = mat_close(v, g[key], rp)
        assert ok, (key, err)


def test_explicit_mesh_any_edge_order(ctx, golden):
    """The DROPS shim uploads a level with the triangulation's own edge numbering: numbering, pattern and
    values must not depend on the global edge ids (permuted here at random)."""
    g = golden("sphere_p2_n8.npz")
    om = O.brick(int(g["n"]), a=float(g["a"]))
    perm = np.random.default_rng(7).permutation(om.ne)  # old edge id -> new edge id
    edge_v = np.empty_like(om.edge_v)
    edge_v[perm] = om.edge_v[:, ::-1]  # and each edge's vertices swapped
    ls_edge = np.empty(om.ne)
    ls_edge[perm] = g["ls_edge"]
    ctx.mesh_upload(om.coords, om.tet_v, perm[om.tet_e].astype(np.int32), edge_v)
    ctx.levelset_upload(g["ls_vert"], ls_edge)
    na, nd = ctx.distribute_dofs(tf.P2IF)
    assert na == int(g["n_active"]) and nd == int(g["n_dofs"])
    dv, de, act, l2g = ctx.dofs()
    assert np.array_equal(l2g, g["loc2glo"])
    ctx.setup_fe_system([tf.FORM_M, tf.FORM_A, tf.FORM_CN], tf.RHS_SPHERE_XYZ, [0, 0, 0, 1.0, 13.0])
    for f, key in ((tf.FORM_M, "M"), (tf.FORM_A, "A"), (tf.FORM_CN, "C")):
        rp, ci, v = ctx.matrix(f)
        assert np.array_equal(rp, g["rowptr"]) and np.array_equal(ci, g["colind"])
        ok, err = mat_close(v, g[key], rp)
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


ELLIPSOID = [0.05, -0.03, 0.02, 1.2, 0.8, 0.7] + list(np.linalg.qr(np.arange(9.0).reshape(3, 3) + np.eye(3))[0].ravel())


@pytest.mark.parametrize("asm", [tf.ASM_KERNEL_PAIR, tf.ASM_KERNEL_FP64])
@pytest.mark.parametrize("n,kind,par", [(32, tf.LS_SPHERE, [0, 0, 0, 1.0]), (28, tf.LS_TORUS, [1.0, 0.4, 2]),
                                        (30, tf.LS_ELLIPSOID, ELLIPSOID)])
def test_p2_against_oracle_mid_size(ctx, n, kind, par, asm):
    """P2 level set on n^3 cubes: GPU (pair and FP64 forms) vs oracle, pattern bit-exact, values 1e-12."""
    a = 5.0 / 3.0
    om = brick(ctx, n, a)
    ctx.levelset_analytic(kind, par, True)
    na, nd = ctx.distribute_dofs(tf.P2IF)
    lv, le = O.levelset(om, kind, par, True)
    st, ona, ond, odv, ode, oact = O.distribute_dofs(om, lv, le, True)
    assert (na, nd) == (ona, ond)
    ctx.assemble_options(asm)
    try:
        ctx.setup_fe_system([tf.FORM_M, tf.FORM_A, tf.FORM_CN], tf.RHS_SPHERE_XYZ, [0, 0, 0, 1.0, 13.0])
    finally:
        ctx.assemble_options(tf.ASM_KERNEL_PAIR)
    opts = O.make_opts(True, [O.FORM_M, O.FORM_A, O.FORM_CN], O.RHS_SPHERE_XYZ, [0, 0, 0, 1.0, 13.0])
    st, rp, ci, vals, rhs = O.assemble(om, lv, le, oact, odv, ode, ond, opts)
    for f in (tf.FORM_M, tf.FORM_A, tf.FORM_CN):
        grp, gci, gv = ctx.matrix(f)
        assert np.array_equal(grp, rp) and np.array_equal(gci, ci)
        ok, err = mat_close(gv, vals[f], grp)
        print(n, kind, asm, f, err)
        assert ok, err
    ok, err = mat_close(ctx.vec_download(tf.VEC_RHS), rhs)
    assert ok, err


@pytest.mark.parametrize("asm", [tf.ASM_KERNEL_PAIR, tf.ASM_KERNEL_FP64])
@pytest.mark.parametrize("n,kind,par,p2ls", [(24, tf.LS_SPHERE, [0, 0, 0, 1.0], False),
                                             (24, tf.LS_TORUS, [1.0, 0.4, 2], True),
                                             (20, tf.LS_ELLIPSOID, ELLIPSOID, True)])
def test_p1_against_oracle_mid_size(ctx, n, kind, par, p2ls, asm):
    """P1 forms on n^3 cubes, GPU (pair and FP64) vs oracle: a P1 level set (constant normal per tet) and
    P2 level sets (normal per point, volume rule per tet); pattern bit-exact, values 1e-12."""
    a = 5.0 / 3.0
    om = brick(ctx, n, a)
    ctx.levelset_analytic(kind, par, p2ls)
    na, nd = ctx.distribute_dofs(tf.P1IF)
    lv, le = O.levelset(om, kind, par, p2ls)
    st, ona, ond, odv, ode, oact = O.distribute_dofs(om, lv, le, False)
    assert (na, nd) == (ona, ond)
    ctx.assemble_options(asm)
    try:
        ctx.setup_fe_system([tf.FORM_M, tf.FORM_A, tf.FORM_CN], tf.RHS_SPHERE_XYZ, [0, 0, 0, 1.0, 13.0])
    finally:
        ctx.assemble_options(tf.ASM_KERNEL_PAIR)
    opts = O.make_opts(False, [O.FORM_M, O.FORM_A, O.FORM_CN], O.RHS_SPHERE_XYZ, [0, 0, 0, 1.0, 13.0])
    st, rp, ci, vals, rhs = O.assemble(om, lv, le, oact, odv, ode, ond, opts)
    for f in (tf.FORM_M, tf.FORM_A, tf.FORM_CN):
        grp, gci, gv = ctx.matrix(f)
        assert np.array_equal(grp, rp) and np.array_equal(gci, ci)
        ok, err = mat_close(gv, vals[f], grp)
        print(n, kind, p2ls, asm, f, err)
        assert ok, err
    ok, err = mat_close(ctx.vec_download(tf.VEC_RHS), rhs)
    assert ok, err


@pytest.mark.parametrize("method,side", [(0, "right"), (1, "left")])
def test_gmres_parity(ctx, golden, method, side):
    """GMRES(20) with Jacobi, right (0) and left (1) preconditioning, against DROPS's own GMRES
    (num/krylovsolver.h:320-463) on the torus system M + A + h C_n: iterations within 2 of the
    reference's, solution within 1e-9."""
    t, g = golden("torus_p1_n16.npz"), golden("ch_torus_p1_n16.npz")
    ctx.matrix_upload(t["rowptr"], t["colind"], t["S"])
    ctx.vec_upload(tf.VEC_B, t["rhs"])
    ctx.vec_fill(tf.VEC_X, len(t["rhs"]), 0.0)
    st, it, res = ctx.gmres_jacobi(tf.MAT_USER, tf.VEC_B, tf.VEC_X, restart=20, tol=1e-10, method=method)
    rit = int(g[f"gmres_{side}_iters"])
    assert st == tf.OK and res <= 1e-10
    assert abs(it - rit) <= 2, (it, rit)
    ok, err = sol_close(ctx.vec_download(tf.VEC_X), g[f"gmres_{side}_x"])
    assert ok, err


def ch_rhs(t, chi, dt, beta, xi=1.0):
    """Right-hand side of a BDF1 Cahn-Hilliard step, f = 0 (surfphasesep.cpp:421-425)."""
    Mc = O.spmv(t["rowptr"], t["colind"], t["M"], chi)
    Mf = O.spmv(t["rowptr"], t["colind"], t["M"], xi * 2 * chi * (1 - chi) * (1 - 2 * chi))
    return np.concatenate([Mc / dt, beta * Mc - Mf])


def test_ch_block_gmres(ctx, golden):
    """One implicit Cahn-Hilliard step against the reference: the block matrix of
    surfphasesep.cpp:431-434 (pattern bit-exact with the reference's block constructor,
    num/spmat.h:718-750; values within 1e-12) and GMRES(50) with nodal block Jacobi from a zero
    guess (iterations within 2 of DROPS's GMRES, solution within 1e-9)."""
    t, g = golden("torus_p1_n16.npz"), golden("ch_torus_p1_n16.npz")
    om, p2, na, nd = setup_case(ctx, t, O.LS_TORUS, [1.0, 0.4, 2])
    ctx.setup_fe_system([tf.FORM_M, tf.FORM_A, tf.FORM_CN])
    dt, eps, rho, beta = float(g["dt"]), float(g["eps"]), float(g["rho"]), float(g["beta_s"])
    ctx.ch_block(1.0 / dt, 1.0, rho, eps * eps, beta)
    rp, ci, B = ctx.matrix(tf.MAT_BLOCK)
    assert np.array_equal(rp, g["B_rowptr"]) and np.array_equal(ci, g["B_colind"])
    ok, err = mat_close(B, g["B"], rp)
    assert ok, err
    ctx.vec_upload(tf.VEC_B, ch_rhs(t, g["chi0"], dt, beta))
    ctx.vec_fill(tf.VEC_X, 2 * nd, 0.0)
    st, it, res = ctx.gmres_jacobi(tf.MAT_BLOCK, tf.VEC_B, tf.VEC_X, restart=50, tol=1e-10, max_iter=20000)
    assert st == tf.OK and res <= 1e-10, (st, it, res)
    assert abs(it - int(g["block_iters"])) <= 2, (it, int(g["block_iters"]))
    ok, err = sol_close(ctx.vec_download(tf.VEC_X), g["block_x"])
    assert ok, err


def test_legacy_numbering(ctx, golden):
    """CreateNumbOnInterfaceVertex: 8 unknowns (plane), 1156 (sphere r=0.31 on 20^3), error at a vertex plane."""
    g = golden("legacy_numbering.npz")
    brick(ctx, (10, 1, 1), orig=np.zeros(3), e=np.eye(3))
    ctx.levelset_analytic(tf.LS_PLANE, [1, 0, 0, 0.41], True)
    na, nd = ctx.create_numb_on_interface_p1()
    assert nd == int(g["plane_n_dofs"]) == 8 and na == int(g["plane_n_active"])
    assert np.array_equal(ctx.dofs()[0], g["plane_dof_vert"])
    ctx.levelset_analytic(tf.LS_PLANE, [1, 0, 0, 0.4], True)
    with pytest.raises(tf.TraceFEMError) as ei:
        ctx.create_numb_on_interface_p1()
    assert ei.value.status == tf.ERR_ZERO_NODE
    brick(ctx, (20, 20, 20), orig=np.zeros(3), e=np.eye(3))
    ctx.levelset_analytic(tf.LS_SPHERE, [0.5, 0.5, 0.5, 0.31], True)
    na, nd = ctx.create_numb_on_interface_p1()
    assert nd == int(g["sphere_n_dofs"]) == 1156 and na == int(g["sphere_n_active"])
    assert np.array_equal(ctx.dofs()[0], g["sphere_dof_vert"])


LEGACY_F = [1.0, 0, 0, -0.5, 0, 0, 0, 1.0, 0, 0]  # f = 1 + x y - z / 2, the harness's test function


def test_legacy_forms_match_reference(ctx, golden):
    """SetupInterfaceMassP1 / SetupLBP1 / SetupInterfaceRhsP1 on the legacy numbering, unit sphere on 10^3:
    pattern bit-exact, values within 1e-12 of the reference's."""
    g = golden("legacy_forms_sphere_n10.npz")
    brick(ctx, int(g["n"]), float(g["a"]))
    ctx.levelset_upload(g["ls_vert"], g["ls_edge"])
    na, nd = ctx.create_numb_on_interface_p1()
    assert na == int(g["n_active"]) and nd == int(g["n_dofs"])
    assert np.array_equal(ctx.dofs()[0], g["dof_vert"])
    nnz = ctx.setup_interface_p1_legacy(float(g["alpha"]), float(g["D"]), LEGACY_F)
    assert nnz == len(g["colind"])
    for f, key in ((tf.FORM_M, "M"), (tf.FORM_A, "A")):
        rp, ci, v = ctx.matrix(f)
        assert np.array_equal(rp, g["rowptr"]) and np.array_equal(ci, g["colind"])
        ok, err = mat_close(v, g[key], rp)
        assert ok, (key, err)
    ok, err = mat_close(ctx.vec_download(tf.VEC_RHS), g["rhs"])
    assert ok, err
    with pytest.raises(tf.TraceFEMError):
        ctx.matrix(tf.FORM_CN)


@pytest.mark.parametrize("n,kind,par,alpha,D,f", [
    (14, O.LS_TORUS, [1.0, 0.4, 2], 1.0, 1.0, [0.5, 1, -1, 0.25, 0.3, 0, -0.2, 0, 0.1, 0]),
    (11, O.LS_SPHERE, [0.1, -0.2, 0.05, 0.8], 0.3, 2.5, None),
])
def test_legacy_forms_match_oracle(ctx, n, kind, par, alpha, D, f):
    om = brick(ctx, n, 1.6)
    ctx.levelset_analytic(kind, par, True)
    lv, le = O.levelset(om, kind, par, True)
    na, nd = ctx.create_numb_on_interface_p1()
    dv = ctx.dofs()[0]
    st, ona, ond, odv = O.numb_on_interface_p1(om, lv, le)
    assert st == O.OK and np.array_equal(dv, odv) and nd == ond
    ctx.vec_fill(tf.VEC_RHS, nd, 7.0)
    nnz = ctx.setup_interface_p1_legacy(alpha, D, f)
    st, rp, ci, M, A, rhs = O.assemble_legacy_p1(om, lv, le, odv, ond, alpha, D, f if f is not None else [0.0] * 10)
    assert st == O.OK and nnz == len(ci)
    for form, ref in ((tf.FORM_M, M), (tf.FORM_A, A)):
        grp, gci, v = ctx.matrix(form)
        assert np.array_equal(grp, rp) and np.array_equal(gci, ci)
        ok, err = mat_close(v, ref, grp)
        assert ok, err
    if f is not None:
        ok, err = mat_close(ctx.vec_download(tf.VEC_RHS), rhs)
        assert ok, err
    else:  # no rhs requested: the vector is left alone
        assert np.all(ctx.vec_download(tf.VEC_RHS) == 7.0)


def test_ch_steps_parity(ctx, golden):
    """Three warm-started BDF1 steps on the torus (P1, n=16) against the reference's block
    constructor and GMRES(50): iterations within 2 per step, state within 1e-9 after each step."""
    t, g = golden("torus_p1_n16.npz"), golden("ch_torus_p1_n16.npz")
    om, p2, na, nd = setup_case(ctx, t, O.LS_TORUS, [1.0, 0.4, 2])
    ctx.setup_fe_system([tf.FORM_M, tf.FORM_A, tf.FORM_CN])
    dt, eps, rho, beta, xi = float(g["dt"]), float(g["eps"]), float(g["rho"]), float(g["beta_s"]), float(g["xi"])
    ctx.vec_upload(tf.VEC_X, np.concatenate([g["chi0"], np.zeros(nd)]))
    for k in range(len(g["steps_iters"])):
        st, its, res = ctx.ch_steps(1, dt, 1.0, eps, beta, xi, rho, restart=50, tol=1e-10)
        assert st == tf.OK and np.all(res <= 1e-10)
        assert abs(int(its[0]) - int(g["steps_iters"][k])) <= 2, (k, its, g["steps_iters"])
        ok, err = sol_close(ctx.vec_download(tf.VEC_X), g["steps_X"][k])
        assert ok, (k, err)


def oracle_ch_adaptive(g, P, chi0):
    """surfphasesep.cpp:397-483 (adaptive BDF1/BDF2) restated on the oracle's GMRES (CPU)."""
    rp, ci, M = g["rowptr"], g["colind"], g["M"]
    m = len(rp) - 1
    f0p = lambda c: P["xi"] * 2 * c * (1 - c) * (1 - 2 * c)
    mv = lambda x: O.spmv(rp, ci, M, x)

    def solve(alpha, b, x0):
        brp, bci, bv = O.ch_block(rp, ci, M, g["A"], g["C"], alpha, 1.0, P["rho"], P["eps"] ** 2, P["beta"])
        st, x, it, res = O.gmres_jacobi(brp, bci, bv, b, x0=x0, restart=50, tol=1e-10, max_iter=50000, block=True)
        assert st == O.OK
        return x

    def F(e, dt):
        if e == 0:
            return P["dt0"]
        return min(max(P["F_rho"] * np.sqrt(P["F_tol"] / e) * dt, P["F_min"]), P["F_max"])

    X = np.concatenate([chi0, np.zeros(m)])
    prev = None
    t, dt, e, i, dts, tries = 0.0, P["dt0"], 0.0, 0, [], []
    while t < P["t_final"]:
        i += 1
        t_prev, dt_prev, n = t, dt, 0
        while True:
            n += 1
            dt = F(e, dt)
            t = t_prev + dt
            chi = X[:m]
            Mc = mv(chi)
            X1 = solve(1 / dt, np.concatenate([Mc / dt, P["beta"] * Mc - mv(f0p(chi))]), X)
            if i == 1:
                X2 = X1
                break
            r = dt / dt_prev
            ce = (1 + r) * chi - r * prev
            b = np.concatenate([((1 + r) / dt) * Mc - (r * r / (1 + r) / dt) * mv(prev),
                                P["beta"] * mv(ce) - mv(f0p(ce))])
            X2 = solve((1 + 2 * r) / (1 + r) / dt, b, X1)
            d = X2[:m] - X1[:m]
            e = np.sqrt(d @ mv(d) / (X2[:m] @ mv(X2[:m])))
            if not (e > P["F_tol"] and P["F_min"] < dt < P["F_max"]):
                break
        prev = X[:m].copy()
        X = X2
        dts.append(dt)
        tries.append(n)
    return t, np.array(dts), np.array(tries), X


def test_ch_adaptive_parity(ctx, golden):
    """Adaptive BDF1/BDF2 Cahn-Hilliard steps (surfphasesep.cpp:397-483) on the torus (P1, n=16): the same
    step sizes, retries and state as the oracle restatement."""
    g = golden("torus_p1_n16.npz")
    om, p2, na, nd = setup_case(ctx, g, O.LS_TORUS, [1.0, 0.4, 2])
    ctx.setup_fe_system([tf.FORM_M, tf.FORM_A, tf.FORM_CN])
    h = 2 * float(g["a"]) / int(g["n"])
    # an attempt grows dt to 2.6e-3 and is rejected; steps 3, 4 and 6 retry, dt shrinks; dt >= 1e-3 keeps
    # GMRES(50) with nodal block Jacobi converging on both the BDF1 and the BDF2 systems
    P = dict(t_final=0.014, dt0=2e-3, F_tol=1e-2, F_rho=0.9, F_min=1e-3, F_max=4e-3, eps=0.02, beta=0.0, xi=1.0,
             rho=h)
    rng = np.random.default_rng(3)
    chi0 = 0.5 + rng.uniform(-0.05, 0.05, nd)
    ctx.vec_upload(tf.VEC_X, np.concatenate([chi0, np.zeros(nd)]))
    te, dts, errs, tries, its = ctx.ch_steps_adaptive(P["t_final"], P["dt0"], P["F_tol"], P["F_rho"], P["F_min"],
                                                      P["F_max"], 1.0, P["eps"], P["beta"], P["xi"], P["rho"])
    ot, odts, otries, OX = oracle_ch_adaptive(g, P, chi0)
    assert len(dts) == len(odts) and np.array_equal(tries, otries), (dts, odts, tries, otries)
    assert np.allclose(dts, odts, rtol=1e-6, atol=0) and abs(te - ot) <= 1e-9
    assert np.any(tries > 1) and dts.min() < P["dt0"]  # the controller rejected steps and shrank dt
    X = ctx.vec_download(tf.VEC_X)
    # ~20 solves to 1e-10, each GPU and CPU iterate within the solver tolerance of the other
    assert np.linalg.norm(X[:nd] - OX[:nd]) <= 1e-7 * np.linalg.norm(OX[:nd])


def test_ch_stats(ctx, golden, tmp_path):
    """Integrals of the per-step statistics (surfphasesep.cpp:324-345) after three CH steps on the torus,
    against the same formulas on the reference's M and A: area 1'M1, raft fraction 1'M chi / area,
    perimeter eps chi'A chi, Lyapunov energy (M1)'f0(chi) + eps^2/2 chi'A chi, f0(c) = xi (c (1 - c))^2."""
    import json

    import scipy.sparse as sp

    g = golden("torus_p1_n16.npz")
    om, p2, na, nd = setup_case(ctx, g, O.LS_TORUS, [1.0, 0.4, 2])
    ctx.setup_fe_system([tf.FORM_M, tf.FORM_A, tf.FORM_CN])
    dt, eps, h, xi = 1e-3, 0.02, 2 * float(g["a"]) / int(g["n"]), 0.7
    rng = np.random.default_rng(5)
    ctx.vec_upload(tf.VEC_X, np.concatenate([0.5 + rng.uniform(-0.01, 0.01, nd), np.zeros(nd)]))
    ctx.ch_steps(3, dt, 1.0, eps, 0.0, xi, h, restart=50, tol=1e-10)
    chi = ctx.vec_download(tf.VEC_CHI)
    st = ctx.ch_stats(eps, xi)
    M = sp.csr_matrix((g["M"], g["colind"], g["rowptr"]))
    A = sp.csr_matrix((g["A"], g["colind"], g["rowptr"]))
    one = np.ones(nd)
    area = one @ (M @ one)
    f0 = xi * (chi * (1 - chi)) ** 2
    want = {"Integral.SurfacaAreaP1": area, "Integral.FESolution.RaftFraction": (M @ chi) @ one / area,
            "Integral.FESolution.PerimeterEstimate": eps * (chi @ (A @ chi)),
            "Integral.FESolution.LyapunovEnergy": (M @ one) @ f0 + 0.5 * eps * eps * (chi @ (A @ chi)),
            "c_h.Max": chi.max(), "c_h.Min": chi.min()}
    for k, v in want.items():
        assert abs(st[k] - v) <= 1e-12 * abs(v), (k, st[k], v)
    tree = ctx.write_ch_stats(str(tmp_path / "t_3.json"), t=3 * dt, h=h, eps=eps, xi=xi)
    back = json.load(open(tmp_path / "t_3.json"))
    assert back == tree and back["DOF"]["c_h"] == nd and back["Integral"]["FESolution"]["RaftFraction"] > 0


def test_patch_topology_bitexact(ctx, golden):
    """make_patch facets, boundary flags and vertices of the reference's area test
    (sphere r=0.5 on [-1,1]^3, 8^3 cubes, vertices on the sphere included) bit for bit."""
    g = golden("area_sphere05_n8.npz")
    brick(ctx, 8, 1.0)
    ctx.levelset_analytic(tf.LS_SPHERE, [0, 0, 0, 0.5], True)
    pats = ctx.patches(g["patch_tets"])
    fo = vo = 0
    for i, t in enumerate(g["patch_tets"]):
        f, b, v = pats[i]
        k, nv = int(g["n_facets"][t]), int(g["patch_nverts"][i])
        assert np.array_equal(f, g["patch_facets"][3 * fo:3 * (fo + k)].reshape(-1, 3))
        assert np.array_equal(b, g["patch_boundary"][fo:fo + k])
        assert np.array_equal(v, g["patch_verts"][4 * vo:4 * (vo + nv)].reshape(-1, 4))
        fo += k
        vo += nv


def _pair_forms(sort, fe, kind, par, p2ls, n):
    """M, A, C_n values and the load vector from a fresh context whose TF_PREP_SORT is `sort`."""
    import os

    old = os.environ.get("TF_PREP_SORT")
    os.environ["TF_PREP_SORT"] = sort
    try:
        c = tf.TraceFEM()
    finally:
        if old is None:
            os.environ.pop("TF_PREP_SORT", None)
        else:
            os.environ["TF_PREP_SORT"] = old
    try:
        c.brick_cube(n, 5.0 / 3.0)
        c.levelset_analytic(kind, par, p2ls)
        c.distribute_dofs(fe)
        c.setup_fe_system([tf.FORM_M, tf.FORM_A, tf.FORM_CN], tf.RHS_SPHERE_XYZ, [0, 0, 0, 1.0, 13.0])
        return [c.matrix(f)[2] for f in (tf.FORM_M, tf.FORM_A, tf.FORM_CN)] + [c.vec_download(tf.VEC_RHS)]
    finally:
        c.close()


@pytest.mark.parametrize("fe,kind,par,p2ls", [(tf.P2IF, tf.LS_ELLIPSOID, ELLIPSOID, True),
                                              (tf.P1IF, tf.LS_SPHERE, [0, 0, 0, 1.0], False),
                                              (tf.P1IF, tf.LS_TORUS, [1.0, 0.4, 2], True)])
def test_prep_order_leaves_forms_unchanged(ctx, fe, kind, par, p2ls):
    """The pair forms' per-tet pass runs its threads ordered by the tets' sign patterns (the default) or in tet
    order (TF_PREP_SORT=0).  Each thread writes its own tet's record, so the forms are bit-identical."""
    a = _pair_forms("1", fe, kind, par, p2ls, 24)
    b = _pair_forms("0", fe, kind, par, p2ls, 24)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
