"""The C oracle against golden vectors produced by the DROPS reference itself.

Fixtures come from tests/golden/make_golden.py, which runs the reference's own
BrickBuilderCL, DistributeDOFs, setupFESystem and PCGSolverCL<JACPcCL>.  These
tests pin the oracle before it is used as the checker of the CUDA path.
"""
import numpy as np
import pytest

from oracle import pyoracle as O
from tests.helpers import loc2glo, mat_close, sha, sol_close

SYSTEMS = [
    ("c1_sphere_p1_n16.npz", O.LS_SPHERE, [0, 0, 0, 1.0]),
    ("sphere_p2_n8.npz", O.LS_SPHERE, [0, 0, 0, 1.0]),
    ("torus_p1_n16.npz", O.LS_TORUS, [1.0, 0.4, 2]),
    ("torus_p2_n10.npz", O.LS_TORUS, [1.0, 0.4, 2]),
]


@pytest.mark.parametrize("name,kind,par", SYSTEMS)
def test_mesh_levelset_dofs_bitexact(golden, name, kind, par):
    g = golden(name)
    mesh = O.brick(int(g["n"]), a=float(g["a"]))
    assert sha(mesh.coords.ravel()) == str(g["coords_sha"])
    assert sha(mesh.tet_v.astype(np.int64).ravel()) == str(g["tet_v_sha"])
    pairs = np.sort(mesh.edge_v[mesh.tet_e], axis=2).astype(np.int64)
    assert sha(pairs.ravel()) == str(g["tet_edge_pairs_sha"])
    lv, le = O.levelset(mesh, kind, par, p2=bool(g["ls_p2"]))
    assert np.array_equal(lv, g["ls_vert"]) and np.array_equal(le, g["ls_edge"])
    p2 = bool(g["p2"])
    st, na, nd, dv, de, act = O.distribute_dofs(mesh, lv, le, p2)
    assert st == O.OK and na == int(g["n_active"]) and nd == int(g["n_dofs"])
    assert np.array_equal(np.nonzero(act)[0], g["active_tets"])
    assert np.array_equal(loc2glo(mesh, act, dv, de, p2), g["loc2glo"])


@pytest.mark.parametrize("name,kind,par", SYSTEMS)
def test_assembly_matches_reference(golden, name, kind, par):
    g = golden(name)
    p2 = bool(g["p2"])
    mesh = O.brick(int(g["n"]), a=float(g["a"]))
    lv, le = O.levelset(mesh, kind, par, p2=bool(g["ls_p2"]))
    st, na, nd, dv, de, act = O.distribute_dofs(mesh, lv, le, p2)
    opts = O.make_opts(p2, [O.FORM_M, O.FORM_A, O.FORM_CN], O.RHS_SPHERE_XYZ, [0, 0, 0, 1.0, 13.0])
    st, rp, ci, vals, rhs = O.assemble(mesh, lv, le, act, dv, de, nd, opts)
    assert st == O.OK
    assert np.array_equal(rp, g["rowptr"]) and np.array_equal(ci, g["colind"])
    for f, key in ((O.FORM_M, "M"), (O.FORM_A, "A"), (O.FORM_CN, "C")):
        ok, err = mat_close(vals[f], g[key], g["rowptr"])
        assert ok, (key, err)
    ok, err = mat_close(rhs, g["rhs"])
    assert ok, err


@pytest.mark.parametrize("name,kind,par", [s for s in SYSTEMS if "p1" in s[0]])
def test_wind_convection_matches_reference(golden, name, kind, par):
    """N_P1P1 (surfactant/ifacetransp.h:1590-1600): int (w . grad_Gamma phi_j) phi_i with the reference's
    vecP2IF wind interpolated at vertices and edge midpoints; a form that is not symmetric."""
    g = golden(name)
    mesh = O.brick(int(g["n"]), a=float(g["a"]))
    lv, le = O.levelset(mesh, kind, par, p2=False)
    st, na, nd, dv, de, act = O.distribute_dofs(mesh, lv, le, False)
    opts = O.make_opts(False, [O.FORM_M, O.FORM_N], wind=(g["wind_vert"], g["wind_edge"]))
    st, rp, ci, vals, rhs = O.assemble(mesh, lv, le, act, dv, de, nd, opts)
    assert st == O.OK
    assert np.array_equal(rp, g["rowptr"]) and np.array_equal(ci, g["colind"])
    ok, err = mat_close(vals[O.FORM_N], g["N"], g["rowptr"])
    assert ok, err
    ok, err = mat_close(vals[O.FORM_M], g["M"], g["rowptr"])
    assert ok, err
    # not symmetric: N differs from its transpose
    import scipy.sparse as sp
    Nm = sp.csr_matrix((g["N"], g["colind"], g["rowptr"]))
    assert abs(Nm - Nm.T).max() > 1e-3 * abs(Nm).max()


@pytest.mark.parametrize("name,kind,par", [s for s in SYSTEMS if "p1" in s[0]])
def test_laplace_m_degenerate_matches_reference(golden, name, kind, par):
    """LaplaceM_P1P1 (surfactant/ifacetransp.h:1533-1544) with the degenerate mobility chi (1 - chi), cut off
    at 0 (buildMobility :1176-1190), chi given per interface DOF."""
    g = golden(name)
    mesh = O.brick(int(g["n"]), a=float(g["a"]))
    lv, le = O.levelset(mesh, kind, par, p2=False)
    st, na, nd, dv, de, act = O.distribute_dofs(mesh, lv, le, False)
    opts = O.make_opts(False, [O.FORM_LAPM], chi=g["chi"], degenerate=True)
    st, rp, ci, vals, rhs = O.assemble(mesh, lv, le, act, dv, de, nd, opts)
    assert st == O.OK and np.array_equal(ci, g["colind"])
    ok, err = mat_close(vals[O.FORM_LAPM], g["LapM"], g["rowptr"])
    assert ok, err


@pytest.mark.parametrize("name", ["c1_sphere_p1_n16.npz", "sphere_p2_n8.npz", "torus_p1_n16.npz"])
def test_pcg_jacobi_matches_reference(golden, name):
    g = golden(name)
    rp, ci = g["rowptr"], g["colind"]
    st, x, it, res = O.pcg_jacobi(rp, ci, g["S"], g["rhs"], tol=1e-10)
    assert st == O.OK and res <= 1e-10
    assert abs(it - int(g["iters"])) <= 1
    ok, err = sol_close(x, g["x"])
    assert ok, err


@pytest.mark.parametrize("side,method", [("right", 0), ("left", 1)])
def test_gmres_jacobi_matches_reference(golden, side, method):
    """DROPS GMRES(20) with JACPcCL (num/krylovsolver.h:320-463) on the torus system M + A + h C_n:
    the oracle takes the same iteration count and lands on the same solution."""
    t, g = golden("torus_p1_n16.npz"), golden("ch_torus_p1_n16.npz")
    st, x, it, res = O.gmres_jacobi(t["rowptr"], t["colind"], t["S"], t["rhs"], restart=20, tol=1e-10, method=method)
    assert st == O.OK and it == int(g[f"gmres_{side}_iters"])
    assert abs(res - float(g[f"gmres_{side}_resid"])) <= 1e-14
    ok, err = sol_close(x, g[f"gmres_{side}_x"], 1e-12)
    assert ok, err


def ch_rhs(t, chi, dt, beta, xi=1.0):
    """Right-hand side of a BDF1 Cahn-Hilliard step, f = 0 (surfphasesep.cpp:421-425)."""
    Mc = O.spmv(t["rowptr"], t["colind"], t["M"], chi)
    Mf = O.spmv(t["rowptr"], t["colind"], t["M"], xi * 2 * chi * (1 - chi) * (1 - 2 * chi))
    return np.concatenate([Mc / dt, beta * Mc - Mf])


def test_ch_block_and_gmres_match_reference(golden):
    """The 2x2 block matrix of surfphasesep.cpp:431-434 from the reference's block constructor
    (num/spmat.h:718-750) bit for bit, and DROPS GMRES(50) with nodal block Jacobi on it: the same
    iteration count, one solve from zero and three warm-started BDF1 steps."""
    t, g = golden("torus_p1_n16.npz"), golden("ch_torus_p1_n16.npz")
    rp, ci = t["rowptr"], t["colind"]
    dt, eps, rho, beta = float(g["dt"]), float(g["eps"]), float(g["rho"]), float(g["beta_s"])
    brp, bci, bv = O.ch_block(rp, ci, t["M"], t["A"], t["C"], 1 / dt, 1.0, rho, eps * eps, beta)
    assert np.array_equal(brp, g["B_rowptr"]) and np.array_equal(bci, g["B_colind"]) and np.array_equal(bv, g["B"])
    st, x, it, res = O.gmres_jacobi(brp, bci, bv, ch_rhs(t, g["chi0"], dt, beta), restart=50, tol=1e-10,
                                    max_iter=20000, block=True)
    assert st == O.OK and it == int(g["block_iters"])
    ok, err = sol_close(x, g["block_x"], 1e-12)
    assert ok, err
    m = len(rp) - 1
    X = np.concatenate([g["chi0"], np.zeros(m)])
    for k in range(len(g["steps_iters"])):
        st, X, it, res = O.gmres_jacobi(brp, bci, bv, ch_rhs(t, X[:m], dt, beta), x0=X, restart=50, tol=1e-10,
                                        max_iter=20000, block=True)
        assert st == O.OK and abs(it - int(g["steps_iters"][k])) <= 1, (k, it, g["steps_iters"])
        ok, err = sol_close(X, g["steps_X"][k], 1e-12)
        assert ok, (k, err)


def test_ch_steps_degenerate_mobility_wind_match_reference(golden):
    """BDF1 steps with LaplaceM_P1P1 reassembled from the current chi (degenerate mobility) and the wind
    block alpha M + N, against the reference's setupFESystem, block constructor and GMRES."""
    t, g = golden("torus_p1_n16.npz"), golden("ch_torus_p1_n16.npz")
    rp, ci = t["rowptr"], t["colind"]
    m = len(rp) - 1
    dt, eps, rho, beta = float(g["dt"]), float(g["eps"]), float(g["rho"]), float(g["beta_s"])
    mesh = O.brick(int(g["n"]), a=float(g["a"]))
    lv, le = O.levelset(mesh, O.LS_TORUS, [1.0, 0.4, 2], p2=False)
    st, na, nd, dv, de, act = O.distribute_dofs(mesh, lv, le, False)
    X = np.concatenate([g["dm_chi0"], np.zeros(m)])
    for k in range(len(g["dm_steps_iters"])):
        st, _, _, vals, _ = O.assemble(mesh, lv, le, act, dv, None, m,
                                       O.make_opts(False, [O.FORM_LAPM], chi=X[:m], degenerate=True))
        brp, bci, bv = O.ch_block(rp, ci, t["M"], t["A"], t["C"], 1 / dt, 1.0, rho, eps * eps, beta,
                                  Amob=vals[O.FORM_LAPM], N=t["N"])
        if k == 0:
            ok, err = mat_close(bv, g["dm_B0"], g["B_rowptr"], 1e-15)
            assert ok, err
        st, X, it, res = O.gmres_jacobi(brp, bci, bv, ch_rhs(t, X[:m], dt, beta), x0=X, restart=50, tol=1e-10,
                                        max_iter=20000, block=True)
        assert st == O.OK and abs(it - int(g["dm_steps_iters"][k])) <= 1, (k, it, g["dm_steps_iters"])
        ok, err = sol_close(X, g["dm_steps_X"][k], 1e-12)
        assert ok, (k, err)


def test_lincomb_matches_reference(golden):
    g = golden("c1_sphere_p1_n16.npz")
    h = 2 * float(g["a"]) / int(g["n"])
    ok, err = mat_close(g["M"] + g["A"] + h * g["C"], g["S"], g["rowptr"])
    assert ok, err


def test_surface_area_golden(golden):
    """tests/principallattice.cpp:316-347: area 3.0909 (rel 1e-4), per-tet areas and patches."""
    g = golden("area_sphere05_n8.npz")
    assert abs(float(g["surface"]) - 3.0909) / 3.0909 < 1e-4
    mesh = O.brick(8, a=1.0)
    assert sha(mesh.coords.ravel()) == str(g["coords_sha"])
    lv, le = O.levelset(mesh, O.LS_SPHERE, [0, 0, 0, 0.5], p2=True)
    # the reference test visits every tet (vertices with phi == 0 included);
    # the P1 hat functions sum to one, so the mass entries of a tet sum to its area
    opts = O.make_opts(False, [O.FORM_M])
    per_tet = np.zeros(mesh.nt)
    for t in range(mesh.nt):
        ls10 = np.concatenate([lv[mesh.tet_v[t]], le[mesh.tet_e[t]]])
        st, forms, _, nf = O.local_forms(mesh.coords[mesh.tet_v[t]], ls10, opts)
        assert st == O.OK and nf == int(g["n_facets"][t])
        per_tet[t] = forms[O.FORM_M].sum()
    assert np.abs(per_tet - g["per_tet"]).max() <= 1e-14
    assert abs(per_tet.sum() - float(g["surface"])) <= 1e-12
    fo = vo = 0
    for i, t in enumerate(g["patch_tets"]):
        ls10 = np.concatenate([lv[mesh.tet_v[t]], le[mesh.tet_e[t]]])
        st, f, b, v = O.make_patch(ls10)
        k = int(g["n_facets"][t])
        nv = int(g["patch_nverts"][i])
        assert st == O.OK
        assert np.array_equal(f, g["patch_facets"][3 * fo:3 * (fo + k)].reshape(-1, 3))
        assert np.array_equal(b, g["patch_boundary"][fo:fo + k])
        assert np.array_equal(v, g["patch_verts"][4 * vo:4 * (vo + nv)].reshape(-1, 4))
        fo += k
        vo += nv


def test_legacy_numbering_golden(golden):
    """tests/interfaceP1FE.cpp: 8 (plane), 1156 (sphere); a plane through
    vertices makes distance() throw in the reference as shipped."""
    g = golden("legacy_numbering.npz")
    cases = {
        "plane": ((10, 1, 1), [1, 0, 0, 0.41]),
        "plane2": ((10, 1, 1), [1, 0, 0, 0.4]),
        "sphere": ((20, 20, 20), None),
    }
    for c, (n, par) in cases.items():
        mesh = O.brick(n, orig=np.zeros(3), e=np.eye(3))
        if par is None:
            lv, le = O.levelset(mesh, O.LS_SPHERE, [0.5, 0.5, 0.5, 0.31], p2=True)
        else:
            lv, le = O.levelset(mesh, O.LS_PLANE, par, p2=True)
        st, na, nd, dv = O.numb_on_interface_p1(mesh, lv, le)
        if int(g[c + "_status"]) != 0:
            assert st == O.ERR_ZERO_NODE
            continue
        assert st == O.OK and nd == int(g[c + "_n_dofs"]) and na == int(g[c + "_n_active"])
        assert np.array_equal(dv, g[c + "_dof_vert"])
    assert int(g["sphere_n_dofs"]) == 1156 and int(g["plane_n_dofs"]) == 8


LEGACY_F = [1.0, 0, 0, -0.5, 0, 0, 0, 1.0, 0, 0]  # f = 1 + x y - z / 2, the harness's test function


def test_oracle_legacy_forms_match_reference(golden):
    """SetupInterfaceMassP1 (alpha on the off-diagonal only), SetupLBP1 (facet normals, no halving on lattice
    faces) and SetupInterfaceRhsP1 (planar pieces of the regular children) of the reference, on the unit sphere
    with the legacy interface numbering."""
    g = golden("legacy_forms_sphere_n10.npz")
    mesh = O.brick(int(g["n"]), a=float(g["a"]))
    st, rp, ci, M, A, rhs = O.assemble_legacy_p1(mesh, g["ls_vert"], g["ls_edge"], g["dof_vert"], int(g["n_dofs"]),
                                                 float(g["alpha"]), float(g["D"]), LEGACY_F)
    assert st == O.OK
    assert np.array_equal(rp, g["rowptr"]) and np.array_equal(ci, g["colind"])
    assert np.array_equal(g["A_rowptr"], g["rowptr"]) and np.array_equal(g["A_colind"], g["colind"])
    for v, ref in ((M, g["M"]), (A, g["A"]), (rhs, g["rhs"])):
        assert np.max(np.abs(v - ref)) <= 1e-12 * np.max(np.abs(ref)), np.max(np.abs(v - ref)) / np.max(np.abs(ref))


def test_vecdesc_binary_layout(golden):
    """VecDescBaseCL::Write(os, binary=true) (misc/problem.h:928-944), written by the reference itself: a
    64-bit count, then the doubles; the solution vector of the C1 system."""
    import os
    import struct

    path = os.path.join(os.path.dirname(__file__), "golden", "c1_sphere_p1_n16_x.vec")
    raw = open(path, "rb").read()
    (n,) = struct.unpack("<Q", raw[:8])
    x = np.frombuffer(raw[8:], dtype="<f8")
    g = golden("c1_sphere_p1_n16.npz")
    assert n == len(g["x"]) == len(x) and len(raw) == 8 + 8 * n
    assert np.array_equal(x, g["x"])


def quaqua_system(g, mesh, lv, le, grad):
    """The oracle's isoparametric P2 forms of the fixture's case, scattered in tet order."""
    import scipy.sparse as sp

    st, na, m, dv, de, act = O.distribute_dofs(mesh, lv, le, True)
    assert st == O.OK and m == int(g["n_dofs"])
    tets = np.nonzero(act)[0]
    M, A, b, npts, newton = O.quaqua_elements(mesh, lv, le, tets, grad=grad)
    I = np.concatenate([dv[mesh.tet_v[tets]], de[mesh.tet_e[tets]]], axis=1)
    rows, cols = np.repeat(I, 10, axis=1).ravel(), np.tile(I, (1, 10)).ravel()
    Ms = sp.coo_matrix((M.ravel(), (rows, cols)), shape=(m, m)).tocsr()
    As = sp.coo_matrix((A.ravel(), (rows, cols)), shape=(m, m)).tocsr()
    rhs = np.zeros(m)
    np.add.at(rhs, I.ravel(), b.ravel())
    return Ms, As, rhs, npts, newton


def test_quaqua_p2_matches_reference(golden):
    """Isoparametric P2 TraceFEM (surfactant.cpp:1581-1640): the recovered gradient
    (num/gradient_recovery.cpp:82), the QuaQua mapper (levelset/levelsetmapper.cpp, Newton form) and
    LocalMassP2CL / LocalLaplaceBeltramiP2CL / LocalVectorP2CL against the reference's own accumulation on
    the unit sphere (8^3 cubes)."""
    import scipy.sparse as sp

    from tests.helpers import sparse_close

    g = golden("quaqua_sphere_p2_n8.npz")
    n, a = int(g["n"]), float(g["a"])
    mesh = O.brick(n, a=a)
    lv, le = O.levelset(mesh, O.LS_SPHERE, [0, 0, 0, 1.0], True)
    gv, ge = O.grad_recovery(mesh, lv, le)
    assert np.abs(gv - g["grad_vert"]).max() <= 1e-14 and np.abs(ge - g["grad_edge"]).max() <= 1e-14
    Ms, As, rhs, npts, newton = quaqua_system(g, mesh, lv, le, (gv, ge))
    m = int(g["n_dofs"])
    Mg = sp.csr_matrix((g["M"], g["M_colind"], g["M_rowptr"]), shape=(m, m))
    Ag = sp.csr_matrix((g["A"], g["A_colind"], g["A_rowptr"]), shape=(m, m))
    for X, G in ((Ms, Mg), (As, Ag)):
        ok, err = sparse_close(X, G)
        assert ok, err
    ok, err = mat_close(rhs, g["rhs"])
    assert ok, err
    assert abs(Ms.sum() - 4 * np.pi) < 2e-2  # the discrete sphere's area
    assert newton.sum() > 0 and newton.max() <= 10 * npts.max()
