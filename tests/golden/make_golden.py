"""Regenerates the golden fixtures in this folder from the DROPS reference itself.

Runs oracle/_ref/ref_harness (built from the reference sources by
oracle/build_ref.sh) on small cases of the TraceFEM path and stores what the
reference computed as compressed .npz files.  Level-set values on edges are
re-indexed from the reference's edge order to this library's brick edge
numbering by the edge's two vertex indices (vertex order is identical).  Large
integer arrays that are only checked for bit-exactness are stored as SHA-256
digests.

    python tests/golden/make_golden.py            (needs the reference sources)
"""
import hashlib
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)
from oracle import pyoracle as O  # noqa: E402
from tfg import read_tfg  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def run(*args, keep_vec=None):
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "out.bin")
        subprocess.check_call([HARNESS, *args, out], cwd=d, stdout=subprocess.DEVNULL)
        if keep_vec and os.path.exists(out + ".vec"):  # VecDescCL::Write(binary) of the solution
            with open(out + ".vec", "rb") as src, open(os.path.join(HERE, keep_vec), "wb") as dst:
                dst.write(src.read())
        return read_tfg(out)


def edge_map(mesh, ref_edge_v):
    key = {tuple(sorted(p)): i for i, p in enumerate(mesh.edge_v.tolist())}
    return np.array([key[tuple(sorted(p))] for p in ref_edge_v.reshape(-1, 2).tolist()], dtype=np.int64)


def system_case(name, fe, ls, shape, n, a, solve, keep_vec=None):
    d = run("system", fe, ls, shape, str(n), repr(a), "1" if solve else "0", keep_vec=keep_vec)
    mesh = O.brick(n, a=a)
    emap = edge_map(mesh, d["edge_v"])
    ls_edge = np.empty(mesh.ne)
    ls_edge[emap] = d["ls_edge"]
    tev = np.sort(d["tet_ev"].reshape(-1, 6, 2), axis=2)
    out = dict(
        n=n, a=a, p2=int(fe == "p2"), ls_p2=int(ls == "lsP2"), shape=shape,
        coords_sha=sha(d["coords"]), tet_v_sha=sha(d["tet_v"].astype(np.int64)),
        tet_edge_pairs_sha=sha(tev.astype(np.int64)),
        ls_vert=d["ls_vert"], ls_edge=ls_edge,
        n_active=int(d["n_active"][0]), n_dofs=int(d["n_dofs"][0]),
        active_tets=d["active_tets"].astype(np.int32), loc2glo=d["loc2glo"].astype(np.int32),
        rowptr=d["M.rowptr"], colind=d["M.colind"].astype(np.int32),
        M=d["M.vals"], A=d["A.vals"], C=d["C.vals"], rhs=d["rhs"],
        ref_time_dofs=d["time_dofs"][0], ref_time_assemble=d["time_assemble"][0],
    )
    if "N.vals" in d:
        # N_P1P1 with the harness wind; nodal wind values per vertex / edge (xyz), edges in this library's order
        assert np.array_equal(d["N.rowptr"], d["M.rowptr"]) and np.array_equal(d["N.colind"], d["M.colind"])
        wind_edge = np.empty((mesh.ne, 3))
        wind_edge[emap] = d["wind_edge"].reshape(-1, 3)
        out.update(N=d["N.vals"], wind_vert=d["wind_vert"].reshape(-1, 3), wind_edge=wind_edge)
    if "LapM.vals" in d:
        # LaplaceM_P1P1 with the degenerate mobility of the harness chi (per interface DOF)
        assert np.array_equal(d["LapM.rowptr"], d["M.rowptr"]) and np.array_equal(d["LapM.colind"], d["M.colind"])
        out.update(LapM=d["LapM.vals"], chi=d["chi"])
    if solve:
        assert np.array_equal(d["S.rowptr"], d["M.rowptr"]) and np.array_equal(d["S.colind"], d["M.colind"])
        out.update(S=d["S.vals"], x=d["x"], iters=int(d["iters"][0]), resid=float(d["resid"][0]),
                   ref_time_solve=d["time_solve"][0])
    np.savez_compressed(os.path.join(HERE, name), **out)
    print(name, "active", out["n_active"], "dofs", out["n_dofs"], "nnz", len(out["colind"]))


def refine_case(name, fe, ls, shape, n, a, width, clevel, flevel, solve):
    """Narrow-band refinement of the brick (AdapTriangCL::MakeInitialTriang with DistMarkingStrategyCL) and the
    TraceFEM system on the last triangulation level.  The mesh is pinned by the per-level tet counts, each
    triangulation tet's level and a digest of its four vertices' coordinates in order (independent of how the
    vertices are numbered)."""
    d = run("system_ref", fe, ls, shape, str(n), repr(a), "1" if solve else "0", repr(width), str(clevel),
            str(flevel))
    tet_xyz = d["coords"].reshape(-1, 3)[d["tet_v"].reshape(-1, 4)]
    out = dict(
        n=n, a=a, width=width, clevel=clevel, flevel=flevel, p2=int(fe == "p2"), ls_p2=int(ls == "lsP2"),
        shape=shape, tets_per_level=d["tets_per_level"], tet_level=d["tet_level"].astype(np.int8),
        tet_xyz_sha=sha(tet_xyz), nt=len(d["tet_level"]), ref_time_refine=d["time_refine"][0],
        n_active=int(d["n_active"][0]), n_dofs=int(d["n_dofs"][0]),
        active_tets=d["active_tets"].astype(np.int32), loc2glo=d["loc2glo"].astype(np.int32),
        rowptr=d["M.rowptr"], colind=d["M.colind"].astype(np.int32),
        M=d["M.vals"], A=d["A.vals"], C=d["C.vals"], rhs=d["rhs"],
    )
    if solve:
        assert np.array_equal(d["S.rowptr"], d["M.rowptr"]) and np.array_equal(d["S.colind"], d["M.colind"])
        out.update(S=d["S.vals"], x=d["x"], iters=int(d["iters"][0]), resid=float(d["resid"][0]))
    np.savez_compressed(os.path.join(HERE, name), **out)
    print(name, "levels", out["tets_per_level"].tolist(), "tets", out["nt"], "dofs", out["n_dofs"])


REFINE_MESHES = [  # shape, n, a, width, coarse, fine
    ("sphere", 6, 5.0 / 3.0, 0.2, 0, 3),
    ("torus", 5, 1.6, 0.05, 0, 3),
    ("sphere", 5, 5.0 / 3.0, 0.0, 1, 2),
    ("torus", 4, 1.6, 0.3, 1, 3),
    ("sphere", 3, 5.0 / 3.0, 0.5, 0, 4),
]


def refine_meshes_case():
    """Refined meshes only (up to four levels, 330k tets), pinned by digests."""
    rows = []
    for shape, n, a, width, cl, fl in REFINE_MESHES:
        d = run("system_ref", "p1", "lsP2", shape, str(n), repr(a), "-1", repr(width), str(cl), str(fl))
        tet_xyz = d["coords"].reshape(-1, 3)[d["tet_v"].reshape(-1, 4)]
        rows.append(dict(per_level=d["tets_per_level"], xyz=sha(tet_xyz), lvl=sha(d["tet_level"].astype(np.int8)),
                         t=d["time_refine"][0]))
    np.savez_compressed(
        os.path.join(HERE, "refine_meshes.npz"),
        shape=np.array([c[0] for c in REFINE_MESHES]), n=np.array([c[1] for c in REFINE_MESHES]),
        a=np.array([c[2] for c in REFINE_MESHES]), width=np.array([c[3] for c in REFINE_MESHES]),
        clevel=np.array([c[4] for c in REFINE_MESHES]), flevel=np.array([c[5] for c in REFINE_MESHES]),
        per_level=np.array([",".join(map(str, r["per_level"].tolist())) for r in rows]),
        tet_xyz_sha=np.array([r["xyz"] for r in rows]), tet_level_sha=np.array([r["lvl"] for r in rows]),
        ref_time_refine=np.array([r["t"] for r in rows]))
    print("refine meshes", [r["per_level"].tolist() for r in rows])


def ch_refined_case(n=6, a=1.62, width=0.1, clevel=0, flevel=2, steps=3):
    """Cahn-Hilliard BDF1 steps (the reference's block constructor and GMRES(50)) on the brick refined
    towards the torus first, as the surface driver does (surfphasesep.cpp:170-181, 414-440)."""
    d = run("gmres_ref", str(n), repr(a), str(steps), repr(width), str(clevel), str(flevel))
    tet_xyz = d["coords"].reshape(-1, 3)[d["tet_v"].reshape(-1, 4)]
    m = int(d["n_dofs"][0])
    out = dict(n=n, a=a, width=width, clevel=clevel, flevel=flevel, tet_xyz_sha=sha(tet_xyz), n_dofs=m,
               dt=d["dt"][0], eps=d["eps"][0], rho=d["rho"][0], beta_s=d["beta_s"][0], xi=d["xi"][0],
               chi0=d["chi0"], block_iters=int(d["block_iters"][0]), block_x=d["block_x"],
               steps_iters=d["steps_iters"], steps_X=d["steps_X"].reshape(steps, 2 * m))
    np.savez_compressed(os.path.join(HERE, f"ch_torus_refined_n{n}.npz"), **out)
    print("ch refined", n, "dofs", m, "block", out["block_iters"], "steps", out["steps_iters"].tolist())


def rules_case():
    """The 64 refinement rules of geom/topo.cpp: children per edge pattern, local points in order."""
    d = run("rules")
    np.savez_compressed(os.path.join(HERE, "refine_rules.npz"), nch=d["nch"].astype(np.int32),
                        children=d["children"].astype(np.int32).reshape(64, 8, 4))


def area_case():
    d = run("area")
    np.savez_compressed(
        os.path.join(HERE, "area_sphere05_n8.npz"), surface=d["surface"][0], per_tet=d["per_tet"],
        n_facets=d["n_facets"].astype(np.int32), patch_tets=d["patch_tets"].astype(np.int32),
        patch_nverts=d["patch_nverts"].astype(np.int32), patch_facets=d["patch_facets"].astype(np.int32),
        patch_boundary=d["patch_boundary"].astype(np.int32), patch_verts=d["patch_verts"],
        tet_v_sha=sha(d["tet_v"].astype(np.int64)), coords_sha=sha(d["coords"]))
    print("area", d["surface"][0])


def legacy_case():
    out = {}
    for c in ("plane", "plane2", "sphere"):
        d = run("legacy_numb", c)
        out[c + "_status"] = int(d["status"][0])
        out[c + "_n_dofs"] = int(d["n_dofs"][0])
        out[c + "_n_active"] = int(d["n_active"][0])
        if "dof_vert" in d:
            out[c + "_dof_vert"] = d["dof_vert"].astype(np.int32)
    np.savez_compressed(os.path.join(HERE, "legacy_numbering.npz"), **out)
    print("legacy", {k: v for k, v in out.items() if not k.endswith("dof_vert")})


def legacy_forms_case(n=10, a=1.6):
    d = run("legacy_forms", str(n), repr(a))
    mesh = O.brick(n, a=a)
    emap = edge_map(mesh, d["edge_v"])
    ls_edge = np.empty(mesh.ne)
    ls_edge[emap] = d["ls_edge"]
    np.savez_compressed(
        os.path.join(HERE, f"legacy_forms_sphere_n{n}.npz"), n=n, a=a, alpha=float(d["alpha"][0]), D=float(d["D"][0]),
        ls_vert=d["ls_vert"], ls_edge=ls_edge, dof_vert=d["dof_vert"].astype(np.int32),
        n_active=int(d["n_active"][0]), n_dofs=int(d["n_dofs"][0]),
        rowptr=d["M.rowptr"], colind=d["M.colind"].astype(np.int32), M=d["M.vals"],
        A_rowptr=d["A.rowptr"], A_colind=d["A.colind"].astype(np.int32), A=d["A.vals"], rhs=d["rhs"],
        tet_v_sha=sha(d["tet_v"].astype(np.int64)), coords_sha=sha(d["coords"]))
    print("legacy forms", n, "dofs", int(d["n_dofs"][0]), "nnz", len(d["M.colind"]))


def ch_case(n=16, a=1.6, steps=3):
    """GMRES with point Jacobi (both sides) on M + A + h C_n, the 2x2 Cahn-Hilliard block matrix and
    warm-started BDF1 steps (plain; degenerate mobility + wind) on the P1 torus, all by the reference's
    own GMRES and block constructor."""
    d = run("gmres", str(n), repr(a), str(steps))
    t = np.load(os.path.join(HERE, "torus_p1_n16.npz"))
    assert np.array_equal(d["M.rowptr"], t["rowptr"]) and np.array_equal(d["M.colind"], t["colind"])
    assert np.array_equal(d["M.vals"], t["M"]) and np.array_equal(d["S.vals"], t["S"]) and np.array_equal(d["rhs"], t["rhs"])
    out = dict(n=n, a=a, n_dofs=int(d["n_dofs"][0]))
    for k in ("dt", "eps", "rho", "beta_s", "xi"):
        out[k] = float(d[k][0])
    for side in ("right", "left"):
        assert int(d[f"gmres_{side}_ok"][0]) == 1
        out[f"gmres_{side}_iters"] = int(d[f"gmres_{side}_iters"][0])
        out[f"gmres_{side}_resid"] = float(d[f"gmres_{side}_resid"][0])
        out[f"gmres_{side}_x"] = d[f"gmres_{side}_x"]
    out.update(chi0=d["chi0"], B_rowptr=d["B.rowptr"], B_colind=d["B.colind"].astype(np.int32), B=d["B.vals"])
    assert int(d["block_ok"][0]) == 1
    out.update(block_iters=int(d["block_iters"][0]), block_resid=float(d["block_resid"][0]), block_x=d["block_x"])
    out.update(steps_iters=d["steps_iters"].astype(np.int32), steps_resid=d["steps_resid"],
               steps_X=d["steps_X"].reshape(steps, -1))
    assert np.array_equal(d["dm_B0.rowptr"], d["B.rowptr"]) and np.array_equal(d["dm_B0.colind"], d["B.colind"])
    out.update(dm_chi0=d["dm_chi0"], dm_B0=d["dm_B0.vals"], dm_steps_iters=d["dm_steps_iters"].astype(np.int32),
               dm_steps_resid=d["dm_steps_resid"], dm_steps_X=d["dm_steps_X"].reshape(steps, -1))
    np.savez_compressed(os.path.join(HERE, f"ch_torus_p1_n{n}.npz"), **out)
    print("ch", n, "dofs", out["n_dofs"], "gmres", out["gmres_right_iters"], out["gmres_left_iters"], "block",
          out["block_iters"], "steps", out["steps_iters"].tolist(), "dm steps", out["dm_steps_iters"].tolist())


def quaqua_case(n=8, a=5.0 / 3.0):
    """Isoparametric P2 TraceFEM with the reference's QuaQua mapper on the unit sphere: the recovered
    gradient, LocalMassP2CL, LocalLaplaceBeltramiP2CL and LocalVectorP2CL (f = 13 xyz at the base points)."""
    d = run("quaqua", str(n), repr(a))
    mesh = O.brick(n, a=a)
    emap = edge_map(mesh, d["edge_v"])
    lv, le = O.levelset(mesh, O.LS_SPHERE, [0, 0, 0, 1.0], True)
    assert np.array_equal(lv, d["ls_vert"]) and np.array_equal(le[emap], d["ls_edge"])
    grad_edge = np.empty((mesh.ne, 3))
    grad_edge[emap] = d["grad_edge"].reshape(-1, 3)
    out = dict(n=n, a=a, n_dofs=int(d["n_dofs"][0]), grad_vert=d["grad_vert"].reshape(-1, 3), grad_edge=grad_edge,
               M_rowptr=d["M.rowptr"], M_colind=d["M.colind"].astype(np.int32), M=d["M.vals"],
               A_rowptr=d["A.rowptr"], A_colind=d["A.colind"].astype(np.int32), A=d["A.vals"], rhs=d["rhs"])
    np.savez_compressed(os.path.join(HERE, f"quaqua_sphere_p2_n{n}.npz"), **out)
    print("quaqua", n, "dofs", out["n_dofs"], "nnz", len(out["M"]), "area", out["M"].sum())


if __name__ == "__main__":
    if not os.path.exists(HARNESS):
        subprocess.check_call([os.path.join(ROOT, "oracle", "build_ref.sh")])
    system_case("c1_sphere_p1_n16.npz", "p1", "lsP1", "sphere", 16, 5.0 / 3.0, True, keep_vec="c1_sphere_p1_n16_x.vec")
    system_case("sphere_p2_n8.npz", "p2", "lsP2", "sphere", 8, 5.0 / 3.0, True)
    system_case("torus_p1_n16.npz", "p1", "lsP1", "torus", 16, 1.6, True)
    system_case("torus_p2_n10.npz", "p2", "lsP2", "torus", 10, 1.6, False)
    area_case()
    legacy_case()
    legacy_forms_case()
    ch_case()
    quaqua_case()
    refine_case("refine_sphere_p1_n4.npz", "p1", "lsP2", "sphere", 4, 5.0 / 3.0, 0.1, 0, 2, True)
    refine_case("refine_torus_p2_n3.npz", "p2", "lsP2", "torus", 3, 1.62, 0.05, 0, 1, False)
    rules_case()
    refine_meshes_case()
    ch_refined_case()
