"""Narrow-band refinement on the host against the reference: the sequential form (tf_refine_band) and the
device engine's kernel bodies run as host loops.

The fixtures come from the reference's own AdapTriangCL::MakeInitialTriang with DistMarkingStrategyCL
(oracle/ref_harness.cpp system_ref, tests/golden/make_golden.py): per-level tet counts, each triangulation tet's
level and a digest of its vertices' coordinates in tet order and local vertex order.  The refinement rules are
compared with the reference's table of geom/topo.cpp.  No device is needed; tests/test_gpu_refine.py runs the
device engine.
"""
import hashlib

import numpy as np
import pytest

import drops_gb300 as tf
from oracle import pyoracle as O
from tests.helpers import loc2glo

SPHERE = [0.0, 0.0, 0.0, 1.0]
TORUS = [1.0, 0.4, 2]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def kind_par(shape):
    return (tf.LS_SPHERE, SPHERE) if shape == "sphere" else (tf.LS_TORUS, TORUS)


def refined(shape, n, a, width, cl, fl):
    om = O.brick(int(n), a=float(a))
    kind, par = kind_par(shape)
    return tf.refine_band(om.coords, om.tet_v, kind, par, float(width), int(cl), int(fl))


def test_rules_match_reference(golden):
    g = golden("refine_rules.npz")
    nch, ch = tf.refine_rules()
    assert np.array_equal(nch, g["nch"])
    assert np.array_equal(ch, g["children"])
    # rule 0 keeps the tet, rule 63 is the regular red refinement into eight children
    assert nch[0] == 1 and list(ch[0, 0]) == [0, 1, 2, 3] and nch[63] == 8


def _rows():
    import os

    path = os.path.join(os.path.dirname(__file__), "golden", "refine_meshes.npz")
    g = np.load(path)
    return [(str(g["shape"][i]), int(g["n"][i]), float(g["a"][i]), float(g["width"][i]), int(g["clevel"][i]),
             int(g["flevel"][i]), i) for i in range(len(g["n"]))]


@pytest.mark.parametrize("shape,n,a,width,cl,fl,i", _rows())
def test_refined_mesh_matches_reference(golden, shape, n, a, width, cl, fl, i):
    """Tet order, local vertex order and coordinates bit for bit, up to four levels and 330k tets."""
    g = golden("refine_meshes.npz")
    r = refined(shape, n, a, width, cl, fl)
    assert ",".join(map(str, r["tets_per_level"].tolist())) == str(g["per_level"][i])
    assert r["last_level"] == fl
    assert sha(r["tet_level"].astype(np.int8)) == str(g["tet_level_sha"][i])
    assert sha(r["coords"][r["tet_v"]]) == str(g["tet_xyz_sha"][i])
    # a conforming mesh: every interior face is shared by exactly two tets
    faces = np.sort(r["tet_v"][:, [[1, 2, 3], [0, 2, 3], [0, 1, 3], [0, 1, 2]]].reshape(-1, 3), axis=1)
    _, cnt = np.unique(faces, axis=0, return_counts=True)
    assert cnt.max() == 2
    # the tets fill the box: volumes add up to (2a)^3
    X = r["coords"][r["tet_v"]]
    vol = np.abs(np.linalg.det(X[:, 1:] - X[:, :1])).sum() / 6.0
    assert abs(vol - (2 * a) ** 3) <= 1e-9 * (2 * a) ** 3


def parallel_host(shape, n, a, width, cl, fl):
    """The device engine's kernel bodies run as host loops (tf_refine_band_parallel_host, outside the header)."""
    import ctypes as C

    L = tf.load_library()
    om = O.brick(int(n), a=float(a))
    kind, par = kind_par(shape)
    par = np.asarray(par, np.float64)
    h = C.c_void_p()
    st = L.tf_refine_band_parallel_host(C.c_int64(len(om.coords)), om.coords.ctypes.data_as(C.c_void_p),
                                        C.c_int64(len(om.tet_v)), om.tet_v.ctypes.data_as(C.c_void_p), C.c_int(kind),
                                        par.ctypes.data_as(C.c_void_p), C.c_int(len(par)), C.c_double(width),
                                        C.c_int(cl), C.c_int(fl), C.byref(h))
    assert st == tf.OK, st
    nv, ne, nt = C.c_int64(), C.c_int64(), C.c_int64()
    ll, steps = C.c_int(), C.c_int()
    L.tf_refined_info(h, C.byref(nv), C.byref(ne), C.byref(nt), C.byref(ll), C.byref(steps))
    co = np.empty((nv.value, 3))
    tv = np.empty((nt.value, 4), np.int32)
    tl = np.empty(nt.value, np.int32)
    pl = np.empty(ll.value + 1, np.int64)
    p = lambda x: x.ctypes.data_as(C.c_void_p)
    L.tf_refined_get(h, p(co), p(tv), None, None, p(tl), p(pl))
    L.tf_refined_free(h)
    return co, tv, tl, pl


@pytest.mark.parametrize("shape,n,a,width,cl,fl,i", _rows())
def test_parallel_engine_matches_reference(golden, shape, n, a, width, cl, fl, i):
    """The data-parallel engine (level-synchronous passes, scans, two-phase edge table) gives the reference's
    mesh bit for bit; on the device the same bodies run as kernels."""
    g = golden("refine_meshes.npz")
    co, tv, tl, pl = parallel_host(shape, n, a, width, cl, fl)
    assert ",".join(map(str, pl.tolist())) == str(g["per_level"][i])
    assert sha(tl.astype(np.int8)) == str(g["tet_level_sha"][i])
    assert sha(co[tv]) == str(g["tet_xyz_sha"][i])


@pytest.mark.parametrize("name", ["refine_sphere_p1_n4.npz", "refine_torus_p2_n3.npz"])
def test_refined_system_mesh_and_oracle_numbering(golden, name):
    """The system fixtures' meshes, and the first-touch numbering of the oracle on the refined mesh against
    the reference's DistributeDOFs there (the checker the GPU tests use is valid on refined meshes)."""
    g = golden(name)
    shape = str(g["shape"])
    r = refined(shape, g["n"], g["a"], g["width"], g["clevel"], g["flevel"])
    assert np.array_equal(r["tets_per_level"], g["tets_per_level"])
    assert np.array_equal(r["tet_level"].astype(np.int8), g["tet_level"])
    assert sha(r["coords"][r["tet_v"]]) == str(g["tet_xyz_sha"])
    mesh = O.Mesh(r["coords"], r["tet_v"], r["tet_e"], r["edge_v"])
    kind, par = kind_par(shape)
    lv, le = O.levelset(mesh, kind, par, bool(g["ls_p2"]))
    p2 = bool(g["p2"])
    st, na, nd, dv, de, act = O.distribute_dofs(mesh, lv, le, p2)
    assert st == 0 and na == int(g["n_active"]) and nd == int(g["n_dofs"])
    assert np.array_equal(np.nonzero(act)[0], g["active_tets"])
    assert np.array_equal(loc2glo(mesh, act, dv, de, p2), g["loc2glo"])


def test_refine_fine_level_zero_is_the_brick():
    om = O.brick(3, a=1.0)
    r = tf.refine_band(om.coords, om.tet_v, tf.LS_SPHERE, SPHERE, 0.1, 0, 0)
    assert r["last_level"] == 0 and r["steps"] == 0
    assert np.array_equal(r["coords"][r["tet_v"]], om.coords[om.tet_v])


def test_refine_rejects_bad_input():
    om = O.brick(2, a=1.0)
    with pytest.raises(tf.TraceFEMError):  # fine level below coarse level
        tf.refine_band(om.coords, om.tet_v, tf.LS_SPHERE, SPHERE, 0.1, 2, 1)
    with pytest.raises(tf.TraceFEMError):  # unknown distance kind
        tf.refine_band(om.coords, om.tet_v, 7, SPHERE, 0.1, 0, 1)
    with pytest.raises(tf.TraceFEMError):  # too few parameters
        tf.refine_band(om.coords, om.tet_v, tf.LS_SPHERE, [0.0, 0.0], 0.1, 0, 1)
    with pytest.raises(tf.TraceFEMError):  # negative width
        tf.refine_band(om.coords, om.tet_v, tf.LS_SPHERE, SPHERE, -1.0, 0, 1)
    bad = om.tet_v.copy()
    bad[0] = bad[0][[1, 0, 2, 3]]  # one tet listing its vertices against the others' order
    with pytest.raises(tf.TraceFEMError):
        tf.refine_band(om.coords, bad, tf.LS_SPHERE, SPHERE, 0.1, 0, 1)
    bad = om.tet_v.copy()
    bad[0, 0] = len(om.coords)  # vertex out of range
    with pytest.raises(tf.TraceFEMError):
        tf.refine_band(om.coords, bad, tf.LS_SPHERE, SPHERE, 0.1, 0, 1)
