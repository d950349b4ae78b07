"""ctypes front end of the C oracle (oracle/tracefem_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as
the checker and by bench.py for the CPU baseline.  The product path never
imports it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libtf_oracle.so")

OK = 0
ERR_ZERO_NODE = 2
ERR_ZERO_PATTERN = 3
FORM_M, FORM_A, FORM_CN, FORM_LAPM, FORM_N = 0, 1, 2, 3, 4
NUM_FORMS = 5
LS_SPHERE, LS_TORUS, LS_ELLIPSOID, LS_PLANE = 0, 1, 2, 3
RHS_NONE, RHS_SPHERE_XYZ, RHS_CONST = 0, 1, 2


def build(force=False):
    """Compile the oracle with gcc (no contraction, so x86 and Arm agree)."""
    srcs = [os.path.join(HERE, f) for f in ("tracefem_oracle.c", "mlp_oracle.c")]
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= max(
        [os.path.getmtime(s) for s in srcs] + [os.path.getmtime(os.path.join(HERE, "tracefem_oracle.h"))]
    ):
        return LIB_PATH
    subprocess.check_call(
        ["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", *srcs, "-o", LIB_PATH, "-lm"]
    )
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        i64, i32p, f64p, u8p, i64p = C.c_int64, C.POINTER(C.c_int32), C.POINTER(C.c_double), C.POINTER(C.c_uint8), C.POINTER(C.c_int64)
        L.orc_brick_num_vertices.restype = i64
        L.orc_brick_num_edges.restype = i64
        L.orc_brick_num_tets.restype = i64
        L.orc_ls_value.restype = C.c_double
        L.orc_kahan_dot.restype = C.c_double
        L.orc_mlp_gradient.restype = C.c_double
        _lib = L
    return _lib


_CT_DTYPE = {C.c_int32: np.int32, C.c_int64: np.int64, C.c_double: np.float64, C.c_float: np.float32,
             C.c_uint8: np.uint8, C.c_uint16: np.uint16}


def _p(a, ct):
    """Pointer to a's data as ct*; a must already hold ct's type, contiguous (no silent reinterpretation)."""
    if a is None:
        return None
    want = _CT_DTYPE.get(ct)
    if want is not None and (a.dtype != want or not a.flags["C_CONTIGUOUS"]):
        raise TypeError(f"oracle argument: expected contiguous {np.dtype(want).name}, got {a.dtype}")
    return a.ctypes.data_as(C.POINTER(ct))


def _in(a, dtype):
    """Input array as contiguous dtype (a converted copy is kept alive by the caller's local name)."""
    return None if a is None else np.ascontiguousarray(a, dtype=dtype)


class Mesh:
    def __init__(self, coords, tet_v, tet_e, edge_v):
        self.coords, self.tet_v, self.tet_e, self.edge_v = coords, tet_v, tet_e, edge_v
        self.nv = coords.shape[0]
        self.nt = tet_v.shape[0]
        self.ne = edge_v.shape[0]


def brick(n, a=None, orig=None, e=None):
    """BrickBuilderCL over [-a,a]^3 with n^3 cubes (or explicit orig / e1,e2,e3)."""
    L = lib()
    if isinstance(n, int):
        n = (n, n, n)
    if orig is None:
        orig = np.array([-a, -a, -a], dtype=np.float64)
        e = np.diag([2.0 * a] * 3)
    orig = np.ascontiguousarray(orig, dtype=np.float64)
    e = np.ascontiguousarray(e, dtype=np.float64)
    nv = L.orc_brick_num_vertices(*n)
    ne = L.orc_brick_num_edges(*n)
    nt = L.orc_brick_num_tets(*n)
    coords = np.empty((nv, 3), np.float64)
    tet_v = np.empty((nt, 4), np.int32)
    tet_e = np.empty((nt, 6), np.int32)
    edge_v = np.empty((ne, 2), np.int32)
    L.orc_brick(_p(orig, C.c_double), _p(e[0].copy(), C.c_double), _p(e[1].copy(), C.c_double),
                _p(e[2].copy(), C.c_double), C.c_int(n[0]), C.c_int(n[1]), C.c_int(n[2]),
                _p(coords, C.c_double), _p(tet_v, C.c_int32), _p(tet_e, C.c_int32), _p(edge_v, C.c_int32))
    return Mesh(coords, tet_v, tet_e, edge_v)


def levelset(mesh, kind, par, p2):
    L = lib()
    par = np.ascontiguousarray(par, dtype=np.float64)
    lv = np.empty(mesh.nv, np.float64)
    le = np.empty(mesh.ne, np.float64)
    L.orc_levelset(C.c_int(kind), _p(par, C.c_double), C.c_int(int(p2)), C.c_int64(mesh.nv), C.c_int64(mesh.ne),
                   _p(mesh.coords, C.c_double), _p(mesh.edge_v, C.c_int32), _p(lv, C.c_double), _p(le, C.c_double))
    return lv, le


def distribute_dofs(mesh, ls_vert, ls_edge, p2, dist=0.0):
    L = lib()
    ls_vert, ls_edge = _in(ls_vert, np.float64), _in(ls_edge, np.float64)
    na, nd = C.c_int64(), C.c_int64()
    dv = np.empty(mesh.nv, np.int32)
    de = np.empty(mesh.ne, np.int32)
    act = np.empty(mesh.nt, np.uint8)
    st = L.orc_distribute_dofs(C.c_int64(mesh.nt), _p(mesh.tet_v, C.c_int32), _p(mesh.tet_e, C.c_int32),
                               C.c_int64(mesh.nv), C.c_int64(mesh.ne), _p(ls_vert, C.c_double),
                               _p(ls_edge, C.c_double), C.c_int(int(p2)), C.c_double(dist), C.byref(na),
                               C.byref(nd), _p(dv, C.c_int32), _p(de, C.c_int32), _p(act, C.c_uint8))
    return st, na.value, nd.value, dv, (de if p2 else None), act


def numb_on_interface_p1(mesh, ls_vert, ls_edge, omit_bound=-1.0):
    L = lib()
    ls_vert, ls_edge = _in(ls_vert, np.float64), _in(ls_edge, np.float64)
    na, nd = C.c_int64(), C.c_int64()
    dv = np.empty(mesh.nv, np.int32)
    st = L.orc_numb_on_interface_p1(C.c_int64(mesh.nt), _p(mesh.tet_v, C.c_int32), _p(mesh.tet_e, C.c_int32),
                                    C.c_int64(mesh.nv), _p(mesh.coords, C.c_double), _p(ls_vert, C.c_double),
                                    _p(ls_edge, C.c_double), C.c_double(omit_bound), C.byref(na), C.byref(nd),
                                    _p(dv, C.c_int32))
    return st, na.value, nd.value, dv


class PatchT(C.Structure):
    _fields_ = [("n_facets", C.c_int), ("n_verts", C.c_int), ("n_cut_verts", C.c_int),
                ("facet", (C.c_int * 3) * 16), ("boundary", C.c_int * 16), ("bary", (C.c_double * 4) * 40)]


def make_patch(ls10):
    L = lib()
    ls10 = np.ascontiguousarray(ls10, dtype=np.float64)
    P = PatchT()
    st = L.orc_make_patch(_p(ls10, C.c_double), C.byref(P))
    facets = np.array([[P.facet[i][j] for j in range(3)] for i in range(P.n_facets)], dtype=np.int64).reshape(-1, 3)
    bnd = np.array([P.boundary[i] for i in range(P.n_facets)], dtype=np.int64)
    verts = np.array([[P.bary[i][j] for j in range(4)] for i in range(P.n_verts)]).reshape(-1, 4)
    return st, facets, bnd, verts


class AssembleOpts(C.Structure):
    _fields_ = [("p2", C.c_int), ("forms", C.c_uint), ("rhs_kind", C.c_int), ("rhs_par", C.c_double * 8),
                ("chi", C.POINTER(C.c_double)), ("degenerate", C.c_int),
                ("wind_vert", C.POINTER(C.c_double)), ("wind_edge", C.POINTER(C.c_double))]


def make_opts(p2, forms, rhs_kind=RHS_NONE, rhs_par=(), chi=None, degenerate=False, wind=None):
    """wind: (wind_vert (nv, 3), wind_edge (ne, 3)) for FORM_N, the P2 wind at vertices and edge midpoints."""
    o = AssembleOpts()
    o.p2 = int(p2)
    o.forms = sum(1 << f for f in forms)
    o.rhs_kind = rhs_kind
    for i, v in enumerate(rhs_par):
        o.rhs_par[i] = v
    chi = _in(chi, np.float64)
    o._chi_keep = chi
    o.chi = _p(chi, C.c_double) if chi is not None else None
    o.degenerate = int(degenerate)
    if wind is not None:
        wv, we = (_in(np.asarray(w, dtype=np.float64).reshape(-1), np.float64) for w in wind)
        o._wind_keep = (wv, we)
        o.wind_vert, o.wind_edge = _p(wv, C.c_double), _p(we, C.c_double)
    return o


def assemble(mesh, ls_vert, ls_edge, active, dof_vert, dof_edge, m, opts):
    """Returns (status, rowptr, colind, {form: vals}, rhs)."""
    L = lib()
    ls_vert, ls_edge = _in(ls_vert, np.float64), _in(ls_edge, np.float64)
    active, dof_vert, dof_edge = _in(active, np.uint8), _in(dof_vert, np.int32), _in(dof_edge, np.int32)
    rowptr = np.empty(m + 1, np.int64)
    colind_p = C.POINTER(C.c_int32)()
    nnz = C.c_int64()
    vals_p = (C.POINTER(C.c_double) * NUM_FORMS)()
    rhs = np.empty(m, np.float64)
    st = L.orc_assemble(C.c_int64(mesh.nt), _p(mesh.tet_v, C.c_int32), _p(mesh.tet_e, C.c_int32),
                        _p(mesh.coords, C.c_double), _p(ls_vert, C.c_double), _p(ls_edge, C.c_double),
                        _p(active, C.c_uint8), _p(dof_vert, C.c_int32),
                        _p(dof_edge, C.c_int32) if dof_edge is not None else None, C.c_int64(m), C.byref(opts),
                        _p(rowptr, C.c_int64), C.byref(colind_p), C.byref(nnz), vals_p, _p(rhs, C.c_double))
    if st != OK:
        return st, None, None, None, None
    libc = C.CDLL(None)
    n = nnz.value
    colind = np.ctypeslib.as_array(colind_p, shape=(max(n, 1),))[:n].copy()
    libc.free(colind_p)
    vals = {}
    for f in range(NUM_FORMS):
        if vals_p[f]:
            vals[f] = np.ctypeslib.as_array(vals_p[f], shape=(max(n, 1),))[:n].copy()
            libc.free(vals_p[f])
    return st, rowptr, colind, vals, rhs


def spmv(rowptr, colind, vals, x):
    L = lib()
    m = len(rowptr) - 1
    y = np.empty(m, np.float64)
    rowptr = np.ascontiguousarray(rowptr, dtype=np.int64)
    colind = np.ascontiguousarray(colind, dtype=np.int32)
    vals = np.ascontiguousarray(vals, dtype=np.float64)
    L.orc_spmv(C.c_int64(m), _p(rowptr, C.c_int64), _p(colind, C.c_int32), _p(vals, C.c_double),
               _p(np.ascontiguousarray(x, dtype=np.float64), C.c_double), _p(y, C.c_double))
    return y


def pcg_jacobi(rowptr, colind, vals, b, x0=None, max_iter=100000, tol=1e-10, rel=True):
    L = lib()
    rowptr, colind, vals = _in(rowptr, np.int64), _in(colind, np.int32), _in(vals, np.float64)
    m = len(rowptr) - 1
    x = np.zeros(m) if x0 is None else np.array(x0, dtype=np.float64)
    it = C.c_int(max_iter)
    t = C.c_double(tol)
    st = L.orc_pcg_jacobi(C.c_int64(m), _p(rowptr, C.c_int64), _p(colind, C.c_int32), _p(vals, C.c_double),
                          _p(np.ascontiguousarray(b, dtype=np.float64), C.c_double), _p(x, C.c_double),
                          C.byref(it), C.byref(t), C.c_int(int(rel)))
    return st, x, it.value, t.value


def gmres_jacobi(rowptr, colind, vals, b, x0=None, restart=50, max_iter=100000, tol=1e-10, rel=True, method=0,
                 block=False):
    L = lib()
    rowptr, colind, vals = _in(rowptr, np.int64), _in(colind, np.int32), _in(vals, np.float64)
    m = len(rowptr) - 1
    x = np.zeros(m) if x0 is None else np.array(x0, dtype=np.float64)
    it = C.c_int(max_iter)
    t = C.c_double(tol)
    st = L.orc_gmres(C.c_int64(m), _p(rowptr, C.c_int64), _p(colind, C.c_int32), _p(vals, C.c_double),
                     _p(np.ascontiguousarray(b, dtype=np.float64), C.c_double), _p(x, C.c_double),
                     C.c_int(restart), C.byref(it), C.byref(t), C.c_int(int(rel)), C.c_int(method), C.c_int(int(block)))
    return st, x, it.value, t.value


def ch_block(rowptr, colind, M, A, Cn, alpha, mob, rho, eps2, beta, Amob=None, N=None):
    """Block matrix of surfphasesep.cpp:431-434; Amob (A_deg) replaces A in the upper-right block, N is added to
    the upper-left one."""
    L = lib()
    rowptr, colind = _in(rowptr, np.int64), _in(colind, np.int32)
    M, A, Cn = _in(M, np.float64), _in(A, np.float64), _in(Cn, np.float64)
    Amob, N = _in(Amob, np.float64), _in(N, np.float64)
    m = len(rowptr) - 1
    nnz = len(colind)
    brp = np.empty(2 * m + 1, np.int64)
    bci = np.empty(4 * nnz, np.int32)
    bv = np.empty(4 * nnz, np.float64)
    L.orc_ch_block(C.c_int64(m), _p(rowptr, C.c_int64), _p(colind, C.c_int32), _p(M, C.c_double),
                   _p(A, C.c_double), _p(Cn, C.c_double), _p(Amob, C.c_double), _p(N, C.c_double),
                   C.c_double(alpha), C.c_double(mob), C.c_double(rho),
                   C.c_double(eps2), C.c_double(beta), _p(brp, C.c_int64), _p(bci, C.c_int32), _p(bv, C.c_double))
    return brp, bci, bv


def assemble_legacy_p1(mesh, ls_vert, ls_edge, dof_vert, m, alpha, D, fpar):
    """SetupInterfaceMassP1 / SetupLBP1 / SetupInterfaceRhsP1: (status, rowptr, colind, M, A, rhs)."""
    L = lib()
    rowptr = np.empty(m + 1, np.int64)
    colind_p = C.POINTER(C.c_int32)()
    m_p, a_p = C.POINTER(C.c_double)(), C.POINTER(C.c_double)()
    nnz = C.c_int64()
    rhs = np.empty(m, np.float64)
    fpar = np.ascontiguousarray(fpar, dtype=np.float64)
    dof_vert = np.ascontiguousarray(dof_vert, dtype=np.int32)
    ls_vert, ls_edge = _in(ls_vert, np.float64), _in(ls_edge, np.float64)
    st = L.orc_assemble_legacy_p1(C.c_int64(mesh.nt), _p(mesh.tet_v, C.c_int32), _p(mesh.tet_e, C.c_int32),
                                  _p(mesh.coords, C.c_double), _p(ls_vert, C.c_double), _p(ls_edge, C.c_double),
                                  _p(dof_vert, C.c_int32), C.c_int64(m), C.c_double(alpha), C.c_double(D),
                                  _p(fpar, C.c_double), _p(rowptr, C.c_int64), C.byref(colind_p), C.byref(nnz),
                                  C.byref(m_p), C.byref(a_p), _p(rhs, C.c_double))
    if st != OK:
        return st, None, None, None, None, None
    libc = C.CDLL(None)
    n = nnz.value
    take = lambda p, ct: np.ctypeslib.as_array(p, shape=(max(n, 1),))[:n].copy()
    colind, Mv, Av = take(colind_p, C.c_int32), take(m_p, C.c_double), take(a_p, C.c_double)
    for p in (colind_p, m_p, a_p):
        libc.free(p)
    return st, rowptr, colind, Mv, Av, rhs


def set_threads(n):
    lib().orc_set_threads(C.c_int(n))


def local_forms(xv, ls10, opts, wind_loc=None):
    """Element matrices of one tet: returns (status, {form: (nl, nl)}, rhs[nl], n_facets).
    wind_loc: (10, 3) P2 wind at the tet's 4 vertices and 6 edge midpoints (FORM_N)."""
    L = lib()
    xv = np.ascontiguousarray(xv, dtype=np.float64)
    ls10 = np.ascontiguousarray(ls10, dtype=np.float64)
    wl = None if wind_loc is None else np.ascontiguousarray(wind_loc, dtype=np.float64).reshape(-1)
    out = np.zeros((NUM_FORMS, 100))
    rhs = np.zeros(10)
    nf = C.c_int()
    st = L.orc_local_forms(_p(xv, C.c_double), _p(ls10, C.c_double), C.byref(opts), None,
                           _p(wl, C.c_double) if wl is not None else None,
                           _p(out, C.c_double), _p(rhs, C.c_double), C.byref(nf))
    nl = 10 if opts.p2 else 4
    return st, {f: out[f, :nl * nl].reshape(nl, nl) for f in range(NUM_FORMS)}, rhs[:nl], nf.value


# ---- per-DOF MLP of the learned warm start ---------------------------------
MLP_IN, MLP_WEIGHTS = 80, 16640


def bf16_bits(a):
    """float32 array -> BF16 bit patterns (uint16), round to nearest even."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return u.astype(np.uint16)


def bf16_value(bits):
    return (np.asarray(bits, dtype=np.uint16).astype(np.uint32) << 16).view(np.float32)


def mlp_forward(w, X, exact=False):
    L = lib()
    w = np.ascontiguousarray(w, dtype=np.float32)
    X = np.ascontiguousarray(X, dtype=np.uint16)
    n = X.shape[0]
    out = np.empty((n, 2), np.float32)
    L.orc_mlp_forward(_p(w, C.c_float), _p(X, C.c_uint16), C.c_int64(n), C.c_int(int(exact)), _p(out, C.c_float))
    return out


def mlp_gradient(w, X, Y, exact=False):
    L = lib()
    w = np.ascontiguousarray(w, dtype=np.float32)
    X = np.ascontiguousarray(X, dtype=np.uint16)
    Y = np.ascontiguousarray(Y, dtype=np.float32)
    g = np.empty(MLP_WEIGHTS, np.float32)
    loss = L.orc_mlp_gradient(_p(w, C.c_float), _p(X, C.c_uint16), _p(Y, C.c_float), C.c_int64(X.shape[0]),
                              C.c_int(int(exact)), _p(g, C.c_float))
    return g, loss


class _QQCtx(C.Structure):
    _fields_ = [("coords", C.c_void_p), ("tet_v", C.c_void_p), ("tet_e", C.c_void_p), ("ls_vert", C.c_void_p),
                ("ls_edge", C.c_void_p), ("grad_vert", C.c_void_p), ("grad_edge", C.c_void_p), ("tol", C.c_double),
                ("armijo", C.c_double), ("maxiter", C.c_int), ("max_damping", C.c_int), ("rhs_c", C.c_double)]


def grad_recovery(mesh, ls_vert, ls_edge):
    """averaging_P2_gradient_recovery (num/gradient_recovery.cpp:82-89): (grad_vert[nv,3], grad_edge[ne,3])."""
    L = lib()
    nv, ne, nt = mesh.nv, mesh.ne, mesh.nt
    gv, ge = np.zeros((nv, 3)), np.zeros((ne, 3))
    L.orc_grad_recovery(C.c_int64(nt), _p(mesh.tet_v, C.c_int32), _p(mesh.tet_e, C.c_int32), _p(mesh.coords, C.c_double),
                        C.c_int64(nv), C.c_int64(ne), _p(_in(ls_vert, np.float64), C.c_double),
                        _p(_in(ls_edge, np.float64), C.c_double), _p(gv, C.c_double), _p(ge, C.c_double))
    return gv, ge


def _qq_ctx(mesh, ls_vert, ls_edge, gv, ge, rhs_c=13.0, tol=1e-13, maxiter=100, armijo=1e-4, max_damping=8):
    q = _QQCtx()
    keep = (mesh.coords, mesh.tet_v, mesh.tet_e, _in(ls_vert, np.float64), _in(ls_edge, np.float64),
            _in(gv, np.float64), _in(ge, np.float64))
    q.coords, q.tet_v, q.tet_e = keep[0].ctypes.data, keep[1].ctypes.data, keep[2].ctypes.data
    q.ls_vert, q.ls_edge, q.grad_vert, q.grad_edge = (k.ctypes.data for k in keep[3:])
    q.tol, q.armijo, q.maxiter, q.max_damping, q.rhs_c = tol, armijo, maxiter, max_damping, rhs_c
    return q, keep


def quaqua_point(mesh, ls_vert, ls_edge, grad, t, b0):
    """One base point of tet t's point b0: (base tet, base bary, dh, Jacobian 3x3, Newton iterations)."""
    q, keep = _qq_ctx(mesh, ls_vert, ls_edge, *grad)
    bt, it, dh = C.c_int64(), C.c_int(), C.c_double()
    bb, J = np.zeros(4), np.zeros(9)
    st = lib().orc_qq_point(C.byref(q), C.c_int64(int(t)), _p(np.ascontiguousarray(b0, dtype=np.float64), C.c_double),
                            C.byref(bt), _p(bb, C.c_double), C.byref(dh), _p(J, C.c_double), C.byref(it))
    if st:
        raise RuntimeError(f"orc_qq_point: status {st}")
    return bt.value, bb, dh.value, J.reshape(3, 3), it.value


def quaqua_elements(mesh, ls_vert, ls_edge, tets, rhs_c=13.0, tol=1e-13, maxiter=100, armijo=1e-4, max_damping=8,
                    grad=None):
    """LocalMassP2CL / LocalLaplaceBeltramiP2CL / LocalVectorP2CL with the QuaQua mapper for the tets `tets`:
    (M[k,10,10], A[k,10,10], b[k,10], points[k], newton iterations[k])."""
    L = lib()
    gv, ge = grad if grad is not None else grad_recovery(mesh, ls_vert, ls_edge)
    q, keep = _qq_ctx(mesh, ls_vert, ls_edge, gv, ge, rhs_c, tol, maxiter, armijo, max_damping)
    k = len(tets)
    M, A, b = np.zeros((k, 10, 10)), np.zeros((k, 10, 10)), np.zeros((k, 10))
    npts, newton = np.zeros(k, np.int32), np.zeros(k, np.int32)
    Mt, At, bt = np.zeros(100), np.zeros(100), np.zeros(10)
    ip, it = C.c_int(), C.c_int()
    for i, t in enumerate(tets):
        st = L.orc_qq_local(C.byref(q), C.c_int64(int(t)), _p(Mt, C.c_double), _p(At, C.c_double), _p(bt, C.c_double),
                            C.byref(ip), C.byref(it))
        if st:
            raise RuntimeError(f"orc_qq_local: status {st} at tet {t}")
        M[i], A[i], b[i] = Mt.reshape(10, 10), At.reshape(10, 10), bt
        npts[i], newton[i] = ip.value, it.value
    del keep
    return M, A, b, npts, newton
