"""drops_gb300: the TraceFEM path of DROPS on GB300 (sm_103a).

The compute path is libtracefem.so (CUDA, built by drops_gb300/build.py) with
the C ABI declared in include/tracefem.h.  This module is a thin ctypes front
end over that ABI, named after the reference's interface:

    ctx = TraceFEM()
    ctx.brick(orig, e1, e2, e3, n1, n2, n3)          # BrickBuilderCL
    ctx.levelset_analytic(LS_SPHERE, [0, 0, 0, 1])     # LSInit / LinearLSInit
    n_active, n = ctx.distribute_dofs(P1IF)            # IdxDescCL::DistributeDOFs
    nnz = ctx.setup_fe_system([FORM_M, FORM_A, FORM_CN], RHS_SPHERE_XYZ, [...])
    ctx.lincomb([FORM_M, FORM_A, FORM_CN], [1, 1, h])  # MatrixCL LinComb ctor
    it, res = ctx.pcg_jacobi(MAT_SYS, VEC_RHS, VEC_X, tol=1e-10)   # PCGSolverCL<JACPcCL>

There is no CPU fallback: if the library is missing or no suitable GPU is
present, constructing a context raises.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libtracefem.so")

# status codes
OK, ERR_CUDA, ERR_ZERO_NODE, ERR_ZERO_PATTERN, ERR_BAD_INPUT, ERR_NOT_CONVERGED, ERR_CAPACITY, ERR_WATCHDOG, ERR_NO_DEVICE, \
    ERR_INTERNAL = range(10)
P1IF, P2IF = 1, 2
FORM_M, FORM_A, FORM_CN, FORM_LAPM = 0, 1, 2, 3
MAT_SYS, MAT_BLOCK, MAT_USER = 4, 5, 6
FORM_N = 7  # N_P1P1, wind convection (tf_wind_upload)
CH_DEGENERATE_MOBILITY, CH_WIND = 1, 2  # tf_ch_options
VEC_RHS, VEC_X, VEC_B, VEC_CHI, VEC_T0, VEC_T1, VEC_T2, VEC_T3 = range(8)
LS_SPHERE, LS_TORUS, LS_ELLIPSOID, LS_PLANE = range(4)
RHS_NONE, RHS_SPHERE_XYZ, RHS_CONST = range(3)
PREC_FP64, PREC_MIXED = 0, 1
ORTH_MGS, ORTH_CGS2 = 0, 1
SPMV_KERNEL_FP64, SPMV_KERNEL_PAIR = 0, 1  # tf_spmv_options
ASM_KERNEL_PAIR, ASM_KERNEL_FP64 = 0, 1  # tf_assemble_options
PCG_FP64_CLASSIC, PCG_FP64_CG1 = 0, 1  # tf_pcg_options
MLP_IN, MLP_WEIGHTS = 80, 16640
K_CLASSIFY, K_NUMBER, K_ASSEMBLE, K_PATTERN, K_SCATTER, K_SPMV, K_PCG, K_GMRES, K_LEVELSET, K_BATCH = range(10)
KERNEL_NAMES = ["classify", "number", "assemble", "pattern", "scatter", "spmv", "pcg", "gmres", "levelset", "batch"]

# every symbol include/tracefem.h declares
EXPORTS = [
    "tf_create", "tf_destroy", "tf_last_error", "tf_status_string", "tf_stream", "tf_mesh_brick", "tf_mesh_upload",
    "tf_mesh_info", "tf_mesh_download", "tf_levelset_upload", "tf_levelset_analytic", "tf_levelset_download",
    "tf_distribute_dofs", "tf_create_numb_on_interface_p1", "tf_dofs_download", "tf_dofs_info", "tf_setup_interface_p1_legacy", "tf_patches_download", "tf_setup_fe_system",
    "tf_matrix_info", "tf_matrix_download", "tf_matrix_upload", "tf_lincomb", "tf_ch_block", "tf_vec_upload",
    "tf_vec_download", "tf_vec_size", "tf_vec_fill", "tf_spmv", "tf_spmv_options", "tf_assemble_options", "tf_pcg_jacobi", "tf_gmres_jacobi", "tf_pcg_jacobi_noalloc", "tf_ch_steps",
    "tf_mesh_brick_batch", "tf_levelset_analytic_batch", "tf_batch_info", "tf_batch_lincomb", "tf_batch_pcg_jacobi",
    "tf_batch_tune", "tf_batch_config", "tf_mlp_init", "tf_mlp_get_weights", "tf_mlp_set_weights", "tf_mlp_forward",
    "tf_mlp_gradient", "tf_mlp_train", "tf_ch_features", "tf_ch_steps_learned", "tf_gmres_options", "tf_pcg_options", "tf_autotune", "tf_autotune_info", "tf_setup_quaqua_p2", "tf_timing_enable",
    "tf_timing_get", "tf_timing_reset", "tf_launch_count", "tf_marker_record", "tf_marker_elapsed", "tf_flush_l2", "tf_spmv_timed", "tf_stream_read_timed", "tf_wind_upload", "tf_vec_write", "tf_vec_read", "tf_ch_stats", "tf_ch_steps_adaptive", "tf_ch_options",
    "tf_host_alloc", "tf_host_free", "tf_mesh_refine_band", "tf_refine_band", "tf_refined_info", "tf_refined_get",
    "tf_refined_free", "tf_refine_rules",
]


class TraceFEMError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"[{status}] {msg}")
        self.status = status


_lib = None


def load_library(path=LIB_PATH):
    """Loads libtracefem.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with drops_gb300.build.build() (nvcc, sm_103a)")
    L = C.CDLL(path)
    L.tf_last_error.restype = C.c_char_p
    L.tf_status_string.restype = C.c_char_p
    L.tf_stream.restype = C.c_void_p
    L.tf_launch_count.restype = C.c_int64
    L.tf_host_alloc.restype = C.c_void_p
    L.tf_host_alloc.argtypes = [C.c_size_t]
    L.tf_host_free.argtypes = [C.c_void_p]
    L.tf_refined_free.argtypes = [C.c_void_p]
    L.tf_refined_free.restype = None
    _lib = L
    return L


def refine_band(coords, tet_v, kind, par, width, coarse_level, fine_level):
    """Narrow-band refinement (AdapTriangCL::MakeInitialTriang with DistMarkingStrategyCL) of a level-0 mesh on
    the host, no device needed.  Returns a dict: coords, tet_v, tet_e, edge_v, tet_level, tets_per_level,
    last_level, steps; raises TraceFEMError on bad input."""
    L = load_library()
    coords = np.ascontiguousarray(coords, dtype=np.float64)
    tet_v = np.ascontiguousarray(tet_v, dtype=np.int32)
    par = np.ascontiguousarray(par, dtype=np.float64)
    h = C.c_void_p()
    st = L.tf_refine_band(C.c_int64(coords.size // 3), _dp(coords), C.c_int64(tet_v.size // 4), _ip(tet_v),
                          C.c_int(kind), _dp(par), C.c_int(par.size), C.c_double(width), C.c_int(coarse_level),
                          C.c_int(fine_level), C.byref(h))
    if st != OK:
        raise TraceFEMError(st, L.tf_status_string(st).decode())
    try:
        nv, ne, nt = C.c_int64(), C.c_int64(), C.c_int64()
        ll, steps = C.c_int(), C.c_int()
        L.tf_refined_info(h, C.byref(nv), C.byref(ne), C.byref(nt), C.byref(ll), C.byref(steps))
        out = dict(coords=np.empty((nv.value, 3)), tet_v=np.empty((nt.value, 4), np.int32),
                   tet_e=np.empty((nt.value, 6), np.int32), edge_v=np.empty((ne.value, 2), np.int32),
                   tet_level=np.empty(nt.value, np.int32), tets_per_level=np.empty(ll.value + 1, np.int64))
        L.tf_refined_get(h, _dp(out["coords"]), _ip(out["tet_v"]), _ip(out["tet_e"]), _ip(out["edge_v"]),
                         _ip(out["tet_level"]), _lp(out["tets_per_level"]))
    finally:
        L.tf_refined_free(h)
    out.update(last_level=ll.value, steps=steps.value)
    return out


def refine_rules():
    """The 64 refinement rules: (nch[64], children[64, 8, 4]) local points, -1 past nch."""
    L = load_library()
    nch = np.empty(64, np.int32)
    ch = np.empty((64, 8, 4), np.int32)
    st = L.tf_refine_rules(_ip(nch), _ip(ch))
    if st != OK:
        raise TraceFEMError(st, L.tf_status_string(st).decode())
    return nch, ch


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32)) if a is not None else None


def _lp(a):
    return a.ctypes.data_as(C.POINTER(C.c_int64)) if a is not None else None


class TraceFEM:
    """One device context (tf_context)."""

    def __init__(self, device=0):
        self.L = load_library()
        h = C.c_void_p()
        st = self.L.tf_create(C.byref(h), C.c_int(device))
        if st != OK:
            raise TraceFEMError(st, self.L.tf_status_string(st).decode() + " (no sm_103a-capable GPU / driver)")
        self.h = h
        self.fe = None
        self.m = 0
        self.batch_count = 0

    def close(self):
        if self.h:
            self.L.tf_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st):
        if st != OK:
            raise TraceFEMError(st, self.L.tf_last_error(self.h).decode())

    def call(self, name, *args):
        """Raw call; returns the status without raising."""
        return getattr(self.L, name)(self.h, *args)

    # ---- mesh -----------------------------------------------------------
    def brick(self, orig, e1, e2, e3, n1, n2, n3):
        v = [np.ascontiguousarray(x, dtype=np.float64) for x in (orig, e1, e2, e3)]
        self._check(self.L.tf_mesh_brick(self.h, *[_dp(x) for x in v], C.c_int(n1), C.c_int(n2), C.c_int(n3)))
        self._keep = v

    def brick_cube(self, n, a):
        """[-a,a]^3 with n^3 cubes."""
        self.brick([-a, -a, -a], [2 * a, 0, 0], [0, 2 * a, 0], [0, 0, 2 * a], n, n, n)

    def brick_batch(self, n, orig, axes):
        """count independent bricks: n[count,3] cubes, orig[count,3], axes[count,3,3] (rows e1, e2, e3)."""
        n = np.ascontiguousarray(n, dtype=np.int32).reshape(-1, 3)
        orig = np.ascontiguousarray(orig, dtype=np.float64).reshape(-1, 3)
        axes = np.ascontiguousarray(axes, dtype=np.float64).reshape(-1, 9)
        self.batch_count = n.shape[0]
        self._check(self.L.tf_mesh_brick_batch(self.h, C.c_int(n.shape[0]), _ip(n), _dp(orig), _dp(axes)))

    def batch_info(self, nnz=True):
        """Per-instance starts (count+1 each): tets, cut tets, rows, nnz."""
        k = self.batch_count + 1
        t, c, r, z = (np.zeros(k, np.int64) for _ in range(4))
        p = lambda a: a.ctypes.data_as(C.POINTER(C.c_int64))
        self._check(self.L.tf_batch_info(self.h, p(t), p(c), p(r), p(z) if nnz else None))
        return t, c, r, (z if nnz else None)

    def batch_lincomb(self, forms, coeffs):
        """TF_MAT_SYS = sum_k coeffs[i, k] forms[k] on the rows of instance i."""
        f = np.ascontiguousarray(forms, dtype=np.int32)
        co = np.ascontiguousarray(coeffs, dtype=np.float64).reshape(self.batch_count, f.size)
        self._check(self.L.tf_batch_lincomb(self.h, C.c_int(f.size), _ip(f), _dp(co)))

    def batch_pcg_jacobi(self, mat, vec_b, vec_x, tol=1e-10, max_iter=100000, rel=True, precision=PREC_FP64,
                         check=True):
        """One persistent launch over all instances; returns (status, iterations[count], residuals[count])."""
        its = np.zeros(self.batch_count, np.int32)
        res = np.zeros(self.batch_count)
        st = self.L.tf_batch_pcg_jacobi(self.h, C.c_int(mat), C.c_int(vec_b), C.c_int(vec_x), C.c_int(precision),
                                        C.c_int(max_iter), C.c_double(tol), C.c_int(int(rel)), _ip(its), _dp(res))
        if check and st not in (OK, ERR_NOT_CONVERGED):
            self._check(st)
        return st, its, res

    def batch_tune(self, mat, vec_b, precision=PREC_FP64):
        lanes, threads = C.c_int(), C.c_int()
        self._check(self.L.tf_batch_tune(self.h, C.c_int(mat), C.c_int(vec_b), C.c_int(precision), C.byref(lanes),
                                         C.byref(threads)))
        return lanes.value, threads.value

    def batch_config(self, lanes=0, threads=0, use_graph=True):
        self._check(self.L.tf_batch_config(self.h, C.c_int(lanes), C.c_int(threads), C.c_int(int(use_graph))))

    def mesh_upload(self, coords, tet_v, tet_e, edge_v):
        coords = np.ascontiguousarray(coords, dtype=np.float64)
        tet_v = np.ascontiguousarray(tet_v, dtype=np.int32)
        tet_e = np.ascontiguousarray(tet_e, dtype=np.int32)
        edge_v = np.ascontiguousarray(edge_v, dtype=np.int32)
        self._check(self.L.tf_mesh_upload(self.h, C.c_int64(coords.size // 3), _dp(coords), C.c_int64(tet_v.size // 4),
                                          _ip(tet_v), _ip(tet_e), C.c_int64(edge_v.size // 2), _ip(edge_v)))

    def mesh_refine_band(self, kind, par, width, coarse_level, fine_level):
        """Refines the context's mesh towards the zero level of the distance function and replaces it by the last
        triangulation level; returns (last_level, steps)."""
        par = np.ascontiguousarray(par, dtype=np.float64)
        ll, steps = C.c_int(), C.c_int()
        self._check(self.L.tf_mesh_refine_band(self.h, C.c_int(kind), _dp(par), C.c_int(par.size), C.c_double(width),
                                               C.c_int(coarse_level), C.c_int(fine_level), C.byref(ll),
                                               C.byref(steps)))
        self.fe = None
        return ll.value, steps.value

    def mesh_info(self):
        nv, ne, nt = C.c_int64(), C.c_int64(), C.c_int64()
        self._check(self.L.tf_mesh_info(self.h, C.byref(nv), C.byref(ne), C.byref(nt)))
        return nv.value, ne.value, nt.value

    def mesh_download(self):
        nv, ne, nt = self.mesh_info()
        coords = np.empty((nv, 3))
        tv = np.empty((nt, 4), np.int32)
        te = np.empty((nt, 6), np.int32)
        ev = np.empty((ne, 2), np.int32)
        self._check(self.L.tf_mesh_download(self.h, _dp(coords), _ip(tv), _ip(te), _ip(ev)))
        return coords, tv, te, ev

    # ---- level set ---------------------------------------------------------
    def ch_steps_adaptive(self, t_final, dt0, F_tol, F_rho, F_min, F_max, mobility, eps, beta_s, xi, rho_vol,
                          t0=0.0, adaptive=True, max_steps=1000, restart=50, tol=1e-10, max_iter=100000):
        """Adaptive BDF1/BDF2 steps (tf_ch_steps_adaptive): returns (t_end, dts, errors, tries, iterations)."""
        P = ChAdaptParams(t0, t_final, dt0, F_tol, F_rho, F_min, F_max, int(adaptive), max_steps, mobility, eps,
                          beta_s, xi, rho_vol, restart, max_iter, tol)
        n, te = C.c_int(), C.c_double()
        dts, errs = np.zeros(max(max_steps, 1)), np.zeros(max(max_steps, 1))
        tries, its = np.zeros(max(max_steps, 1), np.int32), np.zeros(max(max_steps, 1), np.int32)
        self._check(self.L.tf_ch_steps_adaptive(self.h, C.byref(P), C.byref(n), C.byref(te), _dp(dts), _dp(errs),
                                                tries.ctypes.data_as(C.POINTER(C.c_int)),
                                                its.ctypes.data_as(C.POINTER(C.c_int))))
        k = n.value
        return te.value, dts[:k], errs[:k], tries[:k], its[:k]

    def ch_options(self, flags):
        """Mobility and wind of the CH time loops: CH_DEGENERATE_MOBILITY | CH_WIND (tf_ch_options)."""
        self._check(self.L.tf_ch_options(self.h, C.c_int(flags)))

    def ch_stats(self, eps, xi=1.0):
        """The integrals of the reference's per-step statistics (surfphasesep.cpp:324-345) for TF_VEC_CHI."""
        out = np.zeros(6)
        self._check(self.L.tf_ch_stats(self.h, C.c_double(eps), C.c_double(xi), _dp(out)))
        return {"Integral.SurfacaAreaP1": out[0], "Integral.FESolution.RaftFraction": out[1],
                "Integral.FESolution.PerimeterEstimate": out[2], "Integral.FESolution.LyapunovEnergy": out[3],
                "c_h.Max": out[4], "c_h.Min": out[5]}

    def write_ch_stats(self, path, t, h, eps, xi=1.0, extra=None):
        """One stats/t_<i>.json of the reference's exportStats: dotted keys as nested objects."""
        import json

        flat = {"t": t, "h": h, "DOF.c_h": self.m, "DOF.mu_h": self.m, **self.ch_stats(eps, xi), **(extra or {})}
        tree = {}
        for key, val in flat.items():
            node = tree
            *parents, leaf = key.split(".")
            for p in parents:
                node = node.setdefault(p, {})
            node[leaf] = float(val) if not isinstance(val, (bool, str)) else val
        with open(path, "w") as f:
            json.dump(tree, f, indent=4)
        return tree

    def vec_write(self, vec, path):
        """VecDescCL::Write(os, binary=true): 64-bit count, then the doubles."""
        self._check(self.L.tf_vec_write(self.h, C.c_int(vec), os.fsencode(path)))

    def vec_read(self, vec, path, n_expected=-1):
        """VecDescCL::Read(is, binary=true); a count other than n_expected (>= 0) raises."""
        self._check(self.L.tf_vec_read(self.h, C.c_int(vec), os.fsencode(path), C.c_int64(n_expected)))

    def wind_upload(self, wind_vert, wind_edge):
        """P2 wind for FORM_N: xyz at every vertex (nv, 3) and at every edge midpoint (ne, 3)."""
        wv = np.ascontiguousarray(wind_vert, dtype=np.float64).reshape(-1)
        we = np.ascontiguousarray(wind_edge, dtype=np.float64).reshape(-1)
        nv, ne, _ = self.mesh_info()
        if wv.size != 3 * nv or we.size != 3 * ne:
            raise ValueError("wind_upload: expected (nv, 3) and (ne, 3) arrays")
        self._check(self.L.tf_wind_upload(self.h, wv.ctypes.data_as(C.POINTER(C.c_double)),
                                          we.ctypes.data_as(C.POINTER(C.c_double))))

    def levelset_upload(self, ls_vert, ls_edge=None):
        ls_vert = np.ascontiguousarray(ls_vert, dtype=np.float64)
        ls_edge = None if ls_edge is None else np.ascontiguousarray(ls_edge, dtype=np.float64)
        self._check(self.L.tf_levelset_upload(self.h, _dp(ls_vert), _dp(ls_edge)))

    def levelset_analytic(self, kind, par, p2=False):
        par = np.ascontiguousarray(par, dtype=np.float64)
        self._check(self.L.tf_levelset_analytic(self.h, C.c_int(kind), _dp(par), C.c_int(par.size), C.c_int(int(p2))))

    def levelset_analytic_batch(self, kind, par, p2=False):
        """par[count, npar]: one parameter set per batch instance."""
        par = np.ascontiguousarray(par, dtype=np.float64).reshape(self.batch_count, -1)
        self._check(self.L.tf_levelset_analytic_batch(self.h, C.c_int(kind), _dp(par), C.c_int(par.shape[1]),
                                                      C.c_int(int(p2))))

    def levelset_download(self):
        nv, ne, nt = self.mesh_info()
        lv, le = np.empty(nv), np.empty(ne)
        self._check(self.L.tf_levelset_download(self.h, _dp(lv), _dp(le)))
        return lv, le

    # ---- DOFs ----------------------------------------------------------------
    def distribute_dofs(self, fe, dist=0.0):
        na, nd = C.c_int64(), C.c_int64()
        self._check(self.L.tf_distribute_dofs(self.h, C.c_int(fe), C.c_double(dist), C.byref(na), C.byref(nd)))
        self.fe, self.n_active, self.m = fe, na.value, nd.value
        return na.value, nd.value

    def create_numb_on_interface_p1(self, omit_bound=-1.0):
        na, nd = C.c_int64(), C.c_int64()
        self._check(self.L.tf_create_numb_on_interface_p1(self.h, C.c_double(omit_bound), C.byref(na), C.byref(nd)))
        self.fe, self.n_active, self.m = P1IF, na.value, nd.value
        return na.value, nd.value

    def dofs(self):
        nv, ne, nt = self.mesh_info()
        nl = 10 if self.fe == P2IF else 4
        ntl = C.c_int64()
        self._check(self.L.tf_dofs_info(self.h, C.byref(ntl), None, None))
        self.n_active = ntl.value
        dv = np.empty(nv, np.int32)
        de = np.empty(ne, np.int32) if self.fe == P2IF else None
        act = np.empty(max(self.n_active, 1), np.int32)
        l2g = np.empty(max(self.n_active * nl, 1), np.int32)
        self._check(self.L.tf_dofs_download(self.h, _ip(dv), _ip(de), _ip(act), _ip(l2g)))
        return dv, de, act[: self.n_active], l2g[: self.n_active * nl]

    def patches(self, tets):
        """make_patch topology of the given tets: list of (facets, boundary, verts)."""
        tets = np.ascontiguousarray(tets, dtype=np.int32)
        count = tets.size
        nf = np.zeros(count, np.int32)
        fac = np.zeros((count, 16, 3), np.int32)
        bnd = np.zeros((count, 16), np.int32)
        nv = np.zeros(count, np.int32)
        ver = np.zeros((count, 40, 4))
        self._check(self.L.tf_patches_download(self.h, _ip(tets), C.c_int64(count), _ip(nf), _ip(fac), _ip(bnd),
                                               _ip(nv), _dp(ver)))
        return [(fac[i, :nf[i]], bnd[i, :nf[i]], ver[i, :nv[i]]) for i in range(count)]

    # ---- assembly ----------------------------------------------------------------
    def setup_fe_system(self, forms, rhs_kind=RHS_NONE, rhs_par=()):
        mask = sum(1 << f for f in forms)
        par = np.ascontiguousarray(rhs_par if len(rhs_par) else [0.0], dtype=np.float64)
        nnz = C.c_int64()
        self._check(self.L.tf_setup_fe_system(self.h, C.c_uint(mask), C.c_int(rhs_kind), _dp(par),
                                              C.c_int(len(rhs_par)), C.byref(nnz)))
        return nnz.value

    def setup_interface_p1_legacy(self, alpha, D, fpar=None):
        """SetupInterfaceMassP1 (alpha), SetupLBP1 (D) and, with fpar (10 coefficients of the quadratic
        f), SetupInterfaceRhsP1 on the legacy P1 numbering; returns nnz."""
        par = None if fpar is None else np.ascontiguousarray(fpar, dtype=np.float64)
        if par is not None and par.size != 10:
            raise ValueError("fpar holds the 10 coefficients of a quadratic")
        nnz = C.c_int64()
        self._check(self.L.tf_setup_interface_p1_legacy(self.h, C.c_double(alpha), C.c_double(D),
                                                        None if par is None else _dp(par), C.byref(nnz)))
        return nnz.value

    def matrix(self, mat):
        m, nnz = C.c_int64(), C.c_int64()
        self._check(self.L.tf_matrix_info(self.h, C.c_int(mat), C.byref(m), C.byref(nnz)))
        rp = np.empty(m.value + 1, np.int64)
        ci = np.empty(max(nnz.value, 1), np.int64)
        v = np.empty(max(nnz.value, 1))
        self._check(self.L.tf_matrix_download(self.h, C.c_int(mat), _lp(rp), _lp(ci), _dp(v)))
        return rp, ci[: nnz.value], v[: nnz.value]

    def matrix_upload(self, rowptr, colind, vals):
        rowptr = np.ascontiguousarray(rowptr, dtype=np.int64)
        colind = np.ascontiguousarray(colind, dtype=np.int64)
        vals = np.ascontiguousarray(vals, dtype=np.float64)
        self._check(self.L.tf_matrix_upload(self.h, C.c_int64(rowptr.size - 1), _lp(rowptr), _lp(colind), _dp(vals)))

    def lincomb(self, forms, coeffs):
        f = np.ascontiguousarray(forms, dtype=np.int32)
        c = np.ascontiguousarray(coeffs, dtype=np.float64)
        self._check(self.L.tf_lincomb(self.h, C.c_int(f.size), f.ctypes.data_as(C.POINTER(C.c_int)), _dp(c)))

    def ch_block(self, alpha, mob, rho, eps2, beta, flags=0):
        """TF_MAT_BLOCK of surfphasesep.cpp:431-434; flags: CH_DEGENERATE_MOBILITY | CH_WIND (tf_ch_block)."""
        use_lapm = int(flags)
        self._check(self.L.tf_ch_block(self.h, C.c_double(alpha), C.c_double(mob), C.c_double(rho), C.c_double(eps2),
                                       C.c_double(beta), C.c_int(int(use_lapm))))

    # ---- vectors and solvers --------------------------------------------------------
    def vec_upload(self, vec, data):
        data = np.ascontiguousarray(data, dtype=np.float64)
        self._check(self.L.tf_vec_upload(self.h, C.c_int(vec), C.c_int64(data.size), _dp(data)))

    def vec_download(self, vec, out=None):
        n = C.c_int64()
        self._check(self.L.tf_vec_size(self.h, C.c_int(vec), C.byref(n)))
        if out is None:
            out = np.empty(n.value)
        self._check(self.L.tf_vec_download(self.h, C.c_int(vec), _dp(out), C.c_int64(n.value)))
        return out

    def vec_fill(self, vec, n, value=0.0):
        self._check(self.L.tf_vec_fill(self.h, C.c_int(vec), C.c_int64(n), C.c_double(value)))

    def spmv(self, mat, vec_x, vec_y):
        self._check(self.L.tf_spmv(self.h, C.c_int(mat), C.c_int(vec_x), C.c_int(vec_y)))

    def pcg_jacobi(self, mat, vec_b, vec_x, tol=1e-10, max_iter=100000, rel=True, precision=PREC_FP64, check=True):
        it, t = C.c_int(max_iter), C.c_double(tol)
        st = self.L.tf_pcg_jacobi(self.h, C.c_int(mat), C.c_int(vec_b), C.c_int(vec_x), C.c_int(precision),
                                  C.byref(it), C.byref(t), C.c_int(int(rel)))
        if check and st not in (OK, ERR_NOT_CONVERGED):
            self._check(st)
        return st, it.value, t.value

    def gmres_jacobi(self, mat, vec_b, vec_x, restart=50, tol=1e-10, max_iter=100000, rel=True, method=0,
                     precision=PREC_FP64, check=True):
        it, t = C.c_int(max_iter), C.c_double(tol)
        st = self.L.tf_gmres_jacobi(self.h, C.c_int(mat), C.c_int(vec_b), C.c_int(vec_x), C.c_int(restart),
                                    C.c_int(method), C.c_int(precision), C.byref(it), C.byref(t), C.c_int(int(rel)))
        if check and st not in (OK, ERR_NOT_CONVERGED):
            self._check(st)
        return st, it.value, t.value

    # ---- learned warm start -------------------------------------------------
    def mlp_init(self, seed=1234):
        self._check(self.L.tf_mlp_init(self.h, C.c_uint64(seed)))

    def mlp_weights(self, w=None):
        """Returns the FP32 weights (MLP_WEIGHTS floats); sets them first when w is given."""
        if w is not None:
            w = np.ascontiguousarray(w, dtype=np.float32)
            self._check(self.L.tf_mlp_set_weights(self.h, w.ctypes.data_as(C.POINTER(C.c_float))))
        out = np.empty(MLP_WEIGHTS, np.float32)
        self._check(self.L.tf_mlp_get_weights(self.h, out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    @staticmethod
    def _u16(a):
        return np.ascontiguousarray(a, dtype=np.uint16).ctypes.data_as(C.POINTER(C.c_uint16))

    def mlp_forward(self, X):
        """X: (n, 80) BF16 bit patterns (uint16); returns (n, 2) float32."""
        X = np.ascontiguousarray(X, dtype=np.uint16)
        n = X.shape[0]
        out = np.empty((n, 2), np.float32)
        self._check(self.L.tf_mlp_forward(self.h, X.ctypes.data_as(C.POINTER(C.c_uint16)), C.c_int64(n),
                                          out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    def mlp_gradient(self, X, Y):
        X = np.ascontiguousarray(X, dtype=np.uint16)
        Y = np.ascontiguousarray(Y, dtype=np.float32)
        g = np.empty(MLP_WEIGHTS, np.float32)
        loss = C.c_double()
        self._check(self.L.tf_mlp_gradient(self.h, X.ctypes.data_as(C.POINTER(C.c_uint16)),
                                           Y.ctypes.data_as(C.POINTER(C.c_float)), C.c_int64(X.shape[0]),
                                           g.ctypes.data_as(C.POINTER(C.c_float)), C.byref(loss)))
        return g, loss.value

    def mlp_train(self, X, Y, epochs=1, minibatch_tiles=16, lr=1e-3):
        X = np.ascontiguousarray(X, dtype=np.uint16)
        Y = np.ascontiguousarray(Y, dtype=np.float32)
        loss = C.c_double()
        self._check(self.L.tf_mlp_train(self.h, X.ctypes.data_as(C.POINTER(C.c_uint16)),
                                        Y.ctypes.data_as(C.POINTER(C.c_float)), C.c_int64(X.shape[0]), C.c_int(epochs),
                                        C.c_int(minibatch_tiles), C.c_float(lr), C.byref(loss)))
        return loss.value

    def ch_features(self, vec_cur, vec_old, vec_next=-1):
        m = self.m
        X = np.empty((m, MLP_IN), np.uint16)
        Y = np.empty((m, 2), np.float32)
        self._check(self.L.tf_ch_features(self.h, C.c_int(vec_cur), C.c_int(vec_old), C.c_int(vec_next),
                                          X.ctypes.data_as(C.POINTER(C.c_uint16)),
                                          Y.ctypes.data_as(C.POINTER(C.c_float))))
        return X, (Y if vec_next >= 0 else None)

    def spmv_options(self, kernel=SPMV_KERNEL_FP64):
        """Kernel of tf_spmv: SPMV_KERNEL_FP64 (default) or SPMV_KERNEL_PAIR (FP32 pairs)."""
        self._check(self.L.tf_spmv_options(self.h, C.c_int(kernel)))

    def assemble_options(self, kernel=ASM_KERNEL_PAIR):
        """Arithmetic of the M, A, C_n and load-vector forms: ASM_KERNEL_PAIR (default, FP32 pairs) or ASM_KERNEL_FP64."""
        self._check(self.L.tf_assemble_options(self.h, C.c_int(kernel)))

    def setup_quaqua_p2(self, f_coeff=13.0, newton_tol=1e-13, newton_maxiter=100):
        """Isoparametric P2 forms with the QuaQua mapper into FORM_M, FORM_A and VEC_RHS; returns the largest
        Newton iteration count of a quadrature point."""
        it = C.c_int()
        self._check(self.L.tf_setup_quaqua_p2(self.h, C.c_double(f_coeff), C.c_double(newton_tol),
                                              C.c_int(newton_maxiter), C.byref(it)))
        return it.value

    def autotune(self, on=True):
        self._check(self.L.tf_autotune(self.h, C.c_int(int(on))))

    def autotune_info(self, mat):
        """(spmv_threads, spmv_blocks_per_sm, pcg_kind, spmv_us[4], pcg_us[3]) chosen for a matrix handle."""
        t, b, k = C.c_int(), C.c_int(), C.c_int()
        su, pu = (C.c_float * 4)(), (C.c_float * 3)()
        self._check(self.L.tf_autotune_info(self.h, C.c_int(mat), C.byref(t), C.byref(b), C.byref(k), su, pu))
        return t.value, b.value, k.value, list(su), list(pu)

    def pcg_options(self, fp64_kernel=PCG_FP64_CLASSIC):
        self._check(self.L.tf_pcg_options(self.h, C.c_int(fp64_kernel)))

    def gmres_options(self, orth=ORTH_MGS):
        self._check(self.L.tf_gmres_options(self.h, C.c_int(orth)))

    def ch_steps_learned(self, nsteps, dt, mobility, eps, beta_s, xi, rho_vol, restart=50, tol=1e-10,
                         max_iter=100000, precision=PREC_FP64, learned=True, train_steps=100, epochs=2,
                         minibatch_tiles=16, lr=1e-3, check=True):
        """Cahn-Hilliard steps with the learned warm start; returns (status, iterations[], residuals[], used[])."""
        k = max(nsteps, 1)
        its, res, used = np.zeros(k, np.int32), np.zeros(k), np.zeros(k, np.int32)
        st = self.L.tf_ch_steps_learned(self.h, C.c_int(nsteps), C.c_double(dt), C.c_double(mobility),
                                        C.c_double(eps), C.c_double(beta_s), C.c_double(xi), C.c_double(rho_vol),
                                        C.c_int(restart), C.c_double(tol), C.c_int(max_iter), C.c_int(precision),
                                        C.c_int(int(learned)),  # 0 plain, 1 projection + MLP, 2 extrapolation, 3 projection
                                        C.c_int(train_steps), C.c_int(epochs), C.c_int(minibatch_tiles),
                                        C.c_float(lr), _ip(its), _dp(res), _ip(used))
        if check:
            self._check(st)
        return st, its[:nsteps], res[:nsteps], used[:nsteps]

    def ch_steps(self, nsteps, dt, mobility, eps, beta_s, xi, rho_vol, restart=50, tol=1e-10, max_iter=100000,
                 warm=True, check=True):
        """Cahn-Hilliard BDF1 steps (tf_ch_steps); returns (status, iterations[], residuals[])."""
        its = np.zeros(max(nsteps, 1), np.int32)
        res = np.zeros(max(nsteps, 1))
        st = self.L.tf_ch_steps(self.h, C.c_int(nsteps), C.c_double(dt), C.c_double(mobility), C.c_double(eps),
                                C.c_double(beta_s), C.c_double(xi), C.c_double(rho_vol), C.c_int(restart),
                                C.c_double(tol), C.c_int(max_iter), C.c_int(int(warm)),
                                its.ctypes.data_as(C.POINTER(C.c_int)), _dp(res))
        if check and st != OK:
            self._check(st)
        return st, its[:nsteps], res[:nsteps]

    # ---- instrumentation ------------------------------------------------------------------
    def timing(self, on=True):
        self._check(self.L.tf_timing_enable(self.h, C.c_int(int(on))))

    def timing_reset(self):
        self._check(self.L.tf_timing_reset(self.h))

    def timing_get(self, kernel):
        ms, n = C.c_double(), C.c_int64()
        self._check(self.L.tf_timing_get(self.h, C.c_int(kernel), C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def launch_count(self):
        return int(self.L.tf_launch_count(self.h))

    def marker(self, slot):
        self._check(self.L.tf_marker_record(self.h, C.c_int(slot)))

    def elapsed_ms(self, a, b):
        ms = C.c_double()
        self._check(self.L.tf_marker_elapsed(self.h, C.c_int(a), C.c_int(b), C.byref(ms)))
        return ms.value

    def flush_l2(self):
        self._check(self.L.tf_flush_l2(self.h))

    def stream_read_timed(self, nbytes, reps=10, cold=1):
        """Device time (ms) of each of `reps` coalesced reads of nbytes (the streaming floor of that size);
        cold: 0 warm, 1 L2 flushed by writing (dirty), 2 flushed by reading (clean)."""
        out = np.zeros(reps, dtype=np.float32)
        self._check(self.L.tf_stream_read_timed(self.h, C.c_int64(int(nbytes)), C.c_int(reps), C.c_int(int(cold)),
                                                out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    def spmv_timed(self, mat, vec_x, vec_y, reps=10, cold=1):
        """Device time (ms) of each of `reps` SpMV calls; cold: 0 warm, 1 L2 flushed by writing, 2 by reading."""
        out = np.zeros(reps, dtype=np.float32)
        self._check(self.L.tf_spmv_timed(self.h, C.c_int(mat), C.c_int(vec_x), C.c_int(vec_y), C.c_int(reps),
                                         C.c_int(int(cold)), out.ctypes.data_as(C.POINTER(C.c_float))))
        return out


class ChAdaptParams(C.Structure):
    """tf_ch_adapt_params: adaptive BDF1/BDF2 control of surfphasesep.cpp:397-483."""
    _fields_ = [("t0", C.c_double), ("t_final", C.c_double), ("dt0", C.c_double), ("F_tol", C.c_double),
                ("F_rho", C.c_double), ("F_min", C.c_double), ("F_max", C.c_double), ("adaptive", C.c_int),
                ("max_steps", C.c_int), ("mobility", C.c_double), ("eps", C.c_double), ("beta_s", C.c_double),
                ("xi", C.c_double), ("rho_vol", C.c_double), ("restart", C.c_int), ("max_iter", C.c_int),
                ("tol", C.c_double)]


class PinnedArray:
    """A numpy view of page-locked host memory (tf_host_alloc)."""

    def __init__(self, n, dtype=np.float64):
        L = load_library()
        dt = np.dtype(dtype)
        self.nbytes = max(int(n) * dt.itemsize, 1)
        self.ptr = L.tf_host_alloc(self.nbytes)
        if not self.ptr:
            raise MemoryError("tf_host_alloc failed")
        self.array = np.ctypeslib.as_array((C.c_byte * self.nbytes).from_address(self.ptr)).view(dt)[: int(n)]

    def free(self):
        if self.ptr:
            load_library().tf_host_free(C.c_void_p(self.ptr))
            self.ptr = None
