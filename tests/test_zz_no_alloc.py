"""The allocation-free PCG entry point (tf_pcg_jacobi_noalloc).

Callers that cannot allocate device memory -- applications that manage all
GPU memory through their own pool, real-time loops that must not trigger the
implicit synchronisation of cudaMalloc/cudaFree -- call tf_pcg_jacobi_noalloc
with their own device buffers; its
work vectors live in a fixed device array of the library.  This test drives it
through the C ABI twice in a row and checks both results against the regular
context-based entry point tf_pcg_jacobi on the same system.  The test itself
allocates its device buffers with the CUDA runtime; only the entry point under
test must not.  Further cases: the solution against the reference's own
golden solution, max_iter = 0, a budget too small to converge (against the
oracle's PCG), an initial guess that is already converged, free device memory
unchanged by the calls, and thirty solves of a 36,606-row P2 system in a row that
agree bit for bit.
"""
import ctypes as C

import numpy as np
import pytest

import drops_gb300 as tf
from oracle import pyoracle as O
from tests.helpers import SOL_RTOL, sol_close

pytestmark = pytest.mark.gpu

MAX_ROWS = 262144  # TF_NOALLOC_MAX_ROWS in include/tracefem.h


def _cudart():
    for name in ("libcudart.so.13", "libcudart.so.12", "libcudart.so"):
        try:
            return C.CDLL(name)
        except OSError:
            pass
    pytest.fail("the CUDA runtime library is not loadable")


class DevArray:
    """A device copy of a numpy array, owned by the test."""

    def __init__(self, rt, arr):
        self.rt = rt
        self.arr = np.ascontiguousarray(arr)
        self.ptr = C.c_void_p()
        assert rt.cudaMalloc(C.byref(self.ptr), C.c_size_t(max(self.arr.nbytes, 1))) == 0
        assert rt.cudaMemcpy(self.ptr, self.arr.ctypes.data_as(C.c_void_p), C.c_size_t(self.arr.nbytes), 1) == 0

    def get(self):
        out = np.empty_like(self.arr)
        assert self.rt.cudaMemcpy(out.ctypes.data_as(C.c_void_p), self.ptr, C.c_size_t(out.nbytes), 2) == 0
        return out

    def free(self):
        if self.ptr:
            self.rt.cudaFree(self.ptr)
            self.ptr = None


@pytest.mark.parametrize("name", ["c1_sphere_p1_n16.npz", "sphere_p2_n8.npz"])
def test_noalloc_pcg_matches_context_pcg(golden, name):
    from drops_gb300 import build

    build.build()
    g = golden(name)
    rowptr, colind, S, rhs = g["rowptr"], g["colind"], g["S"], g["rhs"]
    m = len(rhs)
    # the existing entry point on the same system
    with tf.TraceFEM() as ctx:
        ctx.matrix_upload(rowptr, colind, S)
        ctx.vec_upload(tf.VEC_B, rhs)
        ctx.vec_fill(tf.VEC_X, m, 0.0)
        st, it_ref, res_ref = ctx.pcg_jacobi(tf.MAT_USER, tf.VEC_B, tf.VEC_X, tol=1e-10)
        assert st == tf.OK
        x_ref = ctx.vec_download(tf.VEC_X)
    L = tf.load_library()
    rt = _cudart()
    rp = DevArray(rt, rowptr.astype(np.int32))
    ci = DevArray(rt, colind.astype(np.int32))
    va = DevArray(rt, S.astype(np.float64))
    b = DevArray(rt, rhs.astype(np.float64))
    try:
        for call in range(2):  # two calls in a row share the library's scratch array
            x = DevArray(rt, np.zeros(m))
            it, tol = C.c_int(100000), C.c_double(1e-10)
            st = L.tf_pcg_jacobi_noalloc(C.c_int64(m), rp.ptr, ci.ptr, va.ptr, b.ptr, x.ptr, C.byref(it), C.byref(tol),
                                         C.c_int(1), None)
            assert st == tf.OK, (call, st)
            assert tol.value <= 1e-10 and abs(it.value - it_ref) <= 1, (it.value, it_ref)
            xs = x.get()
            x.free()
            ok, err = sol_close(xs, x_ref, SOL_RTOL)
            assert ok, (call, err)
        # the reference's own solution of the same system
        ok, err = sol_close(xs, g["x"], SOL_RTOL)
        assert ok, err
        # max_iter = 0: no iteration, not converged, the initial relative residual (x = 0: 1)
        x = DevArray(rt, np.zeros(m))
        it, tol = C.c_int(0), C.c_double(1e-10)
        st = L.tf_pcg_jacobi_noalloc(C.c_int64(m), rp.ptr, ci.ptr, va.ptr, b.ptr, x.ptr, C.byref(it), C.byref(tol),
                                     C.c_int(1), None)
        assert st == tf.ERR_NOT_CONVERGED and it.value == 0 and abs(tol.value - 1.0) < 1e-14, (st, it.value, tol.value)
        assert np.array_equal(x.get(), np.zeros(m))
        x.free()
        # five iterations cannot reach 1e-10: not converged, the oracle's residual after five steps
        x = DevArray(rt, np.zeros(m))
        it, tol = C.c_int(5), C.c_double(1e-10)
        st = L.tf_pcg_jacobi_noalloc(C.c_int64(m), rp.ptr, ci.ptr, va.ptr, b.ptr, x.ptr, C.byref(it), C.byref(tol),
                                     C.c_int(1), None)
        ost, ox, oit, ores = O.pcg_jacobi(rowptr.astype(np.int64), colind.astype(np.int64), S, rhs, max_iter=5, tol=1e-10)
        assert st == tf.ERR_NOT_CONVERGED and it.value == 5 == oit, (st, it.value, oit)
        assert abs(tol.value - ores) <= 1e-9 * ores, (tol.value, ores)
        ok, err = sol_close(x.get(), ox, 1e-12)
        assert ok, err
        x.free()
        # an initial guess that already meets the tolerance: no iteration, converged, x untouched
        x = DevArray(rt, xs)
        it, tol = C.c_int(100), C.c_double(1e-10)
        st = L.tf_pcg_jacobi_noalloc(C.c_int64(m), rp.ptr, ci.ptr, va.ptr, b.ptr, x.ptr, C.byref(it), C.byref(tol),
                                     C.c_int(1), None)
        assert st == tf.OK and it.value == 0 and tol.value <= 1e-10, (st, it.value, tol.value)
        assert np.array_equal(x.get(), xs)
        x.free()
        # sizes beyond the fixed scratch array are refused before any device work
        it, tol = C.c_int(10), C.c_double(1e-10)
        st = L.tf_pcg_jacobi_noalloc(C.c_int64(MAX_ROWS + 1), rp.ptr, ci.ptr, va.ptr, b.ptr, b.ptr, C.byref(it),
                                     C.byref(tol), C.c_int(1), None)
        assert st == tf.ERR_CAPACITY
    finally:
        for d in (rp, ci, va, b):
            d.free()


def test_noalloc_pcg_repeatable_and_allocation_free():
    """Thirty solves in a row on a 36,606-row P2 system (sphere, 48^3 cubes) give
    bitwise identical solutions, iteration counts and residuals (a race on the
    shared scratch array between blocks would show up as a difference), and
    the device's free memory is the same before and after them."""
    from drops_gb300 import build

    build.build()
    with tf.TraceFEM() as ctx:
        n, a = 48, 5.0 / 3.0
        ctx.brick_cube(n, a)
        ctx.levelset_analytic(tf.LS_SPHERE, [0, 0, 0, 1.0], p2=True)
        ctx.distribute_dofs(tf.P2IF)
        ctx.setup_fe_system([tf.FORM_M, tf.FORM_A, tf.FORM_CN], tf.RHS_SPHERE_XYZ, [0, 0, 0, 1.0, 13.0])
        ctx.lincomb([tf.FORM_M, tf.FORM_A, tf.FORM_CN], [1.0, 1.0, 2 * a / n])
        rowptr, colind, S = ctx.matrix(tf.MAT_SYS)
        rhs = ctx.vec_download(tf.VEC_RHS)
    m = len(rhs)
    assert m == 36606 <= MAX_ROWS
    L = tf.load_library()
    rt = _cudart()
    rp = DevArray(rt, rowptr.astype(np.int32))
    ci = DevArray(rt, colind.astype(np.int32))
    va = DevArray(rt, S.astype(np.float64))
    b = DevArray(rt, rhs.astype(np.float64))
    x = DevArray(rt, np.zeros(m))
    zero = np.zeros(m)
    try:
        free0, total = C.c_size_t(), C.c_size_t()
        assert rt.cudaMemGetInfo(C.byref(free0), C.byref(total)) == 0
        first = None
        for call in range(30):
            assert rt.cudaMemcpy(x.ptr, zero.ctypes.data_as(C.c_void_p), C.c_size_t(zero.nbytes), 1) == 0
            it, tol = C.c_int(100000), C.c_double(1e-10)
            st = L.tf_pcg_jacobi_noalloc(C.c_int64(m), rp.ptr, ci.ptr, va.ptr, b.ptr, x.ptr, C.byref(it),
                                         C.byref(tol), C.c_int(1), None)
            assert st == tf.OK, (call, st)
            got = (x.get(), it.value, tol.value)
            if first is None:
                first = got
            else:
                assert np.array_equal(got[0], first[0]) and got[1:] == first[1:], (call, got[1:], first[1:])
        free1 = C.c_size_t()
        assert rt.cudaMemGetInfo(C.byref(free1), C.byref(total)) == 0
        assert free1.value == free0.value, (free0.value, free1.value)
        _, ox, _, _ = O.pcg_jacobi(rowptr.astype(np.int64), colind.astype(np.int64), S, rhs, tol=1e-10)
        ok, err = sol_close(first[0], ox, SOL_RTOL)
        assert ok, err
    finally:
        for d in (rp, ci, va, b, x):
            d.free()
