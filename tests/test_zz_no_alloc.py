"""The allocation-free PCG entry point (tf_pcg_jacobi_noalloc).

Callers that cannot allocate device memory -- applications that manage all
GPU memory through their own pool, real-time loops that must not trigger the
implicit synchronisation of cudaMalloc/cudaFree -- call tf_pcg_jacobi_noalloc
with their own device buffers; its
work vectors live in a fixed device array of the library.  This test drives it
through the C ABI twice in a row and checks both results against the regular
context-based entry point tf_pcg_jacobi on the same system.  The test itself
allocates its device buffers with the CUDA runtime; only the entry point under
test must not.
"""
import ctypes as C

import numpy as np
import pytest

import drops_gb300 as tf
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
        # sizes beyond the fixed scratch array are refused before any device work
        it, tol = C.c_int(10), C.c_double(1e-10)
        st = L.tf_pcg_jacobi_noalloc(C.c_int64(MAX_ROWS + 1), rp.ptr, ci.ptr, va.ptr, b.ptr, b.ptr, C.byref(it),
                                     C.byref(tol), C.c_int(1), None)
        assert st == tf.ERR_CAPACITY
    finally:
        for d in (rp, ci, va, b):
            d.free()
