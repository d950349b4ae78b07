"""Shared comparison helpers for the parity tests."""
import hashlib

import numpy as np

# FP64 matrix entries, per entry: |a_ij - b_ij| <= MAT_RTOL * s_i, where s_i is
# the scale of row i, max(max_k |b_ik|, MAT_FLOOR * max|b|).  An entry that is a
# sum with cancellation is judged against the size of its row, not its own
# size.  Rows whose largest entry is below MAT_FLOOR * max|b| belong to DOFs
# whose surface piece is tiny; their entries come from facets spanned by cut
# points a short distance apart, where two correct evaluations of the same
# formulas round differently by up to ~1e-17 * max|b| (measured on the P1
# torus: the C restatement against the reference 4e-18, the CUDA path 1.1e-17),
# so they are held to MAT_RTOL * MAT_FLOOR * max|b| absolutely.
# Load vectors have no row scale and an odd f (13xyz) makes entries cancel to
# ~1e-16 * max|b|: they are compared norm-wise, |a_i - b_i| <= MAT_RTOL * max|b|
# (VEC_FLOOR = 1).
MAT_RTOL = 1e-12
MAT_FLOOR = 1e-4
VEC_FLOOR = 1.0
# solutions: ||x - x_ref||_2 <= 1e-9 ||x_ref||_2
SOL_RTOL = 1e-9


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def entry_scale(b, rowptr=None, floor=None):
    """Per-entry scale s: the row maximum of |b| (rowptr given) or |b_i| (a vector), at least floor * max|b|
    (floor: MAT_FLOOR for a matrix, VEC_FLOOR for a vector)."""
    b = np.abs(np.asarray(b, dtype=np.float64))
    if not b.size:
        return b
    if floor is None:
        floor = VEC_FLOOR if rowptr is None else MAT_FLOOR
    lo = floor * b.max()
    if rowptr is None:
        return np.maximum(b, lo)
    rowptr = np.asarray(rowptr, dtype=np.int64)
    cnt = np.diff(rowptr)
    rowmax = np.zeros(len(cnt))
    nz = cnt > 0
    rowmax[nz] = np.maximum.reduceat(b, rowptr[:-1][nz])
    return np.maximum(np.repeat(rowmax, cnt), lo)


def mat_close(a, b, rowptr=None, rtol=MAT_RTOL, floor=None):
    """(ok, worst |a - b| / s) with the per-entry scale s of entry_scale."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if not b.size:
        return True, 0.0
    err = float((np.abs(a - b) / entry_scale(b, rowptr, floor)).max())
    return err <= rtol, err


def entry_rel_err(a, b, floor=1e-12):
    """Worst plain relative error |a_ij - b_ij| / |b_ij| over the entries with |b_ij| > floor * max|b|
    (reported beside mat_close; cancellation makes it larger than the row-scaled error)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    sel = np.abs(b) > floor * np.abs(b).max()
    return float((np.abs(a - b)[sel] / np.abs(b[sel])).max()) if sel.any() else 0.0


def sol_close(x, xr, rtol=SOL_RTOL):
    err = np.linalg.norm(x - xr) / np.linalg.norm(xr)
    return err <= rtol, err


def loc2glo(mesh, active, dof_vert, dof_edge, p2):
    ts = np.nonzero(active)[0]
    if p2:
        return np.concatenate([dof_vert[mesh.tet_v[ts]], dof_edge[mesh.tet_e[ts]]], axis=1).ravel()
    return dof_vert[mesh.tet_v[ts]].ravel()


def sparse_close(X, G, rtol=MAT_RTOL, floor=MAT_FLOOR):
    """mat_close for two scipy sparse matrices whose patterns may differ (entries missing from one
    count as zeros): |X_ij - G_ij| <= rtol * max(max_k |G_ik|, floor * max|G|).  Returns (ok, worst)."""
    import scipy.sparse as sp

    X, G = sp.csr_matrix(X), sp.csr_matrix(G)
    D = abs(X - G).tocsr()
    if D.nnz == 0:
        return True, 0.0
    rowmax = abs(G).max(axis=1).toarray().ravel()
    s = np.maximum(rowmax, floor * abs(G).max())
    worst = float(D.multiply(1.0 / s[:, None]).max())
    return worst <= rtol, worst
