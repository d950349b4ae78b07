"""Shared comparison helpers for the parity tests."""
import hashlib

import numpy as np

# FP64 matrix entries: |a - b| <= 1e-12 * max|b| over the matrix (entries whose
# rows carry only a vanishing surface area, ~1e-32, are compared in that norm).
MAT_RTOL = 1e-12
# solutions: ||x - x_ref||_2 <= 1e-9 ||x_ref||_2
SOL_RTOL = 1e-9


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def mat_close(a, b, rtol=MAT_RTOL):
    a = np.asarray(a)
    b = np.asarray(b)
    scale = np.abs(b).max() if b.size else 1.0
    err = np.abs(a - b).max() / scale if b.size else 0.0
    return err <= rtol, err


def sol_close(x, xr, rtol=SOL_RTOL):
    err = np.linalg.norm(x - xr) / np.linalg.norm(xr)
    return err <= rtol, err


def loc2glo(mesh, active, dof_vert, dof_edge, p2):
    ts = np.nonzero(active)[0]
    if p2:
        return np.concatenate([dof_vert[mesh.tet_v[ts]], dof_edge[mesh.tet_e[ts]]], axis=1).ravel()
    return dof_vert[mesh.tet_v[ts]].ravel()
