"""The benchmark workload at its own size, through the CUDA path, against the oracle.

P2 TraceFEM surface Poisson on the sphere |x| = 1 in [-5/3, 5/3]^3 split into
96^3 Kuhn cubes (5,308,416 tets; 71,328 cut tets, 145,206 DOFs, 3,304,002
non-zeros), P2 level set, f = 13 xyz at ext(x), A = M + A_LB + h C_n, Jacobi-PCG
to relative residual 1e-10.  Checked:
  - cut tets, DOF numbering (Loc2Glo) and CSR pattern bit for bit (SHA-256);
  - M, A, C_n per entry within 1e-12 of their row's scale and the load vector
    within 1e-12 of its largest entry (tests/helpers.py), with the worst plain
    per-entry relative error printed beside;
  - the mixed-precision, the FP64 and the FP64 single-barrier PCG solutions
    within 1e-9 of the oracle's FP64 PCG solution; the FP64 residual of each
    on the GPU's own system (host arithmetic) within 1.01e-10, and on the
    oracle's system within 1.1e-10 (the two systems differ by the forms'
    rounding, ~1e-12 of the row scale, which moves the residual by ~1e-12).
The oracle (C restatement of the reference, pinned to the reference's own
outputs by tests/test_oracle_golden.py) takes a few seconds on this size.
"""
import numpy as np
import pytest

import drops_gb300 as tf
from oracle import pyoracle as O
from tests.helpers import entry_rel_err, loc2glo, mat_close, sha, sol_close

pytestmark = pytest.mark.gpu

N, HALF = 96, 5.0 / 3.0
SPHERE = [0.0, 0.0, 0.0, 1.0]
RHS = [0.0, 0.0, 0.0, 1.0, 13.0]


def test_p2_sphere96_against_oracle():
    from drops_gb300 import build

    build.build()
    h = 2 * HALF / N
    forms = [tf.FORM_M, tf.FORM_A, tf.FORM_CN]
    with tf.TraceFEM() as ctx:
        ctx.brick_cube(N, HALF)
        ctx.levelset_analytic(tf.LS_SPHERE, SPHERE, p2=True)
        na, m = ctx.distribute_dofs(tf.P2IF)
        ctx.setup_fe_system(forms, tf.RHS_SPHERE_XYZ, RHS)
        ctx.lincomb(forms, [1.0, 1.0, h])
        dv, de, act, l2g = ctx.dofs()
        mats = {f: ctx.matrix(f) for f in forms}
        rhs = ctx.vec_download(tf.VEC_RHS)
        xs = {}
        for key, prec, k64 in (("mixed", tf.PREC_MIXED, tf.PCG_FP64_CLASSIC), ("fp64", tf.PREC_FP64, tf.PCG_FP64_CLASSIC),
                               ("fp64_cg1", tf.PREC_FP64, tf.PCG_FP64_CG1)):
            ctx.pcg_options(k64)
            ctx.vec_fill(tf.VEC_X, m, 0.0)
            st, it, res = ctx.pcg_jacobi(tf.MAT_SYS, tf.VEC_RHS, tf.VEC_X, tol=1e-10, precision=prec)
            assert st == tf.OK and res <= 1e-10, (key, st, res)
            xs[key] = ctx.vec_download(tf.VEC_X)
        ctx.pcg_options(tf.PCG_FP64_CLASSIC)

    O.set_threads(0)
    mesh = O.brick(N, a=HALF)
    lv, le = O.levelset(mesh, O.LS_SPHERE, SPHERE, True)
    st, ona, om, odv, ode, oact = O.distribute_dofs(mesh, lv, le, True)
    assert st == O.OK and (na, m) == (ona, om) == (71328, 145206)
    assert sha(act) == sha(np.nonzero(oact)[0].astype(act.dtype))
    assert sha(l2g) == sha(loc2glo(mesh, oact, odv, ode, True).astype(l2g.dtype))
    opts = O.make_opts(True, forms, O.RHS_SPHERE_XYZ, RHS)
    st, orp, oci, vals, orhs = O.assemble(mesh, lv, le, oact, odv, ode, m, opts)
    assert st == O.OK and len(oci) == 3304002
    report, fails = {}, []
    for f, name in zip(forms, ("M", "A", "C_n")):
        rp, ci, v = mats[f]
        assert sha(rp.astype(np.int64)) == sha(orp.astype(np.int64)) and sha(ci.astype(np.int32)) == sha(oci)
        ok, err = mat_close(v, vals[f], orp)
        report[name] = (err, entry_rel_err(v, vals[f]))
        if not ok:
            fails.append(name)
    ok, err = mat_close(rhs, orhs)
    report["rhs"] = (err, entry_rel_err(rhs, orhs))
    if not ok:
        fails.append("rhs")
    S = vals[O.FORM_M] + vals[O.FORM_A] + h * vals[O.FORM_CN]
    st, ox, oit, ores = O.pcg_jacobi(orp, oci, S, orhs, tol=1e-10)
    assert st == O.OK
    Sg = mats[tf.FORM_M][2] + mats[tf.FORM_A][2] + h * mats[tf.FORM_CN][2]
    for name, x in xs.items():
        r = np.linalg.norm(orhs - O.spmv(orp, oci, S, x)) / np.linalg.norm(orhs)
        rg = np.linalg.norm(rhs - O.spmv(orp, oci, Sg, x)) / np.linalg.norm(rhs)
        ok, err = sol_close(x, ox)
        report[f"x_{name}"] = (err, r, rg)
        if not ok or rg > 1.01e-10 or r > 1.1e-10:
            fails.append(f"x_{name}")
    for k, vs in report.items():
        print(f"{k}: " + " ".join(f"{a:.3e}" for a in vs))
    assert not fails, (fails, report)
