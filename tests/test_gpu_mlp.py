"""Warm-start MLP on the tensor cores: forward and gradients against the CPU oracle, training, features, and
the learned Cahn-Hilliard warm start against the plain previous-state warm start."""
import numpy as np
import pytest

import drops_gb300 as tf
from oracle import pyoracle as O
from tests.test_mlp_oracle import random_problem

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from drops_gb300 import build

    build.build()
    c = tf.TraceFEM()
    yield c
    c.close()


@pytest.mark.parametrize("n", [1, 128, 300, 1000])
def test_mlp_forward_matches_oracle(ctx, n):
    w, X, _ = random_problem(n, 100 + n)
    ctx.mlp_weights(w)
    pred = ctx.mlp_forward(X)
    ref = O.mlp_forward(w, X)
    scale = max(1.0, float(np.max(np.abs(ref))))
    # BF16 activations: an FP32 sum that lands on the other side of a rounding
    # boundary than the oracle's moves one activation by one BF16 step
    assert np.max(np.abs(pred - ref)) <= 2e-2 * scale, np.max(np.abs(pred - ref))
    assert np.mean(np.abs(pred - ref)) <= 2e-3 * scale


@pytest.mark.parametrize("n", [128, 333, 2048])
def test_mlp_gradient_matches_oracle(ctx, n):
    w, X, Y = random_problem(n, 200 + n)
    ctx.mlp_weights(w)
    g, loss = ctx.mlp_gradient(X, Y)
    og, oloss = O.mlp_gradient(w, X, Y)
    assert abs(loss - oloss) <= 1e-2 * oloss
    assert np.linalg.norm(g - og) <= 2e-2 * np.linalg.norm(og), np.linalg.norm(g - og) / np.linalg.norm(og)
    # per layer as well
    for l in range(4):
        a, b = g[l * 5120:(l + 1) * 5120], og[l * 5120:(l + 1) * 5120]
        assert np.linalg.norm(a - b) <= 3e-2 * np.linalg.norm(b) + 1e-9, l
    # weights unchanged by a gradient evaluation
    assert np.array_equal(ctx.mlp_weights(), w)


def test_mlp_training_fits_a_smooth_map(ctx):
    rng = np.random.default_rng(5)
    n = 4096
    x = np.zeros((n, 80), np.float32)
    x[:, :70] = rng.uniform(-1, 1, (n, 70))
    x[:, 70] = 1
    X = O.bf16_bits(x)
    xv = O.bf16_value(X)
    Y = np.stack([np.sin(xv[:, 0]) + 0.5 * xv[:, 1], xv[:, 2] * xv[:, 3]], axis=1).astype(np.float32)
    ctx.mlp_init(7)
    _, l0 = ctx.mlp_gradient(X, Y)
    for _ in range(30):
        l1 = ctx.mlp_train(X, Y, epochs=1, minibatch_tiles=8, lr=3e-3)
    assert l1 < 0.2 * l0, (l0, l1)


def _torus(ctx, n=16, a=1.6):
    ctx.brick_cube(n, a)
    ctx.levelset_analytic(tf.LS_TORUS, [1.0, 0.4, 2], False)
    na, nd = ctx.distribute_dofs(tf.P1IF)
    ctx.setup_fe_system([tf.FORM_M, tf.FORM_A, tf.FORM_CN])
    return nd, 2 * a / n


def _bf16(v):
    return O.bf16_bits(np.asarray(v, dtype=np.float64).astype(np.float32))


def test_ch_features_bitexact(ctx):
    nd, h = _torus(ctx)
    rng = np.random.default_rng(3)
    states = [np.concatenate([0.5 + rng.uniform(-0.01, 0.01, nd), rng.uniform(-0.1, 0.1, nd)])]
    ctx.vec_upload(tf.VEC_X, states[0])
    for _ in range(3):
        ctx.ch_steps(1, 1e-3, 1.0, 0.02, 0.0, 1.0, h, tol=1e-10)
        states.append(ctx.vec_download(tf.VEC_X))
    xo, xn, xx = states[1], states[2], states[3]
    ctx.vec_upload(tf.VEC_T0, xn)
    ctx.vec_upload(tf.VEC_T1, xo)
    ctx.vec_upload(tf.VEC_T2, xx)
    X, Y = ctx.ch_features(tf.VEC_T0, tf.VEC_T1, tf.VEC_T2)
    # restatement
    m = nd
    rp, ci, _ = ctx.matrix(tf.FORM_M)
    s_c = np.sqrt(np.sum((xn[:m] - xo[:m]) ** 2) / m)
    s_w = np.sqrt(np.sum((xn[m:] - xo[m:]) ** 2) / m)
    S_w = np.sqrt(np.sum(xn[m:] ** 2) / m)
    coords, tv, te, ev = ctx.mesh_download()
    dv, _, act, l2g = ctx.dofs()
    lv, _ = ctx.levelset_download()
    first = {}
    for r, d in enumerate(l2g):
        first.setdefault(int(d), r // 4)
    ref = np.zeros((m, 80), np.uint16)
    for i in range(m):
        row = [i] + [int(j) for j in ci[rp[i]:rp[i + 1]] if j != i][:15]
        f = np.zeros(80)
        for s, j in enumerate(row):
            f[4 * s:4 * s + 4] = [2.0 * (xn[j] - 0.5), (xn[j] - xo[j]) / s_c, xn[m + j] / S_w,
                                  (xn[m + j] - xo[m + j]) / s_w]
        ref[i, :64] = _bf16(f[:64])
        v = int(np.nonzero(dv == i)[0][0])
        t = tv[act[first[i]]]
        p = coords[t]
        fv = lv[t]
        e = p[1:] - p[0]
        g = np.zeros(3)
        for k in range(3):
            aa, bb = e[(k + 1) % 3], e[(k + 2) % 3]
            cr = np.array([aa[1] * bb[2] - aa[2] * bb[1], aa[2] * bb[0] - aa[0] * bb[2], aa[0] * bb[1] - aa[1] * bb[0]])
            g = g + (fv[k + 1] - fv[0]) * cr
        nn = np.sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2])
        ref[i, 64:67] = O.bf16_bits(coords[v].astype(np.float32))
        ref[i, 67:70] = O.bf16_bits((g * (1.0 / nn)).astype(np.float32))
        ref[i, 70] = O.bf16_bits(np.float32([1.0]))[0]
    assert np.array_equal(X, ref), np.argwhere(X != ref)[:5]
    # targets: deviation of the increment from linear extrapolation
    yref = np.stack([((xx[:m] - xn[:m]) - (xn[:m] - xo[:m])) / s_c,
                     ((xx[m:] - xn[m:]) - (xn[m:] - xo[m:])) / s_w], axis=1).astype(np.float32)
    assert np.array_equal(Y, yref)


def test_learned_warm_start_converges_and_gains(ctx):
    """Same CH run four times: previous-state warm start (the reference's), linear extrapolation, the
    minimal-residual projection onto the last 6 states, and that projection with the MLP's correction
    added to its basis (trained online on steps 1..12).  Every solve reaches the tolerance and the final
    states agree.  In total GMRES iterations: learned < extrapolated < previous state, and projected <
    extrapolated; the learned run stays within 5% of the projection without the network (the network's
    own contribution, printed)."""
    nd, h = _torus(ctx, 20)
    rng = np.random.default_rng(21)
    x0 = np.concatenate([0.5 + rng.uniform(-0.01, 0.01, nd), np.zeros(nd)])
    args = (24, 1e-3, 1.0, 0.02, 0.0, 1.0, h)
    runs = {}
    for mode in (0, 2, 3, 1):
        ctx.mlp_init(3)
        ctx.vec_upload(tf.VEC_X, x0)
        st, its, res, used = ctx.ch_steps_learned(*args, learned=mode, train_steps=12, epochs=3, lr=2e-3)
        assert st == tf.OK and np.all(res <= 1e-10)
        runs[mode] = (its, used.astype(bool), ctx.vec_download(tf.VEC_X))
        print("mode", mode, "iterations", int(its.sum()), its.tolist(), "used", int(used.sum()))
    it_p, used_p, xp = runs[0]
    assert not used_p.any()
    for mode in (2, 3, 1):
        its, u, x = runs[mode]
        assert np.linalg.norm(x - xp) <= 1e-6 * np.linalg.norm(xp)
        assert u.sum() >= 3, (mode, u)
    tot = {k: int(v[0].sum()) for k, v in runs.items()}
    assert tot[1] < tot[2] < tot[0], tot
    assert tot[3] < tot[2], tot
    assert tot[1] <= 1.05 * tot[3], tot
