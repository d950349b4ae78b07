"""The CPU oracle of the warm-start MLP: its backward pass against finite differences (host only)."""
import numpy as np

from oracle import pyoracle as O


def random_problem(n, seed):
    rng = np.random.default_rng(seed)
    w = np.zeros(O.MLP_WEIGHTS, np.float32)
    for l, (rows, fan_in) in enumerate(((64, 71), (64, 65), (64, 65), (2, 65))):
        W = w[l * 64 * 80:(l * 64 + rows) * 80].reshape(rows, 80)
        W[:, :fan_in] = rng.uniform(-1, 1, (rows, fan_in)) * np.sqrt(3.0 / fan_in)
    x = np.zeros((n, 80), np.float32)
    x[:, :70] = rng.standard_normal((n, 70))
    x[:, 70] = 1.0
    X = O.bf16_bits(x)
    Y = rng.standard_normal((n, 2)).astype(np.float32)
    return w, X, Y


def test_mlp_oracle_gradient_matches_finite_differences():
    w, X, Y = random_problem(37, 7)
    g, loss = O.mlp_gradient(w, X, Y, exact=True)
    rng = np.random.default_rng(3)
    real = np.nonzero(g)[0]
    for i in rng.choice(real, 40, replace=False):
        h = np.float32(1e-3 * max(1.0, abs(w[i])))
        wp, wm = w.copy(), w.copy()
        wp[i] += h
        wm[i] -= h
        lp = O.mlp_gradient(wp, X, Y, exact=True)[1]
        lm = O.mlp_gradient(wm, X, Y, exact=True)[1]
        fd = (lp - lm) / (float(wp[i]) - float(wm[i]))
        assert abs(fd - g[i]) <= 1e-4 * max(1e-3, abs(g[i])) + 1e-7, (i, fd, g[i])


def test_mlp_oracle_bf16_emulation_close_to_exact():
    w, X, Y = random_problem(64, 11)
    g0, l0 = O.mlp_gradient(w, X, Y, exact=True)
    g1, l1 = O.mlp_gradient(w, X, Y, exact=False)
    assert abs(l0 - l1) <= 2e-2 * l0
    assert np.linalg.norm(g1 - g0) <= 5e-2 * np.linalg.norm(g0)
    p0 = O.mlp_forward(w, X, exact=True)
    p1 = O.mlp_forward(w, X, exact=False)
    assert np.max(np.abs(p1 - p0)) <= 5e-2 * np.max(np.abs(p0))
    # padding rows / columns carry no gradient
    G = g1[:3 * 64 * 80].reshape(3, 64, 80)
    assert np.all(G[0, :, 71:] == 0) and np.all(G[1:, :, 65:] == 0)
    assert np.all(g1[3 * 64 * 80 + 2 * 80:] == 0)
