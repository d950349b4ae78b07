"""Synthetic problem families (host only)."""
import numpy as np

from drops_gb300.workloads import ellipsoid_batch


def test_ellipsoid_batch_distribution_and_reproducibility():
    W = ellipsoid_batch(64, nmin=16, nmax=64, seed=1000)
    assert W["n"].shape == (64, 3) and np.all(W["n"][:, 0] == W["n"][:, 1]) and np.all(W["n"][:, 0] == W["n"][:, 2])
    assert W["n"].min() >= 16 and W["n"].max() <= 64
    semi = W["par"][:, 3:6]
    assert semi.min() >= 0.6 and semi.max() <= 1.4
    assert np.all(np.linalg.norm(W["par"][:, :3], axis=1) <= 0.1)
    for q in W["par"][:, 6:].reshape(-1, 3, 3):
        assert np.allclose(q @ q.T, np.eye(3), atol=1e-12) and abs(np.linalg.det(q) - 1.0) < 1e-12
    assert np.allclose(W["h"], 2 * (5.0 / 3.0) / W["n"][:, 0])
    W2 = ellipsoid_batch(64, nmin=16, nmax=64, seed=1000)
    assert all(np.array_equal(W[k], W2[k]) for k in W)
    # instance i depends on seed + i only
    W3 = ellipsoid_batch(8, nmin=16, nmax=64, seed=1004)
    assert np.array_equal(W3["par"][0], W["par"][4])
