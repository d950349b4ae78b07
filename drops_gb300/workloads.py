"""Synthetic problem families of the TraceFEM path (seeded, reproducible).

The reference runs its surface problems on Kuhn bricks (geom/builder.cpp:99-180)
with analytic level sets (surfactant/Surface.hpp); these helpers produce the
parameters of such problems for the batched calls of the library.
"""
import numpy as np

BOX = 5.0 / 3.0  # half-width of the cube [-5/3, 5/3]^3 the surface Poisson problems live in


def haar_rotation(rng):
    """Uniformly distributed rotation (QR of a Gaussian matrix, signs fixed, det +1)."""
    q, r = np.linalg.qr(rng.standard_normal((3, 3)))
    q = q * np.sign(np.diag(r))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def ellipsoid_batch(count, nmin=16, nmax=64, seed=1000, box=BOX, axes_range=(0.6, 1.4), centre_radius=0.1):
    """`count` independent ellipsoid problems; instance i draws from seed + i.

    Per instance: mesh n^3 cubes of [-box, box]^3 with n uniform in
    [nmin, nmax]; semi-axes uniform in axes_range; a uniformly random rotation;
    the centre uniform in the ball of radius centre_radius.  Returns a dict
    with n[count,3], orig[count,3], axes[count,3,3] (rows e1, e2, e3),
    par[count,15] (TF_LS_ELLIPSOID parameters: centre, semi-axes, rotation Q
    row-major, phi = |diag(1/a,1/b,1/c) Q^T (x - c)| - 1) and h[count] (mesh
    width, the scale of the normal-gradient stabilisation).
    """
    n = np.empty((count, 3), np.int32)
    orig = np.empty((count, 3))
    axes = np.empty((count, 3, 3))
    par = np.empty((count, 15))
    h = np.empty(count)
    for i in range(count):
        rng = np.random.default_rng(seed + i)
        k = int(rng.integers(nmin, nmax + 1))
        semi = rng.uniform(axes_range[0], axes_range[1], 3)
        q = haar_rotation(rng)
        d = rng.standard_normal(3)
        d /= np.linalg.norm(d)
        centre = d * centre_radius * rng.uniform() ** (1.0 / 3.0)
        n[i] = k
        orig[i] = -box
        axes[i] = np.diag([2.0 * box] * 3)
        par[i, :3] = centre
        par[i, 3:6] = semi
        par[i, 6:] = q.ravel()
        h[i] = 2.0 * box / k
    return {"n": n, "orig": orig, "axes": axes, "par": par, "h": h}
