"""y_Ax (num/spmat.h:1684-1709) through tf_spmv: the FP32-pair kernel and the FP64-FMA kernel against the
oracle's FP64 product."""
import numpy as np
import pytest

import drops_gb300 as tf
from oracle import pyoracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctxs():
    from drops_gb300 import build

    build.build()
    pair, native = tf.TraceFEM(), tf.TraceFEM()
    pair.spmv_options(tf.SPMV_KERNEL_PAIR)
    native.spmv_options(tf.SPMV_KERNEL_FP64)
    yield pair, native
    pair.close()
    native.close()


def _spmv(ctx, rp, ci, v, x):
    ctx.matrix_upload(rp, ci, v)
    ctx.vec_upload(tf.VEC_X, x)
    ctx.spmv(tf.MAT_USER, tf.VEC_X, tf.VEC_T0)
    return ctx.vec_download(tf.VEC_T0)


# pair arithmetic carries ~48 significant bits: per product ~3 * 2^-48 relative, summed over the row
PAIR_REL = 3e-13
# FP64 FMA chain against the oracle's FP64 sum: a few ulps of sum |a_ij x_j|
FP64_REL = 4e-15


def _check(y, rp, ci, v, x, rel=PAIR_REL):
    """Per row: |y_i - (A x)_i| <= rel * sum_j |a_ij x_j|."""
    ref = O.spmv(rp, ci, v, x)
    mag = O.spmv(rp, ci, np.abs(v), np.abs(x))
    err = np.abs(y - ref)
    bound = rel * mag + 1e-300
    assert np.all(err <= bound), (np.max(err / bound), int(np.argmax(err / bound)))
    return ref


@pytest.mark.parametrize("name,key", [("c1_sphere_p1_n16.npz", "S"), ("sphere_p2_n8.npz", "M"),
                                      ("torus_p1_n16.npz", "A"), ("torus_p2_n10.npz", "C")])
def test_spmv_matches_oracle(ctxs, golden, name, key):
    g = golden(name)
    rp, ci, v = g["rowptr"], g["colind"], g[key]
    rng = np.random.default_rng(11)
    for x in (rng.uniform(-1, 1, len(rp) - 1), g["x"] if "x" in g else rng.standard_normal(len(rp) - 1)):
        ys = [_spmv(c, rp, ci, v, x) for c in ctxs]
        _check(ys[0], rp, ci, v, x, PAIR_REL)
        _check(ys[1], rp, ci, v, x, FP64_REL)
        # within the 1e-12 parity bound of each other
        assert np.max(np.abs(ys[0] - ys[1])) <= 1e-12 * max(np.max(np.abs(ys[1])), 1e-300)


def test_spmv_wide_range(ctxs):
    """Row scaling covers rows of any magnitude; non-zero x outside [2^-74, 2^100] takes the FP64 path in the
    same launch; a non-finite matrix value keeps the matrix on the FP64 kernel."""
    rng = np.random.default_rng(5)
    m = 3000
    rp = np.arange(0, 7 * m + 1, 7, dtype=np.int64)
    ci = np.stack([(np.arange(m) + d) % m for d in (-3, -2, -1, 0, 1, 2, 3)], axis=1).ravel().astype(np.int32)
    ci = np.sort(ci.reshape(m, 7), axis=1).ravel()
    v = rng.uniform(-1, 1, 7 * m)
    scale = 10.0 ** rng.integers(-250, 250, m)  # row magnitudes from 1e-250 to 1e250
    v *= np.repeat(scale, 7)
    v[5::97] *= 1e-20  # entries tiny relative to their row
    x = rng.uniform(-1, 1, m)
    pair, native = ctxs
    _check(_spmv(pair, rp, ci, v, x), rp, ci, v, x, PAIR_REL)
    _check(_spmv(native, rp, ci, v, x), rp, ci, v, x, FP64_REL)
    # x out of the pair range: the flag sends the launch down the FP64 path (FP64 FMAs in CSR order, a few
    # ulps of sum |a_ij x_j| from the oracle and from the balanced FP64 kernel, which splits wide slices)
    x2 = x.copy()
    x2[::500] = 1e-200
    x2[7] = 1e40
    y = _spmv(pair, rp, ci, v, x2)
    _check(y, rp, ci, v, x2, FP64_REL)
    _check(_spmv(native, rp, ci, v, x2), rp, ci, v, x2, FP64_REL)
    # a non-finite value: the FP64 kernel, whose IEEE result the oracle reproduces
    v3 = v.copy()
    v3[100] = np.inf
    y = _spmv(pair, rp, ci, v3, x)
    ref = O.spmv(rp, ci, v3, x)
    assert np.array_equal(np.isfinite(y), np.isfinite(ref))
    fin = np.isfinite(ref)
    assert np.all(np.abs(y[fin] - ref[fin]) <= FP64_REL * O.spmv(rp, ci, np.abs(v3), np.abs(x))[fin])


def _random_csr(rng, lengths, m):
    """Rows of the given lengths; row r holds the distinct columns (r + k s_r) mod m, k < length, sorted."""
    lengths = np.asarray(lengths, dtype=np.int64)
    rp = np.zeros(m + 1, dtype=np.int64)
    rp[1:] = np.cumsum(lengths)
    row = np.repeat(np.arange(m), lengths)
    k = np.arange(rp[-1]) - np.repeat(rp[:-1], lengths)
    ci = (row + k * (1 + (row % 3))) % m  # steps 1..3 < m / max length: distinct per row
    order = np.lexsort((ci, row))
    v = rng.uniform(-1, 1, rp[-1])
    return rp, ci[order].astype(np.int32), v


@pytest.mark.parametrize("case", ["tiny", "empty_rows", "one_long_row", "uneven", "many_slices"])
def test_spmv_balanced_uneven_rows(ctxs, case):
    """The balanced kernel splits the column work of a block's slices evenly over its warps, so slices are
    shared by several warps; uneven rows, empty rows, single-slice matrices and blocks with fewer columns than
    warps must all give the oracle's product, bit-identical from call to call."""
    rng = np.random.default_rng({"tiny": 1, "empty_rows": 2, "one_long_row": 3, "uneven": 4, "many_slices": 5}[case])
    if case == "tiny":
        m = 5
        lengths = np.array([1, 0, 3, 5, 2])
    elif case == "empty_rows":
        m = 3000
        lengths = rng.integers(0, 4, m) * (rng.random(m) < 0.3)
    elif case == "one_long_row":
        m = 2000
        lengths = np.ones(m, dtype=np.int64)
        lengths[777] = 600
    elif case == "uneven":
        m = 40000
        lengths = np.where(rng.random(m) < 0.1, rng.integers(40, 63, m), rng.integers(8, 20, m))
    else:
        m = 300000
        lengths = rng.integers(5, 16, m)
    rp, ci, v = _random_csr(rng, lengths, m)
    x = rng.uniform(-1, 1, m)
    pair, native = ctxs
    y = _spmv(native, rp, ci, v, x)
    _check(y, rp, ci, v, x, FP64_REL)
    assert np.array_equal(y, _spmv(native, rp, ci, v, x))
    yp = _spmv(pair, rp, ci, v, x)
    _check(yp, rp, ci, v, x, PAIR_REL)
    assert np.array_equal(yp, _spmv(pair, rp, ci, v, x))


def test_spmv_split_edges(ctxs):
    """x at the edges of the pair range (2^-74, 2^100, significands with all low bits set, single low bits,
    zeros of both signs): the integer split keeps |x - hi - lo| <= 2^-47 |x|."""
    base = np.array([2.0 ** -74, 2.0 ** 100, 1.0, 0.0, np.nextafter(1.0, 2.0), np.nextafter(2.0, 0.0),
                     1.0 + 2.0 ** -24, 1.0 + 2.0 ** -23 + 2.0 ** -52, np.nextafter(2.0 ** 101, 0.0), 0.1, np.pi])
    x = np.concatenate([base, -base, base * 1.25, base * (1 + 2.0 ** -30), base * 2.0 ** -20, base * 2.0 ** 20])
    mag = np.abs(x)
    x = x[(mag == 0) | ((mag >= 2.0 ** -74) & (mag < 2.0 ** 101))]
    m = len(x)
    rp = np.arange(m + 1, dtype=np.int64)
    ci = np.arange(m, dtype=np.int32)
    v = np.ones(m)
    y = _spmv(ctxs[0], rp, ci, v, x)
    assert np.all(np.abs(y - x) <= 2.0 ** -47 * np.abs(x)), np.max(np.abs(y - x) / np.maximum(np.abs(x), 1e-300))


def test_spmv_pair_large(ctxs):
    """The pair kernel on a matrix of 9M stored entries (a few hundred blocks of 64 slices each, several chunks
    per block) and the default kernel (FP64), bit-identical to a context forced to FP64 at the same launch
    shape; an unknown kernel is refused.  The balanced kernel's warps split a block's column work, so the
    order in which a row's partial sums meet follows the grid: two contexts compare bit for bit only at the
    same shape (the fixed default here, autotuning off in both), and each is checked against the FP64 bound."""
    pair, _ = ctxs
    rng = np.random.default_rng(21)
    m = 400000
    rp, ci, v = _random_csr(rng, rng.integers(18, 26, m), m)
    assert rp[-1] >= 8 << 20
    x = rng.uniform(-1, 1, m)
    _check(_spmv(pair, rp, ci, v, x), rp, ci, v, x, PAIR_REL)
    default, native = tf.TraceFEM(), tf.TraceFEM()
    try:
        with pytest.raises(tf.TraceFEMError):
            default.spmv_options(2)
        native.spmv_options(tf.SPMV_KERNEL_FP64)
        default.autotune(False)
        native.autotune(False)
        y = _spmv(default, rp, ci, v, x)
        _check(y, rp, ci, v, x, FP64_REL)
        assert np.array_equal(y, _spmv(native, rp, ci, v, x))
    finally:
        default.close()
        native.close()
