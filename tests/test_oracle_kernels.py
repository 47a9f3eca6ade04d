"""The oracle's compiled sweeps (oracle/kernels.c) equal its NumPy loops bit for bit."""
import numpy as np
import pytest

from oracle import _ck
from oracle import linalg as ol
from oracle import spectral as osp


@pytest.fixture(scope="module")
def clib():
    try:
        _ck.build()
    except Exception as e:  # pragma: no cover - no gcc
        pytest.skip("gcc unavailable: %s" % e)
    L = _ck.lib()
    assert L is not None
    return L


def numpy_only(fn, *args):
    saved = _ck.lib
    _ck.lib = lambda: None
    try:
        return fn(*args)
    finally:
        _ck.lib = saved


def both(fn, *args):
    a = fn(*[x.copy() if isinstance(x, np.ndarray) else x for x in args])
    b = numpy_only(fn, *[x.copy() if isinstance(x, np.ndarray) else x for x in args])
    return a, b


@pytest.mark.parametrize("n,m", [(4, 1), (9, 3), (33, 17), (64, 40)])
def test_fdma_solve_bitwise(clib, n, m):
    rng = np.random.default_rng(n * 100 + m)
    l, d, u1, u2 = rng.standard_normal(n - 2), 3 + rng.random(n), rng.standard_normal(n - 2), rng.standard_normal(n - 4)
    x = rng.standard_normal((n, m))
    a, b = both(ol.fdma_solve, l, d, u1, u2, x)
    assert np.array_equal(a, b)
    # strided right-hand side (a transposed view): the result lands in the view
    xt = rng.standard_normal((m, n)).T
    a, b = both(ol.fdma_solve, l, d, u1, u2, xt)
    assert np.array_equal(a, b)
    # one system per column (the stacked Poisson systems)
    L2, D2, U1, U2 = (rng.standard_normal((n - 2, m)), 3 + rng.random((n, m)), rng.standard_normal((n - 2, m)),
                      rng.standard_normal((n - 4, m)))
    a, b = both(ol.fdma_solve, L2, D2, U1, U2, x)
    assert np.array_equal(a, b)
    a, b = both(ol.fdma_lu, L2, D2, U1, U2)
    for p, q in zip(a, b):
        assert np.array_equal(p, q)


@pytest.mark.parametrize("n,m", [(2, 1), (7, 5), (65, 33)])
def test_twodma_bitwise(clib, n, m):
    rng = np.random.default_rng(n + m)
    d, u, x = 2 + rng.random(n), rng.standard_normal(n - 2), rng.standard_normal((n, m))
    a, b = both(ol.twodma_solve, d, u, x)
    assert np.array_equal(a, b)
    a, b = both(ol.twodma_solve, d, u, x[:, 0].copy())
    assert np.array_equal(a, b)


@pytest.mark.parametrize("n,m,k", [(5, 1, 2), (17, 4, 2), (64, 9, 1), (40, 3, 3)])
def test_tdma_offset_bitwise(clib, n, m, k):
    rng = np.random.default_rng(n * k + m)
    a, bb, c = rng.standard_normal(n - k), 4 + rng.random(n), rng.standard_normal(n - k)
    rhs = rng.standard_normal((n, m))
    p, q = both(ol.tdma_offset, a, bb, c, rhs, k)
    assert np.array_equal(p, q)
    p, q = both(ol.tdma_offset, a, bb, c, rhs[:, 0].copy(), k)
    assert np.array_equal(p, q) and p.shape == (n,)


@pytest.mark.parametrize("shape,axis", [((3,), 0), ((12, 7), 0), ((7, 12), 1), ((5, 6, 4), 1)])
def test_cheb_diff_bitwise(clib, shape, axis):
    c = np.random.default_rng(len(shape)).standard_normal(shape)
    a, b = both(osp.cheb_diff, c, 2, axis)
    assert np.array_equal(a, b)


def test_fdma_type2_bitwise(clib):
    rng = np.random.default_rng(7)
    n, m = 24, 10
    A = np.diag(2 + rng.random(n)) + np.diag(rng.random(n - 2), 2) + np.diag(rng.random(n - 2), -2) \
        + np.diag(rng.random(n - 4), 4)
    C = np.diag(1 + rng.random(n)) + np.diag(rng.random(n - 2), 2)
    lam = np.concatenate([[0.0], 1 + rng.random(m - 1)])
    x = rng.standard_normal((n, m))
    for singular in (False, True):
        a, b = both(ol.fdma_type2, A, C, lam, x, singular)
        assert np.array_equal(a, b)
