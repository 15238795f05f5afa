"""Daughter tables (pbe_gb300.quadrature) against numpy's Gauss-Legendre and
the moment constraints of docs/theory.md:34-38 (volume per event = parent)."""
import numpy as np
import pytest

import pbe_gb300 as pg
from pbe_gb300 import quadrature as q


@pytest.mark.parametrize("order", [1, 2, 3, 4, 5, 8, 12, 16, 32, 64])
def test_gauss_legendre_matches_numpy(order):
    t, w = q.gauss_legendre(order)
    tr, wr = np.polynomial.legendre.leggauss(order)
    assert np.max(np.abs(t - tr)) < 4e-16
    assert np.max(np.abs(w - wr)) < 4e-15


def test_symmetric_and_erosion():
    assert q.moments(*q.symmetric_binary()) == (2.0, 1.0)
    nu, vol = q.moments(*q.symmetric_binary_split(16))
    assert abs(nu - 2.0) < 1e-15 and abs(vol - 1.0) < 1e-15
    nu, vol = q.moments(*q.erosion(0.05))
    assert nu == 2.0 and abs(vol - 1.0) < 1e-15


@pytest.mark.parametrize("order", [2, 4, 8, 16])
def test_uniform_daughter(order):
    t, bw = q.uniform(order)
    assert np.all((t > 0) & (t < 1))
    nu, vol = q.moments(t, bw)
    assert abs(nu - 2.0) < 1e-14 and abs(vol - 1.0) < 1e-14


@pytest.mark.parametrize("p", [0.0, 1.0, 2.0, 3.0])
@pytest.mark.parametrize("order", [4, 8])
def test_power_law_daughter(p, order):
    t, bw = q.power_law(p, order)
    assert len(t) == 2 * order
    nu, vol = q.moments(t, bw)
    assert abs(nu - (p + 2.0) / (p + 1.0)) < 1e-14
    assert abs(vol - 1.0) < 1e-14


def test_power_law_noninteger_exponent_converges():
    t, bw = q.power_law(0.5, 16)
    nu, vol = q.moments(t, bw)
    # t^0.5 is not smooth at 0: the error decays like order^-3
    assert abs(nu - 2.5 / 1.5) < 5e-5
    assert abs(vol - 1.0) < 1e-7


# ---- the C ABI builder (pbe_daughter_table) gives the same tables ---------------
def _c_table(kind, order=0, param=0.0, param2=0.0):
    import ctypes

    lib = pg.load()
    n = ctypes.c_int()
    assert lib.pbe_daughter_table(kind, order, param, param2, None, None, 0, ctypes.byref(n)) == 0
    t = np.zeros(n.value)
    bw = np.zeros(n.value)
    assert lib.pbe_daughter_table(kind, order, param, param2, t.ctypes.data, bw.ctypes.data,
                                  n.value, ctypes.byref(n)) == 0
    return t, bw


@pytest.mark.parametrize("order", [1, 2, 4, 8, 16, 31])
def test_c_abi_tables_match_python(order):
    np.testing.assert_array_equal(_c_table(pg._lib.DAUGHTER_SYMMETRIC), pg.quadrature.symmetric_binary())
    np.testing.assert_array_equal(_c_table(pg._lib.DAUGHTER_EROSION, param=0.05),
                                  pg.quadrature.erosion(0.05))
    t, bw = _c_table(pg._lib.DAUGHTER_UNIFORM, order)
    rt, rbw = pg.quadrature.uniform(order)
    np.testing.assert_allclose(t, rt, rtol=0, atol=2e-16)
    np.testing.assert_allclose(bw, rbw, rtol=1e-14)
    for p, split in ((2.0, 0.0), (0.5, 0.3), (-0.5, 0.5)):
        t, bw = _c_table(pg._lib.DAUGHTER_POWERLAW, order, p, split)
        rt, rbw = pg.quadrature.power_law(p, order, split or 0.5)
        np.testing.assert_allclose(t, rt, rtol=0, atol=2e-16)
        np.testing.assert_allclose(bw, rbw, rtol=1e-13)


def test_c_abi_table_rejects_bad_input():
    import ctypes

    lib = pg.load()
    n = ctypes.c_int()
    buf = np.zeros(4)
    assert lib.pbe_daughter_table(9, 4, 0.0, 0.0, None, None, 0, ctypes.byref(n)) == 1
    assert lib.pbe_daughter_table(pg._lib.DAUGHTER_EROSION, 0, 1.5, 0.0, None, None, 0, ctypes.byref(n)) == 1
    assert lib.pbe_daughter_table(pg._lib.DAUGHTER_POWERLAW, 4, -1.0, 0.0, None, None, 0, ctypes.byref(n)) == 1
    assert lib.pbe_daughter_table(pg._lib.DAUGHTER_UNIFORM, 0, 0.0, 0.0, None, None, 0, ctypes.byref(n)) == 1
    # capacity too small for 8 entries
    assert lib.pbe_daughter_table(pg._lib.DAUGHTER_UNIFORM, 8, 0.0, 0.0, buf.ctypes.data,
                                  buf.ctypes.data, 4, ctypes.byref(n)) == 1
