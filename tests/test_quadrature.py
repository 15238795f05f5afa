"""Daughter tables (pbe_gb300.quadrature) against numpy's Gauss-Legendre and
the moment constraints of docs/theory.md:34-38 (volume per event = parent)."""
import numpy as np
import pytest

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
