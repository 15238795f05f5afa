"""Daughter-distribution quadrature tables (t_q, bw_q) for the breakage RHS.

The breakage kernels evaluate, for parent x_j and table entry q, a fragment of
volume x_j t_q carrying bw_q fragments per breakage event
(reference include/pbe_cuda/breakage.cuh:43-50, docs/api.md:185-192,
docs/theory.md:122-148). The reference documents four daughter
distributions and builds only the first three in its examples; all four are
built here from the mathematics:

  symmetric binary  b(v|v') = 2 delta(v - v'/2)        t = {1/2}, bw = {2}
  erosion (eps)     delta(v - eps v') + delta(v - (1-eps) v')
                                                       t = {1-eps, eps}, bw = {1, 1}
  uniform           b(v|v') = 2 / v'                   Gauss-Legendre on (0,1), bw = 2 w
  power law (p)     b(v|v') = C v^p with the volume constraint
                    int_0^v' v b dv = v'  =>  C = (p+2) / v'^(p+1), so in
                    t = v/v':  b dv = (p+2) t^p dt,    bw = (p+2) t^p w
                    on a two-interval Gauss-Legendre rule over (0, s) and
                    (s, 1); s = 1/2 (the reference does not state a split).
                    Fragments per event: (p+2)/(p+1).

Gauss-Legendre nodes are computed by Newton iteration on the three-term
recurrence of the Legendre polynomials (Golub & Welsch give the same nodes).
"""
from __future__ import annotations

import math

import numpy as np


def gauss_legendre(order: int) -> tuple[np.ndarray, np.ndarray]:
    """Nodes and weights of the `order`-point Gauss-Legendre rule on [-1, 1]."""
    if order < 1:
        raise ValueError("order must be >= 1")
    n = order
    x = np.empty(n)
    w = np.empty(n)
    for i in range(n):
        # Tricomi's initial guess for the i-th root (descending)
        z = math.cos(math.pi * (i + 0.75) / (n + 0.5))
        for _ in range(100):
            p0, p1 = 1.0, z
            for k in range(2, n + 1):
                p0, p1 = p1, ((2 * k - 1) * z * p1 - (k - 1) * p0) / k
            if n == 1:
                p0, p1 = 1.0, z
            dp = n * (z * p1 - p0) / (z * z - 1.0) if n > 1 else 1.0
            dz = p1 / dp
            z -= dz
            if abs(dz) < 1e-16:
                break
        p0, p1 = 1.0, z
        for k in range(2, n + 1):
            p0, p1 = p1, ((2 * k - 1) * z * p1 - (k - 1) * p0) / k
        dp = n * (z * p1 - p0) / (z * z - 1.0) if n > 1 else 1.0
        x[i] = z
        w[i] = 2.0 / ((1.0 - z * z) * dp * dp)
    order_idx = np.argsort(x)
    return x[order_idx], w[order_idx]


def gauss_legendre_01(order: int, a: float = 0.0, b: float = 1.0) -> tuple[np.ndarray, np.ndarray]:
    """Gauss-Legendre rule mapped to (a, b)."""
    x, w = gauss_legendre(order)
    h = 0.5 * (b - a)
    return a + h * (x + 1.0), h * w


def symmetric_binary() -> tuple[np.ndarray, np.ndarray]:
    return np.array([0.5]), np.array([2.0])


def symmetric_binary_split(n_quad: int) -> tuple[np.ndarray, np.ndarray]:
    """The symmetric binary daughter written as n_quad coincident entries
    t = 1/2 with bw = 2/n_quad each (same RHS as n_quad = 1 up to rounding)."""
    return np.full(n_quad, 0.5), np.full(n_quad, 2.0 / n_quad)


def erosion(eps: float) -> tuple[np.ndarray, np.ndarray]:
    if not (0.0 < eps < 1.0):
        raise ValueError("eps must be in (0, 1)")
    return np.array([1.0 - eps, eps]), np.array([1.0, 1.0])


def uniform(order: int) -> tuple[np.ndarray, np.ndarray]:
    t, w = gauss_legendre_01(order)
    return t, 2.0 * w


def power_law(p: float, order: int, split: float = 0.5) -> tuple[np.ndarray, np.ndarray]:
    """b(v|v') = (p+2) v^p / v'^(p+1) on a two-interval rule (2*order points)."""
    if p <= -1.0:
        raise ValueError("power-law exponent must be > -1")
    t1, w1 = gauss_legendre_01(order, 0.0, split)
    t2, w2 = gauss_legendre_01(order, split, 1.0)
    t = np.concatenate([t1, t2])
    w = np.concatenate([w1, w2])
    return t, (p + 2.0) * t ** p * w


def moments(t: np.ndarray, bw: np.ndarray) -> tuple[float, float]:
    """(fragments per event, volume fraction per event) of a table."""
    return float(np.sum(bw)), float(np.sum(bw * t))
