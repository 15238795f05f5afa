"""Pins the CPU oracle to the reference: tests/golden/golden_ref.npz holds RHS
vectors computed by the reference's own CUDA kernels (built unmodified from
its sources, launched with its launch geometry) on a GB300, for every
aggregation kernel (3 grids x 2 populations) and every selection x daughter
pair, generated by tests/golden/make_golden.py. CPU only.

Bound per bin: |oracle - golden| <= 1e-12 * scale + misplaced + 1e-280 where
`misplaced` covers near-tie pairs whose logarithm bracket may round
differently in the host's and the device's log (see oracle/pbe_oracle.cpp).
The reference sums with atomics, so its last bits vary from run to run."""
import os

import numpy as np
import pytest

import pyoracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden_ref.npz")
TOL, FLOOR = 1e-12, 1e-280


def _cases(prefix):
    z = np.load(GOLDEN)
    keys = sorted({k.rsplit("/", 1)[0] for k in z.files if k.startswith(prefix)})
    return z, keys


def test_golden_file_is_complete():
    z, agg = _cases("agg/")
    _, brk = _cases("brk/")
    assert len(agg) == 3 * 2 * 6
    assert len(brk) == 3 * 2 * 4 * 4


@pytest.mark.parametrize("key", _cases("agg/")[1])
def test_oracle_aggregation_matches_reference_kernels(key):
    z = np.load(GOLDEN)
    x, N, p, gold = z[key + "/x"], z[key + "/N"], z[key + "/params"], z[key + "/rhs"]
    n, lx0, ilr, k, b0, bbr, bsh = p
    out, scale, mis, code = pyoracle.aggregation_rhs(N, x, int(k), b0, bbr, bsh, lx0, ilr,
                                                     exact_bracket=False, with_misplaced=True)
    assert code == 0
    err = np.abs(out - gold)
    assert np.all(err <= TOL * scale + mis + FLOOR), (key, float(np.max(err / np.maximum(scale, 1e-300))))


@pytest.mark.parametrize("key", _cases("brk/")[1])
def test_oracle_breakage_matches_reference_kernels(key):
    z = np.load(GOLDEN)
    x, N, p, gold = z[key + "/x"], z[key + "/N"], z[key + "/params"], z[key + "/rhs"]
    t_q, bw_q = z[key + "/t_q"], z[key + "/bw_q"]
    n, nq, sel, S0, vref, alpha, vmin = p
    out, scale, code = pyoracle.breakage_rhs(N, x, t_q, bw_q, int(sel), S0, vref, alpha, vmin)
    assert code == 0
    err = np.abs(out - gold)
    assert np.all(err <= TOL * scale + FLOOR), (key, float(np.max(err / np.maximum(scale, 1e-300))))
