"""Mesh-field (structure-of-arrays) layout <-> packed cells (pbe_batch_from_soa,
pbe_batch_to_soa): ragged cells, a leading dimension above n_cells, entries
beyond a cell's sections untouched, exact round trip, and an RK4 step taken on
the packed state and scattered back equal to the step of the packed input."""
import numpy as np
import pytest

import pbe_gb300 as pg
from gpu_util import t

pytestmark = pytest.mark.gpu


def _plan(rng, n_cells=77, n_max=70):
    x = 1e-18 * 2.0 ** (np.arange(n_max) / 4)
    cell_n = rng.integers(1, n_max + 1, size=n_cells)
    cell_n[:3] = [1, n_max, 33]
    t_q, bw_q = pg.quadrature.uniform(2)
    return x, cell_n, pg.BatchPlan([x], cell_n, np.zeros(n_cells, dtype=int), 5, 1, t_q, bw_q)


def test_soa_round_trip_and_untouched_entries():
    import torch

    rng = np.random.default_rng(8)
    x, cell_n, plan = _plan(rng)
    with plan:
        n_cells, n_max, ld = len(cell_n), int(cell_n.max()), len(cell_n) + 13
        soa = rng.normal(size=(n_max, ld))
        mask = np.arange(n_max)[:, None] < np.concatenate([cell_n, np.zeros(ld - n_cells, int)])[None, :]
        dsoa = t(soa.ravel())
        dN = t(np.full(plan.total, np.nan))
        assert plan.from_soa(dsoa, ld, dN) == 0
        torch.cuda.synchronize()
        N = dN.cpu().numpy()
        for c in range(n_cells):
            o = plan.offsets[c]
            np.testing.assert_array_equal(N[o:o + cell_n[c]], soa[:cell_n[c], c])
        back = t(np.full(n_max * ld, -7.0))
        assert plan.to_soa(dN, back, ld) == 0
        torch.cuda.synchronize()
        b = back.cpu().numpy().reshape(n_max, ld)
        np.testing.assert_array_equal(b[mask], soa[mask])
        assert np.all(b[~mask] == -7.0)
        assert plan.from_soa(dsoa, n_cells - 1, dN) == pg.ERR_INVALID_VALUE
        assert plan.to_soa(dN, 0, ld) == pg.ERR_INVALID_DEVICE_POINTER


def test_integration_through_the_mesh_layout():
    import torch

    rng = np.random.default_rng(9)
    x, cell_n, plan = _plan(rng, n_cells=40)
    with plan:
        n_cells, n_max, ld = len(cell_n), int(cell_n.max()), len(cell_n)
        soa = np.zeros((n_max, ld))
        for c in range(n_cells):
            soa[:cell_n[c], c] = pg.grids.lognormal_ic(x[:cell_n[c]], cell_n[c] // 3, 1.0, 1e12)
        prm = t(pg.batch.cell_params(n_cells, beta_br=6.73e-18, beta_sh=66.67, S0=1e-3,
                                     v_ref=float(x[20])))
        packed = np.concatenate([soa[:cell_n[c], c] for c in range(n_cells)])
        ref = t(packed)
        assert plan.rk4(ref, prm, 0.5, 3) == 0
        dsoa = t(soa.ravel())
        dN = t(np.zeros(plan.total))
        assert plan.from_soa(dsoa, ld, dN) == 0
        assert plan.rk4(dN, prm, 0.5, 3) == 0
        assert plan.to_soa(dN, dsoa, ld) == 0
        torch.cuda.synchronize()
        got = dsoa.cpu().numpy().reshape(n_max, ld)
        R = ref.cpu().numpy()
        for c in range(n_cells):
            o = plan.offsets[c]
            np.testing.assert_array_equal(got[:cell_n[c], c], R[o:o + cell_n[c]])
