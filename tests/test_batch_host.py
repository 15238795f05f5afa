"""Batched-cell API on the host (no GPU): plan argument checks that return
before any CUDA call, the parameter-row layout, and the seeded batched-cell
workload."""
import ctypes

import numpy as np
import pytest

import pbe_gb300 as pg


def _create(grids, cell_n, cell_grid, kernel=5, selection=-1, t_q=None, bw_q=None):
    lib = pg.load()
    grid_n = np.ascontiguousarray([len(g) for g in grids], dtype=np.int32)
    grid_x = np.ascontiguousarray(np.concatenate(grids), dtype=np.float64)
    cn = np.ascontiguousarray(cell_n, dtype=np.int32)
    cg = np.ascontiguousarray(cell_grid, dtype=np.int32)
    nq = 0 if t_q is None else len(t_q)
    tq = None if t_q is None else np.ascontiguousarray(t_q, dtype=np.float64)
    bw = None if bw_q is None else np.ascontiguousarray(bw_q, dtype=np.float64)
    h = ctypes.c_void_p()
    code = lib.pbe_batch_create(ctypes.byref(h), len(grid_n), grid_n.ctypes.data,
                                grid_x.ctypes.data, len(cn), cn.ctypes.data, cg.ctypes.data,
                                kernel, selection, nq, None if tq is None else tq.ctypes.data,
                                None if bw is None else bw.ctypes.data, 0, None)
    return code, h


G = [pg.grids.geometric_pow2(40, 1e-21, 8.0)]


@pytest.mark.parametrize("case", [
    dict(cell_n=[41], cell_grid=[0]),                                 # cell longer than its grid
    dict(cell_n=[0], cell_grid=[0]),                                  # empty cell
    dict(cell_n=[10], cell_grid=[1]),                                 # unknown grid
    dict(cell_n=[10], cell_grid=[-1]),
    dict(cell_n=[10], cell_grid=[0], kernel=6),                       # bad kernel type
    dict(cell_n=[10], cell_grid=[0], kernel=-1, selection=-1),        # nothing to compute
    dict(cell_n=[10], cell_grid=[0], selection=4, t_q=[0.5], bw_q=[2.0]),
    dict(cell_n=[10], cell_grid=[0], selection=0, t_q=[1.5], bw_q=[1.0]),   # t_q > 1
    dict(cell_n=[10], cell_grid=[0], selection=0, t_q=[0.0], bw_q=[1.0]),   # t_q <= 0
    dict(cell_n=[10], cell_grid=[0], selection=0),                    # no daughter table
    dict(grids=[G[0][::-1]], cell_n=[10], cell_grid=[0]),             # decreasing pivots
    dict(grids=[np.r_[G[0][:5], G[0][4:]]], cell_n=[10], cell_grid=[0]),    # repeated pivot
    dict(grids=[np.r_[-1.0, G[0]]], cell_n=[10], cell_grid=[0]),      # non-positive pivot
    dict(grids=[np.r_[1e-310, G[0]]], cell_n=[10], cell_grid=[0]),    # subnormal pivot
])
def test_plan_creation_rejects_bad_input_on_host(case):
    case = dict(case)
    grids = case.pop("grids", G)
    code, h = _create(grids, **case)
    assert code == pg.ERR_INVALID_VALUE
    assert not h.value


def test_null_plan_calls():
    lib = pg.load()
    assert lib.pbe_batch_destroy(None) == 0
    assert lib.pbe_batch_offsets(None, None) == pg.ERR_INVALID_VALUE
    assert lib.pbe_batch_rhs(None, None, None, None, None) == pg.ERR_INVALID_VALUE
    assert lib.pbe_batch_rk4(None, None, None, 0.1, 1, None) == pg.ERR_INVALID_VALUE
    assert lib.pbe_batch_rk4_percell(None, None, None, 0.1, 1, None) == pg.ERR_INVALID_VALUE
    assert lib.pbe_batch_schedule(None, None, None) == pg.ERR_INVALID_VALUE


def test_cell_params_layout_and_defaults():
    assert ctypes.sizeof(pg.BatchCellParams) == 64
    p = pg.batch.cell_params(3, beta_sh=[1.0, 2.0, 3.0], S0=5.0)
    assert p.shape == (3, 8)
    assert list(p[1]) == [1.0, 0.0, 2.0, 5.0, 1.0, 1.0, 0.0, 0.0]
    with pytest.raises(TypeError):
        pg.batch.cell_params(2, G=3.0)


def test_batched_cells_workload_is_seeded_and_in_range():
    a = pg.grids.config_batched_cells(n_cells=256)
    b = pg.grids.config_batched_cells(n_cells=256)
    assert np.array_equal(a["N"], b["N"]) and np.array_equal(a["cell_n"], b["cell_n"])
    n, g, p = a["cell_n"], a["cell_grid"], a["params"]
    assert n.min() >= 64 and n.max() <= 3840 and np.all(n % 64 == 0)
    assert set(np.unique(g)) <= {0, 1, 2, 3}
    G = 0.75 * p[:, 2]
    assert G.min() >= 10.0 and G.max() <= 200.0
    assert p[:, 5].min() >= 0.5 and p[:, 5].max() <= 1.5
    assert np.all(p[:, 1] == 6.73e-18) and np.all(p[:, 3] == 1e-3)
    assert len(a["N"]) == n.sum()
    # x_ref is the cell's middle pivot
    for c in range(10):
        assert p[c, 4] == a["grids"][g[c]][n[c] // 2]
    # each cell's N sums to the stated total
    off = np.r_[0, np.cumsum(n)]
    tot = np.array([a["N"][off[c]:off[c + 1]].sum() for c in range(len(n))])
    np.testing.assert_allclose(tot, 1e13, rtol=1e-12)
