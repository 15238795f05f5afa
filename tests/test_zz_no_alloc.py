"""pbe_aggregation_rhs_noalloc: the aggregation entry point for callers that
cannot let a library allocate device memory (solvers that give the whole GPU
to their own allocator, codes that forbid allocation during time stepping,
plug-in interfaces with no way to pass a workspace). Its scratch is a fixed
device array inside the library instead of a pool allocation.

Checked through the C ABI against the allocating entry point
(pbe_aggregation_rhs_ex, same mode) on two calls in a row, with the per-bin
tolerance of the other parity tests; that its calls take nothing from the
library's scratch pool and leave the device's free memory unchanged; and the
size limit (n <= 32768) is rejected with cudaErrorInvalidValue. This file is
collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

import pbe_gb300 as pg
from gpu_util import agg_params, assert_close, oracle_agg, t

pytestmark = pytest.mark.gpu

NOALLOC_MAX_N = 32768


def _noalloc():
    fn = pg.load().pbe_aggregation_rhs_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p] * 3 + [ctypes.POINTER(pg.AggregationParams), ctypes.c_int,
                                           ctypes.c_void_p]
    return fn


def _inputs(n, q):
    x = pg.grids.geometric_pow2(n, 1e-21, q)
    N = pg.grids.lognormal_ic(x, n // 8, 1.0, 1e14)
    return x, N


@pytest.mark.parametrize("mode", [pg.MODE_GATHER, pg.MODE_SCATTER], ids=["gather", "scatter"])
def test_noalloc_matches_allocating_entry_point(mode):
    import torch

    fn = _noalloc()
    stream = torch.cuda.current_stream().cuda_stream or None
    # two sizes, alternating, so each call finds the previous call's contents
    cases = []
    for n, q in ((3000, 128.0), (1200, 64.0)):
        x, N = _inputs(n, q)
        p = agg_params(n, 5, 0.0, 6.73e-18, 66.67, x)
        tN, tx = t(N), t(x)
        want = torch.zeros(n, dtype=torch.float64, device="cuda")
        assert pg.aggregation_rhs(tN, tx, want, p, mode=mode) == 0
        torch.cuda.synchronize()
        _, scale, _ = oracle_agg(N, x, p)
        cases.append((tN, tx, p, want.cpu().numpy(), scale))
    for call in range(2):
        for tN, tx, p, want, scale in cases:
            got = torch.zeros(p.n, dtype=torch.float64, device="cuda")
            code = fn(tN.data_ptr(), tx.data_ptr(), got.data_ptr(), p, mode, stream)
            assert code == 0, pg.error_string(code)
            torch.cuda.synchronize()
            assert_close(got.cpu().numpy(), want, scale, "noalloc call %d n=%d" % (call, p.n))


def test_noalloc_calls_allocate_nothing():
    """After a first call (which loads the kernels and looks up the array's
    address), further calls must neither draw on the library's scratch pool
    (its high-water mark stays 0 after a reset) nor change the device's free
    memory."""
    import torch

    fn = _noalloc()
    n = 2500
    x, N = _inputs(n, 128.0)
    p = agg_params(n, 5, 0.0, 6.73e-18, 66.67, x)
    tN, tx = t(N), t(x)
    out = torch.zeros(n, dtype=torch.float64, device="cuda")
    # the allocating entry point once, so the pool exists and its mark can be read
    assert pg.aggregation_rhs(tN, tx, out, p) == 0
    for mode in (pg.MODE_GATHER, pg.MODE_SCATTER):
        assert fn(tN.data_ptr(), tx.data_ptr(), out.data_ptr(), p, mode, None) == 0
    torch.cuda.synchronize()
    pg.scratch_pool_usage(reset_high=True)
    reserved0, high0 = pg.scratch_pool_usage()
    free0 = torch.cuda.mem_get_info()[0]
    for k in range(6):
        mode = pg.MODE_GATHER if k % 2 == 0 else pg.MODE_SCATTER
        assert fn(tN.data_ptr(), tx.data_ptr(), out.data_ptr(), p, mode, None) == 0
    torch.cuda.synchronize()
    reserved1, high1 = pg.scratch_pool_usage()
    free1 = torch.cuda.mem_get_info()[0]
    assert high0 == 0 and high1 == 0, "noalloc calls drew %d bytes from the scratch pool" % high1
    assert reserved1 == reserved0
    assert free1 == free0, "device free memory changed by %d bytes" % (free0 - free1)
    # the allocating entry point does draw on the pool: the check sees it
    assert pg.aggregation_rhs(tN, tx, out, p) == 0
    torch.cuda.synchronize()
    assert pg.scratch_pool_usage()[1] > 0


def test_noalloc_rejects_sizes_beyond_its_array():
    import torch

    fn = _noalloc()
    n = NOALLOC_MAX_N + 1
    x, N = _inputs(n, 512.0)
    p = agg_params(n, 0, 1e-15, 0.0, 0.0, x)
    rhs = torch.zeros(n, dtype=torch.float64, device="cuda")
    assert fn(t(N).data_ptr(), t(x).data_ptr(), rhs.data_ptr(), p, pg.MODE_GATHER, None) == \
        pg.ERR_INVALID_VALUE
    torch.cuda.synchronize()
    assert float(rhs.abs().max()) == 0.0   # nothing was launched
