"""The reference's own unit-test assertions (tests/unit/test_aggregation.cpp,
tests/unit/test_breakage.cpp; restated in refsuite.py) replayed against the
GPU library through the C ABI, in both accumulation modes."""
import pytest

import pbe_gb300 as pg
import refsuite as rs
from gpu_util import gpu_agg, gpu_brk

pytestmark = pytest.mark.gpu

MODES = [pg.MODE_GATHER, pg.MODE_SCATTER]


def _agg(mode):
    def f(N, x, p):
        if N is None:
            import torch

            tx = torch.tensor(x, device="cuda")
            rhs = torch.zeros(len(x), dtype=torch.float64, device="cuda")
            return pg.aggregation_rhs(None, tx, rhs, pg.AggregationParams(**p), mode=mode), None
        return gpu_agg(N, x, pg.AggregationParams(**p), mode)
    return f


def _brk(mode):
    def f(N, x, t_q, bw_q, p):
        if N is None:
            import torch

            c = lambda a: torch.tensor(a, device="cuda")  # noqa: E731
            rhs = torch.zeros(len(x), dtype=torch.float64, device="cuda")
            return pg.breakage_rhs(None, c(x), c(t_q), c(bw_q), rhs, pg.BreakageParams(**p),
                                   mode=mode), None
        return gpu_brk(N, x, t_q, bw_q, pg.BreakageParams(**p), mode)
    return f


@pytest.mark.parametrize("mode", MODES, ids=["gather", "scatter"])
class TestAggregation:
    @pytest.mark.parametrize("name,k,b0,bbr,bsh", rs.AGG_CASES)
    def test_smoke(self, mode, name, k, b0, bbr, bsh):
        rs.agg_smoke(_agg(mode), k, b0, bbr, bsh)

    @pytest.mark.parametrize("name,k,b0,bbr,bsh", rs.AGG_CASES)
    def test_volume_conserved(self, mode, name, k, b0, bbr, bsh):
        rs.agg_volume_conserved(_agg(mode), k, b0, bbr, bsh)

    def test_zero_population(self, mode):
        rs.agg_zero_population(_agg(mode))

    def test_self_collision(self, mode):
        rs.agg_self_collision(_agg(mode))

    def test_total_number_nonincreasing(self, mode):
        rs.agg_total_number_nonincreasing(_agg(mode))

    def test_invalid_n(self, mode):
        rs.agg_invalid_n(_agg(mode))

    def test_null_pointer(self, mode):
        rs.agg_null_pointer(_agg(mode))


@pytest.mark.parametrize("mode", MODES, ids=["gather", "scatter"])
class TestBreakage:
    @pytest.mark.parametrize("name,sel,kw", rs.BRK_SMOKE)
    def test_smoke(self, mode, name, sel, kw):
        rs.brk_smoke(_brk(mode), sel, kw)

    @pytest.mark.parametrize("name,sel,kw", rs.BRK_SMOKE)
    def test_volume_conserved(self, mode, name, sel, kw):
        rs.brk_volume_conserved(_brk(mode), sel, kw)

    def test_zero_population(self, mode):
        rs.brk_zero_population(_brk(mode))

    def test_death_constant(self, mode):
        rs.brk_death_constant(_brk(mode))

    def test_total_number_nondecreasing(self, mode):
        rs.brk_total_number_nondecreasing(_brk(mode))

    def test_threshold_suppresses(self, mode):
        rs.brk_threshold_suppresses(_brk(mode))

    def test_invalid_n(self, mode):
        rs.brk_invalid_n(_brk(mode))

    def test_null_pointer(self, mode):
        rs.brk_null_pointer(_brk(mode))
