"""The C-ABI library loads without a GPU, exports every function declared in
include/pbe_gb300.h, has the reference's struct layouts, and rejects bad
arguments on the host (these paths return before any CUDA call)."""
import ctypes
import os
import re

import pytest

import pbe_gb300 as pg

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "pbe_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^[A-Za-z_][\w \*]*?\b(pbe_\w+)\s*\(", src, flags=re.M)))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("pbe_aggregation_rhs", "pbe_breakage_rhs", "pbe_aggregation_rhs_ex",
                 "pbe_breakage_rhs_ex", "pbe_aggregation_workspace_bytes",
                 "pbe_breakage_workspace_bytes", "pbe_error_string", "pbe_version"):
        assert must in names


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(pg.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_struct_layouts_match_reference():
    # pbe_cuda::AggregationParams: int, pad, 2 doubles, int(enum), pad, 3 doubles, int, pad
    A = pg.AggregationParams
    assert ctypes.sizeof(A) == 64
    assert [getattr(A, f).offset for f in ("n", "log_x0", "inv_log_r", "kernel_type", "beta0",
                                           "beta_br", "beta_sh", "block_size")] == \
        [0, 8, 16, 24, 32, 40, 48, 56]
    B = pg.BreakageParams
    assert ctypes.sizeof(B) == 56
    assert [getattr(B, f).offset for f in ("n", "n_quad", "selection", "S0", "v_ref", "alpha",
                                           "v_min", "block_size")] == [0, 4, 8, 16, 24, 32, 40, 48]


def test_defaults_match_reference():
    a = pg.AggregationParams()
    assert (a.n, a.log_x0, a.inv_log_r, a.kernel_type, a.beta0, a.beta_br, a.beta_sh,
            a.block_size) == (0, 0.0, 0.0, 0, 1.0, 0.0, 0.0, 256)
    b = pg.BreakageParams()
    assert (b.n, b.n_quad, b.selection, b.S0, b.v_ref, b.alpha, b.v_min, b.block_size) == \
        (0, 0, 0, 1.0, 1.0, 1.0, 0.0, 256)


FAKE = 0x10000  # never dereferenced: every case below is rejected on the host


@pytest.mark.parametrize("kw,code", [
    (dict(n=0), pg.ERR_INVALID_VALUE),
    (dict(n=-3), pg.ERR_INVALID_VALUE),
    (dict(n=64, kernel_type=6), pg.ERR_INVALID_VALUE),
    (dict(n=64, kernel_type=-1), pg.ERR_INVALID_VALUE),
    (dict(n=64, block_size=2048), pg.ERR_INVALID_CONFIGURATION),
])
def test_aggregation_host_errors(kw, code):
    lib = pg.load()
    p = pg.AggregationParams(**kw)
    assert lib.pbe_aggregation_rhs(FAKE, FAKE, FAKE, p, None) == code


@pytest.mark.parametrize("which", [0, 1, 2])
def test_aggregation_null_pointers(which):
    lib = pg.load()
    ptrs = [FAKE, FAKE, FAKE]
    ptrs[which] = None
    assert lib.pbe_aggregation_rhs(*ptrs, pg.AggregationParams(n=64), None) == \
        pg.ERR_INVALID_DEVICE_POINTER
    # n <= 0 is reported before null pointers, like the reference (aggregation.cu:23-24)
    assert lib.pbe_aggregation_rhs(*ptrs, pg.AggregationParams(n=0), None) == pg.ERR_INVALID_VALUE


@pytest.mark.parametrize("kw,code", [
    (dict(n=0, n_quad=1), pg.ERR_INVALID_VALUE),
    (dict(n=64, n_quad=0), pg.ERR_INVALID_VALUE),
    (dict(n=64, n_quad=1, selection=4), pg.ERR_INVALID_VALUE),
    (dict(n=64, n_quad=1, block_size=0), pg.ERR_INVALID_VALUE),
    (dict(n=64, n_quad=1, block_size=4096), pg.ERR_INVALID_CONFIGURATION),
    (dict(n=1 << 20, n_quad=1 << 12), pg.ERR_INVALID_VALUE),
])
def test_breakage_host_errors(kw, code):
    lib = pg.load()
    p = pg.BreakageParams(**kw)
    assert lib.pbe_breakage_rhs(FAKE, FAKE, FAKE, FAKE, FAKE, p, None) == code


@pytest.mark.parametrize("which", range(5))
def test_breakage_null_pointers(which):
    lib = pg.load()
    ptrs = [FAKE] * 5
    ptrs[which] = None
    assert lib.pbe_breakage_rhs(*ptrs, pg.BreakageParams(n=64, n_quad=1), None) == \
        pg.ERR_INVALID_DEVICE_POINTER


def test_workspace_queries():
    assert pg.aggregation_workspace_bytes(0) == 0
    assert pg.aggregation_workspace_bytes(16384) > 16384 * 8 * 6
    assert pg.breakage_workspace_bytes(16384, 16, pg.MODE_GATHER) > 16384 * 16 * 20
    assert pg.breakage_workspace_bytes(16384, 16, pg.MODE_SCATTER) == 0
    assert pg.breakage_workspace_bytes(0, 16) == 0


def test_version_and_error_strings():
    lib = pg.load()
    assert lib.pbe_version() == 100
    assert "invalid argument" in pg.error_string(1)
