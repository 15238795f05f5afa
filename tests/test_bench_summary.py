"""bench.py's summary of the extra sections, on the sections file of a real
GB300 run (tests/golden/bench_sections_sample.json): every key the summary
reads must exist, so the one JSON line is printed."""
import importlib.util
import json
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_summary_of_a_real_sections_file():
    with open(os.path.join(ROOT, "tests", "golden", "bench_sections_sample.json")) as f:
        sections = json.load(f)
    out = _bench().summarize(sections, 870.0)
    assert set(out) >= {"reference_kernels_sm103a", "vjp_rhs_ratio_n16384", "other_mode",
                        "batched_config3", "adjoint_config4", "classes_config5"}
    assert out["batched_config3"]["roofline_frac"] is not None
    json.dumps(out)


def test_summary_of_no_sections():
    assert _bench().summarize({}, 1.0) == {}


def test_vjp_instruction_model_counts_pairs_and_clips():
    """vjp_lane_fp64_instr: 7 FP64 instructions per pair j < k, one fewer when
    the pair's bracket j + Ld[k - j] reaches n - 1 (clipped), on a small
    geometric grid, against a direct count over the pairs."""
    import numpy as np

    b = _bench()
    for n, q in ((300, 16.0), (257, 4.0), (64, 1.0)):
        x = 1e-21 * np.exp2(np.arange(n) / q)
        v = x[0] + x
        L = np.searchsorted(x, v, side="right") - 1
        L = np.where(v >= x[-1], b.LAG_CLIP, L)
        want = 0
        for j in range(n):
            for k in range(j + 1, n):
                clipped = L[k - j] >= b.LAG_CLIP or j + L[k - j] >= n - 1
                want += 6 if clipped else 7
        assert b.vjp_lane_fp64_instr(x) == want
