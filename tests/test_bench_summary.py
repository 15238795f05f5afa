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
