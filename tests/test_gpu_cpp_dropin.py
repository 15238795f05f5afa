"""The C++ drop-in boundary exercised by compiled C++ callers.

1. The reference's six example programs (examples/*/main.cpp with
   examples/common/pbe_examples_utils.hpp, staged unchanged into oracle/_ref/
   by oracle/build_ref.sh) are compiled with the host C++ compiler against
   this repository's include/pbe_cuda headers and linked twice:
     - to libpbe_gb300.so (this library), and
     - to liboracle_ref_dropin.so (oracle/ref_dropin_shim.cpp: the same C++
       API running the reference's own kernels, built unmodified from its
       sources).
   Both binaries run on the GPU; every number they print must agree (to the
   printed digits; quantities at machine precision, below 1e-9, only need to
   stay there), except the wall time. The final errors are also checked
   against the values the reference documents for its examples
   (docs/examples.md "Expected output": e.g. N_tot error ~1.7e-4 and M1 at
   machine precision for the constant-kernel case).
2. tests/cpp/dropin_check.cpp: pbe_cuda::launch_* and the C ABI give bitwise
   the same results in gather mode (RHS and VJP, every kernel and selection),
   and the C++ calls return the reference's error codes.
"""
from __future__ import annotations

import concurrent.futures
import importlib.util
import os
import re
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_EXAMPLES = os.path.join(ROOT, "oracle", "_ref", "examples")
LIBDIR = os.path.join(ROOT, "pbe-fixed-pivot-cuda_gb300", "lib")
ORACLE_BUILD = os.path.join(ROOT, "oracle", "_build")
INCLUDE = os.path.join(ROOT, "include")

EXAMPLES = ["aggregation_constant", "aggregation_sum", "aggregation_product",
            "breakage_linear_symmetricbinary", "breakage_linear_uniform", "flocculation_two_stage"]

# final error lines and the values docs/examples.md of the reference gives for them
# ("~" values: two significant digits; None = "at machine precision")
DOCUMENTED = {
    "aggregation_constant": {"N_tot error": 1.7e-4, "M1 error": None},
    "aggregation_sum": {"M0 error": 1.4e-4, "M1 error": 1.6e-4},
    "aggregation_product": {"M0 error": 1.7e-4, "M2 error": 4.8e-3, "M1 error": 1.6e-4},
    # docs/examples.md gives "N_tot error ~1e-04" here, but the program as shipped
    # prints machine precision on both libraries: with the linear selection
    # function dN_tot/dt = S0 M1 / v_ref is constant, so explicit Euler is exact
    "breakage_linear_symmetricbinary": {"N_tot error": None, "V_tot error": None},
    "breakage_linear_uniform": {"M0 error": 2.2e-4, "M1 error": 1.8e-4},
}

_NUM = re.compile(r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?")


def _build_mod():
    spec = importlib.util.spec_from_file_location(
        "pbe_build_for_tests", os.path.join(ROOT, "pbe-fixed-pivot-cuda_gb300", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _compile(src_args, out, link):
    b = _build_mod()
    cuda = b._cuda_home()
    cmd = ["g++", "-std=c++17", "-O2", "-I" + INCLUDE, "-I" + os.path.join(cuda, "include"),
           *src_args, *link, *b._cuda_libdirs(cuda), "-lcudart", "-o", out]
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert proc.returncode == 0, "compile failed: %s\n%s" % (" ".join(cmd), proc.stdout)
    return out


def _link_ours():
    return ["-L" + LIBDIR, "-lpbe_gb300", "-Wl,-rpath," + LIBDIR]


def _link_ref():
    return ["-L" + ORACLE_BUILD, "-loracle_ref_dropin", "-Wl,-rpath," + ORACLE_BUILD, "-lcuda"]


@pytest.fixture(scope="module")
def example_bins(tmp_path_factory):
    if not os.path.isfile(os.path.join(REF_EXAMPLES, "common", "pbe_examples_utils.hpp")):
        pytest.fail("reference examples not staged under oracle/_ref/examples "
                    "(run oracle/build_ref.sh where the reference checkout exists)")
    out = tmp_path_factory.mktemp("examples")
    jobs = []
    for ex in EXAMPLES:
        src = [os.path.join(REF_EXAMPLES, ex, "main.cpp"), "-I" + os.path.join(REF_EXAMPLES, "common")]
        jobs.append((ex, "ours", src, str(out / (ex + ".gb300")), _link_ours()))
        jobs.append((ex, "ref", src, str(out / (ex + ".ref")), _link_ref()))
    bins = {}
    with concurrent.futures.ThreadPoolExecutor(max_workers=8) as pool:
        futs = {pool.submit(_compile, s, o, l): (ex, kind) for ex, kind, s, o, l in jobs}
        for f, key in futs.items():
            bins[key] = f.result()
    return bins


def _run(path):
    env = dict(os.environ)
    env.pop("PBE_GB300_MODE", None)
    proc = subprocess.run([path], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                          timeout=300, env=env)
    assert proc.returncode == 0, "%s exited %d:\n%s" % (path, proc.returncode, proc.stdout[-3000:])
    return proc.stdout


def _quantum(tok: str) -> float:
    """One unit in the last printed digit of a number token."""
    mant, _, exp = tok.lower().partition("e")
    dec = len(mant.split(".")[1]) if "." in mant else 0
    return 10.0 ** (-dec + (int(exp) if exp else 0))


def _compare_outputs(ours: str, ref: str, name: str):
    lo = [ln for ln in ours.splitlines() if "Wall time" not in ln]
    lr = [ln for ln in ref.splitlines() if "Wall time" not in ln]
    assert len(lo) == len(lr), "%s: %d vs %d output lines" % (name, len(lo), len(lr))
    checked = 0
    for a, b in zip(lo, lr):
        ta, tb = _NUM.findall(a), _NUM.findall(b)
        assert len(ta) == len(tb), "%s: line differs:\n  ours: %s\n  ref : %s" % (name, a, b)
        for xa, xb in zip(ta, tb):
            if xa == xb:
                checked += 1
                continue
            fa, fb = float(xa), float(xb)
            if abs(fa) < 1e-9 and abs(fb) < 1e-9:      # machine-precision quantities
                checked += 1
                continue
            q = max(_quantum(xa), _quantum(xb))
            assert abs(fa - fb) <= q * 1.0001, \
                "%s: %s vs %s differ beyond the printed digits:\n  ours: %s\n  ref : %s" % (
                    name, xa, xb, a, b)
            checked += 1
    return checked


def _final_errors(text: str) -> dict:
    out = {}
    for m in re.finditer(r"^\s*([A-Za-z0-9_]+ error)\s*:\s*([-+0-9.eE]+)", text, re.M):
        out[m.group(1)] = float(m.group(2))
    return out


@pytest.mark.parametrize("name", EXAMPLES)
def test_reference_example_same_output_on_both_libraries(example_bins, name):
    ours = _run(example_bins[(name, "ours")])
    ref = _run(example_bins[(name, "ref")])
    n = _compare_outputs(ours, ref, name)
    assert n > 10
    # the words (PASS / WARN verdicts, labels) are the same too
    words = lambda txt: [_NUM.sub("#", ln) for ln in txt.splitlines() if "Wall time" not in ln]  # noqa: E731
    assert words(ours) == words(ref), "%s: the printed text differs" % name
    errs, rerrs = _final_errors(ours), _final_errors(ref)
    notes = []
    for key, want in DOCUMENTED.get(name, {}).items():
        assert key in errs and key in rerrs, "%s: no '%s' line in:\n%s" % (name, key, ours[-1500:])
        got = errs[key]
        in_doc = (rerrs[key] < 1e-10) if want is None else (0.4 * want <= rerrs[key] <= 2.5 * want)
        if not in_doc:
            # the reference's own program disagrees with its documentation: the
            # comparison with the reference's kernels above is the check
            notes.append("%s: reference prints %g, docs give %s" % (key, rerrs[key], want))
            continue
        if want is None:
            assert got < 1e-10, "%s: %s = %g, documented at machine precision" % (name, key, got)
        else:
            assert 0.4 * want <= got <= 2.5 * want, \
                "%s: %s = %g, documented ~%g" % (name, key, got, want)
    print("%s: %d printed numbers equal on both libraries; final errors %s (reference %s)%s"
          % (name, n, errs, rerrs, ("; " + "; ".join(notes)) if notes else ""))


def test_cpp_api_bitwise_equals_c_abi(tmp_path):
    exe = _compile([os.path.join(ROOT, "tests", "cpp", "dropin_check.cpp")],
                   str(tmp_path / "dropin_check"), _link_ours())
    out = _run(exe)
    print(out)
    assert "ALL OK" in out
    assert "FAIL" not in out
