"""Build recipe for libpbe_gb300.so and for the CPU oracle used by the tests.

The library is compiled with nvcc for sm_103a only (one -gencode), three
translation units in parallel, and linked into lib/libpbe_gb300.so (CUDA
runtime linked statically, so the .so loads without a GPU). Rebuilds only what
is older than its sources.

    python pbe-fixed-pivot-cuda_gb300/build.py          # library + oracle
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libpbe_gb300.so")
PROBE_LIB = os.path.join(LIBDIR, "libpbe_probe.so")

ORACLE = os.path.join(ROOT, "oracle")
ORACLE_BUILD = os.path.join(ORACLE, "_build")
ORACLE_LIB = os.path.join(ORACLE_BUILD, "liboracle.so")
REF_RUNNER_LIB = os.path.join(ORACLE_BUILD, "libref_runner.so")
# the reference's C++ API over its own kernels (ref_dropin_shim.cpp + ref_runner.cpp)
REF_DROPIN_LIB = os.path.join(ORACLE_BUILD, "liboracle_ref_dropin.so")

SOURCES = ["aggregation.cu", "breakage.cu", "vjp.cu", "api.cu", "noalloc.cu",
           "batch_kernels.cu", "batch.cu", "adjoint.cu", "death_gemm.cu",
           "batch_vjp.cu", "batch_implicit.cu", "batch_soa.cu", "daughter.cpp"]
ARCH = ["-gencode=arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-O3"]


def _cuda_home() -> str:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.isfile(os.path.join(cand, "bin", "nvcc")):
            return cand
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found (set CUDA_HOME)")


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps if os.path.exists(d))


def _run(cmd: list[str], cwd: str | None = None) -> None:
    proc = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("command failed (%d): %s\n%s" % (proc.returncode, " ".join(cmd), proc.stdout))


def _cuda_libdirs(cuda: str) -> list[str]:
    """-L flags for libcudart and the libcuda stub (x86_64 and aarch64 layouts)."""
    out = []
    for d in ("lib64", os.path.join("lib64", "stubs"), os.path.join("targets", "sbsa-linux", "lib", "stubs"),
              os.path.join("targets", "x86_64-linux", "lib", "stubs")):
        p = os.path.join(cuda, d)
        if os.path.isdir(p):
            out.append("-L" + p)
    return out


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    for dp, _, fs in os.walk(INCLUDE):
        hs += [os.path.join(dp, f) for f in fs]
    return hs


def build_library(force: bool = False) -> str:
    """Compile the csrc sources (CUDA for sm_103a, host C++) and link lib/libpbe_gb300.so."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    nvcc = os.path.join(_cuda_home(), "bin", "nvcc")
    hdrs = _headers()
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        objs.append(o)
        if force or not _newer(o, [s] + hdrs):
            jobs.append([nvcc, *ARCH, *NVCC_FLAGS, "-I" + INCLUDE, "-I" + CSRC, "-c", s, "-o", o])
    if jobs:
        with concurrent.futures.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            list(ex.map(_run, jobs))
    if force or jobs or not _newer(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-Xcompiler", "-fPIC", *objs, "-o", LIB])
    return LIB


def build_probe(force: bool = False) -> str:
    """lib/libpbe_probe.so: the FP64 throughput probe bench.py uses as roofline peak."""
    os.makedirs(LIBDIR, exist_ok=True)
    src = os.path.join(CSRC, "peak_probe.cu")
    if force or not _newer(PROBE_LIB, [src]):
        nvcc = os.path.join(_cuda_home(), "bin", "nvcc")
        _run([nvcc, *ARCH, "-O3", "-std=c++17", "-shared", "-Xcompiler", "-fPIC", src, "-o", PROBE_LIB])
    return PROBE_LIB


def build_oracle(force: bool = False) -> None:
    """CPU oracle (g++), the reference-kernel runner, and the reference cubins
    (only where the reference sources exist; elsewhere the cubins already built
    are used)."""
    os.makedirs(ORACLE_BUILD, exist_ok=True)
    src = os.path.join(ORACLE, "pbe_oracle.cpp")
    if force or not _newer(ORACLE_LIB, [src]):
        # no FMA contraction: identical oracle results on x86_64 and aarch64
        _run(["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
              src, "-o", ORACLE_LIB])
    cuda = _cuda_home()
    rsrc = os.path.join(ORACLE, "ref_runner.cpp")
    if force or not _newer(REF_RUNNER_LIB, [rsrc]):
        libdirs = _cuda_libdirs(cuda)
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I" + os.path.join(cuda, "include"),
              rsrc, *libdirs, "-lcuda", "-o", REF_RUNNER_LIB])
    shim = os.path.join(ORACLE, "ref_dropin_shim.cpp")
    if force or not _newer(REF_DROPIN_LIB, [rsrc, shim] + _headers()):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I" + os.path.join(cuda, "include"),
              "-I" + INCLUDE, shim, rsrc, *_cuda_libdirs(cuda), "-lcudart", "-lcuda", "-ldl",
              "-o", REF_DROPIN_LIB])
    ref_script = os.path.join(ORACLE, "build_ref.sh")
    _run(["sh", ref_script])


def build_all(force: bool = False) -> None:
    with concurrent.futures.ThreadPoolExecutor(max_workers=3) as ex:
        futs = [ex.submit(build_library, force), ex.submit(build_oracle, force),
                ex.submit(build_probe, force)]
        for f in futs:
            f.result()


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print("built", LIB)
