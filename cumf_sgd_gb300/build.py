"""Build recipe for the native library, the command-line tools and the oracle.

Outputs (all git-ignored, rebuilt on every machine):
  cumf_sgd_gb300/lib/libcumf_sgd.so   the C-ABI library (CUDA kernels for sm_103a + host code)
  cumf_sgd_gb300/bin/cumf_sgd         drop-in for singleGPU/cumf_sgd (main.cpp)
  cumf_sgd_gb300/bin/cumf_predict     evaluator (mf-predict -e 0/1/2/5/6/10-13)
  cumf_sgd_gb300/bin/cumf_transform   rating text -> binary records (data/netflix/transform)
Translation units compile in parallel; nothing here needs cmake.
"""
from __future__ import annotations

import concurrent.futures as cf
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
BINDIR = os.path.join(PKG, "bin")
LIB = os.path.join(LIBDIR, "libcumf_sgd.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
LIB_SOURCES = [
    "sgd_update.cu",
    "prep.cu",
    "api_io.cpp",
    "api_train.cpp",
    "stream_train.cpp",
    "noalloc.cu",
    "tc_gemm.cu",
    "mlp.cu",
    "batch.cu",
    "text_parse.cu",
    "eval.cu",
    "strata.cu",
    "hot_rows.cu",
]
TOOLS = {"cumf_sgd": "cli_main.cpp", "cumf_predict": "predict_main.cpp", "cumf_transform": "transform_main.cpp"}


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers() -> list[str]:
    hs = [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs


def _compile(src: str, verbose_ptxas: bool) -> str:
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, src + ".o")
    if not _stale(obj, [path] + _headers() + [os.path.abspath(__file__)]):
        return obj
    common = ["-O3", "-std=c++17", "-I", INCLUDE, "-I", CSRC, "-Xcompiler", "-fPIC,-Wall"]
    if src.endswith(".cu"):
        cmd = [nvcc(), *ARCH, "-lineinfo", "--expt-relaxed-constexpr", *common, "-c", path, "-o", obj]
        if verbose_ptxas:
            cmd.insert(1, "-Xptxas=-v")
    else:
        cmd = [nvcc(), "-x", "c++", *common, "-c", path, "-o", obj]
    _run(cmd)
    return obj


def build(verbose: bool = False, verbose_ptxas: bool = False, jobs: int | None = None) -> str:
    """Compiles the library and tools; returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(BINDIR, exist_ok=True)
    srcs = LIB_SOURCES + list(TOOLS.values())
    jobs = jobs or min(len(srcs), max(1, os.cpu_count() or 1))
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = dict(zip(srcs, ex.map(lambda s: _compile(s, verbose_ptxas), srcs)))
    lib_objs = [objs[s] for s in LIB_SOURCES]
    if _stale(LIB, lib_objs):
        _run([nvcc(), *ARCH, "-shared", "-o", LIB, *lib_objs, "-lpthread"])
    for tool, src in TOOLS.items():
        exe = os.path.join(BINDIR, tool)
        if _stale(exe, [objs[src], LIB]):
            _run([nvcc(), "-o", exe, objs[src], "-L", LIBDIR, "-lcumf_sgd",
                  "-Xlinker", "-rpath,$ORIGIN/../lib"])
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, verbose_ptxas="-v" in sys.argv)
