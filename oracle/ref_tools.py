"""Runs the reference's own trainers built by ref_build.sh (oracle/_ref/).

TEST INFRASTRUCTURE ONLY: imported by tests/ and by bench.py's baseline legs (the reference
arm and the reference-kernel / cpu_baseline keys), never by the cumf_sgd_gb300 package.

  cumf_sgd_ref   the reference GPU trainer, singleGPU/ built unmodified for sm_103a (with the
                 two-function __shfl shim).  Its update kernel is
                 sgd_k128_kernel_hogwild_warp32_lrate (sgd_k128_kernel_hogwild_warp32.h:3-104),
                 one persistent launch for all iterations (sgd_kernel.cu:212-244), which prints
                 update_per_sec = nnz * iterations / (host clock() time around the launch and
                 its cudaDeviceSynchronize).  It seeds its id shuffle from time() and its
                 sampling from clock(), so two runs differ.
  mf-train       LIBMF's CPU trainer (test/mf-train.cpp, test/mf.cpp:2932-3097): prints
                 "computation time" and "perf: X updates/second" (mf.cpp:3093-3097).
  mf-predict     its evaluator (test/mf-predict.cpp), "RMSE = x.xxxx" for -e 0.
"""
from __future__ import annotations

import os
import re
import subprocess
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")


def tool(name: str) -> str:
    return os.path.join(REF_DIR, name)


def available(*names: str) -> bool:
    return all(os.access(tool(n), os.X_OK) for n in names)


def build_info() -> str:
    path = os.path.join(REF_DIR, "BUILD_INFO")
    return open(path).read().strip() if os.path.exists(path) else ""


def write_records(records: np.ndarray, path: str) -> None:
    """12-byte {int32 u, int32 v, float32 r} records, the format both trainers read."""
    np.ascontiguousarray(records).tofile(path)


def cumf_flags(workers: int, iters: int, k: int = 128, lam: float = 0.05, alpha: float = 0.08,
               beta: float = 0.3, grid=(1, 1, 1, 1)) -> list:
    """The reference's canonical run flags (data/netflix/run.sh:3) with the given workers."""
    u, v, x, y = grid
    return ["-l", str(lam), "-a", str(alpha), "-b", str(beta), "-u", str(u), "-v", str(v), "-x", str(x),
            "-y", str(y), "-s", str(workers), "-k", str(k), "-t", str(iters)]


def run_reference_gpu(train_path: str, model_path: str, workers: int, iters: int = 20, gpu: int = 0,
                      timeout: float = 600.0, **kw) -> dict:
    """Trains with the reference GPU trainer; returns its printed update_per_sec, the process
    wall time and the return code (the model is written to model_path)."""
    cmd = [tool("cumf_sgd_ref"), "-g", str(gpu)] + cumf_flags(workers, iters, **kw) + [train_path, model_path]
    t0 = time.perf_counter()
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=timeout)
    wall = time.perf_counter() - t0
    ups = re.findall(r"update_per_sec:([0-9.eE+-]+)", r.stdout)
    return {"rc": r.returncode, "update_per_sec": float(ups[0]) if ups else None, "wall_s": wall,
            "tail": (r.stdout[-400:] + r.stderr[-400:]) if r.returncode else ""}


def run_libmf(train_path: str, model_path: str, iters: int, threads: int, k: int = 128, l2: float = 0.05,
              timeout: float = 1800.0) -> dict:
    """LIBMF mf-train with `threads` threads and 2*threads+1 blocks per dimension (LIBMF's
    advice, test/README), quiet; returns its perf line and computation time."""
    cmd = [tool("mf-train"), "-l2", str(l2), "-k", str(k), "-t", str(iters), "-s", str(threads),
           "-n", str(2 * threads + 1), "--quiet", train_path, model_path]
    t0 = time.perf_counter()
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=timeout)
    wall = time.perf_counter() - t0
    perf = re.findall(r"perf: ([0-9.eE+-]+)", r.stdout)
    comp = re.findall(r"computation time:\s*([0-9.eE+-]+)", r.stdout)
    return {"rc": r.returncode, "perf": float(perf[0]) if perf else None,
            "computation_s": float(comp[0]) if comp else None, "wall_s": wall,
            "tail": (r.stdout[-400:] + r.stderr[-400:]) if r.returncode else ""}


def libmf_rmse(test_path: str, model_path: str) -> float:
    """mf-predict -e 0: the RMSE line of the reference's evaluator."""
    r = subprocess.run([tool("mf-predict"), "-e", "0", test_path, model_path],
                       capture_output=True, text=True, timeout=600)
    got = re.findall(r"RMSE = ([0-9.eE+-]+)", r.stdout)
    if r.returncode != 0 or not got:
        raise RuntimeError("mf-predict failed: " + r.stdout[-300:] + r.stderr[-300:])
    return float(got[0])
