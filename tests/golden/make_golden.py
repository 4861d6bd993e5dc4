"""Generates the golden fixtures in this directory from the reference's own code.

Runs the tools that oracle/ref_build.sh compiles from the reference sources (where the
reference tree is mounted):
  ref_layout  - singleGPU/sgd.cu gen_random_map / shuffle_problem / grid_problem /
                collect_data / scale_problem / scale_model / shuffle_model
  ref_rmse    - test/mf.cpp read_problem + mf_load_model + calc_rmse (full precision)
  mf-predict  - test/mf-predict.cpp "-e 0" output line
Usage: python tests/golden/make_golden.py   (rewrites layout_*.npz and rmse.npz)
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle  # noqa: E402

NODE = oracle.NODE

# (name, m, n, nnz, seed, ux, vy, k)
LAYOUT_CASES = [
    ("layout_1x1", 137, 61, 3000, 12345, 1, 1, 8),
    ("layout_2x3", 211, 97, 5000, 777, 2, 3, 4),
    ("layout_3x2", 90, 40, 2500, 1796309857, 3, 2, 4),
    ("layout_4x4", 64, 64, 4096, 1, 4, 4, 4),
    ("layout_empty_rows", 500, 300, 700, 42, 2, 2, 4),
]


def make_records(m: int, n: int, nnz: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    rec = np.empty(nnz, dtype=NODE)
    rec["u"] = rng.integers(0, m, nnz)
    rec["v"] = rng.integers(0, n, nnz)
    rec["u"][0], rec["v"][0] = m - 1, n - 1  # pin the extent
    rec["r"] = rng.integers(1, 6, nnz).astype(np.float32) + rng.random(nnz).astype(np.float32) * (seed % 2)
    return rec


def layout_fixtures(tmp: str) -> None:
    for name, m, n, nnz, seed, ux, vy, k in LAYOUT_CASES:
        rec = make_records(m, n, nnz, seed)
        res = oracle.ref_layout(rec, seed, ux, vy, k, tmp)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), records=rec, seed=seed, ux=ux, vy=vy, k=k,
                            **{key: np.asarray(val) for key, val in res.items()})
        print("wrote", name)


def rmse_fixtures(tmp: str) -> None:
    rng = np.random.default_rng(2024)
    cases = []
    for i, (m, n, k, nnz) in enumerate([(50, 40, 8, 900), (300, 120, 128, 5000), (20, 10, 32, 200)]):
        P = (rng.standard_normal((m, k)) * 0.3).astype(np.float32)
        Q = (rng.standard_normal((n, k)) * 0.3).astype(np.float32)
        b = np.float32(3.25)
        te = np.empty(nnz, dtype=NODE)
        te["u"] = rng.integers(0, m + 5, nnz)  # some ids outside the model -> b
        te["v"] = rng.integers(0, n + 3, nnz)
        te["r"] = rng.integers(1, 6, nnz).astype(np.float32)
        if i == 2:
            P[3, 0] = np.nan  # NaN prediction -> b
        tpath, mpath = os.path.join(tmp, f"te{i}.bin"), os.path.join(tmp, f"m{i}.model")
        te.tofile(tpath)
        with open(mpath, "wb") as f:
            np.array([0, m, n, k], dtype=np.int32).tofile(f)
            np.array([b], dtype=np.float32).tofile(f)
            P.tofile(f)
            Q.tofile(f)
        full = oracle.ref_rmse(tpath, mpath)
        out = subprocess.run([os.path.join(oracle.REF_DIR, "mf-predict"), "-e", "0", tpath, mpath,
                              os.path.join(tmp, "o")], capture_output=True, text=True, check=True).stdout
        line = [ln for ln in out.splitlines() if ln.startswith("RMSE = ")][0]
        cases.append(dict(P=P, Q=Q, b=b, te=te, rmse=full, line=line))
        print("rmse case", i, full, line)
    np.savez_compressed(os.path.join(HERE, "rmse.npz"),
                        **{f"{key}{i}": np.asarray(c[key]) for i, c in enumerate(cases) for key in c})


def main() -> None:
    if not oracle.reference_available():
        oracle.build_reference()
    with tempfile.TemporaryDirectory() as tmp:
        layout_fixtures(tmp)
        rmse_fixtures(tmp)


if __name__ == "__main__":
    main()
