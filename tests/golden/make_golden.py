"""Generates the golden fixtures in this directory from the reference's own code.

Runs the tools that oracle/ref_build.sh compiles from the reference sources (where the
reference tree is mounted):
  ref_layout  - singleGPU/sgd.cu gen_random_map / shuffle_problem / grid_problem /
                collect_data / scale_problem / scale_model / shuffle_model
  ref_rmse    - test/mf.cpp read_problem + mf_load_model + calc_rmse (full precision)
  mf-predict  - test/mf-predict.cpp "-e 0" output line
  transform   - data/netflix/transform.cpp (rating text -> 12-byte records)
  ref_rmse    - (with "all") every mf-predict criterion of test/mf.cpp
Usage: python tests/golden/make_golden.py [text|eval]   (rewrites layout_*.npz, rmse.npz, text.npz
and eval.npz, or only the named set)
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


EVAL_CRITERIA = (0, 1, 2, 5, 6, 10, 11, 12, 13)


def eval_fixtures(tmp: str) -> None:
    """All mf-predict criteria from the reference's own test/mf.cpp functions: signed ratings
    (positives are r > 0 for LOGLOSS, ACCURACY, MPR and AUC), ids outside the model, a NaN
    prediction, duplicate (u, v) pairs and rows that are all positive."""
    rng = np.random.default_rng(77)
    out = {}
    for i, (m, n, k, nnz, nonneg) in enumerate([(40, 30, 8, 600, False), (120, 90, 32, 3000, False),
                                                (25, 18, 16, 300, True)]):
        scale = 0.3 if not nonneg else 0.5
        P = (rng.standard_normal((m, k)) * scale).astype(np.float32)
        Q = (rng.standard_normal((n, k)) * scale).astype(np.float32)
        if nonneg:  # positive predictions for GKL
            P, Q = np.abs(P), np.abs(Q)
        b = np.float32(0.5)
        te = np.empty(nnz, dtype=NODE)
        te["u"] = rng.integers(0, m + 4, nnz)
        te["v"] = rng.integers(0, n + 3, nnz)
        te["r"] = rng.integers(1, 6, nnz).astype(np.float32) if nonneg else \
            rng.choice(np.array([-1, 0, 1, 2, 3.5], dtype=np.float32), nnz)
        te["u"][:5], te["v"][:5], te["r"][:5] = 2, 3, np.float32(2.0)  # duplicate positives
        full_u = m + 1  # a row outside the model whose test entries cover most columns
        cols = np.arange(0, n + 1)
        extra = np.zeros(len(cols), dtype=NODE)
        extra["u"], extra["v"], extra["r"] = full_u, cols, np.float32(1.0)
        te = np.concatenate([te, extra])
        if i == 1:
            P[3, 0] = np.nan
        tpath, mpath = os.path.join(tmp, f"ev{i}.bin"), os.path.join(tmp, f"ev{i}.model")
        te.tofile(tpath)
        with open(mpath, "wb") as f:
            np.array([0, m, n, k], dtype=np.int32).tofile(f)
            np.array([b], dtype=np.float32).tofile(f)
            P.tofile(f)
            Q.tofile(f)
        crit = oracle.ref_criteria(tpath, mpath)
        out.update({f"P{i}": P, f"Q{i}": Q, f"b{i}": b, f"te{i}": te,
                    f"crit{i}": np.array([crit[c] for c in EVAL_CRITERIA])})
        print("eval case", i, {c: round(crit[c], 6) for c in EVAL_CRITERIA})
    np.savez_compressed(os.path.join(HERE, "eval.npz"), criteria=np.array(EVAL_CRITERIA), **out)


def text_cases() -> dict:
    """Rating texts the reference's transform accepts: MatrixMarket-style headers, integer and
    decimal ratings in many spellings (exact float ties, the float range ends, subnormals,
    inf/nan), ids with signs and leading zeros, and whitespace/header layouts."""
    rng = np.random.default_rng(99)
    head = b"%%MatrixMarket matrix coordinate real general\n% synthetic ratings\n1000 400 5000\n"
    cases = {}
    lines = [b"%d %d %d" % (rng.integers(0, 1000), rng.integers(0, 400), rng.integers(1, 6)) for _ in range(2000)]
    cases["mm_int"] = head + b"\n".join(lines) + b"\n"
    fmts = ["%.1f", "%.2f", "%.3f", "%.9g", "%.17g", "%.6e", "%g", "%.12f", "%.18e"]
    vals = np.concatenate([rng.uniform(0, 5, 1500), rng.normal(0, 20, 700), 10.0 ** rng.uniform(-40, 38, 600),
                           -(10.0 ** rng.uniform(-44, 30, 200))])
    special = [b"0.1", b"0.2", b"0.3", b"1e-3", b"2.5E+1", b"+4", b"007", b"-0.0", b"4.", b".5", b"-.25",
               b"1.000000000000000000", b"3.4028235677973366e38", b"3.4028234663852886e38",
               b"3.4028235677973365e38", b"1.4e-45", b"7.006492321624086e-46", b"7.006492321624087e-46",
               b"1.1754943508222875e-38", b"0.000000000000000000000000000000000000000001",
               b"123456789012345678", b"16777217", b"16777219", b"9007199254740993", b"1.000000059604644775",
               b"1.000000059604644776", b"0.1000000014901161193", b"33554431", b"1e39", b"1e-50",
               b"inf", b"-inf", b"INF", b"Infinity", b"nan", b"-nan", b"NaN", b"5e0", b"5E-0", b"0e10",
               b"00000000000000000000000000000000000000000000000001.5", b"1234567890123456789e-30"]
    toks = [(fmts[i % len(fmts)] % x).encode() for i, x in enumerate(vals)] + special
    ids = [b"+12", b"0003", b"-5", b"2147483647", b"-2147483648", b"0", b"+0", b"-0"]
    lines = []
    for i, t in enumerate(toks):
        u = ids[i % len(ids)] if i % 7 == 0 else b"%d" % rng.integers(0, 100000)
        lines.append(u + b" " + (b"%d" % rng.integers(0, 5000)) + b" " + t)
    cases["decimals"] = head + b"\n".join(lines) + b"\n"
    ws = [b" ", b"\t", b"  ", b" \t ", b"\r\n", b"\n\n", b"\v", b"\f"]
    parts = []
    for i in range(600):
        rec = [b"%d" % rng.integers(0, 50), b"%d" % rng.integers(0, 50), b"%.2f" % rng.uniform(1, 5)]
        parts.append(ws[rng.integers(0, len(ws))].join(rec) + ws[rng.integers(0, len(ws))])
    cases["whitespace"] = b"h1 with spaces  \r\n\th2\nh3\n   " + b"".join(parts) + b"7 8 9.5"  # no final newline
    cases["header_blank"] = b"h1\n\nh3\n1 2 3\n4 5 6\n"
    cases["header_empty_first"] = b"\n1 2 3\n4 5 6.25\n"
    cases["header_short"] = b"only one line"
    cases["empty"] = b""
    cases["one_record_spanning_lines"] = head + b"1\n2\n3.5\n"
    return cases


def text_fixtures(tmp: str) -> None:
    out = {}
    for name, text in text_cases().items():
        out["text_" + name] = np.frombuffer(text, dtype=np.uint8)
        out["bin_" + name] = np.frombuffer(oracle.ref_transform(text, tmp), dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, "text.npz"), **out)
    print("wrote text.npz")


def main() -> None:
    if not oracle.reference_available():
        oracle.build_reference()
    with tempfile.TemporaryDirectory() as tmp:
        if len(sys.argv) > 1 and sys.argv[1] == "text":
            text_fixtures(tmp)
            return
        if len(sys.argv) > 1 and sys.argv[1] == "eval":
            eval_fixtures(tmp)
            return
        layout_fixtures(tmp)
        rmse_fixtures(tmp)
        text_fixtures(tmp)
        eval_fixtures(tmp)


if __name__ == "__main__":
    main()
