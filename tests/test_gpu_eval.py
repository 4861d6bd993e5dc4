"""GPU evaluation criteria (mf-predict -e 0/1/2/5/6/10-13) against the reference's own
test/mf.cpp values (golden) and the oracle.  Tolerances: 1e-6 relative for the pointwise
criteria (float terms summed in double in another order), 1e-9 for MPR / AUC (counts of
exact float comparisons; the dot products use the same sequential FMA order)."""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

pytestmark = pytest.mark.gpu

RANKING = (10, 11, 12, 13)


def close(got, ref, c):
    if np.isnan(ref):
        return np.isnan(got)
    tol = 1e-9 if c in RANKING else 1e-6
    return abs(got - ref) <= tol * max(1.0, abs(ref))


def model_of(P, Q, b):
    import cumf_sgd_gb300 as cm
    return cm.MFModel.from_arrays(P, Q, b)


def test_criteria_match_reference(lib, cuda):
    import cumf_sgd_gb300 as cm
    z = np.load(os.path.join(GOLDEN, "eval.npz"))
    for i in range(3):
        te = z[f"te{i}"]
        prob = cm.MFProblem.from_arrays(te["u"], te["v"], te["r"])
        model = model_of(z[f"P{i}"], z[f"Q{i}"], float(z[f"b{i}"]))
        for c, ref in zip(z["criteria"], z[f"crit{i}"]):
            got = cm.evaluate(prob, model, int(c))
            assert close(got, ref, int(c)), (i, int(c), got, ref)


@pytest.mark.parametrize("seed,m,n,k,nnz", [(1, 700, 300, 64, 20000), (2, 90, 1500, 32, 8000)])
def test_criteria_match_oracle_random(lib, cuda, orc, seed, m, n, k, nnz):
    import cumf_sgd_gb300 as cm
    rng = np.random.default_rng(seed)
    P = (rng.standard_normal((m, k)) * 0.2).astype(np.float32)
    Q = (rng.standard_normal((n, k)) * 0.2).astype(np.float32)
    te = np.zeros(nnz, dtype=orc.NODE)
    te["u"] = rng.integers(0, m + 7, nnz)
    te["v"] = rng.integers(0, n + 5, nnz)
    te["r"] = rng.choice(np.array([-2, 0, 1, 3, 4.5], dtype=np.float32), nnz)
    te[100:110] = te[100]  # repeated positives in one row
    prob = cm.MFProblem.from_arrays(te["u"], te["v"], te["r"])
    model = model_of(P, Q, 0.25)
    for c in (1, 5, 6) + RANKING:
        ref = orc.evaluate(te, P, Q, 0.25, c)
        got = cm.evaluate(prob, model, c)
        assert close(got, ref, c), (c, got, ref)


def test_criteria_errors(lib, cuda):
    import cumf_sgd_gb300 as cm
    from cumf_sgd_gb300 import _lib
    P = np.ones((4, 32), np.float32)
    prob = cm.MFProblem.from_arrays([0, 9], [1, 2], [1.0, 2.0], m=5, n=3)
    model = model_of(P, P, 0.0)
    with pytest.raises(cm.CumfError) as e:
        cm.evaluate(prob, model, 3)
    assert e.value.code == _lib.CUMF_ERR_ARG and "unknown evaluation criterion" in str(e.value)
    with pytest.raises(cm.CumfError) as e:
        cm.evaluate(prob, model, 12)  # user 9 lies outside max(5, 4) rows
    assert e.value.code == _lib.CUMF_ERR_RANGE
    empty = cm.MFProblem.from_arrays([], [], [])
    assert cm.evaluate(empty, model, 1) == 0.0
    assert np.isnan(cm.evaluate(empty, model, 10))


def test_predict_tool_prints_reference_lines(lib, cuda, tmp_path):
    z = np.load(os.path.join(GOLDEN, "eval.npz"))
    te, P, Q, b = z["te1"], z["P1"], z["Q1"], z["b1"]
    tpath, mpath = tmp_path / "te.bin", tmp_path / "m.model"
    te.tofile(tpath)
    with open(mpath, "wb") as f:
        np.array([0, P.shape[0], Q.shape[0], P.shape[1]], dtype=np.int32).tofile(f)
        np.array([b], dtype=np.float32).tofile(f)
        P.tofile(f)
        Q.tofile(f)
    exe = os.path.join(ROOT, "cumf_sgd_gb300", "bin", "cumf_predict")
    labels = {0: "RMSE = ", 1: "MAE = ", 5: "LOGLOSS = ", 6: "ACCURACY = ", 10: "Row-wise MPR = ",
              11: "Column-wise MPR = ", 12: "Row-wise AUC = ", 13: "Colmn-wise AUC = "}
    for c, ref in zip(z["criteria"], z["crit1"]):
        c = int(c)
        if c not in labels:
            continue
        out = subprocess.run([exe, "-e", str(c), str(tpath), str(mpath)], capture_output=True, text=True)
        assert out.returncode == 0, out.stdout
        lines = out.stdout.splitlines()
        assert [ln for ln in lines if ln.startswith(labels[c])] == [labels[c] + "%.4f" % ref]
        assert lines[-1].startswith("time elapsed:")
        if c == 0:
            assert lines[0] == "calculating rmse ..."
    out = subprocess.run([exe, "-e", "3", str(tpath), str(mpath)], capture_output=True, text=True)
    assert out.returncode == 1 and out.stdout.strip() == "unknown evaluation criterion"
