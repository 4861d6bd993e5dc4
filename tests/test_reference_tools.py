"""The baseline legs that run the reference's own trainers (oracle/ref_tools.py, used by
bench.py's reference arm and cpu_baseline): LIBMF mf-train on the host cores, with the
warm-up iterations subtracted, and mf-predict's RMSE.  CPU only; skipped where the reference
tools are not built."""
import os
import sys

import numpy as np
import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def ref_tools():
    from oracle import oracle, ref_tools
    try:
        oracle.build_reference()
    except Exception as e:
        pytest.skip(f"reference tools not built: {e}")
    if not ref_tools.available("mf-train", "mf-predict"):
        pytest.skip("reference tools not built on this host")
    return ref_tools


def _planted(m, n, nnz, seed):
    rng = np.random.default_rng(seed)
    P = rng.normal(0, 0.5, (m, 4))
    Q = rng.normal(0, 0.5, (n, 4))
    rec = np.empty(nnz, dtype=[("u", "<i4"), ("v", "<i4"), ("r", "<f4")])
    rec["u"] = rng.integers(0, m, nnz)
    rec["v"] = rng.integers(0, n, nnz)
    rec["r"] = np.clip(np.rint(3.5 + (P[rec["u"]] * Q[rec["v"]]).sum(1) + rng.normal(0, 0.3, nnz)), 1, 5)
    return rec


def test_libmf_baseline_times_iterations_after_warm_up(ref_tools, tmp_path):
    sys.path.insert(0, ROOT)
    import bench
    train = _planted(400, 200, 60_000, 1)
    test = _planted(400, 200, 5_000, 2)
    out = bench.libmf_baseline(ref_tools, train, iters=6, threads=2, tmpdir=str(tmp_path), warm_iters=2, test=test)
    assert out["kind"] == "reference" and out["cores"] == 2 and out["timed_iterations"] == 4
    assert out["value"] > 0 and 0 < out["timed_s"] <= out["computation_s"]
    assert 0.0 < out["test_rmse_mf_predict"] < 2.0
    assert os.path.exists(out["model_path"])


def test_reference_gpu_flags_are_the_canonical_run(ref_tools):
    flags = ref_tools.cumf_flags(7904, 20)
    assert flags == ["-l", "0.05", "-a", "0.08", "-b", "0.3", "-u", "1", "-v", "1", "-x", "1", "-y", "1",
                     "-s", "7904", "-k", "128", "-t", "20"]
