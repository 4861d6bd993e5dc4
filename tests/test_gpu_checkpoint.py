"""Checkpoint / resume of mode-A training (cumf_train_ckpt): a run stopped after some epochs
and resumed from its checkpoint ends with the same factors, bit for bit, as an uninterrupted
run when one worker makes the run deterministic; mismatched or damaged checkpoints are
refused.  Failures are made on the host (stop_after, edited files); no GPU fault is involved."""
import os
import subprocess

import numpy as np
import pytest

import cumf_sgd_gb300 as cm
from conftest import ROOT

pytestmark = pytest.mark.gpu


def problem(seed=3, m=400, n=250, nnz=30000):
    rng = np.random.default_rng(seed)
    rec = np.empty(nnz, dtype=cm.NODE_DTYPE)
    rec["u"] = rng.integers(0, m, nnz)
    rec["v"] = rng.integers(0, n, nnz)
    rec["r"] = rng.integers(1, 6, nnz).astype(np.float32)
    return rec, cm.MFProblem.from_arrays(rec["u"], rec["v"], rec["r"])


def params(**kw):
    base = dict(k=64, num_workers=1, num_iters=10, alpha=0.08, beta=0.3, seed=11, gpu=0, precision="fp16",
                quiet=1)
    base.update(kw)
    return cm.Parameter(**base)


def test_stop_and_resume_is_bit_identical(lib, cuda, tmp_path):
    _, prob = problem()
    full, _, done = cm.sgd_train_ckpt(prob, None, params(), str(tmp_path / "a.ckpt"), every=2)
    assert done == 10
    plain = cm.sgd_train(prob, None, params())
    np.testing.assert_array_equal(full.P, plain.P)
    np.testing.assert_array_equal(full.Q, plain.Q)
    path = str(tmp_path / "b.ckpt")
    part, _, done = cm.sgd_train_ckpt(prob, None, params(), path, every=2, stop_after=5)
    assert done == 5 and os.path.exists(path)
    assert not np.array_equal(part.P, full.P)
    rest, st, done = cm.sgd_train_ckpt(prob, None, params(), path, every=2, resume=True)
    assert done == 10
    np.testing.assert_array_equal(rest.P, full.P)
    np.testing.assert_array_equal(rest.Q, full.Q)
    assert rest.b == full.b


def test_extend_a_finished_run(lib, cuda, tmp_path):
    _, prob = problem(seed=4)
    path = str(tmp_path / "c.ckpt")
    cm.sgd_train_ckpt(prob, None, params(num_iters=6), path, every=3)
    ext, _, done = cm.sgd_train_ckpt(prob, None, params(num_iters=9), path, every=3, resume=True)
    assert done == 9
    ref = cm.sgd_train(prob, None, params(num_iters=9))
    np.testing.assert_array_equal(ext.P, ref.P)
    np.testing.assert_array_equal(ext.Q, ref.Q)


def test_resume_without_a_file_starts_from_scratch(lib, cuda, tmp_path):
    _, prob = problem(seed=5)
    model, _, done = cm.sgd_train_ckpt(prob, None, params(num_iters=4), str(tmp_path / "none.ckpt"), every=0,
                                       resume=True)
    assert done == 4
    np.testing.assert_array_equal(model.P, cm.sgd_train(prob, None, params(num_iters=4)).P)


def test_mismatched_and_damaged_checkpoints_are_refused(lib, cuda, tmp_path):
    from cumf_sgd_gb300 import _lib
    rec, prob = problem(seed=6)
    path = str(tmp_path / "d.ckpt")
    cm.sgd_train_ckpt(prob, None, params(num_iters=4), path, every=2, stop_after=2)

    def refused(pr, par, needle):
        with pytest.raises(cm.CumfError) as e:
            cm.sgd_train_ckpt(pr, None, par, path, every=2, resume=True)
        assert e.value.code == _lib.CUMF_ERR_FORMAT
        assert needle in str(e.value)

    refused(prob, params(num_iters=4, seed=12), "seed")
    refused(prob, params(num_iters=4, precision="bf16"), "k or precision")
    rec2 = rec.copy()
    rec2["r"][17] += 1
    refused(cm.MFProblem.from_arrays(rec2["u"], rec2["v"], rec2["r"]), params(num_iters=4), "training ratings")
    raw = bytearray(open(path, "rb").read())
    raw[-3] ^= 0x40
    open(path, "wb").write(bytes(raw))
    refused(prob, params(num_iters=4), "digest")
    open(path, "wb").write(bytes(raw[:-100]))
    refused(prob, params(num_iters=4), "truncated")


def test_many_workers_resume_quality(lib, cuda, tmp_path):
    rng = np.random.default_rng(9)
    m, n, nnz, rank = 3000, 800, 400000, 8
    Pt, Qt = rng.standard_normal((m, rank)) * 0.5, rng.standard_normal((n, rank)) * 0.5
    u, v = rng.integers(0, m, nnz), rng.integers(0, n, nnz)
    r = np.clip(np.round(3 + (Pt[u] * Qt[v]).sum(1) + rng.standard_normal(nnz) * 0.3), 1, 5).astype(np.float32)
    tr = cm.MFProblem.from_arrays(u[:360000], v[:360000], r[:360000], m=m, n=n)
    te = cm.MFProblem.from_arrays(u[360000:], v[360000:], r[360000:], m=m, n=n)
    par = params(k=128, num_workers=256, num_iters=12)
    path = str(tmp_path / "w.ckpt")
    full = cm.sgd_train(tr, None, par)
    cm.sgd_train_ckpt(tr, None, par, path, every=4, stop_after=6)
    rest, _, done = cm.sgd_train_ckpt(tr, None, par, path, every=4, resume=True)
    assert done == 12
    assert abs(cm.calc_rmse(te, rest) - cm.calc_rmse(te, full)) < 0.01


def test_cli_checkpoint_and_resume(lib, cuda, tmp_path):
    rec, _ = problem(seed=8)
    trp = tmp_path / "train.bin"
    rec.tofile(trp)
    exe = os.path.join(ROOT, "cumf_sgd_gb300", "bin", "cumf_sgd")
    ck = str(tmp_path / "cli.ckpt")
    base = [exe, "-k", "64", "-t", "6", "-s", "4", "--seed", "5", "--quiet", "--checkpoint", ck,
            "--checkpoint-every", "3"]
    res = subprocess.run(base + [str(trp), str(tmp_path / "m1")], capture_output=True, text=True)
    assert res.returncode == 0, res.stdout
    assert os.path.exists(ck)
    res = subprocess.run(base + ["--resume", str(trp), str(tmp_path / "m2")], capture_output=True, text=True)
    assert res.returncode == 0, res.stdout
    # The checkpoint already holds all 6 epochs: resuming trains nothing and writes the same model.
    assert open(tmp_path / "m1", "rb").read() == open(tmp_path / "m2", "rb").read()
