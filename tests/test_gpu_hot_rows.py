"""Copies of the most-rated rows (csrc/hot_rows.cu) against their CPU restatement
(oracle/hot_rows_oracle.py): plan tables, the rewrite of the ratings, spread and merge bit for
bit in every storage type; then cumf_train with and without copies on a skewed problem."""
import numpy as np
import pytest

import cumf_sgd_gb300 as cm
from cumf_sgd_gb300 import synth
from oracle import hot_rows_oracle as ho

pytestmark = pytest.mark.gpu

TORCH_DTYPE = {"fp16": "float16", "fp16sr": "float16", "bf16": "bfloat16", "bf16sr": "bfloat16", "fp32": "float32"}


def _records(nnz, m, n, seed, s_user=0.8, s_item=1.1):
    rng = np.random.default_rng(seed)
    pu = 1.0 / np.arange(1, m + 1) ** s_user
    pv = 1.0 / np.arange(1, n + 1) ** s_item
    rec = np.empty(nnz, dtype=cm.NODE_DTYPE)
    rec["u"] = rng.permutation(m)[rng.choice(m, nnz, p=pu / pu.sum())]
    rec["v"] = rng.permutation(n)[rng.choice(n, nnz, p=pv / pv.sum())]
    rec["r"] = rng.integers(1, 6, nnz).astype(np.float32)
    return rec


@pytest.mark.parametrize("m,n,nnz,per_copy,max_copies", [
    (3000, 700, 60_000, 40, 256),
    (3000, 700, 60_000, 40, 3),
    (3000, 700, 60_000, 1, 7),       # every row with two ratings or more has copies
    (250_000, 5, 400_000, 2000, 256),  # fewer items than plan threads; long runs of users
])
def test_plan_and_assign_match_oracle(lib, cuda, m, n, nnz, per_copy, max_copies):
    import torch
    rec = _records(nnz, m, n, 1)
    d = torch.from_numpy(rec.view(np.uint8).copy()).to(cuda)
    h = cm.HotRows(d.data_ptr(), nnz, m, n, per_copy, max_copies)
    want = ho.plan(rec, m, n, per_copy, max_copies)
    tm, tn, gm, gn = h.tables()
    np.testing.assert_array_equal(tm, want["tab_m"])
    np.testing.assert_array_equal(tn, want["tab_n"])
    np.testing.assert_array_equal(gm, want["grp_m"])
    np.testing.assert_array_equal(gn, want["grp_n"])
    assert (h.m_rows, h.n_rows) == (want["m_rows"], want["n_rows"])
    assert (h.hot_users, h.hot_items) == (len(want["grp_m"]), len(want["grp_n"]))
    assert h.hot_items > 0
    h.assign(d.data_ptr(), nnz)
    torch.cuda.synchronize()
    got = d.cpu().numpy().view(cm.NODE_DTYPE)
    exp = ho.assign(rec, want)
    np.testing.assert_array_equal(got["u"], exp["u"])
    np.testing.assert_array_equal(got["v"], exp["v"])
    np.testing.assert_array_equal(got["r"], rec["r"])
    assert got["u"].max() < h.m_rows and got["v"].max() < h.n_rows
    h.close()


def test_no_row_above_per_copy_means_no_copies(lib, cuda):
    import torch
    rec = _records(5000, 400, 300, 2)
    d = torch.from_numpy(rec.view(np.uint8).copy()).to(cuda)
    h = cm.HotRows(d.data_ptr(), len(rec), 400, 300, 10**9)
    assert (h.m_rows, h.n_rows, h.hot_users, h.hot_items) == (400, 300, 0, 0)
    h.assign(d.data_ptr(), len(rec))
    h.merge(0, 0, 64, "fp16")  # nothing to merge: no factor matrix is touched
    torch.cuda.synchronize()
    np.testing.assert_array_equal(d.cpu().numpy(), rec.view(np.uint8))


@pytest.mark.parametrize("precision", ["fp16", "bf16", "fp32", "bf16sr", "fp16sr"])
def test_spread_and_merge_match_oracle(lib, cuda, precision):
    import torch
    m, n, k, nnz = 500, 120, 64, 30_000
    rec = _records(nnz, m, n, 3)
    d = torch.from_numpy(rec.view(np.uint8).copy()).to(cuda)
    h = cm.HotRows(d.data_ptr(), nnz, m, n, 100, 16)
    tm, tn, gm, gn = h.tables()
    assert h.hot_users > 0 and h.hot_items > 0
    dt = getattr(torch, TORCH_DTYPE[precision])
    P = torch.empty(h.m_rows, k, dtype=dt, device=cuda)
    Q = torch.empty(h.n_rows, k, dtype=dt, device=cuda)
    cm.dev_init_factors(P.data_ptr(), m, k, precision, 3, 1)
    cm.dev_init_factors(Q.data_ptr(), n, k, precision, 3, 2)
    P0, Q0 = P.float().cpu().numpy(), Q.float().cpu().numpy()
    h.spread(P.data_ptr(), Q.data_ptr(), k, precision)
    ho.spread(P0, tm, gm)
    ho.spread(Q0, tn, gn)
    np.testing.assert_array_equal(P.float().cpu().numpy(), P0)
    np.testing.assert_array_equal(Q.float().cpu().numpy(), Q0)
    # every copy drifts on its own, as the epochs leave them
    g = torch.Generator(device=cuda)
    g.manual_seed(4)
    for F in (P, Q):
        F.copy_((F.float() + 0.05 * torch.randn(F.shape, device=cuda, generator=g)).to(dt))
    Pn, Qn = P.float().cpu().numpy(), Q.float().cpu().numpy()
    h.merge(P.data_ptr(), Q.data_ptr(), k, precision)
    ho.merge(Pn, tm, gm, precision)
    ho.merge(Qn, tn, gn, precision)
    np.testing.assert_array_equal(P.float().cpu().numpy(), Pn)
    np.testing.assert_array_equal(Q.float().cpu().numpy(), Qn)
    h.close()


def _train(train, test, spec, **kw):
    prob = cm.MFProblem.from_arrays(train["u"], train["v"], train["r"], m=spec.m, n=spec.n)
    te = cm.MFProblem.from_arrays(test["u"], test["v"], test["r"])
    par = cm.Parameter(k=128, num_workers=0, num_iters=20, lambda_p=0.05, lambda_q=0.05, alpha=0.08, beta=0.3,
                       seed=1, gpu=0, quiet=1, **kw)
    model, st = cm.sgd_train(prob, None, par, with_stats=True)
    return cm.calc_rmse(te, model), st, model


def test_train_with_copies_keeps_quality(lib, cuda):
    """5M ratings of the 480,189 x 17,770 family scaled by 1/20 (Zipf item popularity):
    automatic workers, 20 epochs.  Copies (hot_rows 0.5) cover the most-rated items; the test
    RMSE is no worse than without copies, the default (bound 0.002), and the model has the
    plain shapes."""
    spec = synth.scaled(synth.C2, 0.05)
    train, test = synth.generate(spec, seed=0)
    rm_hot, st_hot, model = _train(train, test, spec, hot_rows=0.5)
    rm_plain, st_plain, _ = _train(train, test, spec)
    assert st_hot.hot_items > 0 and st_hot.extra_rows > 0
    assert st_plain.hot_items == 0 and st_plain.hot_users == 0 and st_plain.extra_rows == 0
    assert model.P.shape == (spec.m, 128) and model.Q.shape == (spec.n, 128)
    assert rm_hot <= rm_plain + 0.002, (rm_hot, rm_plain)


def test_one_worker_has_no_copies(lib, cuda):
    rec = _records(50_000, 300, 40, 5)
    prob = cm.MFProblem.from_arrays(rec["u"], rec["v"], rec["r"], m=300, n=40)
    par = cm.Parameter(k=32, num_workers=1, num_iters=2, seed=1, gpu=0, quiet=1, hot_rows=4.0)
    _, st = cm.sgd_train(prob, None, par, with_stats=True)
    assert st.hot_items == 0 and st.hot_users == 0 and st.extra_rows == 0


def test_checkpoint_records_copies(lib, cuda, tmp_path):
    """A run with copies stops after 2 of 4 epochs and resumes from its checkpoint; a resume
    with another hot_rows setting is refused."""
    rec = _records(400_000, 2000, 300, 6)
    prob = cm.MFProblem.from_arrays(rec["u"], rec["v"], rec["r"], m=2000, n=300)
    path = str(tmp_path / "ck.bin")
    par = cm.Parameter(k=64, num_workers=512, num_iters=4, seed=1, gpu=0, quiet=1, hot_rows=0.5)
    m1, st1, done = cm.sgd_train_ckpt(prob, None, par, path, every=1, stop_after=2)
    assert done == 2 and st1.hot_items > 0
    m2, st2, done = cm.sgd_train_ckpt(prob, None, par, path, every=1, resume=True)
    assert done == 4 and np.isfinite(m2.P).all() and np.isfinite(m2.Q).all()
    with pytest.raises(cm.CumfError, match="hot_rows"):
        cm.sgd_train_ckpt(prob, None, cm.Parameter(**{**par.__dict__, "hot_rows": 2.0}), path, every=1,
                          resume=True)


def test_per_epoch_rmse_and_persistent_launches_with_copies(lib, cuda):
    """With copies, the per-epoch test RMSE (evaluated after each epoch's merge) ends at the
    returned model's RMSE; several epochs per launch (merges after each launch) still train."""
    spec = synth.scaled(synth.C2, 0.02)
    train, test = synth.generate(spec, seed=1)
    prob = cm.MFProblem.from_arrays(train["u"], train["v"], train["r"], m=spec.m, n=spec.n)
    te = cm.MFProblem.from_arrays(test["u"], test["v"], test["r"])
    par = cm.Parameter(k=128, num_workers=0, num_iters=6, alpha=0.08, beta=0.3, seed=2, gpu=0, quiet=1,
                       hot_rows=0.5)
    model, st, rm, _ = cm.sgd_train_ex(prob, te, par)
    assert st.hot_items > 0
    assert abs(rm[-1] - cm.calc_rmse(te, model)) <= 1e-6 and rm[-1] < rm[0]
    par3 = cm.Parameter(**{**par.__dict__, "num_workers": 2048, "epochs_per_launch": 3})
    m3, st3 = cm.sgd_train(prob, None, par3, with_stats=True)
    assert st3.hot_items > 0 and np.isfinite(m3.P).all()
    assert cm.calc_rmse(te, m3) < rm[0]
