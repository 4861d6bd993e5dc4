"""Batched persistent launch of many factorizations against the oracle (one worker per
problem: bit-exact at every lane width), its autotuner (zero learning rate: factors
unchanged; lane widths a problem's k cannot take are refused) and graph replay."""
import numpy as np
import pytest

import cumf_sgd_gb300 as cm

pytestmark = pytest.mark.gpu

SHAPES = [(60, 30, 900, 32), (45, 70, 2000, 64), (80, 40, 3100, 128), (7, 5, 100, 128), (33, 21, 129, 64)]


def make(cuda, seed, workers=1, lr_len=8, min_k=0):
    import torch
    from oracle import oracle
    rng = np.random.default_rng(seed)
    probs, host = [], []
    lr = oracle.lr_table(0.08, 0.3, 0.0, lr_len)
    d_lr = torch.from_numpy(lr).to(cuda)
    for i, (m, n, nnz, k) in enumerate(s for s in SHAPES if s[3] >= min_k):
        rec = np.empty(nnz, dtype=cm.NODE_DTYPE)
        rec["u"], rec["v"] = rng.integers(0, m, nnz), rng.integers(0, n, nnz)
        rec["r"] = rng.integers(1, 6, nnz).astype(np.float32) / np.float32(1.3)
        d_R = torch.from_numpy(rec.view(np.uint8).copy()).to(cuda)
        P = torch.empty(m * k * 2, dtype=torch.uint8, device=cuda)
        Q = torch.empty(n * k * 2, dtype=torch.uint8, device=cuda)
        cm.dev_init_factors(P.data_ptr(), m, k, "fp16", 40 + i, 1)
        cm.dev_init_factors(Q.data_ptr(), n, k, "fp16", 40 + i, 2)
        host.append(dict(rec=rec, m=m, n=n, k=k, seed=40 + i, P=P, Q=Q, d_R=d_R))
        probs.append(dict(d_R=d_R.data_ptr(), nnz=nnz, d_P=P.data_ptr(), m=m, n=n, d_Q=Q.data_ptr(), k=k,
                          num_workers=workers, lambda_p=0.05, lambda_q=0.04, seed=40 + i, d_lr=d_lr.data_ptr(),
                          lr_len=lr_len))
    return probs, host, lr, d_lr


def as_f32(t, rows, k):
    import torch
    return t.view(torch.float16).reshape(rows, k).float().cpu().numpy()


@pytest.mark.parametrize("lanes", [8, 16, 32])
def test_batched_single_worker_bit_exact(lib, orc, cuda, lanes):
    """Each lane width the autotuner can pick (32 lanes only for k >= 64)."""
    import torch
    probs, host, lr, _keep = make(cuda, 1, min_k=64 if lanes == 32 else 0)
    b = cm.Batch(probs)
    b.set_tuning(16, 2, 4, lanes=lanes)
    assert b.info()["lanes"] == lanes
    for ep in range(2):
        b.run(ep, 1, use_graph=(ep == 1))
    torch.cuda.synchronize()
    assert b.status() == 0
    for h in host:
        P = orc.init_factors(h["m"], h["k"], "fp16", h["seed"], 1)
        Q = orc.init_factors(h["n"], h["k"], "fp16", h["seed"], 2)
        orc.sgd_epochs(h["rec"], P, Q, "fp16", 1, lr, 0, 2, 0.05, 0.04, h["seed"], lanes=lanes)
        np.testing.assert_array_equal(as_f32(h["P"], h["m"], h["k"]), P)
        np.testing.assert_array_equal(as_f32(h["Q"], h["n"], h["k"]), Q)


def test_autotune_leaves_factors_unchanged_and_graph_matches_direct(lib, cuda):
    import torch
    probs, host, _, _keep = make(cuda, 2, workers=0)
    b = cm.Batch(probs)
    before = [(h["P"].clone(), h["Q"].clone()) for h in host]
    best = b.autotune()
    torch.cuda.synchronize()
    assert best["epoch_ms"] > 0 and best["order"] in (0, 1, 2)
    assert best["lanes"] in (8, 16)  # a k = 32 problem rules out 32 lanes
    for h, (p0, q0) in zip(host, before):
        assert torch.equal(h["P"], p0) and torch.equal(h["Q"], q0)
    # one worker per problem: the graph replay and a direct launch give the same bits
    probs1, host1, _, _k1 = make(cuda, 3)
    probs2, host2, _, _k2 = make(cuda, 3)
    b1, b2 = cm.Batch(probs1), cm.Batch(probs2)
    b1.run(0, 1, use_graph=True)
    b2.run(0, 1, use_graph=False)
    torch.cuda.synchronize()
    for h1, h2 in zip(host1, host2):
        assert torch.equal(h1["P"], h2["P"]) and torch.equal(h1["Q"], h2["Q"])


def test_batched_hogwild_matches_plain_kernel_quality(lib, cuda):
    """Planted problems of three k: after 15 epochs the batched launch's train RMSE is within
    5% of the plain kernel's on the same problem (Hogwild runs differ run to run)."""
    import torch
    from cumf_sgd_gb300 import synth
    specs = [(synth.scaled(synth.C1, 0.2), 32), (synth.scaled(synth.C1, 0.3), 64), (synth.scaled(synth.C1, 0.25), 128)]
    lr = torch.from_numpy(cm.lr_schedule(0.08, 0.3, 0.0, 24)).to(cuda)
    runs = {}
    for arm in ("plain", "batched"):
        probs, hs = [], []
        for i, (sp, k) in enumerate(specs):
            tr, _ = synth.generate(sp, seed=50 + i, device="cpu")
            scale = np.float32(np.std(tr["r"].astype(np.float64)))
            rec = tr.copy()
            rec["r"] = rec["r"] * np.float32(1.0 / float(scale))
            d_R = torch.from_numpy(rec.view(np.uint8).copy()).to(cuda)
            P = torch.empty(sp.m * k * 2, dtype=torch.uint8, device=cuda)
            Q = torch.empty(sp.n * k * 2, dtype=torch.uint8, device=cuda)
            cm.dev_init_factors(P.data_ptr(), sp.m, k, "fp16", i, 1)
            cm.dev_init_factors(Q.data_ptr(), sp.n, k, "fp16", i, 2)
            lam = float(np.float32(0.05) / scale)
            hs.append((rec, sp, k, P, Q, d_R))
            probs.append(dict(d_R=d_R.data_ptr(), nnz=len(rec), d_P=P.data_ptr(), m=sp.m, n=sp.n, d_Q=Q.data_ptr(),
                              k=k, num_workers=256, lambda_p=lam, lambda_q=lam, seed=i, d_lr=lr.data_ptr(), lr_len=24))
        if arm == "plain":
            for p in probs:
                cm.sgd_update(p["d_R"], p["nnz"], p["d_P"], p["m"], p["d_Q"], p["n"], p["k"], "fp16", 256, 0,
                              p["d_lr"], 0, 15, p["lambda_p"], p["lambda_q"], p["seed"])
        else:
            b = cm.Batch(probs)
            b.run(0, 15, use_graph=True)
        torch.cuda.synchronize()
        out = []
        for rec, sp, k, P, Q, _ in hs:
            Pf, Qf = as_f32(P, sp.m, k), as_f32(Q, sp.n, k)
            pred = (Pf[rec["u"]] * Qf[rec["v"]]).sum(1)
            out.append(float(np.sqrt(np.mean((rec["r"] - pred) ** 2))))
        runs[arm] = out
    for a, b_ in zip(runs["plain"], runs["batched"]):
        assert abs(a - b_) <= 0.05 * a, runs


def test_batched_tuning_refuses_lanes_a_problem_cannot_take(lib, cuda):
    from cumf_sgd_gb300 import _lib
    probs, host, _, _keep = make(cuda, 4)  # includes k = 32: 32 lanes would give one half per lane
    b = cm.Batch(probs)
    with pytest.raises(RuntimeError):
        b.set_tuning(16, 2, 4, lanes=32)
    with pytest.raises(RuntimeError):
        b.set_tuning(16, 2, 4, lanes=12)
    assert b.info()["lanes"] == 16


def test_batched_row_copies_single_worker_bit_exact(lib, orc, cuda):
    """Problems with copies of their most-rated rows (at least 40 ratings per copy): the batch
    runs one launch per epoch and merges the copies after each.  One worker per problem: the
    extended factors equal the oracle's epochs over the rewritten ratings, each followed by
    the restated merge, bit for bit (copies included)."""
    import torch
    from oracle import hot_rows_oracle as ho
    probs, host, lr, _keep = make(cuda, 2)
    plans = []
    for p, h in zip(probs, host):
        plan = cm.HotRows(p["d_R"], p["nnz"], h["m"], h["n"], 40)
        plan.assign(p["d_R"], p["nnz"])
        P = torch.empty(plan.m_rows * h["k"] * 2, dtype=torch.uint8, device=cuda)
        Q = torch.empty(plan.n_rows * h["k"] * 2, dtype=torch.uint8, device=cuda)
        cm.dev_init_factors(P.data_ptr(), h["m"], h["k"], "fp16", h["seed"], 1)
        cm.dev_init_factors(Q.data_ptr(), h["n"], h["k"], "fp16", h["seed"], 2)
        plan.spread(P.data_ptr(), Q.data_ptr(), h["k"], "fp16")
        h.update(P=P, Q=Q, plan=plan)
        p.update(d_P=P.data_ptr(), d_Q=Q.data_ptr(), hot=plan)
        plans.append(plan)
    assert sum(pl.hot_users + pl.hot_items for pl in plans) > 0
    b = cm.Batch(probs)
    b.set_tuning(16, 2, 4, lanes=16)
    b.run(0, 2, use_graph=True)
    torch.cuda.synchronize()
    assert b.status() == 0
    for h in host:
        plan = h["plan"]
        tm, tn, gm, gn = plan.tables()
        want = ho.plan(h["rec"], h["m"], h["n"], 40)
        rec = ho.assign(h["rec"], want)
        P = np.zeros((plan.m_rows, h["k"]), np.float32)
        Q = np.zeros((plan.n_rows, h["k"]), np.float32)
        P[:h["m"]] = orc.init_factors(h["m"], h["k"], "fp16", h["seed"], 1)
        Q[:h["n"]] = orc.init_factors(h["n"], h["k"], "fp16", h["seed"], 2)
        ho.spread(P, tm, gm)
        ho.spread(Q, tn, gn)
        for ep in range(2):
            orc.sgd_epochs(rec, P, Q, "fp16", 1, lr, ep, 1, 0.05, 0.04, h["seed"], lanes=16)
            ho.merge(P, tm, gm, "fp16")
            ho.merge(Q, tn, gn, "fp16")
        np.testing.assert_array_equal(as_f32(h["P"], plan.m_rows, h["k"]), P)
        np.testing.assert_array_equal(as_f32(h["Q"], plan.n_rows, h["k"]), Q)
