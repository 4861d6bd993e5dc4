"""Learned warm start on the GPU: what the trained network gains over the method without it.

An MLP encoder is trained on the tensor cores on (features, solved user row) pairs from plain
SGD solves of c1-shaped planted matrices; then new users join a deployed c1 model.  Their rows
initialised by the network must predict their held-out ratings better than every non-learned
start on the same deployed model (random rows as plain SGD draws them, zero rows, the
network's own input: the rating-centred mean of the rated items' factors, and the plain mean
of those factors scaled to the user's mean rating), far better than random rows, and stay
better than each after the same fold-in epochs (item rows frozen)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

K = 128


def test_mlp_warm_start_beats_non_learned_new_user_rows(lib, cuda):
    import torch
    import cumf_sgd_gb300 as cm
    from cumf_sgd_gb300 import synth
    spec = synth.C1
    sm, _, _ = cm.device_info(0)

    def solve(tr, m, n, seed, iters=20, init=None, te=None, tail_epochs=0, tail_start=0, alpha=0.08):
        prob = cm.MFProblem.from_arrays(tr["u"], tr["v"], tr["r"], m=m, n=n)
        tprob = cm.MFProblem.from_arrays(te["u"], te["v"], te["r"]) if te is not None else None
        par = cm.Parameter(k=K, num_workers=cm.auto_workers(len(tr), sm, K, "fp16"), num_iters=iters, alpha=alpha,
                           beta=0.3, seed=seed, gpu=0, precision="fp16", tail_epochs=tail_epochs,
                           tail_start=tail_start)
        return cm.sgd_train_ex(prob, tprob, par, init)

    def features(rec, m, dQ):
        dR = torch.from_numpy(rec.view(np.uint8).copy()).to(cuda)
        dX = torch.empty(m, K + 3, device=cuda)
        cm.user_features(dR.data_ptr(), len(rec), dQ.data_ptr(), spec.n, K, m, dX.data_ptr())
        return dX

    # training pairs from three solves of the family
    Xs, Ts = [], []
    for s in range(3):
        tr, _ = synth.generate(spec, seed=20 + s, device="cuda")
        model = solve(tr, spec.m, spec.n, seed=20 + s)[0]
        X = features(tr, spec.m, torch.from_numpy(np.ascontiguousarray(model.Q)).to(cuda))
        keep = torch.from_numpy(np.nonzero(np.bincount(tr["u"], minlength=spec.m) > 0)[0]).to(cuda)
        Xs.append(X[keep])
        Ts.append(torch.from_numpy(np.ascontiguousarray(model.P)).to(cuda)[keep])
    X, T = torch.cat(Xs).contiguous(), torch.cat(Ts).contiguous()
    mlp = cm.MLP(K + 3, 512, K, seed=7)
    before = mlp.loss_grad(X.data_ptr(), T.data_ptr(), len(X))
    after = mlp.train(X.data_ptr(), T.data_ptr(), len(X), epochs=30, batch=1024, lr=1e-3, seed=3)
    assert after < 0.5 * before, (before, after)

    # a deployed base model and new users from the same planted model
    new_users = 5000
    b_tr, _, n_tr, n_te = synth.generate_growth(spec, new_users, 0.05, seed=100, device="cuda")
    m_all, n = spec.m + new_users, spec.n
    base = solve(b_tr, spec.m, n, seed=1)[0]
    base_P = torch.from_numpy(np.ascontiguousarray(base.P)).to(cuda)
    base_Q = torch.from_numpy(np.ascontiguousarray(base.Q)).to(cuda)
    local = n_tr.copy()
    local["u"] -= spec.m
    local_te = n_te.copy()
    local_te["u"] -= spec.m
    d_nte = torch.from_numpy(local_te.view(np.uint8).copy()).to(cuda)

    def new_user_rmse(P_new):
        return cm.dev_rmse(d_nte.data_ptr(), len(local_te), P_new.data_ptr(), new_users, base_Q.data_ptr(), n, K,
                           float(base.b))

    rows_mlp = torch.empty(new_users, K, device=cuda)
    Xn = features(local, new_users, base_Q)
    mlp.forward(Xn.data_ptr(), new_users, rows_mlp.data_ptr())
    rng = np.random.default_rng(9)
    rows_rand = torch.from_numpy((rng.random((new_users, K), dtype=np.float32) / np.sqrt(K)).astype(np.float32)).to(cuda)
    # non-learned: the mean of the rated items' rows scaled so its product with that mean is
    # the user's mean rating (the model has no bias term)
    uu = torch.from_numpy(local["u"].astype(np.int64)).to(cuda)
    vv = torch.from_numpy(local["v"].astype(np.int64)).to(cuda)
    rr = torch.from_numpy(local["r"].astype(np.float32)).to(cuda)
    deg = torch.zeros(new_users, device=cuda).index_add_(0, uu, torch.ones_like(rr)).clamp_(min=1)
    mu = torch.zeros(new_users, device=cuda).index_add_(0, uu, rr) / deg
    qbar = torch.sparse.mm(torch.sparse_coo_tensor(torch.stack([uu, vv]), 1.0 / deg[uu], (new_users, n)), base_Q)
    rows_mean = (qbar * (mu / (qbar * qbar).sum(1).clamp_(min=1e-12))[:, None]).contiguous()
    starts = {"mlp": rows_mlp, "random": rows_rand, "zero": torch.zeros(new_users, K, device=cuda),
              "qmean": Xn[:, :K].contiguous(), "mean": rows_mean}
    at_init = {name: new_user_rmse(rows) for name, rows in starts.items()}
    assert at_init["mlp"] < 0.7 * at_init["random"], at_init
    assert all(at_init["mlp"] < v for name, v in at_init.items() if name != "mlp"), at_init

    # the same fold-in epochs from every start (item rows frozen, base rows as deployed)
    g_tr = np.concatenate([b_tr, n_tr])
    final = {}
    for name, rows in starts.items():
        P0 = torch.empty(m_all, K, device=cuda)
        P0[: spec.m] = base_P
        P0[spec.m:] = rows
        init = cm.DeviceModel(P0.data_ptr(), m_all, base_Q.data_ptr(), n, K)
        model = solve(g_tr, m_all, n, seed=5, iters=3, init=init, tail_epochs=3, tail_start=len(b_tr), alpha=0.04)[0]
        P_new = torch.from_numpy(np.ascontiguousarray(model.P[spec.m:])).to(cuda)
        Q_out = np.ascontiguousarray(model.Q)
        assert np.allclose(Q_out, base.Q, rtol=1e-3, atol=1e-3), name  # fold-in left the items alone
        final[name] = new_user_rmse(P_new)
    assert all(final["mlp"] < v for name, v in final.items() if name != "mlp"), (final, at_init)
