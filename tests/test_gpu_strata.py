"""Deterministic stratified schedule (cumf_dev_strata_*, params.deterministic): with every
block of a stratum updated in parallel, the factors equal the serial restatement bit for bit,
and repeated training runs are identical."""
import numpy as np
import pytest

import cumf_sgd_gb300 as cm

pytestmark = pytest.mark.gpu


def problem(m, n, nnz, seed):
    rng = np.random.default_rng(seed)
    rec = np.empty(nnz, dtype=cm.NODE_DTYPE)
    rec["u"] = rng.integers(0, m, nnz)
    rec["v"] = rng.integers(0, n, nnz)
    rec["r"] = (rng.integers(1, 6, nnz) / np.float32(1.7)).astype(np.float32)
    return rec


def lanes_of(k, precision):
    return min(32, k * (4 if precision == "fp32" else 2) // 16)


@pytest.mark.parametrize("precision", ["fp32", "fp16", "bf16", "bf16sr", "fp16sr"])
@pytest.mark.parametrize("k,G", [(128, 16), (32, 7), (64, 40)])
def test_strata_epochs_bit_exact(lib, orc, cuda, precision, k, G):
    import torch
    m, n, nnz = 700, 450, 30000
    rec = problem(m, n, nnz, k + G)
    eb = 4 if precision == "fp32" else 2
    d_R = torch.from_numpy(rec.view(np.uint8).copy()).to(cuda)
    d_S = torch.empty_like(d_R)
    d_off = torch.empty((G * G + 1) * 8, dtype=torch.uint8, device=cuda)
    cm.dev_strata_layout(d_R.data_ptr(), nnz, G, d_S.data_ptr(), d_off.data_ptr())
    keys = (rec["u"] % G) * G + rec["v"] % G
    order = np.argsort(keys, kind="stable")
    assert d_S.cpu().numpy().tobytes() == rec[order].tobytes()
    off = np.concatenate([[0], np.cumsum(np.bincount(keys, minlength=G * G))]).astype(np.uint64)
    assert np.array_equal(d_off.cpu().numpy().view(np.uint64), off)
    P = torch.empty(m * k * eb, dtype=torch.uint8, device=cuda)
    Q = torch.empty(n * k * eb, dtype=torch.uint8, device=cuda)
    cm.dev_init_factors(P.data_ptr(), m, k, precision, 5, 1)
    cm.dev_init_factors(Q.data_ptr(), n, k, precision, 5, 2)
    lr = orc.lr_table(0.08, 0.3, 0.0, 6)
    status = torch.zeros(1, dtype=torch.int32, device=cuda)
    cm.dev_strata_epochs(d_S.data_ptr(), d_off.data_ptr(), G, P.data_ptr(), m, Q.data_ptr(), n, k, precision, lr,
                         0, 3, 0.05, 0.04, 5, status.data_ptr())
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    dt = torch.float32 if precision == "fp32" else (torch.float16 if precision.startswith("fp16") else torch.bfloat16)
    Pg = P.view(dt).float().cpu().numpy().reshape(m, k)
    Qg = Q.view(dt).float().cpu().numpy().reshape(n, k)
    Po = orc.init_factors(m, k, precision, 5, 1)
    Qo = orc.init_factors(n, k, precision, 5, 2)
    assert orc.strata_epochs(rec, Po, Qo, precision, G, lr, 0, 3, 0.05, 0.04, 5, lanes_of(k, precision)) == 0
    np.testing.assert_array_equal(Pg, Po)
    np.testing.assert_array_equal(Qg, Qo)


def test_deterministic_training_is_reproducible(lib, cuda):
    rng = np.random.default_rng(4)
    m, n, nnz, rank = 3000, 900, 300000, 8
    Pt, Qt = rng.standard_normal((m, rank)) * 0.5, rng.standard_normal((n, rank)) * 0.5
    u, v = rng.integers(0, m, nnz), rng.integers(0, n, nnz)
    r = np.clip(np.round(3 + (Pt[u] * Qt[v]).sum(1) + rng.standard_normal(nnz) * 0.3), 1, 5).astype(np.float32)
    tr = cm.MFProblem.from_arrays(u[:270000], v[:270000], r[:270000], m=m, n=n)
    te = cm.MFProblem.from_arrays(u[270000:], v[270000:], r[270000:], m=m, n=n)
    par = cm.Parameter(k=128, num_workers=0, num_iters=10, alpha=0.08, beta=0.3, seed=3, gpu=0, quiet=1,
                       deterministic=1)
    a, st = cm.sgd_train(tr, None, par, with_stats=True)
    b = cm.sgd_train(tr, None, par)
    np.testing.assert_array_equal(a.P, b.P)
    np.testing.assert_array_equal(a.Q, b.Q)
    assert st.num_workers == int(np.sqrt(270000 / 24))  # workers per stratum = groups
    hog = cm.sgd_train(tr, None, cm.Parameter(**{**par.__dict__, "deterministic": 0}))
    assert abs(cm.calc_rmse(te, a) - cm.calc_rmse(te, hog)) < 0.02


def test_deterministic_parameter_errors(lib, cuda):
    from cumf_sgd_gb300 import _lib
    prob = cm.MFProblem.from_arrays([0, 1], [0, 1], [1.0, 2.0])
    for kw in (dict(deterministic=-1), dict(deterministic=1, u_grid=2, v_grid=2),
               dict(deterministic=1, tail_epochs=2, tail_start=1)):
        with pytest.raises(cm.CumfError) as e:
            cm.sgd_train(prob, None, cm.Parameter(k=128, num_workers=4, seed=0, gpu=0, **kw))
        assert e.value.code == _lib.CUMF_ERR_ARG
