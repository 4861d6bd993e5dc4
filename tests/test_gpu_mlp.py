"""Warm-start MLP on the tensor cores against its CPU restatements (oracle/mlp_oracle.py).
Tolerances:
  - against the restatement with the GPU's bf16 roundings (forward_backward_bf16): loss within
    1e-3 and each gradient tensor within 3e-3 relative L2 (fp32 accumulation order and the odd
    value rounded to the other bf16 neighbour are the only differences);
  - against exact FP64: each gradient tensor within its own bound from gradient_bounds (twice
    the bf16-rounded restatement's own distance from FP64, plus 2e-3), about 0.6-1.1%;
  - features within 1e-4 relative (fp32 atomics)."""
import numpy as np
import pytest

import cumf_sgd_gb300 as cm
from oracle import mlp_oracle

pytestmark = pytest.mark.gpu

D_IN, H, D_OUT = 131, 512, 128


def split(g):
    return mlp_oracle.unpack(g, D_IN, H, D_OUT)


@pytest.mark.parametrize("rows", [256, 300, 1000])
def test_mlp_loss_and_gradients_match_fp64(lib, cuda, rows):
    import torch
    rng = np.random.default_rng(rows)
    X = rng.standard_normal((rows, D_IN)).astype(np.float32) * 0.5
    T = rng.standard_normal((rows, D_OUT)).astype(np.float32) * 0.2
    mlp = cm.MLP(D_IN, H, D_OUT, seed=3)
    params = mlp.get(0)
    dX, dT = torch.from_numpy(X).to(cuda), torch.from_numpy(T).to(cuda)
    loss = mlp.loss_grad(dX.data_ptr(), dT.data_ptr(), rows)
    grads = mlp.get(1)
    ref_loss, ref_grads = mlp_oracle.forward_backward(params, X, T, D_IN, H, D_OUT)
    assert abs(loss - ref_loss) <= 0.01 * ref_loss, (loss, ref_loss)
    l16, g16, g64, bounds = mlp_oracle.gradient_bounds(params, X, T, D_IN, H, D_OUT)
    assert abs(loss - l16) <= 1e-3 * l16, (loss, l16)
    for name, g, r16, r64 in zip(mlp_oracle.GRAD_NAMES, split(grads), split(g16), split(g64)):
        e16, e64 = mlp_oracle.rel_err(g, r16), mlp_oracle.rel_err(g, r64)
        assert e16 <= 3e-3, (name, e16)
        assert e64 <= bounds[name], (name, e64, bounds[name])
    Y = torch.empty(rows, D_OUT, device=cuda)
    mlp.forward(dX.data_ptr(), rows, Y.data_ptr())
    torch.cuda.synchronize()
    W1, b1, W2, b2, W3, b3 = split(params)
    ref_y = mlp_oracle.gelu(mlp_oracle.gelu(X @ W1.T + b1) @ W2.T + b2) @ W3.T + b3
    assert np.linalg.norm(Y.cpu().numpy() - ref_y) <= 0.01 * np.linalg.norm(ref_y)


def test_mlp_training_fits_a_smooth_map(lib, cuda):
    import torch
    rng = np.random.default_rng(0)
    rows = 8192
    X = rng.standard_normal((rows, D_IN)).astype(np.float32)
    A = rng.standard_normal((D_IN, D_OUT)).astype(np.float32) / np.sqrt(D_IN)
    T = np.tanh(X @ A).astype(np.float32)
    mlp = cm.MLP(D_IN, H, D_OUT, seed=1)
    dX, dT = torch.from_numpy(X).to(cuda), torch.from_numpy(T).to(cuda)
    before = mlp.loss_grad(dX.data_ptr(), dT.data_ptr(), rows)
    after = mlp.train(dX.data_ptr(), dT.data_ptr(), rows, epochs=20, batch=512, lr=1e-3, seed=2)
    assert after < 0.1 * before, (before, after)


@pytest.mark.parametrize("k", [128, 96, 300])
def test_user_features_match_fp64(lib, cuda, k):
    """Against the float64 restatement (k = 96 and 300: a partial last column pass); every
    call gives the same bits; ratings outside the matrix are left out."""
    import torch
    rng = np.random.default_rng(5)
    m, n, nnz = 500, 200, 20000
    rec = np.empty(nnz, dtype=cm.NODE_DTYPE)
    rec["u"] = rng.integers(0, m - 10, nnz)  # the last users have no ratings
    rec["v"] = rng.integers(0, n, nnz)
    rec["r"] = rng.integers(1, 6, nnz).astype(np.float32)
    rec["u"][:300] = rng.integers(0, 40, 300)  # a few users with many ratings
    Q = (rng.standard_normal((n, k)) * 0.3).astype(np.float32)
    dQ = torch.from_numpy(Q).to(cuda)

    def feats(records):
        dR = torch.from_numpy(records.view(np.uint8).copy()).to(cuda)
        dX = torch.empty(m, k + 3, device=cuda)
        cm.user_features(dR.data_ptr(), len(records), dQ.data_ptr(), n, k, m, dX.data_ptr())
        return dX.cpu().numpy()

    got = feats(rec)
    ref = mlp_oracle.user_features(rec, Q, m, k)
    assert np.abs(got - ref).max() <= 1e-4 * np.abs(ref).max()
    assert (got[-10:] == 0).all()
    assert (feats(rec) == got).all()  # deterministic
    bad = np.empty(7, dtype=cm.NODE_DTYPE)
    bad["u"] = [-1, m, 3, 5, m + 7, 2, 0]
    bad["v"] = [1, 1, -2, n, 0, n + 1, -5]
    bad["r"] = 4.0
    mixed = np.concatenate([bad[:3], rec[:nnz // 2], bad[3:], rec[nnz // 2:]])
    assert (feats(mixed) == got).all()  # out-of-range ratings change nothing


def test_mlp_training_with_a_short_last_batch_continues_across_calls(lib, cuda):
    """Rows not a multiple of the batch (the last, shorter step is a second captured graph),
    and a second call continuing from the first (Adam's step count carries over)."""
    import torch
    rng = np.random.default_rng(4)
    rows = 3000
    X = rng.standard_normal((rows, D_IN)).astype(np.float32)
    A = rng.standard_normal((D_IN, D_OUT)).astype(np.float32) / np.sqrt(D_IN)
    T = np.tanh(X @ A).astype(np.float32)
    mlp = cm.MLP(D_IN, H, D_OUT, seed=7)
    dX, dT = torch.from_numpy(X).to(cuda), torch.from_numpy(T).to(cuda)
    before = mlp.loss_grad(dX.data_ptr(), dT.data_ptr(), rows)
    first = mlp.train(dX.data_ptr(), dT.data_ptr(), rows, epochs=15, batch=512, lr=1e-3, seed=3)
    mid = mlp.loss_grad(dX.data_ptr(), dT.data_ptr(), rows)
    second = mlp.train(dX.data_ptr(), dT.data_ptr(), rows, epochs=15, batch=512, lr=1e-3, seed=4)
    after = mlp.loss_grad(dX.data_ptr(), dT.data_ptr(), rows)
    assert np.isfinite([first, second]).all()
    assert mid < 0.3 * before and after < mid, (before, mid, after)
    assert second < first, (first, second)
    assert mlp.train(dX.data_ptr(), dT.data_ptr(), rows, epochs=0, batch=512, lr=1e-3, seed=5) == 0.0
