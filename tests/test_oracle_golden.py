"""The oracle against golden vectors produced by the reference's own code
(tests/golden/make_golden.py runs singleGPU/sgd.cu and test/mf.cpp compiled unmodified)."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN

LAYOUTS = sorted(glob.glob(os.path.join(GOLDEN, "layout_*.npz")))


@pytest.mark.parametrize("path", LAYOUTS, ids=[os.path.basename(p)[:-4] for p in LAYOUTS])
def test_layout_matches_reference(orc, path):
    g = np.load(path)
    rec = g["records"]
    m, n, seed, ux, vy, k = int(g["m"]), int(g["n"]), int(g["seed"]), int(g["ux"]), int(g["vy"]), int(g["k"])
    # collect_data (sgd.cu:78-96)
    ave, std = orc.collect_data(rec)
    assert np.float32(ave) == g["ave"] and np.float32(std) == g["std"]
    # gen_random_map x2 (sgd.cu:39-53, 656-657)
    pm = orc.gen_random_map(seed, m)
    qm = orc.gen_random_map(seed, n)
    np.testing.assert_array_equal(pm, g["p_map"])
    np.testing.assert_array_equal(qm, g["q_map"])
    # shuffle_problem (sgd.cu:126-134)
    sh = rec.copy()
    sh["u"] = pm[sh["u"]]
    sh["v"] = qm[sh["v"]]
    assert sh.tobytes() == g["shuffled"].tobytes()
    # grid_problem (sgd.cu:411-487): exact in-place order
    gridded, gs, us, vs = orc.grid_problem(sh, m, n, ux, vy)
    np.testing.assert_array_equal(gs, g["grid_size"])
    assert (us, vs) == (int(g["u_seg"]), int(g["v_seg"]))
    assert gridded.tobytes() == g["gridded"].tobytes()
    # scale_problem (sgd.cu:98-124)
    scale = max(np.float32(1e-4), np.float32(std))
    sc = gridded.copy()
    sc["r"] = sc["r"] * np.float32(1.0 / float(scale))
    if ux * vy != 1:
        sc["u"] = sc["u"] % us
        sc["v"] = sc["v"] % vs
    assert sc.tobytes() == g["scaled"].tobytes()


@pytest.mark.parametrize("path", LAYOUTS[:3], ids=[os.path.basename(p)[:-4] for p in LAYOUTS[:3]])
def test_scale_and_unshuffle_model_match_reference(orc, path):
    g = np.load(path)
    m, n, k = int(g["m"]), int(g["n"]), int(g["k"])
    P = ((np.arange(m * k) % 9973).astype(np.float32) * np.float32(0.001) + np.float32(0.5)).reshape(m, k)
    Q = ((np.arange(n * k) % 7919).astype(np.float32) * np.float32(0.002) - np.float32(0.25)).reshape(n, k)
    scale = max(np.float32(1e-4), np.float32(g["std"]))
    inv_p = np.empty(m, np.int32)
    inv_p[g["p_map"]] = np.arange(m)
    inv_q = np.empty(n, np.int32)
    inv_q[g["q_map"]] = np.arange(n)
    for X, inv in ((P, inv_p), (Q, inv_q)):
        orc.lib().or_scale_model(X.ctypes.data, X.shape[0], k, float(scale))
        orc.shuffle_model(X, inv)
    np.testing.assert_array_equal(P, g["P"])
    np.testing.assert_array_equal(Q, g["Q"])
    # The library's export is a gather: out[o] = in[p_map[o]] * sqrt(scale).
    P0 = ((np.arange(m * k) % 9973).astype(np.float32) * np.float32(0.001) + np.float32(0.5)).reshape(m, k)
    f = np.float32(np.sqrt(np.float32(scale)))
    np.testing.assert_array_equal(P0[g["p_map"]] * f, g["P"])


def test_rmse_matches_reference(orc):
    g = np.load(os.path.join(GOLDEN, "rmse.npz"))
    i = 0
    while f"rmse{i}" in g:
        got = orc.calc_rmse(g[f"te{i}"], g[f"P{i}"], g[f"Q{i}"], float(g[f"b{i}"]))
        ref = float(g[f"rmse{i}"])
        assert abs(got - ref) <= 1e-6 * ref, (i, got, ref)
        assert f"RMSE = {got:.4f}" == str(g[f"line{i}"])
        i += 1
    assert i >= 3


def test_lr_table(orc):
    t = orc.lr_table(0.08, 0.3, 0.0, 24)
    # alpha, beta are floats (Parameter, sgd.h:42) widened to double (sgd_kernel.cu:139-146)
    a, b = float(np.float32(0.08)), float(np.float32(0.3))
    expect = np.array([np.float32(a / (1 + b * i ** 1.5)) for i in range(24)], dtype=np.float32)
    np.testing.assert_array_equal(t, expect)


def test_oracle_serial_sgd_reduces_training_error(orc):
    rng = np.random.default_rng(0)
    m, n, k, nnz = 60, 40, 32, 4000
    rec = np.empty(nnz, dtype=orc.NODE)
    rec["u"] = rng.integers(0, m, nnz)
    rec["v"] = rng.integers(0, n, nnz)
    rec["r"] = rng.integers(1, 6, nnz).astype(np.float32)
    P, Q, b, ave, std = orc.train(rec, m, n, k=k, precision="fp32", num_workers=4, num_iters=10, lanes=8)
    P0, Q0, _, _, _ = orc.train(rec, m, n, k=k, precision="fp32", num_workers=4, num_iters=0, lanes=8)
    assert orc.calc_rmse(rec, P, Q, b) < 0.8 * orc.calc_rmse(rec, P0, Q0, b)


def test_half_rounding_matches_numpy(orc):
    x = np.concatenate([np.random.default_rng(1).standard_normal(5000).astype(np.float32) * 4,
                        np.array([65504, 65519.99, 65520, 6.1e-5, 5.96e-8, 2.98e-8, 1e-9, -0.0],
                                 dtype=np.float32)])
    with np.errstate(over="ignore"):
        ref = x.astype(np.float16).view(np.uint16)
    got = np.array([orc.lib().or_half_rn(float(v)) for v in x], dtype=np.uint16)
    np.testing.assert_array_equal(got, ref)


def test_text_oracle_matches_reference_transform(orc):
    """The oracle's strict parse reproduces the records the reference's own transform wrote
    (data/netflix/transform.cpp, compiled from its source) for every text fixture."""
    z = np.load(os.path.join(GOLDEN, "text.npz"))
    names = [k[5:] for k in z.files if k.startswith("text_")]
    assert len(names) >= 8
    for name in names:
        got = orc.parse_text(z["text_" + name].tobytes())
        assert not isinstance(got, tuple), (name, got)
        assert got.tobytes() == z["bin_" + name].tobytes(), name


def test_text_oracle_rejects_malformed_tokens(orc):
    head = b"a\nb\nc\n"
    assert orc.parse_text(head + b"1 2 3\n4 5 x\n") == ("bad", len(head) + 10)
    assert orc.parse_text(head + b"1 2.5 3\n") == ("bad", len(head) + 2)
    assert orc.parse_text(head + b"1 2 0x1p3\n") == ("bad", len(head) + 4)
    assert orc.parse_text(head + b"99999999999 2 3\n") == ("bad", len(head))
    assert orc.parse_text(head + b"1 2 3 4\n") == ("partial", None)


def test_criteria_oracle_matches_reference(orc):
    """Every mf-predict criterion of the oracle against the reference's own test/mf.cpp
    functions (golden values computed with oracle/_ref/ref_rmse ... all)."""
    z = np.load(os.path.join(GOLDEN, "eval.npz"))
    crits = [int(c) for c in z["criteria"]]
    for i in range(3):
        te, P, Q, b = z[f"te{i}"], z[f"P{i}"], z[f"Q{i}"], float(z[f"b{i}"])
        for c, ref in zip(crits, z[f"crit{i}"]):
            got = orc.evaluate(te, P, Q, b, c)
            if np.isnan(ref):
                assert np.isnan(got), (i, c)
            else:
                assert abs(got - ref) <= 1e-6 * max(1.0, abs(ref)), (i, c, got, ref)


def test_oracle_fold_in_freezes_items(orc):
    """freeze_q: item rows are read, never written, and user rows still move (the GPU kernels
    are compared with this bit for bit in test_single_worker_fold_in_bit_exact)."""
    import cumf_sgd_gb300 as cm
    rng = np.random.default_rng(3)
    m, n, k = 30, 12, 64
    rec = np.empty(600, dtype=cm.NODE_DTYPE)
    rec["u"], rec["v"] = rng.integers(0, m, 600), rng.integers(0, n, 600)
    rec["r"] = rng.integers(1, 6, 600).astype(np.float32)
    lr = orc.lr_table(0.08, 0.3, 0.0, 4)
    for precision in ("fp32", "fp16", "bf16", "bf16sr", "fp16sr"):
        P0, Q0 = orc.init_factors(m, k, precision, 2, 1), orc.init_factors(n, k, precision, 2, 2)
        P, Q = P0.copy(), Q0.copy()
        orc.sgd_epochs(rec, P, Q, precision, 1, lr, 0, 2, 0.05, 0.05, 2, freeze_q=1)
        assert np.array_equal(Q, Q0), precision
        assert not np.array_equal(P, P0), precision
        Pu, Qu = P0.copy(), Q0.copy()
        orc.sgd_epochs(rec, Pu, Qu, precision, 1, lr, 0, 2, 0.05, 0.05, 2, freeze_q=0)
        assert not np.array_equal(Qu, Q0) and not np.array_equal(Pu, P), precision
