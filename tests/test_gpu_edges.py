"""Edge cases of the update path: factor rows beyond 4 GB of offset, a rating array longer
than 2^31 records, and empty problems in every mode; the cache of page-locked host buffers."""
import numpy as np
import pytest

import cumf_sgd_gb300 as cm

pytestmark = pytest.mark.gpu


def test_rows_beyond_4gb_offsets_bit_exact(lib, orc, cuda):
    """k = 32 fp16 rows are 64 bytes: users above 2^26 sit more than 4 GB into P.  One
    worker, two epochs; the touched rows equal the oracle run on the same rows renumbered."""
    import torch
    m, n, k, nnz = 80_000_000, 500, 32, 4000
    rng = np.random.default_rng(5)
    users = np.concatenate([rng.choice(np.arange(67_200_000, m), 150, replace=False), np.array([0, 1, 2, 3, 4])])
    rec = np.empty(nnz, dtype=cm.NODE_DTYPE)
    rec["u"] = users[rng.integers(0, len(users), nnz)]
    rec["v"] = rng.integers(0, n, nnz)
    rec["r"] = rng.integers(1, 6, nnz).astype(np.float32) / np.float32(1.3)
    P = torch.empty(m * k, dtype=torch.float16, device=cuda)
    Q = torch.empty(n * k, dtype=torch.float16, device=cuda)
    cm.dev_init_factors(P.data_ptr(), m, k, "fp16", 9, 1)
    cm.dev_init_factors(Q.data_ptr(), n, k, "fp16", 9, 2)
    idx = torch.from_numpy(users.astype(np.int64)).to(cuda)
    P0 = P.view(m, k).index_select(0, idx).float().cpu().numpy()
    Q0 = Q.view(n, k).float().cpu().numpy()
    d_R = torch.from_numpy(rec.view(np.uint8).copy()).to(cuda)
    lr = orc.lr_table(0.08, 0.3, 0.0, 4)
    d_lr = torch.from_numpy(lr).to(cuda)
    status = torch.zeros(1, dtype=torch.int32, device=cuda)
    cm.sgd_update(d_R.data_ptr(), nnz, P.data_ptr(), m, Q.data_ptr(), n, k, "fp16", 1, 0, d_lr.data_ptr(), 0, 2,
                  0.05, 0.05, 3, status.data_ptr())
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    got_P = P.view(m, k).index_select(0, idx).float().cpu().numpy()
    got_Q = Q.view(n, k).float().cpu().numpy()
    remap = {int(u): i for i, u in enumerate(users)}
    small = rec.copy()
    small["u"] = np.array([remap[int(u)] for u in rec["u"]], dtype=np.int32)
    Pr, Qr = P0.copy(), Q0.copy()
    assert orc.sgd_epochs(small, Pr, Qr, "fp16", 1, lr, 0, 2, 0.05, 0.05, 3, lanes=4) == 0
    np.testing.assert_array_equal(got_P, Pr)
    np.testing.assert_array_equal(got_Q, Qr)


def test_more_than_2_31_ratings(lib, cuda):
    """2^31 + 2^20 records built on the device: records below index 2^31 name users 0..999,
    the rest users 1000..1999.  One epoch with auto workers updates both groups (the samples
    reach past 2^31) and leaves every other row as initialised."""
    import torch
    N = (1 << 31) + (1 << 20)
    m, n, k = 3000, 777, 32
    rec = torch.empty((N, 3), dtype=torch.int32, device=cuda)
    chunk = 1 << 28
    for a in range(0, N, chunk):
        b = min(N, a + chunk)
        i = torch.arange(a, b, dtype=torch.int64, device=cuda)
        rec[a:b, 0] = (i % 1000 + (i >= (1 << 31)).to(torch.int64) * 1000).to(torch.int32)
        rec[a:b, 1] = (i % n).to(torch.int32)
        rec[a:b, 2] = torch.full((b - a,), 3.0, device=cuda).view(torch.int32)
        del i
    P = torch.empty(m * k, dtype=torch.float16, device=cuda)
    Q = torch.empty(n * k, dtype=torch.float16, device=cuda)
    cm.dev_init_factors(P.data_ptr(), m, k, "fp16", 4, 1)
    cm.dev_init_factors(Q.data_ptr(), n, k, "fp16", 4, 2)
    P0 = P.view(m, k).float().clone()
    lr = torch.full((4,), 0.01, dtype=torch.float32, device=cuda)
    status = torch.zeros(1, dtype=torch.int32, device=cuda)
    sm, _, _ = cm.device_info(0)
    workers = cm.auto_workers(N, sm, k, "fp16", 0)
    cm.sgd_update(rec.data_ptr(), N, P.data_ptr(), m, Q.data_ptr(), n, k, "fp16", workers, 0, lr.data_ptr(), 0, 1,
                  0.05, 0.05, 7, status.data_ptr())
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    Pf = P.view(m, k).float()
    moved = (Pf != P0).any(1).cpu().numpy()
    assert moved[:1000].all() and moved[1000:2000].all()
    assert not moved[2000:].any()
    assert torch.isfinite(Pf).all()
    del rec


@pytest.mark.parametrize("grid", [(1, 1), (2, 2)])
def test_empty_problem_trains(lib, cuda, grid):
    prob = cm.MFProblem.from_arrays([], [], [], m=7, n=5)
    par = cm.Parameter(k=32, num_workers=4, num_iters=3, u_grid=grid[0], v_grid=grid[1], seed=1, gpu=0, quiet=1)
    model = cm.sgd_train(prob, None, par)
    assert model.P.shape == (7, 32) and model.Q.shape == (5, 32)
    assert np.isfinite(model.P).all() and np.isfinite(model.Q).all()
    assert model.b == 0.0


def test_zero_workers_means_automatic(lib, cuda):
    rng = np.random.default_rng(3)
    nnz, m, n = 200_000, 2000, 500
    prob = cm.MFProblem.from_arrays(rng.integers(0, m, nnz), rng.integers(0, n, nnz),
                                    rng.integers(1, 6, nnz).astype(np.float32), m=m, n=n)
    sm, _, _ = cm.device_info(0)
    for grid in ((1, 1), (2, 2)):
        par = cm.Parameter(k=64, num_workers=0, num_iters=2, u_grid=grid[0], v_grid=grid[1], seed=1, gpu=0, quiet=1)
        _, st = cm.sgd_train(prob, None, par, with_stats=True)
        blocks = grid[0] * grid[1]
        assert st.num_workers == cm.auto_workers(nnz // blocks, sm, 64, "fp16", 0)


def test_copy_bandwidth_probe(lib, cuda):
    """The roofline probe: an L2-resident copy is faster than one that streams from HBM."""
    import ctypes as C
    from cumf_sgd_gb300 import _lib
    l2, hbm = C.c_double(0), C.c_double(0)
    _lib.check(lib.cumf_probe_copy_bandwidth(16 << 20, 200, C.byref(l2), None))
    _lib.check(lib.cumf_probe_copy_bandwidth(1 << 30, 3, C.byref(hbm), None))
    assert hbm.value > 1000 and l2.value > 1.3 * hbm.value
    with pytest.raises(cm.CumfError):
        _lib.check(lib.cumf_probe_copy_bandwidth(8, 1, C.byref(l2), None))


def test_pinned_host_buffers_are_cached_and_released(lib, cuda):
    """A pinned model buffer given back by cumf_free_model serves the next allocation it fits
    (page-locking is the slow part of every training call's export); a request much smaller
    than the cached block gets its own; cumf_release_host_cache empties the cache."""
    import ctypes as C
    from cumf_sgd_gb300 import _lib
    lib.cumf_release_host_cache()

    def alloc(m, n, k):
        mod = _lib.Model()
        assert lib.cumf_alloc_model(m, n, k, C.byref(mod)) == 0
        assert mod.pinned == 1
        return mod

    a = alloc(20_000, 3_000, 128)
    p_addr, q_addr = C.cast(a.P, C.c_void_p).value, C.cast(a.Q, C.c_void_p).value
    assert lib.cumf_free_model(C.byref(a)) == 0
    b = alloc(20_000, 3_000, 128)  # the same sizes come back from the cache
    assert C.cast(b.P, C.c_void_p).value == p_addr and C.cast(b.Q, C.c_void_p).value == q_addr
    arr = np.ctypeslib.as_array(b.P, shape=(20_000 * 128,))
    arr[:] = 1.5  # the reused buffer is ordinary writable host memory
    assert lib.cumf_free_model(C.byref(b)) == 0
    tiny = alloc(10, 10, 128)  # far smaller than the cached P block: not taken from it
    assert C.cast(tiny.P, C.c_void_p).value != p_addr
    assert lib.cumf_free_model(C.byref(tiny)) == 0
    assert lib.cumf_release_host_cache() == 0
    c = alloc(20_000, 3_000, 128)
    assert lib.cumf_free_model(C.byref(c)) == 0
    assert lib.cumf_release_host_cache() == 0
