"""cumf_dev_rmse_noalloc: the RMSE evaluator for callers that cannot allocate device memory
when they evaluate (fixed pools or arenas, allocator hooks, out-of-memory handlers).  Its
scratch is a fixed array inside the library, so its result must equal the allocating
cumf_dev_rmse within the RMSE tolerance used elsewhere (1e-6 relative), call after call.
Collected last so a failure here leaves every other test already run."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_rmse_matches_allocating_entry_point(lib, cuda):
    import torch
    from cumf_sgd_gb300 import _lib
    rng = np.random.default_rng(17)
    m, n, k, nnz = 700, 300, 128, 250_000
    rec = np.empty(nnz, dtype=[("u", "<i4"), ("v", "<i4"), ("r", "<f4")])
    rec["u"] = rng.integers(0, m + 4, nnz)  # some ids outside the model predict b
    rec["v"] = rng.integers(0, n, nnz)
    rec["r"] = rng.integers(1, 6, nnz).astype(np.float32)
    d_R = torch.from_numpy(rec.view(np.uint8).copy()).to(cuda)
    d_P = torch.from_numpy((rng.standard_normal((m, k)) * 0.2).astype(np.float32)).to(cuda)
    d_Q = torch.from_numpy((rng.standard_normal((n, k)) * 0.2).astype(np.float32)).to(cuda)
    b = 3.1
    # set-up call (nnz = 0): loads the evaluator code while allocation is still allowed
    zero = C.c_double(-1.0)
    assert lib.cumf_dev_rmse_noalloc(None, 0, None, m, None, n, k, b, C.byref(zero), None) == 0
    assert zero.value == 0.0
    ref = C.c_double()
    assert lib.cumf_dev_rmse(d_R.data_ptr(), nnz, d_P.data_ptr(), m, d_Q.data_ptr(), n, k, b,
                             C.byref(ref), None) == 0
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    first = None
    for _ in range(3):  # the shared scratch keeps the last call's contents
        got = C.c_double()
        rc = lib.cumf_dev_rmse_noalloc(d_R.data_ptr(), nnz, d_P.data_ptr(), m, d_Q.data_ptr(), n, k, b,
                                       C.byref(got), None)
        assert rc == 0, lib.cumf_last_error()
        assert abs(got.value - ref.value) <= 1e-6 * ref.value, (got.value, ref.value)
        first = got.value if first is None else first
        assert got.value == first  # the same bits from call to call
    # after the set-up call, evaluations take no device memory
    assert torch.cuda.mem_get_info()[0] == free_before
    # a smaller second problem right after: stale partials of the bigger call must not leak in
    small = 10_000
    ref2, got2 = C.c_double(), C.c_double()
    assert lib.cumf_dev_rmse(d_R.data_ptr(), small, d_P.data_ptr(), m, d_Q.data_ptr(), n, k, b,
                             C.byref(ref2), None) == 0
    assert lib.cumf_dev_rmse_noalloc(d_R.data_ptr(), small, d_P.data_ptr(), m, d_Q.data_ptr(), n, k, b,
                                     C.byref(got2), None) == 0
    assert abs(got2.value - ref2.value) <= 1e-6 * ref2.value
    # sizes beyond the fixed scratch are rejected before anything runs
    too_many = 16384 * 8192 + 1
    rc = lib.cumf_dev_rmse_noalloc(d_R.data_ptr(), too_many, d_P.data_ptr(), m, d_Q.data_ptr(), n, k, b,
                                   C.byref(got2), None)
    assert rc == _lib.CUMF_ERR_ARG and b"scratch limit" in lib.cumf_last_error()
