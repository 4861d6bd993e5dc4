"""Host side of the C ABI (no GPU): symbols, CLI parsing, files, shuffle and grid parity."""
import ctypes as C
import glob
import os
import re
import subprocess

import numpy as np
import pytest

import cumf_sgd_gb300 as cm
from cumf_sgd_gb300 import _lib
from conftest import GOLDEN, ROOT


def header_functions():
    txt = open(os.path.join(ROOT, "include", "cumf_sgd.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(cumf_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(lib):
    names = header_functions()
    assert len(names) >= 25
    for name in names:
        assert hasattr(lib, name), name
    assert set(names) == set(_lib.exported_symbols())
    assert lib.cumf_abi_version() == 2


def test_default_params_match_reference(lib):
    p = cm.Parameter.from_c(cm.Parameter().to_c())
    q = _lib.Params()
    lib.cumf_default_params(C.byref(q))
    # Parameter() (singleGPU/sgd.h:45)
    assert (q.k, q.num_workers, q.num_iters, q.gpu) == (80, 12, 30, 3)
    assert np.float32(q.lambda_p) == np.float32(0.05) and q.lrate == 0
    assert np.float32(q.alpha) == np.float32(0.01) and np.float32(q.beta) == np.float32(0.01)
    assert p.k == 80


def test_parse_argument_reference_semantics(lib):
    a = cm.parse_argument(["cumf_sgd", "-g", "1", "-l", "0.05", "-a", "0.08", "-b", "0.3", "-u", "1",
                           "-v", "1", "-x", "2", "-y", "2", "-s", "750", "-k", "128", "-t", "20",
                           "./data/netflix_train.bin"])
    p = a.param
    assert p.num_workers == 752  # rounded up to a multiple of 4 (main.cpp:139)
    assert (p.x_grid, p.y_grid) == (1, 1)  # u*v == 1 forces x = y = 1 (main.cpp:219-223)
    assert (p.k, p.num_iters, p.gpu) == (128, 20, 1)
    assert np.float32(p.alpha) == np.float32(0.08) and np.float32(p.beta) == np.float32(0.3)
    assert a.tr_path == "./data/netflix_train.bin"
    assert a.model_path == "netflix_train.bin.model"  # basename + .model (main.cpp:205-213)
    b = cm.parse_argument(["x", "-l", "0.01,0.02", "-u", "2", "-v", "3", "-x", "2", "-y", "4", "tr", "out.m"])
    assert np.float32(b.param.lambda_p) == np.float32(0.01) and np.float32(b.param.lambda_q) == np.float32(0.02)
    assert (b.param.ux, b.param.vy) == (4, 12) and b.model_path == "out.m"
    c = cm.parse_argument(["x", "--seed", "99", "--precision", "bf16sr", "-p", "te.bin", "tr"])
    assert c.param.seed == 99 and c.param.precision == "bf16sr" and c.va_path == "te.bin"
    assert c.param.hot_rows == 0  # no copies of the most-rated rows by default
    d = cm.parse_argument(["x", "--hot-rows", "0.5", "--deterministic", "3", "tr"])
    assert np.float32(d.param.hot_rows) == np.float32(0.5) and d.param.deterministic == 3


@pytest.mark.parametrize("argv,msg", [
    (["x"], "error"),
    (["x", "-k"], "need to specify number of factors"),
    (["x", "-k", "abc", "tr"], "-k should be followed by a number"),
    (["x", "-s", "4"], "training data not specified"),
    (["x", "--precision", "fp8", "tr"], "unknown precision"),
    (["x", "--hot-rows", "-1", "tr"], "--hot-rows should be 0 or more"),
    (["x", "--hot-rows"], "need to specify a number after --hot-rows"),
])
def test_parse_argument_errors(lib, argv, msg):
    with pytest.raises(ValueError, match=msg):
        cm.parse_argument(argv)


def test_problem_file_roundtrip_and_shards(lib, tmp_path):
    rng = np.random.default_rng(3)
    u = rng.integers(0, 50, 1000)
    v = rng.integers(0, 30, 1000)
    r = rng.random(1000).astype(np.float32) * 5
    prob = cm.MFProblem.from_arrays(u, v, r)
    path = str(tmp_path / "tr.bin")
    prob.write(path)
    assert os.path.getsize(path) == 12 * 1000
    back = cm.read_problem(path, pinned=False)
    assert (back.m, back.n, back.nnz) == (u.max() + 1, v.max() + 1, 1000)
    assert back.records.tobytes() == prob.records.tobytes()
    # trailing partial record is ignored (sgd.cu:237)
    with open(path, "ab") as f:
        f.write(b"\x01\x02\x03\x04\x05")
    assert cm.read_problem(path, pinned=False).nnz == 1000
    # sharded input path0..pathN read in order (sgd.cu:207-217, 272-332)
    base = str(tmp_path / "sh")
    recs = prob.records
    for i, (a, b_) in enumerate([(0, 300), (300, 301), (301, 1000)]):
        recs[a:b_].tofile(base + str(i))
    sh = cm.read_problem(base, pinned=False)
    assert sh.records.tobytes() == recs.tobytes() and sh.m == prob.m


def test_read_problem_errors(lib, tmp_path):
    with pytest.raises(cm.CumfError) as e:
        cm.read_problem(str(tmp_path / "missing.bin"))
    assert e.value.code == _lib.CUMF_ERR_IO
    bad = np.zeros(3, dtype=cm.NODE_DTYPE)
    bad["u"] = [0, -4, 2]
    p = str(tmp_path / "neg.bin")
    bad.tofile(p)
    with pytest.raises(cm.CumfError) as e:
        cm.read_problem(p)
    assert e.value.code == _lib.CUMF_ERR_FORMAT
    empty = str(tmp_path / "empty.bin")
    open(empty, "wb").close()
    pe = cm.read_problem(empty)
    assert (pe.nnz, pe.m, pe.n) == (0, 1, 1)


def test_model_file_layout_roundtrip(lib, tmp_path):
    rng = np.random.default_rng(5)
    P = rng.standard_normal((7, 16)).astype(np.float32)
    Q = rng.standard_normal((5, 16)).astype(np.float32)
    mod = cm.MFModel.from_arrays(P, Q, 1.25)
    path = str(tmp_path / "a.model")
    cm.save_model(mod, path)
    raw = open(path, "rb").read()
    assert len(raw) == 20 + 4 * 16 * (7 + 5)  # main.cpp:247-266
    assert np.frombuffer(raw[:16], np.int32).tolist() == [0, 7, 5, 16]
    assert np.frombuffer(raw[16:20], np.float32)[0] == np.float32(1.25)
    np.testing.assert_array_equal(np.frombuffer(raw[20:20 + 4 * 7 * 16], np.float32).reshape(7, 16), P)
    back = cm.mf_load_model(path)
    np.testing.assert_array_equal(back.P, P)
    np.testing.assert_array_equal(back.Q, Q)
    assert back.b == np.float32(1.25)
    with open(path, "r+b") as f:
        f.truncate(100)
    with pytest.raises(cm.CumfError) as e:
        cm.mf_load_model(path)
    assert e.value.code == _lib.CUMF_ERR_FORMAT
    with pytest.raises(cm.CumfError) as e:
        cm.save_model(mod, str(tmp_path / "no" / "such" / "dir.model"))
    assert e.value.code == _lib.CUMF_ERR_IO


LAYOUTS = sorted(glob.glob(os.path.join(GOLDEN, "layout_*.npz")))


@pytest.mark.parametrize("path", LAYOUTS, ids=[os.path.basename(p)[:-4] for p in LAYOUTS])
def test_library_shuffle_and_grid_match_reference(lib, path):
    g = np.load(path)
    m, n, seed, ux, vy = int(g["m"]), int(g["n"]), int(g["seed"]), int(g["ux"]), int(g["vy"])
    np.testing.assert_array_equal(cm.random_map(seed, m), g["p_map"])
    np.testing.assert_array_equal(cm.random_map(seed, n), g["q_map"])
    rec = np.ascontiguousarray(g["shuffled"].copy())
    gs, us, vs = cm.grid_problem(rec, m, n, ux, vy)
    np.testing.assert_array_equal(gs, g["grid_size"])
    assert (us, vs) == (int(g["u_seg"]), int(g["v_seg"]))
    assert rec.tobytes() == g["gridded"].tobytes()


def test_random_map_matches_glibc_for_large_sizes(lib, orc):
    for seed, size in [(0, 1), (7, 2), (1796309857, 480189), (123, 17770)]:
        np.testing.assert_array_equal(cm.random_map(seed, size), orc.gen_random_map(seed, size))


def test_lr_schedule_and_budget(lib, orc):
    np.testing.assert_array_equal(cm.lr_schedule(0.08, 0.3, 0.001, 30), orc.lr_table(0.08, 0.3, 0.001, 30))
    # ceil(nnz / (workers * 128)) (sgd_kernel.cu:203)
    assert cm.batches_per_worker(99_072_112, 7_696) == 101
    assert cm.batches_per_worker(900_000, 7_904) == 1
    assert cm.batches_per_worker(1, 1) == 1 and cm.batches_per_worker(0, 4) == 0


def test_train_rejects_bad_parameters_without_gpu(lib):
    prob = cm.MFProblem.from_arrays([0, 1], [0, 1], [1.0, 2.0])
    for kw in (dict(k=100), dict(k=128, num_workers=-1), dict(k=128, lanes=3), dict(k=128, num_iters=-1)):
        with pytest.raises(cm.CumfError) as e:
            cm.sgd_train(prob, None, cm.Parameter(**kw))
        assert e.value.code == _lib.CUMF_ERR_ARG


def test_cli_usage_errors(lib):
    exe = os.path.join(ROOT, "cumf_sgd_gb300", "bin", "cumf_sgd")
    res = subprocess.run([exe], capture_output=True, text=True)
    assert res.returncode == 1 and "error" in res.stdout
    res = subprocess.run([exe, "-k", "12x"], capture_output=True, text=True)
    assert res.returncode == 1
    exe2 = os.path.join(ROOT, "cumf_sgd_gb300", "bin", "cumf_predict")
    res = subprocess.run([exe2, "-e", "1", "a", "b"], capture_output=True, text=True)
    assert res.returncode == 1


def test_text_header_skip_follows_fscanf(lib):
    """fscanf("%[^\\n]\\n") three times (transform.cpp:31-33): each call takes a non-empty line
    and the whitespace after it; an empty line stops it."""
    import cumf_sgd_gb300 as cm
    assert cm.text_data_start(b"h1\n\nh3\n1 2 3\n4 5 6\n") == 13
    assert cm.text_data_start(b"\n1 2 3\n") == 0
    assert cm.text_data_start(b"only one line") == 13
    assert cm.text_data_start(b"") == 0
    assert cm.text_data_start(b"a\r\n  b\nc\n\n 1 2 3") == 11
    assert cm.text_data_start(b"a\nb\nc\n1 2 3", header_lines=0) == 0


def test_transform_tool_usage(lib, tmp_path):
    """Usage errors print the reference's message and exit 0 (transform.cpp:11-22)."""
    exe = os.path.join(ROOT, "cumf_sgd_gb300", "bin", "cumf_transform")
    for argv in ([exe], [exe, str(tmp_path / "missing.txt")], [exe, "a", "b"]):
        res = subprocess.run(argv, capture_output=True, text=True)
        assert res.returncode == 0 and res.stdout == "usage: ./transform file_name\n"


def test_checkpoint_arguments_without_gpu(lib, tmp_path):
    import cumf_sgd_gb300 as cm
    from cumf_sgd_gb300 import _lib as L
    prob = cm.MFProblem.from_arrays([0, 1], [0, 1], [1.0, 2.0])
    with pytest.raises(cm.CumfError) as e:
        cm.sgd_train_ckpt(prob, None, cm.Parameter(k=128), "", every=1)
    assert e.value.code == L.CUMF_ERR_ARG
    with pytest.raises(cm.CumfError) as e:
        cm.sgd_train_ckpt(prob, None, cm.Parameter(k=128), str(tmp_path / "x"), every=-1)
    assert e.value.code == L.CUMF_ERR_ARG
    with pytest.raises(cm.CumfError) as e:
        cm.sgd_train_ckpt(prob, None, cm.Parameter(k=128, u_grid=2, v_grid=2), str(tmp_path / "x"))
    assert e.value.code == L.CUMF_ERR_ARG
    exe = os.path.join(ROOT, "cumf_sgd_gb300", "bin", "cumf_sgd")
    res = subprocess.run([exe, "--resume", "train.bin"], capture_output=True, text=True)
    assert res.returncode == 1 and "--checkpoint" in res.stdout


def test_hot_rows_api_refuses_bad_arguments_without_a_gpu(lib):
    """The copies' entry points check their arguments before touching a device."""
    import ctypes as C
    out = C.c_void_p()
    assert lib.cumf_hot_rows_plan(None, 10, 5, 5, 100, 8, None, None) != 0  # no output pointer
    for args in ((None, -1, 5, 5, 100, 8), (None, 10, 0, 5, 100, 8), (None, 10, 5, 5, 0, 8), (None, 10, 5, 5, 100, 0),
                 (None, 10, 5, 5, 100, 8)):  # the last: ratings without a pointer
        assert lib.cumf_hot_rows_plan(*args, C.byref(out), None) != 0
        assert out.value is None
    assert lib.cumf_hot_rows_info(None, None, None, None, None) != 0
    assert lib.cumf_hot_rows_assign(None, None, 0, None) != 0
    assert lib.cumf_hot_rows_merge(None, None, None, 128, 0, None) != 0
    assert lib.cumf_hot_rows_free(None) == 0
    # no copies for one worker, no ratings or a concurrency of 0
    assert lib.cumf_hot_rows_per_copy(10**8, 1, 128, 0, 0, 0.5) == 0
    assert lib.cumf_hot_rows_per_copy(0, 1000, 128, 0, 0, 0.5) == 0
    assert lib.cumf_hot_rows_per_copy(10**8, 1000, 128, 0, 0, 0.0) == 0
