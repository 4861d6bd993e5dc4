"""ctypes front end of the C oracle (oracle.c) and of the reference tools in oracle/_ref.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg, never by the cumf_sgd_gb300 package.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "build")
LIB = os.path.join(BUILD, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
NODE = np.dtype([("u", "<i4"), ("v", "<i4"), ("r", "<f4")])

OR_HALF, OR_BF16, OR_FLOAT = 0, 1, 2
OR_DOT_LANES, OR_DOT_REF = 0, 1
OR_ORDER_WORKER_MAJOR, OR_ORDER_ROUND_ROBIN = 0, 1
KIND = {"fp16": (OR_HALF, 0), "bf16": (OR_BF16, 0), "fp32": (OR_FLOAT, 0),
        "bf16sr": (OR_BF16, 1), "fp16sr": (OR_HALF, 1)}


def build_oracle() -> str:
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "oracle.c")
    hdr = os.path.join(HERE, "oracle.h")
    if (not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(src), os.path.getmtime(hdr))):
        cc = shutil.which("gcc") or "cc"
        res = subprocess.run([cc, "-O2", "-std=gnu11", "-fPIC", "-shared", "-ffp-contract=off",
                              "-o", LIB, src, "-lm", "-lpthread"], capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + res.stderr)
    return LIB


def build_reference() -> bool:
    """Builds oracle/_ref from the reference tree when it is present, or (on the GPU host,
    which has no reference tree) the trainer tools from the sources ref_build.sh staged in
    oracle/_ref/src; returns whether the reference trainers are available."""
    ref = os.environ.get("CUMF_REFERENCE", "/root/reference")
    staged = os.path.isfile(os.path.join(REF_DIR, "src", "singleGPU", "sgd_kernel.cu"))
    if not os.path.isdir(os.path.join(ref, "test")) and not staged:
        return trainers_available()
    script = os.path.join(HERE, "ref_build.sh")
    res = subprocess.run(["bash", script], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("reference build failed:\n" + res.stdout + res.stderr)
    return trainers_available()


def reference_available() -> bool:
    """The reference's host tools built on this machine (goldens: layouts, criteria)."""
    return all(os.access(os.path.join(REF_DIR, t), os.X_OK) for t in ("mf-predict", "ref_layout", "ref_rmse"))


def trainers_available() -> bool:
    """The reference's two trainers: LIBMF mf-train (CPU) and cumf_sgd_ref (the reference GPU
    trainer, singleGPU/, built for sm_103a)."""
    return all(os.access(os.path.join(REF_DIR, t), os.X_OK) for t in ("mf-train", "mf-predict", "cumf_sgd_ref"))


def ref_build_info() -> str:
    path = os.path.join(REF_DIR, "BUILD_INFO")
    return open(path).read().strip() if os.path.exists(path) else ""


class _SgdArgs(C.Structure):
    _fields_ = [("R", C.c_void_p), ("nnz", C.c_int64), ("P", C.c_void_p), ("m", C.c_int32),
                ("Q", C.c_void_p), ("n", C.c_int32), ("k", C.c_int), ("kind", C.c_int),
                ("sr", C.c_int), ("num_workers", C.c_int), ("lanes", C.c_int),
                ("dot_order", C.c_int), ("order", C.c_int), ("lr", C.c_void_p),
                ("first_epoch", C.c_int), ("n_epochs", C.c_int), ("lambda_p", C.c_float),
                ("lambda_q", C.c_float), ("seed", C.c_uint64), ("skipped", C.c_int64),
                ("freeze_q", C.c_int)]


class _TrainArgs(C.Structure):
    _fields_ = [("R", C.c_void_p), ("nnz", C.c_int64), ("m", C.c_int32), ("n", C.c_int32),
                ("k", C.c_int), ("kind", C.c_int), ("sr", C.c_int), ("num_workers", C.c_int),
                ("lanes", C.c_int), ("dot_order", C.c_int), ("order", C.c_int),
                ("num_iters", C.c_int), ("lambda_p", C.c_float), ("lambda_q", C.c_float),
                ("alpha", C.c_float), ("beta", C.c_float), ("lrate", C.c_float),
                ("seed", C.c_uint64), ("u_grid", C.c_int), ("v_grid", C.c_int),
                ("x_grid", C.c_int), ("y_grid", C.c_int), ("P_out", C.c_void_p),
                ("Q_out", C.c_void_p), ("b_out", C.c_float), ("ave", C.c_float),
                ("std_dev", C.c_float)]


class _Sgd64Args(C.Structure):
    _fields_ = [("R", C.c_void_p), ("nnz", C.c_int64), ("P", C.c_void_p), ("m", C.c_int32),
                ("Q", C.c_void_p), ("n", C.c_int32), ("k", C.c_int), ("num_workers", C.c_int),
                ("order", C.c_int), ("lr", C.c_void_p), ("first_epoch", C.c_int), ("n_epochs", C.c_int),
                ("lambda_p", C.c_double), ("lambda_q", C.c_double), ("rscale", C.c_double),
                ("seed", C.c_uint64)]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        _lib = C.CDLL(build_oracle())
        _lib.or_half_rn.restype = C.c_uint16
        _lib.or_half_rn.argtypes = [C.c_float]
        _lib.or_half_to_float.restype = C.c_float
        _lib.or_half_to_float.argtypes = [C.c_uint16]
        _lib.or_bf16_rn.restype = C.c_uint16
        _lib.or_bf16_rn.argtypes = [C.c_float]
        _lib.or_splitmix64.restype = C.c_uint64
        _lib.or_splitmix64.argtypes = [C.c_uint64]
        _lib.or_batch_start.restype = C.c_uint64
        _lib.or_batch_start.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64]
        _lib.or_block_seed.restype = C.c_uint64
        _lib.or_block_seed.argtypes = [C.c_uint64, C.c_int]
        _lib.or_calc_rmse.restype = C.c_double
        _lib.or_calc_rmse.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int32, C.c_void_p,
                                      C.c_int32, C.c_int, C.c_float]
        _lib.or_gen_random_map.argtypes = [C.c_uint32, C.c_int32, C.c_void_p]
        _lib.or_grid_problem.argtypes = [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_int, C.c_int,
                                         C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        _lib.or_collect_data.argtypes = [C.c_void_p, C.c_int64, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        _lib.or_lr_table.argtypes = [C.c_float, C.c_float, C.c_float, C.c_int, C.c_void_p]
        _lib.or_init_factors.argtypes = [C.c_void_p, C.c_int64, C.c_int, C.c_int, C.c_uint64, C.c_uint32]
        _lib.or_sgd_epochs.argtypes = [C.POINTER(_SgdArgs)]
        _lib.or_train.argtypes = [C.POINTER(_TrainArgs)]
        _lib.or_shuffle_model.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_int]
        _lib.or_scale_model.argtypes = [C.c_void_p, C.c_int64, C.c_int, C.c_float]
        _lib.or_sgd_epochs_f64.argtypes = [C.POINTER(_Sgd64Args)]
        _lib.or_sgd_epochs_f64_threads.argtypes = [C.POINTER(_Sgd64Args), C.c_int]
        _lib.or_init_factors_f64.argtypes = [C.c_void_p, C.c_int64, C.c_int, C.c_uint64, C.c_uint32]
        _lib.or_calc_rmse_f64.restype = C.c_double
        _lib.or_calc_rmse_f64.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32,
                                          C.c_int, C.c_double]
        _lib.or_evaluate.argtypes = [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_void_p, C.c_int32,
                                     C.c_void_p, C.c_int32, C.c_int, C.c_float, C.c_int]
        _lib.or_evaluate.restype = C.c_double
        _lib.or_strata_epochs.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int32, C.c_void_p, C.c_int32,
                                          C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int,
                                          C.c_int, C.c_float, C.c_float, C.c_uint64]
        _lib.or_strata_epochs.restype = C.c_int64
        _lib.or_parse_text.argtypes = [C.c_char_p, C.c_int64, C.c_int, C.c_void_p, C.c_int64,
                                        C.POINTER(C.c_int64)]
        _lib.or_parse_text.restype = C.c_int64
        _lib.or_hogwild_threads.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int32, C.c_void_p,
                                            C.c_int32, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int,
                                            C.c_float, C.c_float, C.c_uint64, C.c_int]
    return _lib


def _ptr(a: np.ndarray) -> int:
    assert a.flags.c_contiguous
    return a.ctypes.data


def half_rn(x: float) -> int:
    return lib().or_half_rn(x)


def gen_random_map(seed: int, size: int) -> np.ndarray:
    out = np.zeros(size, dtype=np.int32)
    lib().or_gen_random_map(seed & 0xffffffff, size, _ptr(out))
    return out


def grid_problem(records: np.ndarray, m: int, n: int, ux: int, vy: int):
    rec = np.ascontiguousarray(records.copy())
    gs = np.zeros(ux * vy, dtype=np.int64)
    us, vs = C.c_int64(), C.c_int64()
    lib().or_grid_problem(_ptr(rec), len(rec), m, n, ux, vy, _ptr(gs), C.byref(us), C.byref(vs))
    return rec, gs, us.value, vs.value


def collect_data(records: np.ndarray):
    a, s = C.c_float(), C.c_float()
    rec = np.ascontiguousarray(records)
    lib().or_collect_data(_ptr(rec), len(rec), C.byref(a), C.byref(s))
    return a.value, s.value


def lr_table(alpha: float, beta: float, lrate: float, n: int) -> np.ndarray:
    out = np.zeros(n, dtype=np.float32)
    lib().or_lr_table(alpha, beta, lrate, n, _ptr(out))
    return out


def init_factors(rows: int, k: int, precision: str, seed: int, tag: int) -> np.ndarray:
    out = np.zeros((rows, k), dtype=np.float32)
    lib().or_init_factors(_ptr(out), rows, k, KIND[precision][0], seed, tag)
    return out


def sgd_epochs(records: np.ndarray, P: np.ndarray, Q: np.ndarray, precision: str, num_workers: int,
               lr: np.ndarray, first_epoch: int, n_epochs: int, lambda_p: float, lambda_q: float,
               seed: int, lanes: int = 16, dot_order: int = OR_DOT_LANES,
               order: int = OR_ORDER_ROUND_ROBIN, freeze_q: int = 0) -> int:
    """Serial batch-Hogwild epochs in place on fp32 arrays P, Q (freeze_q: Q is read, never
    written); returns skipped records."""
    rec = np.ascontiguousarray(records)
    lr = np.ascontiguousarray(lr, dtype=np.float32)
    kind, sr = KIND[precision]
    a = _SgdArgs(R=_ptr(rec), nnz=len(rec), P=_ptr(P), m=P.shape[0], Q=_ptr(Q), n=Q.shape[0],
                 k=P.shape[1], kind=kind, sr=sr, num_workers=num_workers, lanes=lanes,
                 dot_order=dot_order, order=order, lr=_ptr(lr), first_epoch=first_epoch,
                 n_epochs=n_epochs, lambda_p=lambda_p, lambda_q=lambda_q, seed=seed, freeze_q=freeze_q)
    lib().or_sgd_epochs(C.byref(a))
    return a.skipped


def hogwild_threads(records: np.ndarray, P: np.ndarray, Q: np.ndarray, num_workers: int,
                    lr: np.ndarray, first_epoch: int, n_epochs: int, lambda_p: float,
                    lambda_q: float, seed: int, threads: int) -> None:
    rec = np.ascontiguousarray(records)
    lr = np.ascontiguousarray(lr, dtype=np.float32)
    lib().or_hogwild_threads(_ptr(rec), len(rec), _ptr(P), P.shape[0], _ptr(Q), Q.shape[0], P.shape[1],
                             num_workers, _ptr(lr), first_epoch, n_epochs, lambda_p, lambda_q, seed,
                             threads)


def train(records: np.ndarray, m: int, n: int, k: int = 128, precision: str = "fp16",
          num_workers: int = 1, num_iters: int = 1, lambda_p: float = 0.05, lambda_q: float = 0.05,
          alpha: float = 0.08, beta: float = 0.3, lrate: float = 0.0, seed: int = 0, lanes: int = 16,
          dot_order: int = OR_DOT_LANES, order: int = OR_ORDER_ROUND_ROBIN, u_grid: int = 1,
          v_grid: int = 1, x_grid: int = 1, y_grid: int = 1):
    """Serial sgd_train; returns (P, Q, b, ave, std_dev)."""
    rec = np.ascontiguousarray(records)
    P = np.zeros((m, k), dtype=np.float32)
    Q = np.zeros((n, k), dtype=np.float32)
    kind, sr = KIND[precision]
    a = _TrainArgs(R=_ptr(rec), nnz=len(rec), m=m, n=n, k=k, kind=kind, sr=sr, num_workers=num_workers,
                   lanes=lanes, dot_order=dot_order, order=order, num_iters=num_iters, lambda_p=lambda_p,
                   lambda_q=lambda_q, alpha=alpha, beta=beta, lrate=lrate, seed=seed, u_grid=u_grid,
                   v_grid=v_grid, x_grid=x_grid, y_grid=y_grid, P_out=_ptr(P), Q_out=_ptr(Q))
    lib().or_train(C.byref(a))
    return P, Q, a.b_out, a.ave, a.std_dev


def calc_rmse(records: np.ndarray, P: np.ndarray, Q: np.ndarray, b: float) -> float:
    rec = np.ascontiguousarray(records)
    P = np.ascontiguousarray(P, dtype=np.float32)
    Q = np.ascontiguousarray(Q, dtype=np.float32)
    return lib().or_calc_rmse(_ptr(rec), len(rec), _ptr(P), P.shape[0], _ptr(Q), Q.shape[0], P.shape[1], b)


def shuffle_model(vec: np.ndarray, inv_map: np.ndarray) -> None:
    inv = np.ascontiguousarray(inv_map.astype(np.int32).copy())
    lib().or_shuffle_model(_ptr(vec), _ptr(inv), vec.shape[0], vec.shape[1])


# ---- reference tools (oracle/_ref), available only where the reference tree was present ----

def ref_layout(records: np.ndarray, seed: int, ux: int, vy: int, k: int, tmpdir: str) -> dict:
    """Runs the reference's sgd.cu host functions on `records` (see ref_layout_driver.cpp)."""
    src = os.path.join(tmpdir, "in.bin")
    out = os.path.join(tmpdir, "out.bin")
    np.ascontiguousarray(records).tofile(src)
    subprocess.run([os.path.join(REF_DIR, "ref_layout"), src, str(seed), str(ux), str(vy), str(k), out],
                   check=True, capture_output=True)
    buf = open(out, "rb").read()
    off = 0

    def take(dtype, count):
        nonlocal off
        a = np.frombuffer(buf, dtype=dtype, count=count, offset=off)
        off += a.nbytes
        return a.copy()

    m, n, ux_, vy_ = take(np.int32, 4)
    nnz = int(take(np.int64, 1)[0])
    ave, std = take(np.float32, 2)
    u_seg, v_seg = take(np.int64, 2)
    res = dict(m=int(m), n=int(n), nnz=nnz, ave=float(ave), std=float(std), u_seg=int(u_seg),
               v_seg=int(v_seg))
    res["p_map"] = take(np.int32, m)
    res["q_map"] = take(np.int32, n)
    res["cont"] = take(np.int32, 8)
    res["grid_size"] = take(np.int64, ux * vy)
    res["shuffled"] = take(NODE, nnz)
    res["gridded"] = take(NODE, nnz)
    res["scaled"] = take(NODE, nnz)
    res["P"] = take(np.float32, m * k).reshape(m, k)
    res["Q"] = take(np.float32, n * k).reshape(n, k)
    return res


def ref_rmse(test_path: str, model_path: str) -> float:
    res = subprocess.run([os.path.join(REF_DIR, "ref_rmse"), test_path, model_path], check=True,
                         capture_output=True, text=True)
    for line in res.stdout.splitlines():
        if line.startswith("RMSE_FULL"):
            return float(line.split()[1])
    raise RuntimeError("ref_rmse printed no RMSE")


def train_f64(records: np.ndarray, m: int, n: int, k: int = 128, num_workers: int = 1, num_iters: int = 20,
              lambda_p: float = 0.05, lambda_q: float = 0.05, alpha: float = 0.08, beta: float = 0.3,
              lrate: float = 0.0, seed: int = 0, order: int = OR_ORDER_ROUND_ROBIN, threads: int = 1):
    """FP64 sgd_train (mode A): the same statistics, id maps, sample schedule and
    learning-rate table as the GPU path, everything else in double; serial when threads == 1,
    else the workers' batches are dealt to `threads` host threads.  Returns (P, Q, b) with
    float64 factors (unscaled, un-permuted)."""
    rec = np.ascontiguousarray(records).copy()
    ave, std = collect_data(rec)
    scale = max(1e-4, float(np.float32(std)))
    pm, qm = gen_random_map(seed, m), gen_random_map(seed, n)
    rec["u"], rec["v"] = pm[rec["u"]], qm[rec["v"]]
    P = np.zeros((m, k), dtype=np.float64)
    Q = np.zeros((n, k), dtype=np.float64)
    lib().or_init_factors_f64(_ptr(P), m, k, seed, 1)
    lib().or_init_factors_f64(_ptr(Q), n, k, seed, 2)
    lr = np.array([alpha / (1 + beta * i ** 1.5) + lrate for i in range(num_iters + 4)], dtype=np.float64)
    a = _Sgd64Args(R=_ptr(rec), nnz=len(rec), P=_ptr(P), m=m, Q=_ptr(Q), n=n, k=k, num_workers=num_workers,
                   order=order, lr=_ptr(lr), first_epoch=0, n_epochs=num_iters, lambda_p=lambda_p / scale,
                   lambda_q=lambda_q / scale, rscale=1.0 / scale, seed=seed)
    if threads > 1:
        lib().or_sgd_epochs_f64_threads(C.byref(a), threads)
    else:
        lib().or_sgd_epochs_f64(C.byref(a))
    f = np.sqrt(scale)
    return P[pm] * f, Q[qm] * f, float(ave) / float(std)


def calc_rmse_f64(records: np.ndarray, P: np.ndarray, Q: np.ndarray, b: float) -> float:
    rec = np.ascontiguousarray(records)
    P = np.ascontiguousarray(P, dtype=np.float64)
    Q = np.ascontiguousarray(Q, dtype=np.float64)
    return lib().or_calc_rmse_f64(_ptr(rec), len(rec), _ptr(P), P.shape[0], _ptr(Q), Q.shape[0], P.shape[1], b)


def parse_text(text: bytes, header_lines: int = 3):
    """Records of a rating text (transform.cpp:31-42, strict form), or ("bad", offset) /
    ("partial", None) when the text is rejected."""
    L = lib()
    bad = C.c_int64(-1)
    n = L.or_parse_text(text, len(text), header_lines, None, 0, C.byref(bad))
    if n == -1:
        return ("bad", bad.value)
    if n == -2:
        return ("partial", None)
    out = np.zeros(n, dtype=NODE)
    L.or_parse_text(text, len(text), header_lines, _ptr(out) if n else None, n, C.byref(bad))
    return out


def ref_transform(text: bytes, tmpdir: str) -> bytes:
    """Output of the reference's own transform (oracle/_ref/transform) for a text."""
    exe = os.path.join(REF_DIR, "transform")
    path = os.path.join(tmpdir, "ratings")
    with open(path, "wb") as f:
        f.write(text)
    subprocess.run([exe, path], check=True, capture_output=True)
    with open(path + ".bin", "rb") as f:
        return f.read()


def evaluate(records: np.ndarray, P: np.ndarray, Q: np.ndarray, b: float, criterion: int,
             prob_m: int = 0, prob_n: int = 0) -> float:
    """mf-predict criterion (test/mf.cpp:3794-4044) of a float model on test records;
    prob_m / prob_n default to the records' extent (as read_problem sets them)."""
    rec = np.ascontiguousarray(records)
    P = np.ascontiguousarray(P, dtype=np.float32)
    Q = np.ascontiguousarray(Q, dtype=np.float32)
    if len(rec):
        prob_m = prob_m or int(rec["u"].max()) + 1
        prob_n = prob_n or int(rec["v"].max()) + 1
    return lib().or_evaluate(_ptr(rec) if len(rec) else None, len(rec), prob_m, prob_n, _ptr(P), P.shape[0],
                             _ptr(Q), Q.shape[0], P.shape[1], b, criterion)


def ref_criteria(test_path: str, model_path: str) -> dict:
    """Every criterion computed by the reference's own test/mf.cpp functions (full precision)."""
    res = subprocess.run([os.path.join(REF_DIR, "ref_rmse"), test_path, model_path, "all"], check=True,
                         capture_output=True, text=True)
    out = {}
    for line in res.stdout.splitlines():
        if line.startswith("RMSE_FULL"):
            out[0] = float(line.split()[1])
        elif line.startswith("CRIT"):
            _, c, v = line.split()
            out[int(c)] = float(v)
    return out


def strata_epochs(records: np.ndarray, P: np.ndarray, Q: np.ndarray, precision: str, groups: int, lr: np.ndarray,
                  first_epoch: int, n_epochs: int, lambda_p: float, lambda_q: float, seed: int, lanes: int) -> int:
    """The deterministic stratified schedule on float32 P, Q in place; returns skipped records."""
    kind, sr = KIND[precision]
    rec = np.ascontiguousarray(records)
    lr = np.ascontiguousarray(lr, dtype=np.float32)
    return lib().or_strata_epochs(_ptr(rec), len(rec), _ptr(P), P.shape[0], _ptr(Q), Q.shape[0], P.shape[1], kind, sr,
                                  lanes, groups, _ptr(lr), first_epoch, n_epochs, lambda_p, lambda_q, seed)
