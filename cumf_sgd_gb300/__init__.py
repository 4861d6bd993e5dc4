"""cumf_sgd_gb300 - GB300-native batch-Hogwild SGD matrix factorization.

Python mirror of cuMF_SGD's host interface over the C ABI in include/cumf_sgd.h:

  Parameter            singleGPU/sgd.h:26-46 (same defaults)
  parse_argument       singleGPU/main.cpp:33-227
  read_problem         singleGPU/sgd.cu:190-335
  sgd_train            singleGPU/sgd.cu:638-690
  save_model           singleGPU/main.cpp:231-273
  mf_load_model        test/mf.cpp:3706-3777
  calc_rmse            test/mf.cpp:3815-3839
  sgd_update           singleGPU/sgd_kernel.cu:125 (device-resident epochs)

All compute runs in libcumf_sgd.so; a missing library raises ImportError at first use.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
from typing import Optional, Sequence

import numpy as np

from . import _lib
from ._lib import CumfError, PRECISIONS, FP16, BF16, FP32, BF16_SR, FP16_SR  # noqa: F401

NODE_DTYPE = np.dtype([("u", "<i4"), ("v", "<i4"), ("r", "<f4")])


@dataclasses.dataclass
class Parameter:
    """Parameter (singleGPU/sgd.h:26-46) with the same defaults, plus seed/precision/lanes."""
    k: int = 80
    num_workers: int = 12
    u_grid: int = 1
    v_grid: int = 1
    x_grid: int = 1
    y_grid: int = 1
    num_iters: int = 30
    gpu: int = 3
    lambda_p: float = 0.05
    lambda_q: float = 0.05
    lrate: float = 0.0
    alpha: float = 0.01
    beta: float = 0.01
    seed: int = 0
    precision: str = "fp16"
    lanes: int = 0
    quiet: bool = True
    epochs_per_launch: int = 0
    verbose_epochs: bool = False
    prefetch: int = -1
    l2_hints: int = -1
    ring: int = -1
    tail_epochs: int = 0
    tail_start: int = 0
    deterministic: int = 0
    hot_rows: Optional[float] = None  # expected workers per copy of a most-rated row; None = library default

    @property
    def ux(self) -> int:
        return self.u_grid * (1 if self.u_grid * self.v_grid == 1 else self.x_grid)

    @property
    def vy(self) -> int:
        return self.v_grid * (1 if self.u_grid * self.v_grid == 1 else self.y_grid)

    def to_c(self) -> _lib.Params:
        p = _lib.Params()
        _lib.check(_lib.load().cumf_default_params(C.byref(p)))
        for f in ("k", "num_workers", "u_grid", "v_grid", "x_grid", "y_grid", "num_iters", "gpu",
                  "lambda_p", "lambda_q", "lrate", "alpha", "beta", "seed", "lanes",
                  "epochs_per_launch", "prefetch", "l2_hints", "ring", "tail_epochs", "tail_start",
                  "deterministic"):
            setattr(p, f, getattr(self, f))
        p.precision = PRECISIONS[self.precision] if isinstance(self.precision, str) else int(self.precision)
        p.quiet = int(bool(self.quiet))
        p.verbose_epochs = int(bool(self.verbose_epochs))
        p.ux, p.vy = self.ux, self.vy
        if self.hot_rows is not None:
            p.hot_rows = float(self.hot_rows)
        return p

    @staticmethod
    def from_c(p: _lib.Params) -> "Parameter":
        inv = {v: k for k, v in PRECISIONS.items()}
        return Parameter(k=p.k, num_workers=p.num_workers, u_grid=p.u_grid, v_grid=p.v_grid,
                         x_grid=p.x_grid, y_grid=p.y_grid, num_iters=p.num_iters, gpu=p.gpu,
                         lambda_p=p.lambda_p, lambda_q=p.lambda_q, lrate=p.lrate, alpha=p.alpha,
                         beta=p.beta, seed=p.seed, precision=inv[p.precision], lanes=p.lanes,
                         quiet=bool(p.quiet), deterministic=p.deterministic, hot_rows=p.hot_rows)


@dataclasses.dataclass
class Argument:
    """Argument (singleGPU/sgd.h:48-77)."""
    param: Parameter
    tr_path: str
    va_path: str
    model_path: str


def parse_argument(argv: Sequence[str]) -> Argument:
    """parse_argument (singleGPU/main.cpp:33-227); argv[0] is the program name."""
    lib = _lib.load()
    arr = (C.c_char_p * len(argv))(*[a.encode() for a in argv])
    out = _lib.Args()
    rc = lib.cumf_parse_args(len(argv), arr, C.byref(out))
    if rc != 0:
        raise ValueError(lib.cumf_last_error().decode())
    return Argument(Parameter.from_c(out.param), out.tr_path.decode(), out.va_path.decode(),
                    out.model_path.decode())


class MFProblem:
    """mf_problem (singleGPU/sgd.h:85-108): m, n, nnz and the 12-byte records R."""

    def __init__(self, c: _lib.Problem):
        self._c = c

    @staticmethod
    def from_arrays(u, v, r, m: Optional[int] = None, n: Optional[int] = None,
                    pinned: bool = False) -> "MFProblem":
        u = np.asarray(u, dtype=np.int32)
        v = np.asarray(v, dtype=np.int32)
        r = np.asarray(r, dtype=np.float32)
        nnz = len(u)
        c = _lib.Problem()
        _lib.check(_lib.load().cumf_alloc_problem(nnz, int(pinned), C.byref(c)))
        prob = MFProblem(c)
        rec = prob.records
        rec["u"], rec["v"], rec["r"] = u, v, r
        c.m = int(m) if m is not None else (int(u.max()) + 1 if nnz else 1)
        c.n = int(n) if n is not None else (int(v.max()) + 1 if nnz else 1)
        c.m, c.n = max(c.m, 1), max(c.n, 1)
        return prob

    @property
    def m(self) -> int:
        return self._c.m

    @property
    def n(self) -> int:
        return self._c.n

    @property
    def nnz(self) -> int:
        return self._c.nnz

    @property
    def records(self) -> np.ndarray:
        """Zero-copy structured view (u, v, r) of the records; the view keeps this problem alive."""
        if self._c.nnz == 0:
            return np.zeros(0, dtype=NODE_DTYPE)
        buf = (C.c_char * (12 * self._c.nnz)).from_address(C.addressof(self._c.R.contents))
        buf._owner = self
        return np.frombuffer(buf, dtype=NODE_DTYPE)

    def write(self, path: str) -> None:
        _lib.check(_lib.load().cumf_write_problem(path.encode(), C.byref(self._c)))

    def __del__(self):
        try:
            if self._c.R:
                _lib.load().cumf_free_problem(C.byref(self._c))
        except Exception:
            pass


def read_problem(path: str, pinned: bool = True) -> MFProblem:
    """read_problem (singleGPU/sgd.cu:190-335)."""
    c = _lib.Problem()
    _lib.check(_lib.load().cumf_read_problem(path.encode(), int(pinned), C.byref(c)))
    return MFProblem(c)


def convert_text(in_path: str, out_path: Optional[str] = None, header_lines: int = 3) -> int:
    """`./transform file_name` (data/netflix/transform.cpp:9-47) parsed on the GPU; returns
    the number of 12-byte records written (to in_path + ".bin" by default)."""
    n = C.c_int64(0)
    _lib.check(_lib.load().cumf_convert_text(in_path.encode(), out_path.encode() if out_path else None,
                                             header_lines, C.byref(n)))
    return n.value


def read_text_problem(path: str, header_lines: int = 3, pinned: bool = True) -> MFProblem:
    """Rating text parsed on the GPU into a problem (what read_problem returns for the
    converted file)."""
    c = _lib.Problem()
    _lib.check(_lib.load().cumf_read_text_problem(path.encode(), header_lines, int(pinned), C.byref(c)))
    return MFProblem(c)


def parse_text_host(text, header_lines: int = 3) -> np.ndarray:
    """Rating text (bytes) -> records with the copies and the parse overlapped in chunks."""
    buf = np.frombuffer(text, dtype=np.uint8) if isinstance(text, (bytes, bytearray)) else text
    n = C.c_int64(0)
    L = _lib.load()
    _lib.check(L.cumf_parse_text_host(buf.ctypes.data, len(buf), header_lines, None, 0, C.byref(n)))
    out = np.zeros(n.value, dtype=NODE_DTYPE)
    _lib.check(L.cumf_parse_text_host(buf.ctypes.data, len(buf), header_lines, out.ctypes.data if n.value else None,
                                      n.value, C.byref(n)))
    return out


def text_data_start(text: bytes, header_lines: int = 3) -> int:
    """Offset of the first data byte after the header lines (transform.cpp:31-33)."""
    out = C.c_int64(0)
    _lib.check(_lib.load().cumf_text_data_start(text, len(text), header_lines, C.byref(out)))
    return out.value


def dev_parse_text(d_text: int, length: int, start: int, d_out: int = 0, cap: int = 0, stream: int = 0) -> int:
    """Device text bytes [start, length) -> records at d_out; returns the record count
    (d_out = 0: count only)."""
    n = C.c_int64(0)
    _lib.check(_lib.load().cumf_dev_parse_text(d_text, length, start, d_out or None, cap, C.byref(n),
                                               stream or None))
    return n.value


class MFModel:
    """mf_model as written to the model file: fp32 P (m x k), Q (n x k) and b."""

    def __init__(self, c: _lib.Model):
        self._c = c

    @staticmethod
    def from_arrays(P: np.ndarray, Q: np.ndarray, b: float) -> "MFModel":
        P = np.ascontiguousarray(P, dtype=np.float32)
        Q = np.ascontiguousarray(Q, dtype=np.float32)
        c = _lib.Model()
        _lib.check(_lib.load().cumf_alloc_model(P.shape[0], Q.shape[0], P.shape[1], C.byref(c)))
        mod = MFModel(c)
        mod.P[...] = P
        mod.Q[...] = Q
        c.b = b
        return mod

    def _view(self, ptr, rows: int) -> np.ndarray:
        """Zero-copy view of a factor matrix; the view keeps this model (and its buffers) alive."""
        if rows * self._c.k == 0:
            return np.zeros((rows, self._c.k), dtype=np.float32)
        buf = (C.c_char * (4 * rows * self._c.k)).from_address(C.addressof(ptr.contents))
        buf._owner = self
        return np.frombuffer(buf, dtype=np.float32).reshape(rows, self._c.k)

    @property
    def P(self) -> np.ndarray:
        return self._view(self._c.P, self._c.m)

    @property
    def Q(self) -> np.ndarray:
        return self._view(self._c.Q, self._c.n)

    @property
    def m(self) -> int:
        return self._c.m

    @property
    def n(self) -> int:
        return self._c.n

    @property
    def k(self) -> int:
        return self._c.k

    @property
    def b(self) -> float:
        return self._c.b

    def __del__(self):
        try:
            if self._c.P or self._c.Q:
                _lib.load().cumf_free_model(C.byref(self._c))
        except Exception:
            pass


@dataclasses.dataclass
class TrainStats:
    prep_ms: float
    train_ms: float
    export_ms: float
    total_ms: float
    updates_per_sec: float
    samples_per_epoch: int
    mean: float
    std_dev: float
    mode: int
    num_workers: int
    lanes: int
    hot_users: int = 0
    hot_items: int = 0
    extra_rows: int = 0


def sgd_train(tr: MFProblem, va: Optional[MFProblem], param: Parameter,
              with_stats: bool = False):
    """sgd_train (singleGPU/sgd.cu:638-690); `tr` is not modified."""
    out = _lib.Model()
    st = _lib.TrainStats()
    p = param.to_c()
    rc = _lib.load().cumf_train(C.byref(tr._c), C.byref(va._c) if va is not None else None,
                                C.byref(p), C.byref(out), C.byref(st))
    _lib.check(rc)
    model = MFModel(out)
    if with_stats:
        stats = TrainStats(**{f: getattr(st, f) for f, _ in _lib.TrainStats._fields_ if f != "reserved_"})
        return model, stats
    return model


def release_host_cache() -> None:
    """Gives the cached page-locked host buffers back to the system (cumf_release_host_cache)."""
    _lib.check(_lib.load().cumf_release_host_cache())


def save_model(model: MFModel, path: str) -> None:
    """save_model (singleGPU/main.cpp:231-273)."""
    _lib.check(_lib.load().cumf_save_model(C.byref(model._c), path.encode()))


def mf_load_model(path: str) -> MFModel:
    """mf_load_model (test/mf.cpp:3706-3777)."""
    c = _lib.Model()
    _lib.check(_lib.load().cumf_load_model(path.encode(), C.byref(c)))
    return MFModel(c)


load_model = mf_load_model


def calc_rmse(prob: MFProblem, model: MFModel) -> float:
    """calc_rmse (test/mf.cpp:3815-3839), evaluated on the GPU."""
    out = C.c_double()
    _lib.check(_lib.load().cumf_rmse(C.byref(prob._c), C.byref(model._c), C.byref(out)))
    return out.value


EVAL_CRITERIA = {"rmse": 0, "mae": 1, "gkl": 2, "logloss": 5, "accuracy": 6, "row_mpr": 10, "col_mpr": 11,
                 "row_auc": 12, "col_auc": 13}


def evaluate(prob: MFProblem, model: MFModel, criterion) -> float:
    """mf-predict -e <criterion> (test/mf.cpp:3841-4044) on the GPU; criterion is LIBMF's
    number or a name of EVAL_CRITERIA."""
    c = EVAL_CRITERIA[criterion] if isinstance(criterion, str) else int(criterion)
    out = C.c_double()
    _lib.check(_lib.load().cumf_evaluate(C.byref(prob._c), C.byref(model._c), c, C.byref(out)))
    return out.value


def lr_schedule(alpha: float, beta: float, lrate: float, n: int) -> np.ndarray:
    """Learning-rate table of singleGPU/sgd_kernel.cu:144-149."""
    out = np.zeros(n, dtype=np.float32)
    _lib.check(_lib.load().cumf_lr_schedule(alpha, beta, lrate, n,
                                            out.ctypes.data_as(C.POINTER(C.c_float))))
    return out


def batches_per_worker(nnz: int, num_workers: int) -> int:
    return int(_lib.load().cumf_batches_per_worker(nnz, num_workers))


def random_map(seed: int, size: int) -> np.ndarray:
    """gen_random_map (singleGPU/sgd.cu:39-53) for a given srand seed."""
    out = np.zeros(size, dtype=np.int32)
    _lib.check(_lib.load().cumf_random_map(seed & 0xffffffff, size,
                                           out.ctypes.data_as(C.POINTER(C.c_int32))))
    return out


def grid_problem(records: np.ndarray, m: int, n: int, ux: int, vy: int):
    """grid_problem (singleGPU/sgd.cu:411-487) in place on a structured record array;
    returns (grid_size, u_seg, v_seg)."""
    assert records.dtype == NODE_DTYPE and records.flags.c_contiguous
    gs = np.zeros(ux * vy, dtype=np.int64)
    us, vs = C.c_int64(), C.c_int64()
    _lib.check(_lib.load().cumf_grid_problem(
        records.ctypes.data_as(C.POINTER(_lib.Node)), len(records), m, n, ux, vy,
        gs.ctypes.data_as(C.POINTER(C.c_int64)), C.byref(us), C.byref(vs)))
    return gs, us.value, vs.value


def device_info(gpu: int = 0):
    sm, ma, mi = C.c_int(), C.c_int(), C.c_int()
    _lib.check(_lib.load().cumf_device_info(gpu, C.byref(sm), C.byref(ma), C.byref(mi)))
    return sm.value, ma.value, mi.value


def default_workers(sm_count: int, k: int, precision: str = "fp16", lanes: int = 0) -> int:
    """Resident workers (one wave) of the update kernel."""
    return int(_lib.load().cumf_default_workers(sm_count, k, PRECISIONS[precision], lanes))


def auto_workers(nnz: int, sm_count: int, k: int, precision: str = "fp16", lanes: int = 0) -> int:
    """Worker count the library picks for nnz ratings (three waves, >= 8 batches each)."""
    return int(_lib.load().cumf_auto_workers(nnz, sm_count, k, PRECISIONS[precision], lanes))


# ---- device-level entry points (integer device addresses, e.g. torch.Tensor.data_ptr()) ----

def sgd_update(d_R: int, nnz: int, d_P: int, m: int, d_Q: int, n: int, k: int, precision: str,
               num_workers: int, lanes: int, d_lr: int, first_epoch: int, n_epochs: int,
               lambda_p: float, lambda_q: float, seed: int, d_status: int = 0,
               stream: int = 0, prefetch: int = -1, l2_hints: int = -1, ring: int = -1,
               freeze_q: int = 0, rows_copied: int = 0) -> None:
    """Batch-Hogwild epochs on caller-owned device buffers (sgd_kernel.cu:212-248)."""
    t = _lib.Tuning(lanes=lanes, prefetch=prefetch, l2_hints=l2_hints, ring=ring, freeze_q=freeze_q,
                    rows_copied=rows_copied)
    _lib.check(_lib.load().cumf_sgd_update_tuned(d_R, nnz, d_P, m, d_Q, n, k, PRECISIONS[precision],
                                                 num_workers, C.byref(t), d_lr, first_epoch, n_epochs,
                                                 lambda_p, lambda_q, seed, d_status or None,
                                                 stream or None))


def dev_init_factors(d: int, rows: int, k: int, precision: str, seed: int, tag: int,
                     stream: int = 0) -> None:
    _lib.check(_lib.load().cumf_dev_init_factors(d, rows, k, PRECISIONS[precision], seed, tag,
                                                 stream or None))


def dev_export_factors(d_in: int, precision: str, d_map: int, rows: int, k: int, factor: float,
                       d_out: int, stream: int = 0) -> None:
    _lib.check(_lib.load().cumf_dev_export_factors(d_in, PRECISIONS[precision], d_map or None,
                                                   rows, k, factor, d_out, stream or None))


def dev_shuffle_scale(d_in: int, d_out: int, nnz: int, d_pmap: int, m: int, d_qmap: int, n: int,
                      scale: float, d_status: int = 0, stream: int = 0) -> None:
    _lib.check(_lib.load().cumf_dev_shuffle_scale(d_in, d_out, nnz, d_pmap or None, m,
                                                  d_qmap or None, n, scale, d_status or None,
                                                  stream or None))


def dev_rating_stats(d_R: int, nnz: int, stream: int = 0):
    mean, std = C.c_double(), C.c_double()
    _lib.check(_lib.load().cumf_dev_rating_stats(d_R, nnz, C.byref(mean), C.byref(std),
                                                 stream or None))
    return mean.value, std.value


class HotRows:
    """Copies of the most-rated rows (cumf_hot_rows_*): plan, assign, spread, merge."""

    def __init__(self, d_R: int, nnz: int, m: int, n: int, per_copy: int, max_copies: int = 256,
                 stream: int = 0):
        self._lib = _lib.load()
        self._h = C.c_void_p()
        _lib.check(self._lib.cumf_hot_rows_plan(d_R, nnz, m, n, per_copy, max_copies, C.byref(self._h),
                                                stream or None))
        mr, nr, hm, hn = (C.c_int32() for _ in range(4))
        _lib.check(self._lib.cumf_hot_rows_info(self._h, C.byref(mr), C.byref(nr), C.byref(hm), C.byref(hn)))
        self.m, self.n = m, n
        self.m_rows, self.n_rows, self.hot_users, self.hot_items = mr.value, nr.value, hm.value, hn.value

    @staticmethod
    def per_copy(nnz: int, num_workers: int, k: int, precision: str, lanes: int, concurrency: float) -> int:
        return int(_lib.load().cumf_hot_rows_per_copy(nnz, num_workers, k, PRECISIONS[precision], lanes,
                                                      concurrency))

    def tables(self):
        """Host copies: (tab_m (m x 2), tab_n (n x 2), grp_m, grp_n); tab rows are {copies, first extra row}."""
        tm = np.zeros((self.m, 2), np.int32)
        tn = np.zeros((self.n, 2), np.int32)
        gm = np.zeros(max(1, self.hot_users), np.int32)
        gn = np.zeros(max(1, self.hot_items), np.int32)
        p = lambda a: a.ctypes.data_as(C.c_void_p)
        _lib.check(self._lib.cumf_hot_rows_tables(self._h, p(tm), p(tn), p(gm), p(gn)))
        return tm, tn, gm[:self.hot_users], gn[:self.hot_items]

    def assign(self, d_R: int, nnz: int, stream: int = 0) -> None:
        _lib.check(self._lib.cumf_hot_rows_assign(self._h, d_R, nnz, stream or None))

    def spread(self, d_P: int, d_Q: int, k: int, precision: str, stream: int = 0) -> None:
        _lib.check(self._lib.cumf_hot_rows_spread(self._h, d_P or None, d_Q or None, k, PRECISIONS[precision],
                                                  stream or None))

    def merge(self, d_P: int, d_Q: int, k: int, precision: str, stream: int = 0) -> None:
        _lib.check(self._lib.cumf_hot_rows_merge(self._h, d_P or None, d_Q or None, k, PRECISIONS[precision],
                                                 stream or None))

    def close(self) -> None:
        if self._h:
            self._lib.cumf_hot_rows_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def dev_rmse(d_R: int, nnz: int, d_P: int, m: int, d_Q: int, n: int, k: int, b: float,
             stream: int = 0) -> float:
    out = C.c_double()
    _lib.check(_lib.load().cumf_dev_rmse(d_R, nnz, d_P, m, d_Q, n, k, b, C.byref(out),
                                         stream or None))
    return out.value


# ---- learned warm start -----------------------------------------------------------------

class MLP:
    """The warm-start encoder: d_in -> hidden -> hidden -> d_out (GELU), bf16 on the tensor
    cores with fp32 master weights (cumf_mlp_* in the C ABI).  Device arrays are passed as
    integer addresses (e.g. torch.Tensor.data_ptr())."""

    def __init__(self, d_in: int, hidden: int = 512, d_out: int = 128, seed: int = 0):
        h = C.c_void_p()
        _lib.check(_lib.load().cumf_mlp_create(d_in, hidden, d_out, seed, C.byref(h)))
        self._h = h
        self.d_in, self.hidden, self.d_out = d_in, hidden, d_out

    def param_count(self) -> int:
        return int(_lib.load().cumf_mlp_param_count(self._h))

    def get(self, which: int = 0) -> np.ndarray:
        out = np.zeros(self.param_count(), dtype=np.float32)
        _lib.check(_lib.load().cumf_mlp_get_params(self._h, out.ctypes.data, len(out), which))
        return out

    def set(self, params: np.ndarray) -> None:
        params = np.ascontiguousarray(params, dtype=np.float32)
        _lib.check(_lib.load().cumf_mlp_set_params(self._h, params.ctypes.data, len(params)))

    def forward(self, d_X: int, rows: int, d_Y: int, stream: int = 0) -> None:
        _lib.check(_lib.load().cumf_mlp_forward(self._h, d_X, rows, d_Y, stream or None))

    def loss_grad(self, d_X: int, d_T: int, rows: int, stream: int = 0) -> float:
        loss = C.c_double()
        _lib.check(_lib.load().cumf_mlp_loss_grad(self._h, d_X, d_T, rows, C.byref(loss), stream or None))
        return loss.value

    def train(self, d_X: int, d_T: int, rows: int, epochs: int, batch: int = 1024, lr: float = 1e-3,
              seed: int = 0, stream: int = 0) -> float:
        loss = C.c_double()
        _lib.check(_lib.load().cumf_mlp_train(self._h, d_X, d_T, rows, epochs, batch, lr, seed, C.byref(loss),
                                              stream or None))
        return loss.value

    def __del__(self):
        try:
            if self._h:
                _lib.load().cumf_mlp_destroy(self._h)
                self._h = None
        except Exception:
            pass


def user_features(d_R: int, nnz: int, d_Q: int, n: int, k: int, m: int, d_X: int, stream: int = 0) -> None:
    """Warm-start features of m users (m x (k+3), fp32) from device ratings and fp32 Q."""
    _lib.check(_lib.load().cumf_user_features(d_R, nnz, d_Q, n, k, m, d_X, stream or None))


class DeviceModel:
    """A starting model whose fp32 factors live in device memory (not owned): P (m x k) and
    Q (n x k) given as device addresses, for sgd_train_ex."""

    def __init__(self, d_P: int, m: int, d_Q: int, n: int, k: int, b: float = 0.0):
        self._c = _lib.Model(fun=0, m=m, n=n, k=k, b=b, pinned=2, P=C.cast(C.c_void_p(d_P), C.POINTER(C.c_float)),
                             Q=C.cast(C.c_void_p(d_Q), C.POINTER(C.c_float)))


def sgd_train_ex(tr: MFProblem, te: Optional[MFProblem], param: Parameter, init=None):
    """sgd_train with optional starting factors and per-epoch test RMSE; returns
    (model, stats, epoch_rmse, epoch_cumulative_train_ms)."""
    out = _lib.Model()
    st = _lib.TrainStats()
    p = param.to_c()
    rm = np.full(max(1, param.num_iters), np.nan)
    ms = np.full(max(1, param.num_iters), np.nan)
    rc = _lib.load().cumf_train_ex(C.byref(tr._c), C.byref(te._c) if te is not None else None, C.byref(p),
                                   C.byref(init._c) if init is not None else None, C.byref(out), C.byref(st),
                                   rm.ctypes.data, ms.ctypes.data)
    _lib.check(rc)
    stats = TrainStats(**{f: getattr(st, f) for f, _ in _lib.TrainStats._fields_ if f != "reserved_"})
    return MFModel(out), stats, rm[:param.num_iters], ms[:param.num_iters]


def sgd_train_ckpt(tr: MFProblem, te: Optional[MFProblem], param: Parameter, path: str, every: int = 1,
                   resume: bool = True, stop_after: int = 0):
    """sgd_train with checkpoints of the in-HBM factors every `every` epochs to `path`;
    resume=True continues from a matching checkpoint; stop_after > 0 ends the call once that
    many epochs are complete.  Returns (model, stats, epochs_done)."""
    out = _lib.Model()
    st = _lib.TrainStats()
    p = param.to_c()
    ck = _lib.Checkpoint(path=path.encode(), every=every, resume=int(resume), stop_after=stop_after)
    done = C.c_int32(0)
    rc = _lib.load().cumf_train_ckpt(C.byref(tr._c), C.byref(te._c) if te is not None else None, C.byref(p),
                                     C.byref(ck), C.byref(out), C.byref(st), C.byref(done))
    _lib.check(rc)
    stats = TrainStats(**{f: getattr(st, f) for f, _ in _lib.TrainStats._fields_ if f != "reserved_"})
    return MFModel(out), stats, done.value


def dev_strata_layout(d_R: int, nnz: int, groups: int, d_out: int, d_block_off: int, stream: int = 0) -> None:
    """Ratings stably sorted into the groups x groups blocks of the deterministic schedule."""
    _lib.check(_lib.load().cumf_dev_strata_layout(d_R, nnz, groups, d_out, d_block_off, stream or None))


def dev_strata_epochs(d_S: int, d_block_off: int, groups: int, d_P: int, m: int, d_Q: int, n: int, k: int,
                      precision: str, lr: np.ndarray, first_epoch: int, n_epochs: int, lambda_p: float,
                      lambda_q: float, seed: int, d_status: int = 0, stream: int = 0) -> None:
    """Epochs of the deterministic stratified schedule on caller-owned device buffers."""
    lr = np.ascontiguousarray(lr, dtype=np.float32)
    _lib.check(_lib.load().cumf_dev_strata_epochs(d_S, d_block_off, groups, d_P, m, d_Q, n, k, PRECISIONS[precision],
                                                  lr.ctypes.data, first_epoch, n_epochs, lambda_p, lambda_q, seed,
                                                  d_status or None, stream or None))


# ---- batched factorizations ------------------------------------------------------------

class Batch:
    """Many independent factorizations in one persistent launch (cumf_batch_* in the C ABI).
    Each problem is a dict with device addresses d_R, d_P, d_Q, d_lr and m, n, nnz, k,
    lambda_p, lambda_q, seed, lr_len and optionally num_workers and hot (a HotRows plan whose
    assign and spread were applied; the batch merges its copies after every epoch)."""

    def __init__(self, problems):
        arr = (_lib.BatchProblem * len(problems))()
        self._plans = [p.get("hot") for p in problems]  # the plans must outlive the batch
        for i, p in enumerate(problems):
            hot = p.get("hot")
            arr[i] = _lib.BatchProblem(d_R=p["d_R"], nnz=p["nnz"], d_P=p["d_P"], m=p["m"], n=p["n"], d_Q=p["d_Q"],
                                       k=p["k"], num_workers=p.get("num_workers", 0), lambda_p=p["lambda_p"],
                                       lambda_q=p["lambda_q"], seed=p["seed"], d_lr=p["d_lr"], lr_len=p["lr_len"],
                                       hot=hot._h.value if hot is not None else None)
        h = C.c_void_p()
        _lib.check(_lib.load().cumf_batch_create(arr, len(problems), C.byref(h)))
        self._h = h

    def set_tuning(self, batches_target: int, order: int, blocks_per_sm: int, lanes: int = 16) -> None:
        t = _lib.BatchTuning(batches_target=batches_target, order=order, blocks_per_sm=blocks_per_sm, lanes=lanes)
        _lib.check(_lib.load().cumf_batch_set_tuning(self._h, C.byref(t)))

    def info(self):
        t = _lib.BatchTuning()
        tasks, samples = C.c_int(), C.c_int64()
        _lib.check(_lib.load().cumf_batch_get_info(self._h, C.byref(t), C.byref(tasks), C.byref(samples)))
        return dict(batches_target=t.batches_target, order=t.order, blocks_per_sm=t.blocks_per_sm,
                    lanes=t.lanes, tasks_per_epoch=tasks.value, samples_per_epoch=samples.value)

    def autotune(self, stream: int = 0):
        t = _lib.BatchTuning()
        ms = C.c_double()
        _lib.check(_lib.load().cumf_batch_autotune(self._h, stream or None, C.byref(t), C.byref(ms)))
        return dict(batches_target=t.batches_target, order=t.order, blocks_per_sm=t.blocks_per_sm,
                    lanes=t.lanes, epoch_ms=ms.value)

    def run(self, first_epoch: int, n_epochs: int, use_graph: bool = True, stream: int = 0) -> None:
        _lib.check(_lib.load().cumf_batch_run(self._h, first_epoch, n_epochs, int(use_graph), stream or None))

    def status(self) -> int:
        st = C.c_int()
        _lib.check(_lib.load().cumf_batch_status(self._h, C.byref(st)))
        return st.value

    def __del__(self):
        try:
            if self._h:
                _lib.load().cumf_batch_destroy(self._h)
                self._h = None
        except Exception:
            pass
