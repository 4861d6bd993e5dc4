"""CPU restatement of the copies of the most-rated rows (cumf_sgd_gb300/csrc/hot_rows.cu).

TEST INFRASTRUCTURE ONLY: imported by tests/, never by the cumf_sgd_gb300 package.

The reference has no such step: its update kernel (singleGPU/sgd_k128_kernel_hogwild_warp32.h
:3-104) reads and writes one user row and one item row per rating.  This module restates the
library's own plan (counts -> copies -> layout of the extra rows), the assignment of ratings
to copies (rating i -> copy i mod copies) and the merge (fp32 mean of the copies summed in copy
order, divided by the copy count, rounded to nearest in the storage type), so that the GPU
tables and merges can be checked bit for bit.
"""
from __future__ import annotations

import numpy as np

from oracle.mlp_oracle import bf16


def copies_of(count: np.ndarray, per_copy: int, max_copies: int) -> np.ndarray:
    count = np.asarray(count, np.int64)
    c = (count + per_copy - 1) // per_copy
    return np.where(count <= per_copy, 1, np.minimum(c, max_copies)).astype(np.int64)


def plan_side(ids: np.ndarray, rows: int, per_copy: int, max_copies: int):
    """(table rows x 2 int32 {copies, first extra row or the row itself}, rows with copies,
    rows including the copies) for one factor matrix."""
    ids = np.asarray(ids, np.int64)
    cnt = np.bincount(ids[(ids >= 0) & (ids < rows)], minlength=rows)
    copies = copies_of(cnt, per_copy, max_copies)
    extra = copies - 1
    first = rows + np.cumsum(extra) - extra
    tab = np.stack([copies, np.where(copies > 1, first, np.arange(rows))], 1).astype(np.int32)
    return tab, np.nonzero(copies > 1)[0].astype(np.int32), rows + int(extra.sum())


def plan(records: np.ndarray, m: int, n: int, per_copy: int, max_copies: int = 256):
    tm, gm, m_rows = plan_side(records["u"], m, per_copy, max_copies)
    tn, gn, n_rows = plan_side(records["v"], n, per_copy, max_copies)
    return {"tab_m": tm, "tab_n": tn, "grp_m": gm, "grp_n": gn, "m_rows": m_rows, "n_rows": n_rows}


def assign(records: np.ndarray, p: dict) -> np.ndarray:
    """The ratings with each id of a row with copies replaced by its copy's row."""
    out = records.copy()
    i = np.arange(len(records), dtype=np.int64)
    for field, tab, rows in (("u", p["tab_m"], len(p["tab_m"])), ("v", p["tab_n"], len(p["tab_n"]))):
        ids = out[field].astype(np.int64)
        ok = (ids >= 0) & (ids < rows)
        c = np.ones_like(ids)
        first = ids.copy()
        c[ok] = tab[ids[ok], 0]
        first[ok] = tab[ids[ok], 1]
        r = i % c
        out[field] = np.where(ok & (c > 1) & (r > 0), first + r - 1, ids).astype(np.int32)
    return out


def _round(x: np.ndarray, precision: str) -> np.ndarray:
    if precision in ("fp16", "fp16sr"):
        return x.astype(np.float16).astype(np.float32)
    if precision in ("bf16", "bf16sr"):
        return bf16(x).astype(np.float32)
    return x.astype(np.float32)


def rows_of(tab: np.ndarray, row: int) -> list:
    c, first = int(tab[row, 0]), int(tab[row, 1])
    return [row] + list(range(first, first + c - 1))


def spread(F: np.ndarray, tab: np.ndarray, grp: np.ndarray) -> None:
    for row in grp:
        for r in rows_of(tab, int(row))[1:]:
            F[r] = F[row]


def merge(F: np.ndarray, tab: np.ndarray, grp: np.ndarray, precision: str) -> None:
    """In place on a float32 array holding storage-type values."""
    for row in grp:
        rows = rows_of(tab, int(row))
        acc = F[rows[0]].astype(np.float32).copy()
        for r in rows[1:]:
            acc = (acc + F[r]).astype(np.float32)
        mean = _round((acc / np.float32(len(rows))).astype(np.float32), precision)
        for r in rows:
            F[r] = mean
