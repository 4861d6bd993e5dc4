"""Seeded synthetic planted-low-rank rating matrices.

The reference measures on Netflix / Yahoo!Music / Hugewiki, which are not available here;
these generators produce matrices with the shapes, sizes and value distributions of the
benchmark configurations instead:

  c1  10,000 x 2,000, 1,000,000 ratings (90/10 split), Zipf(1.0) users and items,
      rank-16 planted factors ~ N(0, 0.25), r = clip(round(3.5 + p.q + N(0, 0.5)), 1, 5)
  c2  480,189 x 17,770, 99,072,112 train + 1,408,395 test, item Zipf exponent fitted so the
      heaviest item has ~230k ratings, user exponent fitted so the heaviest user has ~17k,
      rank-32 planted model, integer 1..5 with mean ~3.6, noise N(0, 0.8)
  c3  1,000,990 x 624,961, 252.8M train + 4.0M test, float ratings on 0..100, rank 48,
      noise with standard deviation 20, clipped
N(mu, v) denotes variance v.  User and item ids are drawn independently from their Zipf
laws over a seeded random relabelling (so popularity is not sorted by id); records come out
in draw order.  Duplicate (u, v) pairs are possible and kept, as independent observations.
Generation runs on torch (CPU or CUDA); only the host copy of the result reaches the
library.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Optional

import numpy as np
import torch

NODE_DTYPE = np.dtype([("u", "<i4"), ("v", "<i4"), ("r", "<f4")])


@dataclasses.dataclass
class PlantedSpec:
    m: int
    n: int
    nnz_train: int
    nnz_test: int
    rank: int
    user_s: float          # Zipf exponent of user ids (or <0: fit to top_user)
    item_s: float          # Zipf exponent of item ids (or <0: fit to top_item)
    factor_var: float      # variance of planted factor entries
    noise_std: float
    offset: float
    gain: float            # r = offset + gain * p.q + noise
    lo: float
    hi: float
    integer: bool
    top_user: int = 0
    top_item: int = 0


C1 = PlantedSpec(m=10_000, n=2_000, nnz_train=900_000, nnz_test=100_000, rank=16, user_s=1.0,
                 item_s=1.0, factor_var=0.25, noise_std=math.sqrt(0.5), offset=3.5, gain=1.0,
                 lo=1, hi=5, integer=True)
C2 = PlantedSpec(m=480_189, n=17_770, nnz_train=99_072_112, nnz_test=1_408_395, rank=32, user_s=-1,
                 item_s=-1, factor_var=1.0 / math.sqrt(32), noise_std=math.sqrt(0.8), offset=3.6,
                 gain=1.0, lo=1, hi=5, integer=True, top_user=17_000, top_item=230_000)
C3 = PlantedSpec(m=1_000_990, n=624_961, nnz_train=252_800_000, nnz_test=4_000_000, rank=48,
                 user_s=-1, item_s=-1, factor_var=1.0 / math.sqrt(48), noise_std=20.0, offset=50.0,
                 gain=20.0, lo=0, hi=100, integer=False, top_user=20_000, top_item=400_000)


def scaled(spec: PlantedSpec, frac: float) -> PlantedSpec:
    """Same family with users, items and ratings scaled by `frac` (for quick tests)."""
    f = dataclasses.replace(spec)
    f.m = max(16, int(spec.m * frac))
    f.n = max(16, int(spec.n * frac))
    f.nnz_train = max(64, int(spec.nnz_train * frac))
    f.nnz_test = max(16, int(spec.nnz_test * frac))
    f.top_user = int(spec.top_user * frac)
    f.top_item = int(spec.top_item * frac)
    return f


def fit_zipf_exponent(count: int, total: int, top: int) -> float:
    """Exponent s with total / H(count, s) ~= top (bisection on the harmonic sum)."""
    ranks = np.arange(1, count + 1, dtype=np.float64)

    def top_share(s: float) -> float:
        return total / np.sum(ranks ** (-s))

    lo, hi = 0.0, 3.0
    for _ in range(60):
        mid = 0.5 * (lo + hi)
        if top_share(mid) < top:
            lo = mid
        else:
            hi = mid
    return 0.5 * (lo + hi)


def _zipf_sampler(count: int, s: float, gen: torch.Generator, device) -> tuple:
    w = torch.arange(1, count + 1, dtype=torch.float64, device=device).pow(-s)
    cdf = torch.cumsum(w, 0)
    cdf /= cdf[-1].clone()
    relabel = torch.randperm(count, generator=gen, device=device).to(torch.int32)
    return cdf, relabel


def _draw(cdf, relabel, n: int, gen: torch.Generator, device) -> torch.Tensor:
    u = torch.rand(n, dtype=torch.float64, generator=gen, device=device)
    idx = torch.searchsorted(cdf, u).clamp_(max=len(cdf) - 1)
    return relabel[idx]


def generate(spec: PlantedSpec, seed: int = 0, device: Optional[str] = None,
             chunk: int = 1 << 24):
    """Returns (train, test) as numpy structured arrays of 12-byte records."""
    device = torch.device(device or ("cuda" if torch.cuda.is_available() else "cpu"))
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    total = spec.nnz_train + spec.nnz_test
    us = spec.user_s if spec.user_s >= 0 else fit_zipf_exponent(spec.m, total, spec.top_user)
    its = spec.item_s if spec.item_s >= 0 else fit_zipf_exponent(spec.n, total, spec.top_item)
    ucdf, urel = _zipf_sampler(spec.m, us, gen, device)
    icdf, irel = _zipf_sampler(spec.n, its, gen, device)
    sd = math.sqrt(spec.factor_var)
    P = torch.randn(spec.m, spec.rank, generator=gen, device=device) * sd
    Q = torch.randn(spec.n, spec.rank, generator=gen, device=device) * sd

    def block(count: int) -> np.ndarray:
        out = np.empty(count, dtype=NODE_DTYPE)
        for a in range(0, count, chunk):
            b = min(count, a + chunk)
            u = _draw(ucdf, urel, b - a, gen, device)
            v = _draw(icdf, irel, b - a, gen, device)
            dot = (P[u.long()] * Q[v.long()]).sum(1)
            r = spec.offset + spec.gain * dot
            r = r + torch.randn(b - a, generator=gen, device=device) * spec.noise_std
            if spec.integer:
                r = torch.round(r)
            r = r.clamp_(spec.lo, spec.hi)
            out["u"][a:b] = u.cpu().numpy()
            out["v"][a:b] = v.cpu().numpy()
            out["r"][a:b] = r.float().cpu().numpy()
        return out

    return block(spec.nnz_train), block(spec.nnz_test)


def generate_c1(seed: int = 0, device: Optional[str] = None):
    return generate(C1, seed, device)


def generate_growth(spec: PlantedSpec, new_users: int, new_frac: float, seed: int = 0,
                    device: Optional[str] = None, test_frac: float = 0.1, chunk: int = 1 << 24):
    """A base matrix plus growth from one planted model: users [0, spec.m) are the base users
    (Zipf, as `generate`), users [spec.m, spec.m + new_users) are new users drawn uniformly,
    whose ratings add `new_frac` of the base train count.  Returns
    (base_train, base_test, new_train, new_test); tests hold `test_frac` of each part."""
    device = torch.device(device or ("cuda" if torch.cuda.is_available() else "cpu"))
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    m_all = spec.m + new_users
    total = spec.nnz_train + spec.nnz_test
    us = spec.user_s if spec.user_s >= 0 else fit_zipf_exponent(spec.m, total, spec.top_user)
    its = spec.item_s if spec.item_s >= 0 else fit_zipf_exponent(spec.n, total, spec.top_item)
    ucdf, urel = _zipf_sampler(spec.m, us, gen, device)
    icdf, irel = _zipf_sampler(spec.n, its, gen, device)
    sd = math.sqrt(spec.factor_var)
    P = torch.randn(m_all, spec.rank, generator=gen, device=device) * sd
    Q = torch.randn(spec.n, spec.rank, generator=gen, device=device) * sd

    def block(count: int, new: bool) -> np.ndarray:
        out = np.empty(count, dtype=NODE_DTYPE)
        for a in range(0, count, chunk):
            b = min(count, a + chunk)
            if new:
                u = torch.randint(spec.m, m_all, (b - a,), generator=gen, device=device).to(torch.int32)
            else:
                u = _draw(ucdf, urel, b - a, gen, device)
            v = _draw(icdf, irel, b - a, gen, device)
            r = spec.offset + spec.gain * (P[u.long()] * Q[v.long()]).sum(1)
            r = r + torch.randn(b - a, generator=gen, device=device) * spec.noise_std
            if spec.integer:
                r = torch.round(r)
            r = r.clamp_(spec.lo, spec.hi)
            out["u"][a:b] = u.cpu().numpy()
            out["v"][a:b] = v.cpu().numpy()
            out["r"][a:b] = r.float().cpu().numpy()
        return out

    n_new = int(round(spec.nnz_train * new_frac))
    new_test = int(round(n_new * test_frac / (1 - test_frac)))
    return (block(spec.nnz_train, False), block(spec.nnz_test, False), block(n_new, True), block(new_test, True))
