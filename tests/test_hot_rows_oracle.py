"""The CPU restatement of the copies of the most-rated rows on hand-worked cases."""
import numpy as np

from oracle import hot_rows_oracle as ho

NODE = np.dtype([("u", "<i4"), ("v", "<i4"), ("r", "<f4")])


def _rec(v, u=None):
    rec = np.zeros(len(v), NODE)
    rec["v"] = v
    rec["u"] = 0 if u is None else u
    return rec


def test_plan_and_assign_by_hand():
    # item counts 7, 1, 4, 0, 0, 8 with 3 ratings per copy -> copies 3, 1, 2, 1, 1, 3
    v = [0, 0, 0, 0, 0, 0, 0, 1, 2, 2, 2, 2, 5, 5, 5, 5, 5, 5, 5, 5]
    p = ho.plan(_rec(v), 1, 6, per_copy=3)
    np.testing.assert_array_equal(p["tab_n"][:, 0], [3, 1, 2, 1, 1, 3])
    np.testing.assert_array_equal(p["tab_n"][:, 1], [6, 1, 8, 3, 4, 9])  # first extra row, or the row
    np.testing.assert_array_equal(p["grp_n"], [0, 2, 5])
    assert p["n_rows"] == 11
    out = ho.assign(_rec(v), p)
    # rating i of a row with c copies goes to copy i mod c (copy 0 is the row itself)
    np.testing.assert_array_equal(out["v"], [0, 6, 7, 0, 6, 7, 0, 1, 2, 8, 2, 8, 5, 9, 10, 5, 9, 10, 5, 9])
    # the single user row (20 ratings) is capped at max_copies
    p2 = ho.plan(_rec(v), 1, 6, per_copy=3, max_copies=4)
    assert p2["tab_m"][0, 0] == 4 and p2["m_rows"] == 4


def test_copies_share_the_ratings_evenly():
    rng = np.random.default_rng(0)
    v = rng.integers(0, 50, 100_000) ** 2 % 50  # skewed
    p = ho.plan(_rec(v), 1, 50, per_copy=500)
    out = ho.assign(_rec(v), p)
    extra = np.arange(50, p["n_rows"])
    assert set(np.unique(out["v"])) >= set(extra)  # every extra row is used
    for row in p["grp_n"]:
        rows = ho.rows_of(p["tab_n"], row)
        cnt = np.array([(out["v"] == r).sum() for r in rows])
        # positions are random, so each copy's share is binomial around count / copies
        assert cnt.max() - cnt.min() <= 8 * np.sqrt(cnt.mean()) + 2


def test_merge_rounds_the_fp32_mean():
    F = np.array([[1.0, 0.1], [2.0, 0.2], [4.0, 0.3], [9.0, 9.0]], np.float32)
    tab = np.array([[3, 1], [1, 1], [1, 2], [1, 3]], np.int32)
    G = F.copy()
    ho.merge(G, tab, np.array([0], np.int32), "fp16")
    mean = np.float32(np.float32(np.float32(1.0 + 2.0) + 4.0) / np.float32(3))
    assert G[0, 0] == np.float32(np.float16(mean)) and (G[:3, 0] == G[0, 0]).all()
    assert G[3, 0] == 9.0  # a row without copies is untouched
    H = F.copy()
    ho.merge(H, tab, np.array([0], np.int32), "fp32")
    assert H[0, 0] == mean
    S = F.copy()
    ho.spread(S, tab, np.array([0], np.int32))
    assert (S[1] == F[0]).all() and (S[2] == F[0]).all()
