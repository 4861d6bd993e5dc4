"""CPU checks of the MLP restatement that the GPU gradient test relies on: a silent
transposition planted in the restatement (the only square weight, W2, makes one possible)
must exceed the per-tensor bounds that the GPU test applies, so the same mistake in the GPU
backward pass would fail that test."""
import numpy as np
import pytest

from oracle import mlp_oracle as mo

D_IN, H, D_OUT = 131, 512, 128


def _case(rows, seed):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((rows, D_IN)).astype(np.float32) * 0.5
    T = rng.standard_normal((rows, D_OUT)).astype(np.float32) * 0.2
    params = np.concatenate([rng.standard_normal(H * D_IN) / np.sqrt(D_IN), 0.1 * rng.standard_normal(H),
                             rng.standard_normal(H * H) / np.sqrt(H), 0.1 * rng.standard_normal(H),
                             rng.standard_normal(D_OUT * H) / np.sqrt(H), 0.1 * rng.standard_normal(D_OUT)])
    return params.astype(np.float32), X, T


def test_bf16_rounding_matches_round_to_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 3.0e38, 1e-40], np.float64)
    got = mo.bf16(x)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: even mantissa -> 1; 1 + 3*2^-9 rounds up
    assert got[0] == 1.0 and got[1] == 1.0 and got[2] == 1.0 + 2 ** -7 and got[3] == -2.5
    assert np.isfinite(got[4]) and abs(got[4] - 3.0e38) <= 3.0e38 * 2 ** -8
    assert abs(got[5] - 1e-40) <= 2.0 ** -134  # subnormal: half of the 2^-133 step


@pytest.mark.parametrize("rows,seed", [(256, 1), (300, 2)])
def test_bounds_accept_bf16_restatement_and_are_tight(rows, seed):
    params, X, T = _case(rows, seed)
    _, g16, g64, bounds = mo.gradient_bounds(params, X, T, D_IN, H, D_OUT)
    for name, a, b in zip(mo.GRAD_NAMES, mo.unpack(g16, D_IN, H, D_OUT), mo.unpack(g64, D_IN, H, D_OUT)):
        assert mo.rel_err(a, b) <= bounds[name] <= 0.02, (name, bounds[name])


@pytest.mark.parametrize("mistake,caught", [("gW2_transposed", ["W2"]), ("dH1_uses_W2T", ["W1", "b1"])])
def test_planted_transposition_exceeds_the_bounds(mistake, caught):
    params, X, T = _case(256, 3)
    _, _, g64, bounds = mo.gradient_bounds(params, X, T, D_IN, H, D_OUT)
    _, bad = mo.forward_backward_bf16(params, X, T, D_IN, H, D_OUT, mistake=mistake)
    errs = {n: mo.rel_err(a, b) for n, a, b in zip(mo.GRAD_NAMES, mo.unpack(bad, D_IN, H, D_OUT),
                                                    mo.unpack(g64, D_IN, H, D_OUT))}
    for name in caught:
        assert errs[name] > 10 * bounds[name], (name, errs[name], bounds[name])
