"""The numpy NRC restatement's backward pass against finite differences (CPU)."""
import types

import numpy as np

from oracle import nrc_ref as R


def _tiny(seed=0):
    rng = np.random.default_rng(seed)
    info = types.SimpleNamespace(n_levels=3, resolution=[2, 3, 5], level_offset=[0, 27, 27 + 64],
                                 level_size=[27, 64, 64])
    grid = R.Grid(info, [0, 0, 0], [1, 1, 1], table_size=64)
    n_entries = 27 + 64 + 64
    table = rng.normal(size=n_entries * 2) * 0.3
    layers = 3
    w = np.zeros(2 * R.WIDTH * R.IN + R.OUT_PAD * R.IN)
    w[:] = rng.normal(size=w.size) * 0.2
    mlp = R.Mlp(w, layers)
    inp = rng.random((6, 13))
    inp[:, 3:6] = inp[:, 3:6] * 2 - 1
    t = rng.random((6, 3))
    return grid, table, mlp, inp, t, n_entries


def _loss(grid, table, mlp, inp, t):
    X0, _ = R.encode(grid, table, inp, rounding=False)
    y, _ = R.forward(mlp, X0, rounding=False)
    # gradient treats the denominator as a constant: use the same surrogate
    return y


def test_mlp_and_table_gradients_match_finite_differences():
    grid, table, mlp, inp, t, n_entries = _tiny()
    X0, cs = R.encode(grid, table, inp, rounding=False)
    y, acts = R.forward(mlp, X0, rounding=False)
    _, dy = R.loss_and_grad(y, t)
    gW, dX0 = R.backward(mlp, acts, dy, rounding=False)
    gT = R.table_grad(grid, cs, dX0, n_entries)
    den = y * y + 0.01   # held fixed (stop-gradient), as in the loss gradient

    def surrogate():
        X, _ = R.encode(grid, table, inp, rounding=False)
        yy, _ = R.forward(mlp, X, rounding=False)
        return ((yy - t) ** 2 / den).sum() / (inp.shape[0] * 3)

    eps = 1e-6
    rng = np.random.default_rng(1)
    for l in range(mlp.layers):
        rows = 3 if l + 1 == mlp.layers else R.WIDTH
        for _ in range(6):
            r, k = rng.integers(rows), rng.integers(R.IN)
            old = mlp.W[l][r, k]
            mlp.W[l][r, k] = old + eps
            fp = surrogate()
            mlp.W[l][r, k] = old - eps
            fm = surrogate()
            mlp.W[l][r, k] = old
            assert abs((fp - fm) / (2 * eps) - gW[l][r, k]) < 1e-6 + 1e-4 * abs(gW[l][r, k])
    touched = np.nonzero(gT)[0]
    for i in rng.choice(touched, 10, replace=False):
        old = table[i]
        table[i] = old + eps
        fp = surrogate()
        table[i] = old - eps
        fm = surrogate()
        table[i] = old
        assert abs((fp - fm) / (2 * eps) - gT[i]) < 1e-6 + 1e-4 * abs(gT[i])


def test_bf16_rounding_is_round_to_nearest_even():
    x = np.array([1.0, 1.00390625, 1.005859375, -2.5e-3, 3.0e38], np.float32)
    r = R.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0          # tie rounds to even
    assert r[2] == 1.0078125
    assert abs(r[3] - (-2.5e-3)) < 2e-5
