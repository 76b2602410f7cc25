"""The radiance-cache oracle (oracle/nrc_ref.py) on its own: its manual
backpropagation equals finite differences of the loss, and the hash-grid
indexing follows the documented dense / hashed rule."""
import numpy as np

import nrc_ref as N


def _params(rng, log2_table):
    fan = np.repeat([np.sqrt(6 / 32)] + [np.sqrt(6 / 64)] * 5, [2048, 4096, 4096, 4096, 4096, 192])
    return rng.uniform(-1, 1, 18624) * fan, rng.uniform(-0.5, 0.5, 16 * (1 << log2_table) * 2)


def test_backprop_matches_finite_differences():
    rng = np.random.default_rng(0)
    lv = N.level_table(4, 1.3, 10)
    mlp, grid = _params(rng, 10)
    p = rng.random((24, 3)).astype(np.float32)
    t = rng.random((24, 4))
    loss, gm, gg = N.loss_and_grads(mlp, grid, p, t, lv, 10)
    y0, _ = N.forward(mlp, grid, p, lv, 10)
    eps = 1e-6
    for k in [0, 7, 2047, 2048, 5000, 12000, 18431, 18432, 18500, 18623]:
        m2 = mlp.copy()
        m2[k] += eps
        lp = N.surrogate_loss(m2, grid, p, t, lv, 10, y0)
        m2[k] -= 2 * eps
        lm = N.surrogate_loss(m2, grid, p, t, lv, 10, y0)
        assert abs(gm[k] - (lp - lm) / (2 * eps)) <= 1e-6 + 1e-5 * abs(gm[k]), k
    for k in np.nonzero(gg)[0][::97][:12]:
        g2 = grid.copy()
        g2[k] += eps
        lp = N.surrogate_loss(mlp, g2, p, t, lv, 10, y0)
        g2[k] -= 2 * eps
        lm = N.surrogate_loss(mlp, g2, p, t, lv, 10, y0)
        assert abs(gg[k] - (lp - lm) / (2 * eps)) <= 1e-8 + 1e-4 * abs(gg[k]), k
    assert loss > 0


def test_level_table_dense_then_hashed():
    lv = N.level_table(16, 1.447, 19)
    dense = [r for _, r in lv]
    assert dense[0] == 17 and all(r > 0 for r in dense[:4]) and dense[-1] == 0
    first_hashed = dense.index(0)
    assert all(r == 0 for r in dense[first_hashed:])
    assert all((r + 0) ** 3 <= 1 << 19 for r in dense[:first_hashed])


def test_corner_weights_partition_unity():
    rng = np.random.default_rng(1)
    lv = N.level_table(16, 1.447, 12)
    idx, w = N.encode_corners(rng.random((50, 3)).astype(np.float32), lv, 12)
    assert np.allclose(w.sum(axis=2), 1.0)
    assert idx.min() >= 0 and idx.max() < 16 * (1 << 12)
