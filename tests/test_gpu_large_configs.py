"""GPU: the 512 x 12 and 512 x 15 chain-kernel configurations (models of
4097-7680 reactions) against the oracle.

The models are block-diagonal, three reactions and two metabolites per block
(S_b = [[1, -1, 0], [0, 1, -1]]), so the null space is known in closed form
(one column (1, 1, 1)/sqrt(3) per block) and the warmup points are random
combinations of it inside the box; no LP or SVD is needed at these sizes."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _block_model(pkg, blocks, seed):
    rng = np.random.default_rng(seed)
    b = np.arange(blocks)
    row = np.concatenate([2 * b, 2 * b, 2 * b + 1, 2 * b + 1])
    col = np.concatenate([3 * b, 3 * b + 1, 3 * b + 1, 3 * b + 2])
    val = np.concatenate([np.ones(blocks), -np.ones(blocks), np.ones(blocks), -np.ones(blocks)])
    n, m = 3 * blocks, 2 * blocks
    lb = -rng.uniform(5.0, 1000.0, n)
    ub = rng.uniform(5.0, 1000.0, n)
    model = pkg.HostModel(n, m, row, col, val, lb, ub)
    N = np.zeros((n, blocks))
    N[3 * b, b] = N[3 * b + 1, b] = N[3 * b + 2, b] = 1.0 / np.sqrt(3.0)
    # every block's common value t stays within [-5, 5], inside every bound
    warm = N @ (rng.uniform(-0.9, 0.9, (blocks, 64)) * 5.0 * np.sqrt(3.0))
    return model, N, warm


@pytest.mark.parametrize("blocks", [1700, 2400])  # n = 5100 (512 x 12) and 7200 (512 x 15)
def test_intermediate_lengths_match_oracle(pkg, oracle_mod, blocks):
    model, N, warm = _block_model(pkg, blocks, seed=blocks)
    P, T = 24, 30
    with pkg.Sampler(model, warm) as s:
        s.set_null_space(N)
        pts, st = s.sample(P, T, seed=31)
    ref, rst = oracle_mod.sample(model, warm, N, 31, P, T)
    assert np.abs(pts - ref).max() <= 1e-10 * max(1.0, np.abs(ref).max())
    assert st["accepted"] == rst["accepted"] == P * T
    assert st["rejected"] == rst["rejected"] and st["reprojections"] == rst["reprojections"]
    assert (pts >= model.lb[:, None] - 1e-9).all() and (pts <= model.ub[:, None] + 1e-9).all()
