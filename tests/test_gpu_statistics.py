"""GPU: statistical parity and feasibility of emitted samples.

The second correctness level for the sampler: on independent chains (disjoint
chain ids, so the two sample sets are independent), the per-flux means and
standard deviations of the CUDA sampler's points agree with the oracle's
within 3 standard errors, and every emitted sample satisfies
lb - 1e-9 <= v <= ub + 1e-9 and |S v|_inf <= 1e-8."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import dense_S

pytestmark = pytest.mark.gpu


def _z_scores(a, b):
    """z of the mean and of the standard deviation difference per flux (rows), chains in columns."""
    na, nb = a.shape[1], b.shape[1]
    ma, mb = a.mean(axis=1), b.mean(axis=1)
    va, vb = a.var(axis=1, ddof=1), b.var(axis=1, ddof=1)
    moving = (va > 1e-18) | (vb > 1e-18)
    se_m = np.sqrt(va / na + vb / nb)
    sa, sb = np.sqrt(va), np.sqrt(vb)
    # standard error of a sample standard deviation with the sample's own kurtosis
    def se_sd(x, s, nx):
        k = ((x - x.mean(axis=1, keepdims=True)) ** 4).mean(axis=1) / np.maximum(s ** 4, 1e-300)
        return s * np.sqrt(np.maximum(k - 1.0, 1e-12) / (4.0 * nx))
    se_s = np.sqrt(se_sd(a, sa, na) ** 2 + se_sd(b, sb, nb) ** 2)
    zm = np.where(moving, (ma - mb) / np.where(moving, se_m, 1.0), 0.0)
    zs = np.where(moving, (sa - sb) / np.where(moving, se_s, 1.0), 0.0)
    return zm, zs, moving


@pytest.mark.parametrize("steps", [30, 200])
def test_flux_moments_match_oracle_within_3_se(pkg, small_model, golden, oracle_mod, steps):
    P = 3000
    with pkg.Sampler(small_model, golden["warmup"]) as s:
        s.set_null_space(golden["N"])
        gpu, _ = s.sample(P, steps, seed=5)
    cpu, _ = oracle_mod.sample(small_model, golden["warmup"], golden["N"], 5, P, steps, chain_offset=10 ** 6)
    zm, zs, moving = _z_scores(gpu, cpu)
    k = int(moving.sum())
    # 3 standard errors per flux; over k fluxes a few |z| > 3 are expected by chance
    # (P(|z| > 3) = 0.27 %), so at most 2 may exceed 3 and none may exceed 4.5.
    assert k > 50
    assert np.abs(zm).max() <= 4.5 and int((np.abs(zm) > 3).sum()) <= 2, np.sort(np.abs(zm))[-5:]
    assert np.abs(zs).max() <= 4.5 and int((np.abs(zs) > 3).sum()) <= 2, np.sort(np.abs(zs))[-5:]


def test_every_emitted_sample_is_feasible(pkg, small_model, golden):
    """FEASIBLE mode: warmups projected once, every emitted point projected if needed.

    (In REFERENCE mode the warmup points are used as given; the fixture's are
    rounded to 6 decimals by %f, |S w| = 5e-6, so between the reference's
    10-step checks a point carries up to that residual, as the reference's
    would; bounds hold in both modes.)"""
    S = dense_S(small_model)
    lb, ub = golden["lb"][:, None], golden["ub"][:, None]
    with pkg.Sampler(small_model, golden["warmup"], mode=pkg.MODE_FEASIBLE) as s:
        s.set_null_space(golden["N"])
        for steps in (1, 9, 10, 11, 57, 300):
            pts, st = s.sample(500, steps, seed=steps)
            assert (pts >= lb - 1e-9).all() and (pts <= ub + 1e-9).all()
            assert np.abs(S @ pts).max() <= 1e-8, steps
            assert st["max_residual"] <= 1e-8 and st["max_bound_violation"] <= 1e-9
    with pkg.Sampler(small_model, golden["warmup"]) as s:
        s.set_null_space(golden["N"])
        pts, st = s.sample(500, 57, seed=3)
        assert (pts >= lb - 1e-9).all() and (pts <= ub + 1e-9).all()
