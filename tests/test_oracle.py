"""CPU: the oracle pinned against the golden vectors (no GPU needed)."""
from __future__ import annotations

import json

import numpy as np
import pytest

from conftest import GOLDEN, dense_S
from oracle import reference_py


def _kat():
    return json.loads((GOLDEN / "philox_kat.json").read_text())


@pytest.mark.parametrize("case", range(3))
def test_philox_kat_c_oracle(oracle_mod, case):
    k = _kat()[case]
    out = oracle_mod.philox([int(x, 16) for x in k["ctr"]], [int(x, 16) for x in k["key"]])
    assert out == [int(x, 16) for x in k["out"]]


@pytest.mark.parametrize("case", range(3))
def test_philox_kat_python(case):
    k = _kat()[case]
    out = reference_py.philox4x32_10([int(x, 16) for x in k["ctr"]], [int(x, 16) for x in k["key"]])
    assert out == [int(x, 16) for x in k["out"]]


def test_stream_helpers_agree(oracle_mod):
    rng = np.random.default_rng(0)
    for _ in range(200):
        seed = int(rng.integers(0, 2**63))
        chain = int(rng.integers(0, 2**40))
        step = int(rng.integers(0, 2**31))
        att = int(rng.integers(0, 5))
        W = int(rng.integers(1, 100000))
        assert oracle_mod.warmup_index(seed, chain, step, att, W) == reference_py.warmup_index(seed, chain, step, att, W)
        u = oracle_mod.step_uniform(seed, chain, step)
        assert u == reference_py.step_uniform(seed, chain, step)
        assert 0.0 < u < 1.0


def test_warmup_index_in_range_and_uniform(oracle_mod):
    W = 7
    counts = np.zeros(W)
    for s in range(7000):
        r = oracle_mod.warmup_index(99, 3, s, 0, W)
        assert 0 <= r < W
        counts[r] += 1
    assert np.all(np.abs(counts - 1000) < 5 * np.sqrt(1000))


def test_c_oracle_matches_golden(oracle_mod, golden, small_model):
    g = golden
    pts, st = oracle_mod.sample(small_model, g["warmup"], g["N"], int(g["seed"]), int(g["chains"]), int(g["steps"]))
    ref = g["points"]
    assert np.abs(pts - ref).max() <= 1e-10 * max(1.0, np.abs(ref).max())
    assert st["rejected"] == int(g["rejected"])
    assert st["accepted"] == int(g["chains"]) * int(g["steps"])


def test_centre_matches_golden(oracle_mod, golden):
    c = oracle_mod.centre(golden["warmup"])
    assert np.allclose(c, golden["centre"], rtol=0, atol=1e-12)


def test_null_space_rule(golden, small_model):
    S = dense_S(small_model)
    N = reference_py.null_space_sts(S)
    assert N.shape == golden["N"].shape
    assert np.abs(S @ N).max() < 1e-10
    assert np.allclose(N.T @ N, np.eye(N.shape[1]), atol=1e-10)
    # same subspace as the committed basis
    P1 = N @ N.T
    P2 = golden["N"] @ golden["N"].T
    assert np.abs(P1 - P2).max() < 1e-10


def test_oracle_invariants(oracle_mod, golden, small_model):
    g = golden
    pts, _ = oracle_mod.sample(small_model, g["warmup"], g["N"], 11, 32, 25)
    lb, ub = g["lb"][:, None], g["ub"][:, None]
    assert (pts >= lb - 1e-9).all() and (pts <= ub + 1e-9).all()


def test_oracle_zero_steps_gives_zeros(oracle_mod, golden, small_model):
    """The reference clears the points before the launch (ACHRCuda.cu:739)."""
    pts, st = oracle_mod.sample(small_model, golden["warmup"], golden["N"], 1, 4, 0)
    assert np.all(pts == 0.0) and st["accepted"] == 0


def test_oracle_threads_do_not_change_results(oracle_mod, golden, small_model):
    g = golden
    a, _ = oracle_mod.sample(small_model, g["warmup"], g["N"], 5, 16, 20, threads=1)
    b, _ = oracle_mod.sample(small_model, g["warmup"], g["N"], 5, 16, 20, threads=4)
    assert np.array_equal(a, b)


def test_oracle_chain_offset(oracle_mod, golden, small_model):
    """Chain ids, not launch positions, key the random stream."""
    g = golden
    a, _ = oracle_mod.sample(small_model, g["warmup"], g["N"], 5, 10, 15)
    b, _ = oracle_mod.sample(small_model, g["warmup"], g["N"], 5, 4, 15, chain_offset=6)
    assert np.array_equal(a[:, 6:10], b)


def test_oracle_matlab_centre_weights_differ(oracle_mod, golden, small_model):
    g = golden
    a, _ = oracle_mod.sample(small_model, g["warmup"], g["N"], 5, 2, 15, centre_offset=0)
    b, _ = oracle_mod.sample(small_model, g["warmup"], g["N"], 5, 2, 15, centre_offset=1)
    assert not np.array_equal(a, b)


def test_oracle_degenerate_direction_is_rejected(oracle_mod, pkg):
    """All warmup points equal the centre: u = 0/0 for every step; the reference
    would read past thrust's end(); here every attempt is a rejection and the
    chain stops after max_attempts."""
    n = 3
    model = pkg.HostModel(n, 1, np.array([0, 0]), np.array([0, 1]), np.array([1.0, -1.0]), np.full(n, -1.0),
                          np.full(n, 1.0))
    warm = np.zeros((n, 4))
    N = np.array([[1, 0], [1, 0], [0, 1.0]]) / np.array([np.sqrt(2), 1.0])
    pts, st = oracle_mod.sample(model, warm, N, 3, 2, 5, max_attempts=50)
    assert st["stuck_chains"] == 2 and st["accepted"] == 0 and st["rejected"] == 100
    assert np.all(pts == 0.0)


def test_refined_null_space_is_orthogonal_to_rows_at_rounding_level(golden, small_model):
    from cases import refined_null_space

    S = dense_S(small_model)
    N = refined_null_space(S, golden["N"])
    assert N.shape == golden["N"].shape
    assert np.abs(S @ N).max() < 1.5e-15 < np.abs(S @ golden["N"]).max()
    assert np.abs(N.T @ N - np.eye(N.shape[1])).max() < 1e-14
    # the same subspace, the columns keeping their direction
    assert np.abs(N - golden["N"]).max() < 1e-13


def test_golden_fixture_is_well_conditioned_for_parity(oracle_mod, golden, small_model):
    """The %f fixture the deferred parity checks and smoke() use: a 1e-15 relative change of N moves
    the oracle's points by far less than the 1e-10 bar (chord points rounded to six decimals, by
    contrast, leave direction components near u_tol and move by ~1e-7)."""
    rng = np.random.default_rng(0)
    a, st = oracle_mod.sample(small_model, golden["warmup"], golden["N"], 7, 16, 30)
    b, _ = oracle_mod.sample(small_model, golden["warmup"], golden["N"] * (1 + 1e-15 * rng.standard_normal(golden["N"].shape)),
                             7, 16, 30)
    assert st["reprojections"] > 0
    assert np.abs(a - b).max() / max(1.0, np.abs(a).max()) < 1e-11
