"""GPU parity: the CUDA chain kernel (through the C ABI) against the CPU oracle.

Bar: final points of every chain match the FP64 oracle to <= 1e-10 relative
(to max(1, max|x|)) over the first 50 steps, with the same accepted/rejected
counts; emitted points satisfy lb - 1e-9 <= v <= ub + 1e-9.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import dense_S

pytestmark = pytest.mark.gpu

REL_TOL = 1e-10


def rel_err(a, b):
    return np.abs(a - b).max() / max(1.0, np.abs(b).max())


@pytest.fixture(scope="module")
def sampler(pkg, native, small_model, golden):
    s = pkg.Sampler(small_model, golden["warmup"])
    s.set_null_space(golden["N"])
    yield s
    s.close()


def test_centre_matches_oracle(sampler, oracle_mod, golden):
    c = sampler.centre()
    ref = oracle_mod.centre(golden["warmup"])
    assert np.abs(c - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("steps", [1, 10, 11, 50])
def test_points_match_oracle(sampler, oracle_mod, small_model, golden, steps):
    P = 64
    pts, st = sampler.sample(P, steps, seed=1234)
    ref, rst = oracle_mod.sample(small_model, golden["warmup"], golden["N"], 1234, P, steps)
    assert rel_err(pts, ref) <= REL_TOL
    assert st["accepted"] == rst["accepted"] == P * steps
    assert st["rejected"] == rst["rejected"]
    assert st["checks"] == rst["checks"]
    assert st["reprojections"] == rst["reprojections"]


@pytest.mark.parametrize("steps", [11, 50])
def test_residual_form_reprojection_matches_oracle(pkg, oracle_mod, small_model, golden, steps):
    """reproject_form = 2: the per-chain reprojection as x - S^T (S S^T)^+ S x (pseudo-inverse
    product in FP32 on the residual) gives the oracle's N (N^T x) points within the same tolerance;
    the fixture's %f-rounded warmups make every check reproject."""
    P = 64
    with pkg.Sampler(small_model, golden["warmup"], reproject_form=2) as s:
        s.set_null_space(golden["N"])
        pts, st = s.sample(P, steps, seed=1234)
    ref, rst = oracle_mod.sample(small_model, golden["warmup"], golden["N"], 1234, P, steps)
    assert st["reprojections"] == rst["reprojections"] > 0
    assert rel_err(pts, ref) <= REL_TOL
    assert st["accepted"] == rst["accepted"] == P * steps and st["rejected"] == rst["rejected"]


def test_golden_fixture_points(sampler, golden):
    pts, _ = sampler.sample(int(golden["chains"]), int(golden["steps"]), seed=int(golden["seed"]))
    assert rel_err(pts, golden["points"]) <= REL_TOL


def test_exact_ratio_mode_agrees(pkg, small_model, golden, oracle_mod):
    """Every candidate in FP64 (no FP32 brackets) gives the same points."""
    with pkg.Sampler(small_model, golden["warmup"], exact_ratio=1) as s:
        s.set_null_space(golden["N"])
        a, sa = s.sample(32, 50, seed=77)
    ref, _ = oracle_mod.sample(small_model, golden["warmup"], golden["N"], 77, 32, 50)
    assert rel_err(a, ref) <= REL_TOL
    assert sa["exact_evals"] >= sa["accepted"] * small_model.n_rxns // 2


def test_filter_evaluates_few_candidates(sampler):
    _, st = sampler.sample(64, 50, seed=5)
    # the FP32 brackets leave only a handful of coordinates per step for FP64
    assert st["exact_evals"] < 0.2 * st["accepted"] * sampler.n


@pytest.mark.parametrize("threads", [32, 64, 128])
def test_block_size_does_not_change_points(pkg, small_model, golden, oracle_mod, threads):
    with pkg.Sampler(small_model, golden["warmup"], threads_per_chain=threads) as s:
        s.set_null_space(golden["N"])
        a, _ = s.sample(16, 30, seed=9)
    ref, _ = oracle_mod.sample(small_model, golden["warmup"], golden["N"], 9, 16, 30)
    assert rel_err(a, ref) <= REL_TOL


def test_bitwise_repeatable(sampler):
    a, _ = sampler.sample(40, 25, seed=3)
    b, _ = sampler.sample(40, 25, seed=3)
    assert np.array_equal(a, b)


def test_chain_offset(sampler):
    a, _ = sampler.sample(20, 15, seed=3)
    b, _ = sampler.sample(8, 15, seed=3, chain_offset=12)
    assert np.array_equal(a[:, 12:20], b)


def test_zero_steps_gives_zeros(sampler):
    pts, st = sampler.sample(5, 0, seed=1)
    assert np.all(pts == 0.0) and st["accepted"] == 0


def test_zero_points(sampler):
    pts, st = sampler.sample(0, 10, seed=1)
    assert pts.shape == (sampler.n, 0) and st["accepted"] == 0


def test_bounds_hold(sampler, golden):
    pts, st = sampler.sample(256, 120, seed=21)
    lb, ub = golden["lb"][:, None], golden["ub"][:, None]
    assert (pts >= lb - 1e-9).all() and (pts <= ub + 1e-9).all()
    assert st["max_bound_violation"] <= 1e-9


def test_feasible_mode_emits_feasible_points(pkg, small_model, golden):
    S = dense_S(small_model)
    with pkg.Sampler(small_model, golden["warmup"], mode=pkg.MODE_FEASIBLE) as s:
        s.set_null_space(golden["N"])
        pts, st = s.sample(128, 37, seed=4)  # 37 steps: the last step is not a check step
    assert np.abs(S @ pts).max() <= 1e-8
    lb, ub = golden["lb"][:, None], golden["ub"][:, None]
    assert (pts >= lb - 1e-9).all() and (pts <= ub + 1e-9).all()
    assert st["max_residual"] <= 1e-8
    # the %f-rounded warmups were projected onto null(S) at set-up, so the
    # in-loop residual checks no longer find anything to reproject
    assert st["checks"] > 0 and st["reprojections"] == 0


def test_stuck_chain_reported(pkg):
    """Every warmup point equals the centre: every attempt is rejected and the
    chain stops after max_attempts instead of looping forever."""
    n = 3
    model = pkg.HostModel(n, 1, np.array([0, 0]), np.array([0, 1]), np.array([1.0, -1.0]), np.full(n, -1.0),
                          np.full(n, 1.0))
    with pkg.Sampler(model, np.zeros((n, 4)), max_attempts=50) as s:
        pts, st = s.sample(2, 5, seed=3)
    assert st["stuck_chains"] == 2 and st["accepted"] == 0 and st["rejected"] == 100
    assert np.all(pts == 0.0)


def test_matlab_centre_weights(pkg, small_model, golden, oracle_mod):
    with pkg.Sampler(small_model, golden["warmup"], centre_offset=1) as s:
        s.set_null_space(golden["N"])
        a, _ = s.sample(16, 40, seed=8)
    ref, _ = oracle_mod.sample(small_model, golden["warmup"], golden["N"], 8, 16, 40, centre_offset=1)
    assert rel_err(a, ref) <= REL_TOL


def test_infinite_bounds(pkg, oracle_mod):
    """Free reactions (lb = -inf / ub = +inf) take part in the ratio test as
    never-binding candidates."""
    rng = np.random.default_rng(0)
    n, m = 12, 4
    row = np.repeat(np.arange(m), 3)
    col = rng.choice(n, size=row.size)
    val = rng.choice([-1.0, 1.0, 2.0], size=row.size)
    lb = np.full(n, -10.0)
    ub = np.full(n, 10.0)
    lb[0] = -np.inf
    ub[1] = np.inf
    model = pkg.HostModel(n, m, row, col, val, lb, ub)
    S = dense_S(model)
    from oracle import reference_py
    N = reference_py.null_space_sts(S)
    warm = (N @ rng.standard_normal((N.shape[1], 30))) * 0.5
    warm = np.clip(warm, -5, 5)
    warm = N @ (N.T @ warm)
    with pkg.Sampler(model, warm) as s:
        s.set_null_space(N)
        a, _ = s.sample(16, 30, seed=2)
    ref, _ = oracle_mod.sample(model, warm, N, 2, 16, 30)
    assert rel_err(a, ref) <= REL_TOL


def test_gpu_null_space(pkg, small_model, golden):
    S = dense_S(small_model)
    with pkg.Sampler(small_model, golden["warmup"]) as s:
        N = s.null_space()
    assert N.shape == golden["N"].shape
    assert np.abs(S @ N).max() < 1e-10
    assert np.allclose(N.T @ N, np.eye(N.shape[1]), atol=1e-10)
    assert np.abs(N @ N.T - golden["N"] @ golden["N"].T).max() < 1e-10


def test_gpu_null_space_svd_of_s(pkg, small_model, golden):
    S = dense_S(small_model)
    with pkg.Sampler(small_model, golden["warmup"], null_space=pkg.NULL_SVD_S) as s:
        N = s.null_space()
    assert N.shape == golden["N"].shape
    assert np.abs(S @ N).max() < 1e-12
    assert np.abs(N @ N.T - golden["N"] @ golden["N"].T).max() < 1e-10


def test_gpu_null_space_holding_fixed_reactions(pkg, small_model, golden):
    """ACHR_NULL_FIXED: reactions with lb == ub get a unit row of their own, so the basis spans
    {v : S v = 0, v_i = 0 on them} and a reprojection leaves them where they are."""
    lb, ub = golden["lb"].copy(), golden["ub"].copy()
    fixed = [3, 17, 40]
    lb[fixed] = ub[fixed] = 0.0
    model = pkg.HostModel(small_model.n_rxns, small_model.n_mets, small_model.row, small_model.col,
                          small_model.val, lb, ub)
    S = dense_S(model)
    with pkg.Sampler(model, golden["warmup"], null_space=pkg.NULL_FIXED) as s:
        N = s.null_space()
    A = np.vstack([S, np.eye(S.shape[1])[fixed]])
    lam, V = np.linalg.eigh(A.T @ A)
    ref = V[:, lam < A.shape[1] * lam.max() * 2.2204e-16]
    assert N.shape == ref.shape
    assert np.abs(S @ N).max() < 1e-10 and np.abs(N[fixed]).max() < 1e-12
    assert np.allclose(N.T @ N, np.eye(N.shape[1]), atol=1e-10)
    assert np.abs(N @ N.T - ref @ ref.T).max() < 1e-10


def test_resume_in_segments_equals_one_run(sampler):
    """12 + 9 + 17 steps in three launches give the points of one 38-step launch."""
    torch = pytest.importorskip("torch")
    P, n = 48, sampler.n
    pts = torch.zeros((n, P), dtype=torch.float64, device="cuda")
    acc = torch.zeros((n, P), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    step = 0
    for seg, resume in ((12, False), (9, True), (17, True)):
        st = sampler.sample_resume(P, step, seg, resume, pts.data_ptr(), acc.data_ptr(), P, stream=stream, seed=21,
                                   chain_offset=5, with_stats=True)
        assert st["accepted"] == P * seg
        step += seg
    ref, _ = sampler.sample(P, 38, seed=21, chain_offset=5)
    assert np.array_equal(pts.cpu().numpy(), ref)


def test_resume_rejects_fresh_start_off_zero(sampler, pkg):
    with pytest.raises(pkg.AchrError):
        sampler.sample_resume(4, 3, 5, False, 16, 16, 4)
