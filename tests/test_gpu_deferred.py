"""GPU: sampling with the reference's reprojections deferred to the batched tensor-core pass.

reproject_form = 3 runs every chain to its next check step per launch of the
chain kernel, reprojects every chain whose check fired in one batched pass
(x <- x - S^T (S S^T)^+ S x: FP64 residual and update, three-BF16-split GEMM),
and clips and updates the centre at the start of the next launch, as the
reference does after its per-chain reprojection (ACHRcu/ACHRCuda.cu:325-350).
On the 72 x 95 fixture (%f warmups: every check reprojects) the points must
match the oracle's per-chain N (N^T x) to 1e-10 with equal counts, also when
the run ends on a check step (a launch that only finishes it), across the
chunk boundary of the segment buffers, for stuck chains and in FEASIBLE mode.
"""
from __future__ import annotations

import numpy as np
import pytest

from cases import refined_null_space, rel_err
from conftest import dense_S

pytestmark = pytest.mark.gpu

REL_TOL = 1e-10


@pytest.fixture(scope="module")
def deferred(pkg, native, small_model, golden):
    s = pkg.Sampler(small_model, golden["warmup"], reproject_form=3)
    s.set_null_space(golden["N"])
    yield s
    s.close()


@pytest.mark.parametrize("steps", [1, 9, 10, 11, 20, 21, 50])
def test_deferred_matches_oracle(deferred, oracle_mod, small_model, golden, steps):
    P = 64
    pts, st = deferred.sample(P, steps, seed=1234)
    ref, rst = oracle_mod.sample(small_model, golden["warmup"], golden["N"], 1234, P, steps)
    assert st["segments"] > 0
    for k in ("accepted", "rejected", "checks", "reprojections"):
        assert st[k] == rst[k], (k, st[k], rst[k])
    assert rst["reprojections"] > 0
    assert rel_err(pts, ref) <= REL_TOL


@pytest.mark.parametrize("period,steps", [(1, 12), (7, 30), (25, 60)])
def test_deferred_other_check_periods(pkg, oracle_mod, small_model, golden, period, steps):
    """With 25 steps between checks the points drift far enough from the null space that the
    oracle's N (N^T x) shows the basis's own 1e-15 row-space residue, and one chain's later
    steps amplify it past the bar: both sides use a basis refined to rounding level."""
    N = refined_null_space(dense_S(small_model), golden["N"])
    with pkg.Sampler(small_model, golden["warmup"], reproject_form=3, check_period=period) as s:
        s.set_null_space(N)
        pts, st = s.sample(32, steps, seed=5)
    ref, rst = oracle_mod.sample(small_model, golden["warmup"], N, 5, 32, steps, check_period=period)
    assert st["checks"] == rst["checks"] and st["reprojections"] == rst["reprojections"] > 0
    assert rel_err(pts, ref) <= REL_TOL


def test_deferred_equals_in_kernel_reprojection(pkg, deferred, small_model, golden):
    """Deferred and in-kernel FP64 reprojection agree to the parity tolerance."""
    a, sa = deferred.sample(48, 40, seed=11)
    with pkg.Sampler(small_model, golden["warmup"], reproject_form=1) as s:
        s.set_null_space(golden["N"])
        b, sb = s.sample(48, 40, seed=11)
    assert sb["segments"] == 0 and sa["reprojections"] == sb["reprojections"]
    assert rel_err(a, b) <= REL_TOL


def test_deferred_bitwise_repeatable(deferred):
    a, _ = deferred.sample(40, 33, seed=3)
    b, _ = deferred.sample(40, 33, seed=3)
    assert np.array_equal(a, b)


def test_deferred_chunk_boundary(deferred):
    """More chains than one sweep of the segment buffers holds (131072): the chains of the second
    sweep equal the same chains sampled on their own."""
    P = 131072 + 40
    a, st = deferred.sample(P, 3, seed=9)
    assert st["accepted"] == 3 * P
    b, _ = deferred.sample(40, 3, seed=9, chain_offset=131072)
    c, _ = deferred.sample(8, 3, seed=9)
    assert np.array_equal(a[:, 131072:], b)
    assert np.array_equal(a[:, :8], c)


def test_deferred_stuck_chain_reported(pkg):
    n = 3
    model = pkg.HostModel(n, 1, np.array([0, 0]), np.array([0, 1]), np.array([1.0, -1.0]), np.full(n, -1.0),
                          np.full(n, 1.0))
    with pkg.Sampler(model, np.zeros((n, 4)), max_attempts=50, reproject_form=3) as s:
        pts, st = s.sample(2, 25, seed=3)
    assert st["stuck_chains"] == 2 and st["accepted"] == 0 and st["rejected"] == 100
    assert np.all(pts == 0.0)


def test_deferred_feasible_mode(pkg, small_model, golden):
    S = dense_S(small_model)
    with pkg.Sampler(small_model, golden["warmup"], mode=pkg.MODE_FEASIBLE, reproject_form=3) as s:
        s.set_null_space(golden["N"])
        pts, st = s.sample(128, 37, seed=4)
    assert np.abs(S @ pts).max() <= 1e-8
    lb, ub = golden["lb"][:, None], golden["ub"][:, None]
    assert (pts >= lb - 1e-9).all() and (pts <= ub + 1e-9).all()


def test_deferred_resume_in_segments_equals_one_run(deferred):
    """achr_sample_resume with deferred reprojection: 12 + 9 + 17 steps (the second segment ends on
    a check step) give the points of one 38-step run, bit for bit."""
    torch = pytest.importorskip("torch")
    P, n = 48, deferred.n
    pts = torch.zeros((n, P), dtype=torch.float64, device="cuda")
    acc = torch.zeros((n, P), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    step = 0
    for seg, resume in ((12, False), (9, True), (17, True)):
        st = deferred.sample_resume(P, step, seg, resume, pts.data_ptr(), acc.data_ptr(), P, stream=stream, seed=21,
                                    chain_offset=5, with_stats=True)
        assert st["accepted"] == P * seg and st["segments"] > 0
        step += seg
    ref, _ = deferred.sample(P, 38, seed=21, chain_offset=5)
    assert np.array_equal(pts.cpu().numpy(), ref)
