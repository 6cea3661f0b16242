"""GPU: ratio-test brackets formed in phase A against a separate bracket pass.

With bracket_pass = 0 the chain kernel forms the FP32 ratio-test brackets in
the same pass as the direction d, before the block has reduced ||d||, using a
candidacy-threshold interval bounded through the box (or the longest
hit-and-run direction); bracket_pass = 1 keeps the separate pass after the
norm.  Both must give bitwise identical points and the same counts: on the
72 x 95 fixture (several block sizes), on a 2200-reaction synthetic model (the
384 x 10 configuration), along hit-and-run directions, and for resumed chains
whose centre lies far outside the box, where every step exceeds the bound and
falls back to the separate pass."""
from __future__ import annotations

import importlib

import numpy as np
import pytest

from conftest import dense_S

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

SAME = ("accepted", "rejected", "checks", "reprojections", "stuck_chains")


def _pair(pkg, model, warm, N, P, T, seed, dirs=None, **kw):
    out = []
    for bp in (0, 1):
        with pkg.Sampler(model, warm, bracket_pass=bp, **kw) as s:
            if N is not None:
                s.set_null_space(N)
            if dirs is not None:
                s.set_directions(dirs)
            out.append(s.sample(P, T, seed=seed))
    (a, sa), (b, sb) = out
    assert np.array_equal(a, b)
    for k in SAME:
        assert sa[k] == sb[k], k
    return a, sa


@pytest.mark.parametrize("threads", [0, 32, 128])
def test_fixture_merged_equals_separate(pkg, small_model, golden, oracle_mod, threads):
    a, st = _pair(pkg, small_model, golden["warmup"], golden["N"], 64, 50, 11, threads_per_chain=threads)
    ref, rst = oracle_mod.sample(small_model, golden["warmup"], golden["N"], 11, 64, 50)
    assert np.abs(a - ref).max() <= 1e-10 * max(1.0, np.abs(ref).max())
    assert st["rejected"] == rst["rejected"]


def test_384_thread_model_merged_equals_separate(pkg):
    synth = importlib.import_module("achr_gb300.synthetic")
    spec = synth.SyntheticSpec(2200, 1540, 0.3, 100, 20.0, seed=21)
    row, col, val, lb, ub = synth.make_model(spec)
    model = pkg.HostModel(spec.n_rxns, spec.n_mets, row, col, val, lb, ub)
    warm = synth.interior_chord_warmup(dense_S(model), lb, ub, 2 * spec.n_rxns, seed=spec.seed)
    _, st = _pair(pkg, model, warm, None, 96, 40, 5, threads_per_chain=384)
    assert st["accepted"] == 96 * 40


def test_hit_and_run_merged_equals_separate(pkg, small_model, golden):
    rng = np.random.default_rng(4)
    dirs = golden["N"] @ rng.standard_normal((golden["N"].shape[1], 300))
    dirs[:, :20] *= 50.0  # a spread of lengths: the bound is the longest direction
    _pair(pkg, small_model, golden["warmup"], golden["N"], 64, 60, 8, dirs=dirs)


def test_centre_outside_box_falls_back(pkg, small_model, golden):
    """A resumed centre 40x the box: ||d|| exceeds the bound on every step, so
    the merged brackets are discarded and the separate pass runs."""
    n, P, step0, T = small_model.n_rxns, 32, 100, 30
    x0 = np.repeat(golden["warmup"].mean(axis=1, keepdims=True), P, axis=1)
    far = 40.0 * np.maximum(np.abs(golden["lb"]), np.abs(golden["ub"]))
    W = golden["warmup"].shape[1]
    A0 = np.repeat(((W + step0) * far)[:, None], P, axis=1)
    res = []
    for bp in (0, 1):
        with pkg.Sampler(small_model, golden["warmup"], bracket_pass=bp) as s:
            s.set_null_space(golden["N"])
            x = torch.from_numpy(np.ascontiguousarray(x0)).cuda()
            A = torch.from_numpy(np.ascontiguousarray(A0)).cuda()
            st = s.sample_resume(P, step0, T, True, x.data_ptr(), A.data_ptr(), P, seed=3, with_stats=True)
            torch.cuda.synchronize()
            res.append((x.cpu().numpy(), A.cpu().numpy(), st))
    assert np.array_equal(res[0][0], res[1][0]) and np.array_equal(res[0][1], res[1][1])
    for k in SAME:
        assert res[0][2][k] == res[1][2][k], k
    assert res[0][2]["accepted"] > 0
