"""GPU: batched sampling of several models in one CUDA-graph launch, and the autotuner.

achr_sample_batch groups the models by chain-kernel configuration and runs
each group as one persistent kernel whose CTAs take (model, chain tile) items
from a device work queue; every chain must come out exactly as the same chain
sampled on its own (same seed, chain id = the model's offset in the batch).
"""
from __future__ import annotations

import importlib

import numpy as np
import pytest

from conftest import dense_S

pytestmark = pytest.mark.gpu

REL_TOL = 1e-10


@pytest.fixture(scope="module")
def models(pkg, small_model, golden):
    synth = importlib.import_module("achr_gb300.synthetic")
    out = [(small_model, golden["warmup"], golden["N"])]
    for spec in (synth.SyntheticSpec(300, 210, 0.3, 30, 20.0, seed=11), synth.SyntheticSpec(40, 28, 0.25, 8, 10.0, seed=12)):
        row, col, val, lb, ub = synth.make_model(spec)
        m = pkg.HostModel(spec.n_rxns, spec.n_mets, row, col, val, lb, ub)
        S = dense_S(m)
        warm = synth.interior_chord_warmup(S, lb, ub, 2 * spec.n_rxns, seed=spec.seed)
        from oracle import reference_py
        out.append((m, warm, reference_py.null_space_sts(S)))
    return out


def test_batch_equals_individual_launches(pkg, models):
    torch = pytest.importorskip("torch")
    samplers = []
    for m, w, N in models:
        s = pkg.Sampler(m, w)
        s.set_null_space(N)
        samplers.append(s)
    P = [24, 40, 9]
    T = 35
    outs = [torch.zeros((s.n, p), dtype=torch.float64, device="cuda") for s, p in zip(samplers, P)]
    stream = torch.cuda.current_stream().cuda_stream
    st, ms = pkg.sample_batch(samplers, P, T, [o.data_ptr() for o in outs], P, stream=stream, seed=777)
    assert st["accepted"] == sum(P) * T and st["stuck_chains"] == 0
    assert 0.0 <= st["load_imbalance"] < 1.0 and st["graph_ms"] > 0 and len(ms) == 3
    off = 0
    for s, p, o in zip(samplers, P, outs):
        ref, _ = s.sample(p, T, seed=777, chain_offset=off)
        assert np.array_equal(o.cpu().numpy(), ref)
        off += p
    for s in samplers:
        s.close()


def test_batch_on_default_stream(pkg, models):
    torch = pytest.importorskip("torch")
    m, w, N = models[1]
    with pkg.Sampler(m, w) as s:
        s.set_null_space(N)
        o = torch.zeros((s.n, 10), dtype=torch.float64, device="cuda")
        st, _ = pkg.sample_batch([s], [10], 12, [o.data_ptr()], [10], stream=0, seed=5)
        ref, _ = s.sample(10, 12, seed=5)
        assert st["accepted"] == 120 and np.array_equal(o.cpu().numpy(), ref)


def test_autotune_picks_a_candidate_and_keeps_parity(pkg, models, oracle_mod):
    m, w, N = models[1]
    with pkg.Sampler(m, w) as s:
        s.set_null_space(N)
        t = s.autotune()
        assert t in (32, 64, 128, 256, 320, 384, 512)
        assert s.autotune() == t  # cached for this size on this device
        pts, st = s.sample(20, 30, seed=3)
    ref, rst = oracle_mod.sample(m, w, N, 3, 20, 30)
    assert np.abs(pts - ref).max() <= REL_TOL * max(1.0, np.abs(ref).max())
    assert st["accepted"] == rst["accepted"]


@pytest.fixture(scope="module")
def queue_models(pkg, models):
    """The three models above plus one of 1500 reactions (a fourth configuration, 256 x 8) and the
    72 x 95 fixture once more, so that one queue holds three models."""
    synth = importlib.import_module("achr_gb300.synthetic")
    from oracle import reference_py
    spec = synth.batch_spec(7, 1500)
    row, col, val, lb, ub = synth.make_model(spec)
    m = pkg.HostModel(spec.n_rxns, spec.n_mets, row, col, val, lb, ub)
    S = dense_S(m)
    warm = synth.interior_chord_warmup(S, lb, ub, 2 * spec.n_rxns, seed=spec.seed)
    return models + [(m, warm, reference_py.null_space_sts(S)), models[0]]


def test_batch_work_queue_many_tiles(pkg, queue_models):
    """Enough chains that the queues cut each model into tiles of several sizes, a model with no
    chains, two models sharing one configuration with a third: bitwise equal to separate runs."""
    torch = pytest.importorskip("torch")
    samplers = []
    for m, w, N in queue_models:
        s = pkg.Sampler(m, w)
        s.set_null_space(N)
        samplers.append(s)
    P = [3000, 700, 0, 450, 1234]
    T = 23
    outs = [torch.zeros((s.n, max(p, 1)), dtype=torch.float64, device="cuda") for s, p in zip(samplers, P)]
    stream = torch.cuda.current_stream().cuda_stream
    st, ms = pkg.sample_batch(samplers, P, T, [o.data_ptr() for o in outs], [max(p, 1) for p in P], stream=stream,
                              seed=4242)
    assert st["accepted"] == sum(P) * T and st["stuck_chains"] == 0
    assert 0.0 <= st["load_imbalance"] < 1.0 and ms[2] == 0.0 and min(ms[k] for k in (0, 1, 3, 4)) > 0.0
    off = 0
    for s, p, o in zip(samplers, P, outs):
        if p:
            ref, _ = s.sample(p, T, seed=4242, chain_offset=off)
            assert np.array_equal(o[:, :p].cpu().numpy(), ref)
        off += p
    for s in samplers:
        s.close()


def test_batch_tiles_do_not_change_the_points(pkg, queue_models):
    """The tile setting changes only how the queue cuts the chains: points stay bitwise equal; the
    batch autotuner keeps one of its candidates."""
    torch = pytest.importorskip("torch")
    samplers = []
    for m, w, N in queue_models[:3]:
        s = pkg.Sampler(m, w)
        s.set_null_space(N)
        samplers.append(s)
    P = [900, 333, 77]
    stream = torch.cuda.current_stream().cuda_stream
    outs = [torch.zeros((s.n, p), dtype=torch.float64, device="cuda") for s, p in zip(samplers, P)]
    ptrs = [o.data_ptr() for o in outs]
    saved = pkg.batch_tiles()
    try:
        got = []
        for tiles in (1, 16):
            pkg.set_batch_tiles(tiles)
            pkg.sample_batch(samplers, P, 17, ptrs, P, stream=stream, seed=31)
            got.append([o.cpu().numpy() for o in outs])
        for a, b in zip(*got):
            assert np.array_equal(a, b)
        best = pkg.autotune_batch(samplers, P, 5, ptrs, P, stream=stream, seed=1)
        assert best in (1, 2, 4, 8, 16) and pkg.batch_tiles() == best
        with pytest.raises(pkg.AchrError):
            pkg.set_batch_tiles(0)
    finally:
        pkg.set_batch_tiles(saved)
        for s in samplers:
            s.close()
