"""GPU: failure detection without a fault.  The chain kernel's wait for a staged
warmup column is bounded; wait_limit_ns = -L makes that wait watch a barrier
that nothing completes, so it runs out after L ns every time.  The launch
records the timeout, lets its real copy land, stops, and the call returns
ACHR_ERR_TIMEOUT; the GPU context stays usable."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TIMEOUT = 7  # ACHR_ERR_TIMEOUT


def test_wait_limit_reports_timeout_and_context_stays_usable(pkg, small_model, golden, oracle_mod):
    with pkg.Sampler(small_model, golden["warmup"], wait_limit_ns=-1_000_000) as s:  # 1 ms
        s.set_null_space(golden["N"])
        with pytest.raises(pkg.AchrError) as err:
            s.sample(32, 20, seed=3)
        assert err.value.status == TIMEOUT
        with pytest.raises(pkg.AchrError):  # and again: nothing is left in a broken state
            s.sample(32, 20, seed=3)
    with pkg.Sampler(small_model, golden["warmup"]) as s2:
        s2.set_null_space(golden["N"])
        pts, st = s2.sample(32, 20, seed=3)
    ref, _ = oracle_mod.sample(small_model, golden["warmup"], golden["N"], 3, 32, 20)
    assert st["accepted"] == 32 * 20
    assert np.abs(pts - ref).max() <= 1e-10 * max(1.0, np.abs(ref).max())


def test_generous_wait_limit_changes_nothing(pkg, small_model, golden):
    with pkg.Sampler(small_model, golden["warmup"], wait_limit_ns=500_000_000) as s:
        s.set_null_space(golden["N"])
        a, _ = s.sample(16, 15, seed=2)
    with pkg.Sampler(small_model, golden["warmup"]) as s:
        s.set_null_space(golden["N"])
        b, _ = s.sample(16, 15, seed=2)
    assert np.array_equal(a, b)


def test_batched_queue_reports_timeout_and_device_stays_usable(pkg, small_model, golden):
    """A model whose column waits run out inside the persistent work-queue launch: every CTA that
    takes one of its items records the timeout and leaves the queue, the launch ends, the batch
    call returns ACHR_ERR_TIMEOUT, and the next batch on the same device samples normally."""
    torch = pytest.importorskip("torch")
    bad = pkg.Sampler(small_model, golden["warmup"], wait_limit_ns=-1_000_000)
    good = pkg.Sampler(small_model, golden["warmup"])
    try:
        for s in (bad, good):
            s.set_null_space(golden["N"])
        P = [40, 40]
        outs = [torch.zeros((small_model.n_rxns, p), dtype=torch.float64, device="cuda") for p in P]
        stream = torch.cuda.current_stream().cuda_stream
        with pytest.raises(pkg.AchrError) as err:
            pkg.sample_batch([good, bad], P, 12, [o.data_ptr() for o in outs], P, stream=stream, seed=4)
        assert err.value.status == TIMEOUT
        st, _ = pkg.sample_batch([good], [40], 12, [outs[0].data_ptr()], [40], stream=stream, seed=4)
        ref, _ = good.sample(40, 12, seed=4)
        assert st["accepted"] == 40 * 12 and np.array_equal(outs[0].cpu().numpy(), ref)
    finally:
        bad.close()
        good.close()
